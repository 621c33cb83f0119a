"""
The pipelined group kernel (tvbg_group_run with tpn = TVBG_GROUP_PIPELINED):
two thread teams per CTA, the coupling gather of block b + 1 (transposed:
each lane loads one ring position for the 8 instances) overlapping the
steps of block b.  The same additions in the same order as the plain group
kernel, so every test but the oracle one demands bit-identical results:
every separable model/coupling pair and the Kuramoto sin/cos ring, BOLD and
trace, per-lane step counts, chunked runs, clusters of up to 16 CTAs,
priority-banded batches and the batch tuner's plans.
"""

import numpy as np
import pytest

from conftest import rel_err

import pyoracle as orc
from tvb_hpc import autotune, groups, _native as nat
from test_gpu_groups import setup, kuramoto_setup

pytestmark = pytest.mark.gpu

TOL = 1e-4


def pair(args, kw, gkw=None):
    a = groups.GroupSet(*args, **kw, **(gkw or {}))
    b = groups.GroupSet(*args, **kw, **(gkw or {}))
    return a, b


def pipelined_shape(gs, cluster=None):
    shapes = [s for s in autotune.group_shapes(gs.N, pipelined=True) if s[3] == nat.GROUP_PIPELINED]
    if cluster is not None:
        shapes = [s for s in shapes if s[1] == cluster]
    return shapes[0]


def same(a, b):
    for x, y in ((a.state, b.state), (a.ring, b.ring)):
        assert np.array_equal(x.cpu().numpy(), y.cpu().numpy())
    for x, y in ((a.bold_out, b.bold_out), (a.trace, b.trace)):
        if x is not None:
            assert np.array_equal(x.cpu().numpy(), y.cpu().numpy(), equal_nan=True)


@pytest.mark.parametrize('model_name,cfun_name', [('MPR', 'Linear'), ('MPR', 'Diff'),
                                                  ('Generic2dOscillator', 'Diff'),
                                                  ('G2DO', 'Sigmoidal'), ('Linear', 'Linear')])
def test_pipelined_matches_plain(cuda, model_name, cfun_name):
    args, kw, _ = setup(model_name, cfun_name, I=13, N=84, speeds=(4.0, 6.0))
    a, b = pair(args, kw)
    assert b.can_pipeline
    b.set_shape(*pipelined_shape(b))
    a.run(417)
    b.run(417)
    b.status.check()
    same(a, b)


def test_pipelined_shape_with_short_delay_tables(cuda):
    """Speeds whose delays are too short for the pipelined kernel (d_min =
    5 at 20 mm/ms) keep the plain kernel in their own launches while the
    others pipeline; the whole set equals the plain run bit for bit."""
    args, kw, _ = setup(I=20, speeds=(4.0, 20.0, 6.0))
    a, b = pair(args, kw)
    assert b.can_pipeline and not b.pipe_tab.all()
    b.set_shape(*pipelined_shape(b))
    launches, _ = b.prepare(300)
    assert {cfg.tpn for *_, cfg in launches} == {1, nat.GROUP_PIPELINED}
    a.run(300)
    b.launch(launches)
    b.advance(np.full(b.n_groups, 300))
    b.torch.cuda.synchronize()
    b.status.check()
    same(a, b)


def test_pipelined_kuramoto_sin_cos(cuda):
    args, kw, _ = kuramoto_setup(I=12, speeds=(4.0, ))
    a, b = pair(args, kw)
    b.set_shape(*pipelined_shape(b))
    a.run(600)
    b.run(600)
    same(a, b)


def test_pipelined_bold_trace_ragged_chunks(cuda):
    rng = np.random.default_rng(1)
    steps = rng.integers(300, 900, 11)
    args, kw, _ = setup(I=11, speeds=(6.0, ))
    gkw = dict(bold_period=100, bold_len=11, trace_every=37, trace_len=32, nsteps=steps)
    a, b = pair(args, kw, gkw)
    b.set_shape(*pipelined_shape(b, cluster=3))
    a.run(steps)
    for part in (np.minimum(steps, 250), np.minimum(np.maximum(steps - 250, 0), 1),
                 np.maximum(steps - 251, 0)):
        b.run(part)
    same(a, b)


@pytest.mark.parametrize('N,cluster', [(998, 16), (400, 12), (192, 4), (68, 2)])
def test_pipelined_clusters_vs_oracle(cuda, N, cluster):
    args, kw, x0 = setup('MPR', 'Linear', I=9, N=N, density=0.03 if N > 500 else 0.1,
                         speeds=(4.0, ))
    gs = groups.GroupSet(*args, **kw)
    gs.set_shape(*pipelined_shape(gs, cluster))
    assert gs.cluster == cluster and gs.tpn == nat.GROUP_PIPELINED
    gs.run(240)
    gs.status.check()
    ref = orc.run_groups_like(gs, x0, 240)
    assert rel_err(gs.state.cpu().numpy(), ref['state']) < TOL


def test_pipelined_rejects_short_delays(cuda):
    """Delays shorter than 2K - 1 steps: the host refuses the shape, and a
    table that claims otherwise is refused by the kernel (status, no run)."""
    args, kw, _ = setup('MPR', 'Linear', I=8, speeds=(20.0, ))   # d_min = 5
    gs = groups.GroupSet(*args, **kw)
    assert not gs.can_pipeline
    with pytest.raises(ValueError):
        gs.set_shape(*pipelined_shape(gs))
    gs.can_pipeline = True       # bypass the host checks: the kernel checks dmin itself
    gs.pipe_tab[:] = True
    gs.set_shape(*pipelined_shape(gs))
    x = gs.state.clone()
    gs.run(64, check=False)
    gs.torch.cuda.synchronize()
    with pytest.raises(RuntimeError):
        gs.status.check()
    assert np.array_equal(gs.state.cpu().numpy(), x.cpu().numpy())


def test_banded_batch_matches_solo(cuda):
    """Mixed shapes and priority bands in one graph: each instance's result
    is the one it gets alone on the plain kernel."""
    sets, solo, steps, shapes = [], [], [], []
    for N, I, cl in ((68, 10, 2), (192, 9, 6), (400, 3, 16)):
        rng = np.random.default_rng(N)
        st = rng.integers(50, 300, I)
        args, kw, _ = setup('MPR', 'Linear', I=I, N=N, density=0.1, speeds=(4.0, ))
        sets.append(groups.GroupSet(*args, **kw, nsteps=st))
        solo.append(groups.GroupSet(*args, **kw, nsteps=st))
        steps.append(st)
        shapes.append(pipelined_shape(sets[-1], cl) if N != 192 else (256, 6, 0, 1))
    gb = groups.GroupBatch(sets, steps, shapes=shapes, step_ms=[0.01, 0.02, 0.03])
    assert gb.n_launches > len(sets)      # bands split launches
    gb.capture()
    gb.run()
    for s, o, st in zip(sets, solo, steps):
        o.run(st)
        assert np.array_equal(s.state.cpu().numpy(), o.state.cpu().numpy())


def test_batch_tuner_plan_is_exact(cuda):
    sets, steps, x0s = [], [], []
    for N, I in ((68, 16), (400, 8)):
        rng = np.random.default_rng(N + 1)
        st = rng.integers(200, 2000, I)
        args, kw, x0 = setup('MPR', 'Linear', I=I, N=N, density=0.1, speeds=(4.0, ))
        sets.append(groups.GroupSet(*args, **kw, nsteps=st))
        steps.append(st)
        x0s.append(sets[-1].state.clone())
    ref = [groups.GroupSet(*setup('MPR', 'Linear', I=s.n, N=s.N, density=0.1,
                                  speeds=(4.0, ))[0],
                           **setup('MPR', 'Linear', I=s.n, N=s.N, density=0.1,
                                   speeds=(4.0, ))[1], nsteps=st) for s, st in zip(sets, steps)]
    tb = groups.GroupBatch(sets, steps, shapes='tune')
    tun = tb.tuning
    assert len(tun['shapes']) == 2 and tun['trials']
    for s, x0 in zip(sets, x0s):       # tuning leaves the device state as it was
        assert np.array_equal(s.state.cpu().numpy(), x0.cpu().numpy())
    tb.run()
    for s, r, st in zip(sets, ref, steps):
        r.run(st)
        assert np.array_equal(s.state.cpu().numpy(), r.state.cpu().numpy())


def test_prepare_segments_tables(cuda):
    """prepare_segments builds one table and sets t0 and the step counts of
    each segment in bulk: byte for byte the tables of build_table per
    segment (13 instances: one group with idle lanes; two delay tables)."""
    args, kw, _ = setup('MPR', 'Linear', I=13, N=84, speeds=(4.0, 6.0))
    gs = groups.GroupSet(*args, **kw)
    gs.set_shape(*pipelined_shape(gs))
    segs = [(0, 30), (30, 30), (60, 17), (77, 0)]
    gs.prepare_segments(segs)
    G = gs.n_groups
    got = gs._segments_keep.cpu().numpy().view(nat.GROUP_DTYPE).reshape(len(segs), G)
    for s, (t0, n) in enumerate(segs):
        gs.t[:] = t0
        ref, _ = gs.build_table(n)
        assert got[s].tobytes() == ref.tobytes(), s
