"""
The lane-interleaved group kernel (tvbg_group_run) against the oracle: the
same CUDA-order step and Philox streams as the per-instance kernels, so the
same 1e-4 relative tolerance.  Covers both block lengths, partial groups,
every separable model/coupling pair, BOLD and trace, per-lane step counts,
clusters of 2/4/8 CTAs, several nodes per thread, chunked runs (bit-exact
with one long run) and agreement with the per-step kernel.
"""

import numpy as np
import pytest

from conftest import rel_err, circ_rel_err

import pyoracle as orc
from tvb_hpc import model, coupling, scheme, network, engine, groups

pytestmark = pytest.mark.gpu

TOL = 1e-4


def setup(model_name='Generic2dOscillator', cfun_name='Diff', I=20, N=84, density=0.3,
          speeds=(5.0, 20.0), noise=True, seed=3, dt=0.1):
    w, ln = network.synthetic_connectome(N, density, seed=seed)
    conn = network.Connectivity.from_dense(w, ln)
    rng = np.random.default_rng(seed + 1)
    m = getattr(model, model_name)()
    if model_name == 'MPR':
        x0 = np.stack([rng.uniform(0.05, 0.3, (I, N)), rng.uniform(-1.5, -0.5, (I, N))], -1)
        nparam = rng.uniform(-6, -4, (I, N, 1)).astype(np.float32)
    elif model_name == 'Linear':
        x0 = rng.uniform(-0.5, 0.5, (I, N, m.nsvar))
        nparam = np.float32(-0.3)
    else:
        x0 = rng.uniform(-0.5, 0.5, (I, N, m.nsvar))
        nparam = None
    cf = getattr(coupling, cfun_name)(m)
    scm = scheme.EulerMaryuyamaStep(dt) if noise else scheme.EulerStep(dt)
    args = (m, cf, scm, conn)
    kw = dict(dt=dt, couplings=np.logspace(-2, 0, I).astype(np.float32),
              speeds=np.resize(np.asarray(speeds, np.float32), I), state0=x0.astype(np.float32),
              nparam=nparam, seed=777)
    return args, kw, x0.astype(np.float32)


def make(model_name='Generic2dOscillator', cfun_name='Diff', gkw=None, **kw):
    args, skw, x0 = setup(model_name, cfun_name, **kw)
    gs = groups.GroupSet(*args, **skw, **(gkw or {}))
    return gs, x0


def check(gs, x0, nsteps):
    gs.run(nsteps)
    ref = orc.run_groups_like(gs, x0, nsteps)
    assert rel_err(gs.state.cpu().numpy(), ref['state']) < TOL
    for b in range(gs.n):
        got, r = gs.ring_plain(b), ref['rings'][b]
        np.testing.assert_array_equal(got == 0, r == 0)
        assert rel_err(got, r) < TOL
    return ref


def test_groups_g2dosc_diff_noise(cuda):
    gs, x0 = make()
    assert set(gs.block_k) == {4, 8}          # speed 20: d_min = 5 -> K = 4
    assert gs.n_groups == 4                    # 10 + 10 instances -> 8 + 2 per speed
    check(gs, x0, 403)


@pytest.mark.parametrize('model_name,cfun_name', [('MPR', 'Linear'), ('Linear', 'Diff'),
                                                  ('G2DO', 'Sigmoidal'), ('Linear', 'Linear'),
                                                  ('MPR', 'Diff')])
def test_groups_other_pairs(cuda, model_name, cfun_name):
    gs, x0 = make(model_name, cfun_name, I=9, speeds=(4.0, ))
    check(gs, x0, 300)


def test_groups_bold_and_trace(cuda):
    gs, x0 = make(I=11, speeds=(6.0, ), gkw=dict(bold_period=100, bold_len=11, trace_every=37,
                                                  trace_len=32))
    ref = check(gs, x0, 1150)
    assert rel_err(gs.bold_out.cpu().numpy(), ref['bold_out']) < TOL
    assert rel_err(gs.trace.cpu().numpy(), ref['trace']) < TOL


def test_groups_ragged_steps(cuda):
    "Lanes of one group stop at their own step counts."
    rng = np.random.default_rng(0)
    steps = rng.integers(100, 420, 13)
    gs, x0 = make('MPR', 'Linear', I=13, speeds=(4.0, ), gkw=dict(nsteps=steps))
    gs.run(steps)
    ref = orc.run_groups_like(gs, x0, steps)
    assert rel_err(gs.state.cpu().numpy(), ref['state']) < TOL


@pytest.mark.parametrize('N,threads,cluster', [(300, None, None), (300, 1024, 2),
                                               (998, None, None), (84, 128, 1), (84, 96, 2),
                                               (84, 64, 4), (192, None, 8)])
def test_groups_clusters_and_multinode_threads(cuda, N, threads, cluster):
    gs, x0 = make('MPR', 'Linear', I=9, N=N, density=0.05 if N > 500 else 0.15, speeds=(4.0, ),
                  gkw=dict(threads=threads, cluster=cluster))
    if cluster:
        assert gs.cluster == cluster
    check(gs, x0, 200)


def test_groups_chunks_bit_exact(cuda):
    a, x0 = make(I=9, speeds=(6.0, ), gkw=dict(bold_period=50, bold_len=20))
    b, _ = make(I=9, speeds=(6.0, ), gkw=dict(bold_period=50, bold_len=20))
    a.run(1000)
    for n in (333, 1, 250, 416):
        b.run(n)
    for t_a, t_b in ((a.state, b.state), (a.ring, b.ring), (a.bold_out, b.bold_out)):
        assert np.array_equal(t_a.cpu().numpy(), t_b.cpu().numpy(), equal_nan=True)


def test_groups_match_per_step_kernel(cuda):
    args, kw, x0 = setup(I=12)
    a = groups.GroupSet(*args, **kw)
    b = engine.Sweep(*args, **kw, blocked=False, tpn=2)
    a.run(500)
    b.run(500)
    assert rel_err(a.state.cpu().numpy(), b.state.cpu().numpy()) < TOL


def test_group_batch_graph(cuda):
    """Sets of different N in one graph launch: each instance's result is
    the one it gets alone."""
    sets, solo, steps = [], [], []
    for N, I in ((68, 10), (192, 9), (400, 3)):
        rng = np.random.default_rng(N)
        st = rng.integers(50, 300, I)
        args, kw, x0 = setup('MPR', 'Linear', I=I, N=N, density=0.1, speeds=(4.0, ))
        sets.append(groups.GroupSet(*args, **kw, nsteps=st))
        solo.append(groups.GroupSet(*args, **kw, nsteps=st))
        steps.append(st)
    gb = groups.GroupBatch(sets, steps)
    gb.capture()
    gb.run()
    for s, o, st in zip(sets, solo, steps):
        o.run(st)
        assert np.array_equal(s.state.cpu().numpy(), o.state.cpu().numpy())


def kuramoto_setup(I=20, N=68, speeds=(4.0, 10.0), seed=11, dt=0.1):
    w, ln = network.synthetic_connectome(N, 0.3, seed=seed)
    conn = network.Connectivity.from_dense(w, ln)
    rng = np.random.default_rng(seed)
    m = model.Kuramoto()
    cf = coupling.Kuramoto(m)
    x0 = rng.uniform(0, 2 * np.pi, (I, N, 1)).astype(np.float32)
    omega = rng.normal(2 * np.pi * 0.01, 0.001, (I, N, 1)).astype(np.float32)
    kw = dict(dt=dt, couplings=np.logspace(-2, 1, I).astype(np.float32),
              speeds=np.resize(np.asarray(speeds, np.float32), I), state0=x0, nparam=omega, seed=5)
    return (m, cf, scheme.EulerStep(dt), conn), kw, x0


def test_groups_kuramoto_sin_cos_ring(cuda):
    """The Kuramoto coupling on the group kernel: the ring keeps sin and cos
    of the phase and the coupling sum is cos(x_i) S_sin - sin(x_i) S_cos,
    algebraically the reference's sum of sin(x_j - x_i)."""
    args, kw, x0 = kuramoto_setup()
    gs = groups.GroupSet(*args, **kw)
    assert gs.channels == 2 and set(gs.block_k) == {8}
    gs.run(1000)
    ref = orc.run_groups_like(gs, x0, 1000)
    assert circ_rel_err(gs.state.cpu().numpy(), ref['state']) < TOL
    for b in range(gs.n):
        got, r = gs.ring_plain(b), ref['rings'][b]
        np.testing.assert_array_equal(got == 0, r == 0)
        assert circ_rel_err(got, r) < TOL


def test_groups_kuramoto_matches_per_instance_kernel_and_chunks(cuda):
    args, kw, x0 = kuramoto_setup(I=10, speeds=(4.0, ))
    a = groups.GroupSet(*args, **kw)
    b = engine.Sweep(*args, **kw, tpn=2)
    c = groups.GroupSet(*args, **kw)
    a.run(600)
    b.run(600)
    for n in (250, 1, 349):
        c.run(n)
    assert circ_rel_err(a.state.cpu().numpy(), b.state.cpu().numpy()) < TOL
    assert np.array_equal(a.state.cpu().numpy(), c.state.cpu().numpy())
