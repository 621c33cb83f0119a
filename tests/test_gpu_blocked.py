"""
The time-blocked kernel (K steps per block, padded ring rows) against the
oracle: same step, same Philox stream, so the same 1e-4 relative tolerance.
Covers both block lengths, gather widths, CTA widths, ring placements,
BOLD (lagged one block in the kernel), trace, chunked runs (bit-exact with
one long run) and ragged step counts (not a multiple of K).
"""

import numpy as np
import pytest

from conftest import rel_err

import pyoracle as orc
from tvb_hpc import model, coupling, scheme, network, engine, _native as nat

pytestmark = pytest.mark.gpu

TOL = 1e-4


def make(model_name='G2DO', cfun_name='Diff', I=8, N=84, speeds=(5.0, 20.0), noise=True,
         seed=3, dt=0.1, **kw):
    w, ln = network.synthetic_connectome(N, 0.3, seed=seed)
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
    sw = engine.Sweep(m, cf, scm, conn, dt=dt, couplings=np.logspace(-2, 0, I),
                      speeds=np.resize(np.asarray(speeds, np.float32), I),
                      state0=x0.astype(np.float32), nparam=nparam, seed=777, **kw)
    return sw, x0.astype(np.float32)


def check(sw, x0, nsteps):
    assert np.all(sw.block_k > 0)
    sw.run(nsteps)
    ref = orc.run_sweep_like(sw, x0, nsteps)
    assert rel_err(sw.state.cpu().numpy(), ref['state']) < TOL
    for b in range(sw.n):
        got, r = sw.ring_plain(b), ref['rings'][b]
        np.testing.assert_array_equal(got == 0, r == 0)
        assert rel_err(got, r) < TOL
    return ref


@pytest.mark.parametrize('tpn', [2, 4, 8])
@pytest.mark.parametrize('warps', [3, 8])
def test_blocked_g2do_diff_noise(cuda, tpn, warps):
    sw, x0 = make(tpn=tpn, warps=warps)
    assert set(sw.block_k) == {4, 8}      # speed 20: d_min = 5 -> K = 4
    check(sw, x0, 603)


def test_blocked_k4_and_global_ring(cuda):
    "speed 20 -> d_min = 5 -> K = 4; speed 1 -> 2048-slot ring in global memory."
    sw, x0 = make(speeds=(20.0, 1.0), tpn=4)
    assert set(sw.block_k) == {4, 8}
    flags = sw.build_table(1)['flags']
    assert np.any(flags & nat.F_SMEM_RING) and not np.all(flags & nat.F_SMEM_RING)
    check(sw, x0, 501)


@pytest.mark.parametrize('model_name,cfun_name', [('MPR', 'Linear'), ('Linear', 'Diff'),
                                                  ('G2DO', 'Sigmoidal'), ('Linear', 'Linear'),
                                                  ('Generic2dOscillator', 'Diff')])
def test_blocked_other_pairs(cuda, model_name, cfun_name):
    sw, x0 = make(model_name, cfun_name, I=4, tpn=4)
    check(sw, x0, 400)


def test_blocked_bold_and_trace(cuda):
    sw, x0 = make(I=4, speeds=(6.0, ), tpn=4, bold_period=100, bold_len=11, trace_every=37,
                  trace_len=32)
    ref = check(sw, x0, 1150)
    assert rel_err(sw.bold_out.cpu().numpy(), ref['bold_out']) < TOL
    assert rel_err(sw.bold.cpu().numpy(), ref['bold']) < TOL
    assert rel_err(sw.trace.cpu().numpy(), ref['trace']) < TOL


def test_blocked_bold_large_deviations(cuda):
    """Balloon driven hard (|f-1|, |v-1| > 0.15): the kernel's exact-form
    branch against the FP64 oracle."""
    # dt 1 ms: 3000 steps = 3 s of balloon time, input held at 2.5
    sw, x0 = make('Linear', 'Linear', I=3, noise=False, speeds=(1.0, ), tpn=4, dt=1.0,
                  bold_period=100, bold_len=30)
    x0[:] = 2.5
    sw.state.copy_(sw.torch.from_numpy(x0).cuda())
    sw.nparam.zero_()
    sw.cf_a[:] = 0.0
    sw.run(3000)
    ref = orc.run_sweep_like(sw, x0, 3000, real='f64')
    assert np.abs(ref['bold'][:, 1:]).max() > 0.15
    assert rel_err(sw.bold_out.cpu().numpy(), ref['bold_out']) < TOL


def test_blocked_chunks_bit_exact(cuda):
    a, x0 = make(I=4, tpn=4, bold_period=50, bold_len=20)
    b, _ = make(I=4, tpn=4, bold_period=50, bold_len=20)
    a.run(1000)
    for n in (333, 1, 250, 416):
        b.run(n)
    for t_a, t_b in ((a.state, b.state), (a.ring, b.ring), (a.bold_out, b.bold_out)):
        assert np.array_equal(t_a.cpu().numpy(), t_b.cpu().numpy(), equal_nan=True)


def test_blocked_matches_per_step_kernel(cuda):
    a, x0 = make(I=4, tpn=4, blocked=True)
    b, _ = make(I=4, tpn=4, blocked=False)
    a.run(500)
    b.run(500)
    assert rel_err(a.state.cpu().numpy(), b.state.cpu().numpy()) < TOL
