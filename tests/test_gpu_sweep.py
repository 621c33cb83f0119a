"""
GPU parity of the step kernel against the CPU oracle (same seeded inputs).

Tolerances: deterministic runs within 1e-4 relative state
error of the FP32 restatement over 1000 steps (circular distance for
Kuramoto phases); the error against the FP64 oracle is reported.  Stochastic
runs use the same Philox stream as the oracle, so they are compared the same
way.  Ring addressing is checked by comparing the whole unskewed ring, slot
by slot, with the oracle's plain ring.
"""

import numpy as np
import pytest

from conftest import circ_rel_err, rel_err

import pyoracle as orc
from tvb_hpc import model, coupling, scheme, network, engine, _native as nat

pytestmark = pytest.mark.gpu

TOL = 1e-4


def kuramoto68(I=32, N=68, seed=0, speed=4.0):
    w, ln = network.synthetic_connectome(N, 0.3, seed=seed)
    conn = network.Connectivity.from_dense(w, ln)
    rng = np.random.default_rng(1)
    theta0 = rng.uniform(0, 2 * np.pi, (I, N, 1)).astype(np.float32)
    omega = rng.normal(2 * np.pi * 0.01, 0.001, (I, N, 1)).astype(np.float32)
    G = np.logspace(-2, 1, I).astype(np.float32)
    return conn, theta0, omega, G


def kuramoto_sweep(conn, theta0, omega, G, speed=4.0, **kw):
    osc = model.Kuramoto()
    return engine.Sweep(osc, coupling.Kuramoto(osc), scheme.EulerStep(0.1), conn, dt=0.1,
                        couplings=G, speeds=speed, state0=theta0, nparam=omega, **kw)


def compare_rings(sw, ref, circ=False):
    errs = []
    for b in range(sw.n):
        got = sw.ring_plain(b)
        r = ref['rings'][b]
        assert got.shape == r.shape
        # never-written slots are zero in both: same addressing
        np.testing.assert_array_equal(got == 0, r == 0)
        errs.append(circ_rel_err(got, r) if circ else rel_err(got, r))
    return max(errs)


@pytest.mark.parametrize('tpn', [1, 2, 4, 8])
def test_kuramoto68_parity(cuda, tpn):
    conn, theta0, omega, G = kuramoto68()
    sw = kuramoto_sweep(conn, theta0, omega, G, tpn=tpn)
    assert np.all(sw.build_table(1)['flags'] & nat.F_SMEM_RING)  # 68 x 512 ring fits
    sw.run(1000)
    ref = orc.run_sweep_like(sw, theta0, 1000)
    got = sw.state.cpu().numpy()
    assert circ_rel_err(got, ref['state']) < TOL
    assert compare_rings(sw, ref, circ=True) < TOL
    ref64 = orc.run_sweep_like(sw, theta0, 1000, real='f64')
    err64 = circ_rel_err(got, ref64['state'])
    print('kuramoto N=68 tpn=%d: rel err vs f32 oracle %.2e, vs f64 oracle %.2e'
          % (tpn, circ_rel_err(got, ref['state']), err64))
    assert err64 < 1e-3


def test_global_ring_equals_smem_ring(cuda):
    conn, theta0, omega, G = kuramoto68(I=8)
    a = kuramoto_sweep(conn, theta0, omega, G, tpn=2)
    b = kuramoto_sweep(conn, theta0, omega, G, tpn=2)
    a.run(300)
    launches = b.prepare(300)
    tab = b.build_table(300, smem_allowed=False)
    dev = cuda.from_numpy(tab.view(np.uint8).copy()).cuda()
    b.launch([(dev, b.n, 0, 0)], 2)
    cuda.cuda.synchronize()
    b.status.check()
    del launches
    assert np.array_equal(a.state.cpu().numpy(), b.state.cpu().numpy())
    assert np.array_equal(a.ring.cpu().numpy(), b.ring.cpu().numpy())


def test_chunked_runs_are_bit_exact(cuda):
    conn, theta0, omega, G = kuramoto68(I=8)
    a = kuramoto_sweep(conn, theta0, omega, G, tpn=4)
    b = kuramoto_sweep(conn, theta0, omega, G, tpn=4)
    a.run(1000)
    for n in (250, 250, 333, 167):
        b.run(n)
    assert np.array_equal(a.state.cpu().numpy(), b.state.cpu().numpy())
    assert np.array_equal(a.ring.cpu().numpy(), b.ring.cpu().numpy())


def g2do_set(I=12, N=84, speeds=(1.0, 5.0, 20.0), nsteps=0, **kw):
    w, ln = network.synthetic_connectome(N, 0.3, seed=3)
    conn = network.Connectivity.from_dense(w, ln)
    rng = np.random.default_rng(4)
    x0 = rng.uniform(-0.5, 0.5, (I, N, 2)).astype(np.float32)
    G = np.logspace(-3, 0, I).astype(np.float32)
    sp = np.resize(np.asarray(speeds, np.float32), I)
    m = model.G2DO()
    kw.setdefault('blocked', False)
    sw = engine.Sweep(m, coupling.Diff(m), scheme.EulerMaryuyamaStep(0.1), conn, dt=0.1,
                      couplings=G, speeds=sp, state0=x0, seed=1234567, **kw)
    return sw, x0


@pytest.mark.parametrize('tpn', [1, 4])
def test_g2do_diff_noise_parity(cuda, tpn):
    "G2DO + Diff coupling + Euler-Maruyama with Philox noise (the dense grid's model)."
    sw, x0 = g2do_set(tpn=tpn)
    assert len(set(sw.lognh)) == 3   # rings of 2048, 512 and 128 slots
    flags = sw.build_table(1)['flags']
    assert not np.all(flags & nat.F_SMEM_RING) and np.any(flags & nat.F_SMEM_RING)
    sw.run(600)
    ref = orc.run_sweep_like(sw, x0, 600)
    got = sw.state.cpu().numpy()
    assert rel_err(got, ref['state']) < TOL
    assert compare_rings(sw, ref) < TOL
    ref64 = orc.run_sweep_like(sw, x0, 600, real='f64')
    print('g2do noise: rel err vs f32 %.2e, vs f64 %.2e'
          % (rel_err(got, ref['state']), rel_err(got, ref64['state'])))


def test_generic2d_oscillator_parity(cuda):
    "The CUDA-DSL form of the 2-D oscillator, per-step kernel."
    N, I = 84, 6
    w, ln = network.synthetic_connectome(N, 0.3, seed=12)
    conn = network.Connectivity.from_dense(w, ln)
    x0 = np.random.default_rng(13).uniform(-0.5, 0.5, (I, N, 2)).astype(np.float32)
    m = model.Generic2dOscillator()
    sw = engine.Sweep(m, coupling.Diff(m), scheme.EulerMaryuyamaStep(0.1), conn, dt=0.1,
                      couplings=np.logspace(-3, 0, I), speeds=[2.0, 9.0, 20.0] * 2, state0=x0,
                      seed=5, tpn=2, blocked=False, bold_period=50, bold_len=20)
    sw.run(1000)
    ref = orc.run_sweep_like(sw, x0, 1000)
    assert rel_err(sw.state.cpu().numpy(), ref['state']) < TOL
    assert rel_err(sw.bold_out.cpu().numpy(), ref['bold_out']) < TOL


def test_mpr_linear_noise_parity(cuda):
    "Montbrio-Pazo-Roxin with linear coupling on r (the uneven batch's and the adjoint fit's model)."
    N, I = 84, 8
    w, ln = network.synthetic_connectome(N, 0.3, seed=5)
    conn = network.Connectivity.from_dense(w, ln)
    rng = np.random.default_rng(6)
    x0 = np.stack([rng.uniform(0.05, 0.3, (I, N)), rng.uniform(-1.5, -0.5, (I, N))], -1)
    x0 = x0.astype(np.float32)
    eta = rng.uniform(-6, -4, (I, N, 1)).astype(np.float32)
    m = model.MPR()
    cf = coupling.Linear(m)
    sw = engine.Sweep(m, cf, scheme.EulerMaryuyamaStep(0.1), conn, dt=0.1,
                      couplings=np.linspace(0.1, 1.0, I), speeds=4.0, state0=x0, nparam=eta,
                      seed=99, tpn=2, blocked=False)
    sw.run(800)
    ref = orc.run_sweep_like(sw, x0, 800)
    got = sw.state.cpu().numpy()
    assert rel_err(got, ref['state']) < TOL
    assert compare_rings(sw, ref) < TOL


def test_bold_and_trace_parity(cuda):
    sw, x0 = g2do_set(I=6, speeds=(5.0, ), bold_period=100, bold_len=12, trace_every=50,
                      trace_len=24, tpn=2)
    sw.run(1200)
    ref = orc.run_sweep_like(sw, x0, 1200)
    got_b = sw.bold_out.cpu().numpy()
    assert np.isfinite(got_b).all()
    assert rel_err(got_b, ref['bold_out']) < TOL
    assert rel_err(sw.trace.cpu().numpy(), ref['trace']) < TOL
    assert rel_err(sw.bold.cpu().numpy(), ref['bold']) < TOL
    ref64 = orc.run_sweep_like(sw, x0, 1200, real='f64')
    print('bold: rel err vs f32 %.2e, vs f64 %.2e'
          % (rel_err(got_b, ref['bold_out']), rel_err(got_b, ref64['bold_out'])))


@pytest.mark.parametrize('speed', [100.0, 4.0])
def test_tracka_order_parity(cuda, speed):
    """Track-A step order, including zero delays (speed 100 mm/ms, dt 1 ms,
    trunc).  400 steps: at speed 4 this system amplifies a 1-ulp change of
    the initial state to 4e-6 after 300 steps and 1.5e-4 after 700 (oracle
    runs), so a longer run would test its conditioning, not the kernel."""
    N, I = 40, 6
    w, ln = network.synthetic_connectome(N, 0.3, seed=8)
    conn = network.Connectivity.from_dense(w, ln)
    rng = np.random.default_rng(9)
    theta0 = rng.uniform(0, 2 * np.pi, (I, N, 1)).astype(np.float32)
    osc = model.Kuramoto()
    sw = engine.Sweep(osc, coupling.Kuramoto(osc), scheme.EulerStep(1.0), conn, dt=1.0,
                      couplings=np.linspace(0.5, 3, I), speeds=speed, state0=theta0,
                      nparam=np.float32(0.0628), rounding='trunc', order='tracka', tpn=2)
    if speed == 100.0:
        assert sw.delay_tables[0].min() == 0
        assert sw.build_table(1)['flags'][0] & nat.F_MIDSYNC
    sw.run(400)
    ref = orc.run_sweep_like(sw, theta0, 400)
    assert circ_rel_err(sw.state.cpu().numpy(), ref['state']) < TOL
    assert compare_rings(sw, ref, circ=True) < TOL


def test_dsl_mode_matches_oracle(cuda):
    """CUDA-DSL semantics (truncated f32 DSL delays, fmod wrap, slot-0 state
    0.001) against the oracle, which is pinned to the reference kernel."""
    N, I = 24, 4
    w, ln = network.synthetic_connectome(N, 0.3, seed=7)
    conn = network.Connectivity.from_dense(w, ln)
    omega = np.float32(60.0 * 2.0 * np.float32(3.141593) / 1e3)
    x0 = np.full((I, N, 1), 0.001, np.float32)
    osc = model.Kuramoto()
    sw = engine.Sweep(osc, coupling.Kuramoto(osc), scheme.EulerStep(0.1), conn, dt=0.1,
                      couplings=[0.5, 1.0, 2.0, 4.0], speeds=[2.0, 3.0, 4.0, 5.0], state0=x0,
                      nparam=omega, rounding='dsl', flags=nat.F_WRAP_FMOD, tpn=1)
    sw.run(300)
    ref = orc.run_sweep_like(sw, x0, 300)
    assert circ_rel_err(sw.state.cpu().numpy(), ref['state']) < TOL
    assert compare_rings(sw, ref, circ=True) < TOL


def test_zero_in_degree_and_ragged_sizes(cuda):
    "Nodes without in-edges, N not a multiple of 32, a single instance."
    N = 45
    w, ln = network.synthetic_connectome(N, 0.2, seed=11)
    w[:, :5] = 0
    w[:5, :] = 0
    ln[w == 0] = 0
    conn = network.Connectivity.from_dense(w, ln)
    assert np.any(conn.in_degree == 0)
    x0 = np.random.default_rng(0).uniform(-1, 1, (1, N, 1)).astype(np.float32)
    m = model.Linear()
    sw = engine.Sweep(m, coupling.Diff(m), scheme.EulerStep(0.1), conn, dt=0.1, couplings=[0.3],
                      speeds=7.0, state0=x0, nparam=np.float32(-0.5), tpn=8, blocked=False)
    sw.run(400)
    ref = orc.run_sweep_like(sw, x0, 400)
    assert rel_err(sw.state.cpu().numpy(), ref['state']) < TOL
