"""
Stochastic runs, statistically: the engine's Euler-Maruyama noise is
compared with the oracle on *independent* seeds (different Philox keys, so
no stream is shared) over an ensemble, and with the analytic stationary
variance of the Ornstein-Uhlenbeck process.  Tolerances follow from the
ensemble sizes (stated beside each check).
"""

import numpy as np
import pytest

import pyoracle as orc
from tvb_hpc import model, coupling, scheme, network, engine, groups

pytestmark = pytest.mark.gpu


def test_ou_stationary_variance(cuda):
    """Linear model x' = lam x + sigma dW, no coupling: stationary variance
    sigma^2 / (2 |lam|).  68 nodes x 64 instances x 8 seeds = 34816
    samples of the final state: relative standard error of a variance
    estimate sqrt(2 / n) = 0.8 %; tolerance 4 %."""
    N, I, dt, lam = 68, 64, 0.1, -0.3
    w, ln = network.synthetic_connectome(N, 0.3, seed=0)
    conn = network.Connectivity.from_dense(w, ln)
    m = model.Linear()
    sig = float(m.engine_spec()[2][0])
    xs = []
    for seed in range(8):
        gs = groups.GroupSet(m, coupling.Linear(m), scheme.EulerMaryuyamaStep(dt), conn, dt=dt,
                             couplings=np.zeros(I, np.float32), speeds=np.full(I, 4.0, np.float32),
                             nparam=np.float32(lam), seed=1000 + seed)
        gs.run(5000)     # 500 ms = 150 relaxation times
        xs.append(gs.state.cpu().numpy().ravel())
    x = np.concatenate(xs)
    # discrete-time stationary variance of x' = (1 + lam dt) x + sqrt(dt) sigma z
    var_exact = dt * sig ** 2 / (1 - (1 + lam * dt) ** 2)
    assert abs(x.mean()) < 4 * np.sqrt(var_exact / x.size)
    assert abs(x.var() / var_exact - 1) < 0.04


def test_ensemble_statistics_match_the_oracle_on_other_seeds(cuda):
    """Coupled noisy 2-D oscillators (G2DOsc + Diff, sigma 1e-3 raised to
    2e-2): ensemble mean, variance and FC of the V traces from the engine
    (seeds 0..7) and the FP32 oracle (seeds 100..107).  Tolerances: 0.1 of
    the ensemble standard deviation for the mean, 10 % for the variance,
    0.03 in the mean absolute FC difference (each side averages 8 x 16
    instances of 40 trace rows)."""
    N, I, dt, steps = 68, 16, 0.1, 4000
    w, ln = network.synthetic_connectome(N, 0.3, seed=2)
    conn = network.Connectivity.from_dense(w, ln)
    m = model.Generic2dOscillator()
    m.diffs = (0.02, 0.02)          # engine_spec reads the noise amplitudes from diffs
    cf = coupling.Diff(m)
    G = np.full(I, 0.1, np.float32)
    rng = np.random.default_rng(3)
    x0 = rng.uniform(-0.5, 0.5, (I, N, 2)).astype(np.float32)
    kw = dict(dt=dt, couplings=G, speeds=np.full(I, 4.0, np.float32), state0=x0,
              trace_every=100, trace_len=41, trace_nobs=1)

    def stats(traces):
        tr = np.concatenate(traces)[:, 1:, :, 0]           # [runs, rows, N], drop t = 0
        fc = np.mean([np.corrcoef(t.T) for t in tr], axis=0)
        return tr.mean(), tr.var(), fc

    gpu, ref = [], []
    for s in range(8):
        gs = groups.GroupSet(m, cf, scheme.EulerMaryuyamaStep(dt), conn, seed=s, **kw)
        gs.run(steps)
        gpu.append(gs.trace.cpu().numpy())
        sw = engine.InstanceSet(m, cf, scheme.EulerMaryuyamaStep(dt), conn, seed=100 + s,
                                blocked=False, **kw)
        out = orc.run_sweep_like(sw, x0, steps)
        ref.append(out['trace'])
    mg, vg, fg = stats(gpu)
    mr, vr, fr = stats(ref)
    assert abs(mg - mr) < 0.1 * np.sqrt(vr)
    assert abs(vg / vr - 1) < 0.10
    off = ~np.eye(N, dtype=bool)
    assert np.abs(fg - fr)[off].mean() < 0.03
