"""
The persistent batched path (tvbg_batch_run): instances of different
connectomes, node counts, ring placements and step counts in one batch --
run eagerly and as one captured CUDA graph -- give bit-identical results to
running each connectome's sweep on its own (same kernels, same arithmetic),
and agree with the oracle.
"""

import numpy as np
import pytest

from conftest import rel_err

import pyoracle as orc
from tvb_hpc import model, coupling, scheme, network, engine

pytestmark = pytest.mark.gpu


def mixed_sets(blocked='auto', seed=0):
    out = []
    m = model.MPR()
    cf = coupling.Linear(m)
    for k, (N, dens, I, speed) in enumerate([(68, 0.3, 6, 4.0), (84, 0.3, 5, 6.0),
                                              (150, 0.15, 3, 2.0), (300, 0.08, 2, 4.0)]):
        w, ln = network.synthetic_connectome(N, dens, seed=seed + k)
        conn = network.Connectivity.from_dense(w, ln)
        rng = np.random.default_rng(seed + 10 + k)
        x0 = np.stack([rng.uniform(0.05, 0.3, (I, N)), rng.uniform(-1.5, -0.5, (I, N))], -1)
        eta = rng.uniform(-6, -4, (I, N, 1))
        s = engine.InstanceSet(m, cf, scheme.EulerMaryuyamaStep(0.1), conn, dt=0.1,
                               couplings=np.logspace(-2, -0.5, I), speeds=speed,
                               state0=x0.astype(np.float32), nparam=eta.astype(np.float32),
                               seed=4242 + k, blocked=blocked)
        out.append((s, x0.astype(np.float32), rng.integers(100, 700, I)))
    return out


@pytest.mark.parametrize('graph', [False, True])
def test_batch_equals_separate_sweeps(cuda, graph):
    torch = cuda
    sets = mixed_sets()
    batch = engine.Batch([s for s, _, _ in sets], [n for _, _, n in sets])
    assert len(batch.launches) >= 2          # several CTA widths
    if graph:
        batch.capture()
    batch.run()
    # separate per-set runs through the same kernels, one set at a time
    sets2 = mixed_sets()
    for (a, x0, n), (b, _, _) in zip(sets, sets2):
        solo = engine.Batch([b], [n])
        solo.run()
        assert np.array_equal(a.state.cpu().numpy(), b.state.cpu().numpy())
        assert np.array_equal(a.ring.cpu().numpy(), b.ring.cpu().numpy())


def test_batch_matches_oracle(cuda):
    sets = mixed_sets()
    batch = engine.Batch([s for s, _, _ in sets], [n for _, _, n in sets])
    batch.run()
    for s, x0, n in sets:
        for b in range(s.n):
            one = orc.run_sweep_like(_Sub(s, b), x0[b:b + 1], int(n[b]))
            assert rel_err(s.state.cpu().numpy()[b], one['state'][0]) < 1e-4


class _Sub:
    "View of one instance of an InstanceSet for the oracle wrapper."

    def __init__(self, s, b):
        self._s, self._b = s, b
        self.n = 1
        for k in ('model_id', 'cfun_id', 'row_np', 'col_np', 'w_np', 'dt', 'flags', 'sigma',
                  'consts', 'cf_b', 'cf_p', 'seed', 'trace_every', 'trace_len', 'trace_nobs',
                  'bold_period', 'bold_len', 'N', 'ns', 'delay_tables'):
            setattr(self, k, getattr(s, k))
        self.lognh = s.lognh[b:b + 1]
        self.tab_of = s.tab_of[b:b + 1]
        self.order_flags = s.order_flags[b:b + 1]
        self.cf_a = s.cf_a[b:b + 1]
        self.inst_ids = s.inst_ids[b:b + 1]
        self.nparam = s.nparam[b:b + 1]

    def bold_obs(self):
        return self._s.bold_obs()
