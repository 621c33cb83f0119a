"""
The reduced Wong-Wang and Jansen-Rit models (tvb_hpc/model.py:209-247) on
the GPU against the oracle: per-instance kernels with every coupling
function, and lane-interleaved groups with the separable couplings.
Tolerance: 1e-4 relative state error, as for every parity test.
"""

import numpy as np
import pytest

from conftest import rel_err

import pyoracle as orc
from tvb_hpc import model, coupling, scheme, network, engine, groups

pytestmark = pytest.mark.gpu

TOL = 1e-4


def setup(name, cfun_name, I=10, N=84, speeds=(4.0, ), noise=True, seed=5, dt=0.1):
    w, ln = network.synthetic_connectome(N, 0.3, seed=seed)
    conn = network.Connectivity.from_dense(w, ln)
    rng = np.random.default_rng(seed + 1)
    m = getattr(model, name)()
    if name == 'RWW':
        x0 = rng.uniform(0.05, 0.5, (I, N, 1))
        nparam = np.stack([rng.uniform(0.5, 0.7, (I, N)), rng.uniform(0.3, 0.35, (I, N))], -1)
        G = np.logspace(-2, 0, I)
    else:
        lim = np.array([(lo, hi) for lo, hi in m.limit], float)
        x0 = rng.uniform(lim[:, 0], lim[:, 1], (I, N, 6)) * 0.05
        nparam = np.stack([rng.uniform(5.0, 6.0, (I, N)), rng.uniform(0.5, 0.6, (I, N))], -1)
        G = np.logspace(-3, -1, I)
    cf = getattr(coupling, cfun_name)(m)
    scm = scheme.EulerMaryuyamaStep(dt) if noise else scheme.EulerStep(dt)
    kw = dict(dt=dt, couplings=G.astype(np.float32), speeds=np.resize(np.asarray(speeds, np.float32), I),
              state0=x0.astype(np.float32), nparam=nparam.astype(np.float32), seed=99)
    return (m, cf, scm, conn), kw, x0.astype(np.float32)


@pytest.mark.parametrize('name,cfun_name', [('RWW', 'Linear'), ('RWW', 'Diff'), ('RWW', 'Sigmoidal'),
                                            ('RWW', 'Kuramoto'), ('JansenRit', 'Sigmoidal'),
                                            ('JansenRit', 'Linear')])
def test_per_instance_kernel(cuda, name, cfun_name):
    args, kw, x0 = setup(name, cfun_name)
    sw = engine.Sweep(*args, **kw)
    assert np.all(sw.block_k == 0)
    if name == 'JansenRit':
        assert not (sw.flags & 1)     # zero diffusion: the Euler-Maruyama scheme is Euler
    sw.run(400)
    ref = orc.run_sweep_like(sw, x0, 400)
    assert np.isfinite(ref['state']).all()
    assert rel_err(sw.state.cpu().numpy(), ref['state']) < TOL
    for b in range(sw.n):
        assert rel_err(sw.ring_plain(b), ref['rings'][b]) < TOL


@pytest.mark.parametrize('name,cfun_name', [('RWW', 'Linear'), ('RWW', 'Diff'),
                                            ('JansenRit', 'Sigmoidal'), ('JansenRit', 'Diff')])
def test_group_kernel(cuda, name, cfun_name):
    args, kw, x0 = setup(name, cfun_name, I=12, speeds=(4.0, 10.0))
    gs = groups.GroupSet(*args, **kw)
    gs.run(403)
    ref = orc.run_groups_like(gs, x0, 403)
    assert np.isfinite(ref['state']).all()
    assert rel_err(gs.state.cpu().numpy(), ref['state']) < TOL
    for b in range(gs.n):
        assert rel_err(gs.ring_plain(b), ref['rings'][b]) < TOL
