"""
The node-parallel kernel for one very large network (tvbg_net_run,
bignet.SingleNetwork): against the oracle at N <= 1024 (the oracle's limit),
against the lane-interleaved group kernel with one instance at N = 20000,
chunked runs bit-exact with one run.  Tolerance 1e-4 relative, as everywhere.
"""

import numpy as np
import pytest

from conftest import rel_err

import pyoracle as orc
from tvb_hpc import model, coupling, scheme, network, groups, bignet

pytestmark = pytest.mark.gpu

TOL = 1e-4


def make(name='Generic2dOscillator', cfun_name='Linear', N=1000, degree=40, noise=False, seed=4,
         speed=4.0, dt=0.1, **kw):
    conn = network.synthetic_sparse_connectome(N, degree, seed=seed)
    m = getattr(model, name)()
    rng = np.random.default_rng(seed)
    if name == 'MPR':
        x0 = np.stack([rng.uniform(0.05, 0.3, N), rng.uniform(-1.5, -0.5, N)], -1)
        nparam = rng.uniform(-6, -4, (N, 1))
    else:
        x0 = rng.uniform(-0.5, 0.5, (N, m.nsvar))
        nparam = None
    cf = getattr(coupling, cfun_name)(m)
    scm = scheme.EulerMaryuyamaStep(dt) if noise else scheme.EulerStep(dt)
    net = bignet.SingleNetwork(m, cf, scm, conn, dt, coupling=0.05, speed=speed,
                               state0=x0.astype(np.float32),
                               nparam=None if nparam is None else nparam.astype(np.float32),
                               seed=21, **kw)
    return net, conn, x0.astype(np.float32), nparam


@pytest.mark.parametrize('name,cfun_name,noise', [('Generic2dOscillator', 'Linear', False),
                                                  ('G2DO', 'Diff', False), ('MPR', 'Linear', True),
                                                  ('Linear', 'Sigmoidal', True)])
def test_net_matches_oracle(cuda, name, cfun_name, noise):
    net, conn, x0, nparam = make(name, cfun_name, noise=noise)
    net.run(403)
    npm = net.nparam.cpu().numpy()[None]
    ref = orc.run(net.model_id, net.cfun_id, net.row_np, net.col_np, net.w_np, 1 << net.lognh, 403,
                  net.dt, net.delays[None], [float(net.cf_a)], npm, x0[None],
                  flags=net.flags, sigma=net.sigma, consts=net.consts, cf_b=float(net.cf_b),
                  cf_p=net.cf_p, seed=net.seed, inst_ids=[0])
    assert np.isfinite(ref['state']).all()
    assert rel_err(net.state.cpu().numpy(), ref['state'][0]) < TOL
    got, r = net.ring_plain(), ref['ring'][0]
    np.testing.assert_array_equal(got == 0, r == 0)
    assert rel_err(got, r) < TOL


def test_net_matches_group_kernel_at_large_n(cuda):
    N = 20000
    net, conn, x0, _ = make(N=N, degree=30, block_k=8)
    m = net.model
    gs = groups.GroupSet(m, net.cfun, net.scheme, conn, net.dt, couplings=[float(net.cf_a)],
                         delays=net.delays, state0=x0[None], seed=21, block_k=8)
    net.run(200)
    gs.run(200)
    assert rel_err(net.state.cpu().numpy(), gs.state.cpu().numpy()[0]) < 1e-5


@pytest.mark.parametrize('name,cfun_name,noise,k', [('MPR', 'Linear', True, 8),
                                                    ('G2DO', 'Diff', True, 4),
                                                    ('Linear', 'Sigmoidal', False, 8)])
def test_net_thread_mappings_bit_identical(cuda, name, cfun_name, noise, k):
    "K lanes per node and one thread per node: same sums, same updates."
    a, _, _, _ = make(name, cfun_name, noise=noise, block_k=k, lanes=True)
    b, _, _, _ = make(name, cfun_name, noise=noise, block_k=k, lanes=False)
    a.run(301)
    b.run(301)
    assert np.array_equal(a.state.cpu().numpy(), b.state.cpu().numpy())
    assert np.array_equal(a.ring.cpu().numpy(), b.ring.cpu().numpy())


def test_net_chunks_bit_exact(cuda):
    a, _, _, _ = make(noise=True, name='MPR')
    b, _, _, _ = make(noise=True, name='MPR')
    a.run(500)
    for n in (7, 250, 1, 242):
        b.run(n)
    assert np.array_equal(a.state.cpu().numpy(), b.state.cpu().numpy())
    assert np.array_equal(a.ring.cpu().numpy(), b.ring.cpu().numpy())
