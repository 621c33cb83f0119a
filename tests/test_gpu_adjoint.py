"""
The hand-written adjoint (tvbg_adjoint_mpr + checkpointed recomputation)
against the FP64 oracle: the oracle's own adjoint (an independent C
restatement of the recursion) and central finite differences of the FP64
oracle loss (h = 1e-4).  Tolerance 1e-3 relative (max-norm), as asked of the
FC-fit gradient.  Also the torch.autograd.Function wrapper.
"""

import numpy as np
import pytest

from conftest import rel_err

import pyoracle as orc
from tvb_hpc import network, model, adjoint

pytestmark = pytest.mark.gpu


def problem(N=40, I=3, T=350, C=100, seed=2):
    w, ln = network.synthetic_connectome(N, 0.3, seed=seed)
    conn = network.Connectivity.from_dense(w, ln)
    rng = np.random.default_rng(seed)
    x0 = np.stack([rng.uniform(0.05, 0.3, (I, N)), rng.uniform(-1.5, -0.5, (I, N))], -1)
    x0 = x0.astype(np.float32)
    eta = rng.uniform(-6, -4, (I, N)).astype(np.float32)
    G = np.linspace(0.3, 1.0, I).astype(np.float32)
    target = np.corrcoef(rng.normal(size=(N, 60))).astype(np.float32)
    prob = adjoint.FCFit(conn, 0.1, 4.0, x0, target, T, checkpoint_every=C)
    return prob, conn, x0, eta, G, target


def test_adjoint_matches_fp64_oracle(cuda):
    prob, conn, x0, eta, G, target = problem()
    loss = prob.forward(G, eta).cpu().numpy()
    dG, deta = (t.cpu().numpy() for t in prob.backward())
    d = conn.delays(4.0, 0.1, 'ceil')
    _, consts, _ = model.MPR().engine_spec()
    loss_o, dG_o, deta_o = orc.mpr_adjoint(conn.row, conn.col, conn.wnz, d, G.astype(np.float64),
                                           eta.astype(np.float64), x0.astype(np.float64),
                                           prob.T, 0.1, consts, target)
    assert rel_err(loss, loss_o) < 1e-4
    assert rel_err(dG, dG_o) < 1e-3, (dG, dG_o)
    assert rel_err(deta, deta_o) < 1e-3
    print('adjoint: rel err dG %.2e, deta %.2e vs FP64 oracle' % (rel_err(dG, dG_o),
                                                                     rel_err(deta, deta_o)))
    # central finite differences of the FP64 loss (instance 0)
    h = 1e-4
    f = lambda g, e: orc.mpr_loss(conn.row, conn.col, conn.wnz, d, g, e, x0[0].astype(np.float64),
                                  prob.T, 0.1, consts, target)
    e0 = eta[0].astype(np.float64)
    fd_G = (f(G[0] + h, e0) - f(G[0] - h, e0)) / (2 * h)
    assert abs(dG[0] - fd_G) / abs(fd_G) < 1e-3
    fd_eta = []
    for i in range(4):
        ep, em = e0.copy(), e0.copy()
        ep[i] += h
        em[i] -= h
        fd_eta.append((f(G[0], ep) - f(G[0], em)) / (2 * h))
    assert rel_err(deta[0, :4], np.array(fd_eta)) < 1e-3


def test_adjoint_autograd_function(cuda):
    torch = cuda
    prob, conn, x0, eta, G, target = problem(I=2, T=200)
    Gt = torch.tensor(G, device='cuda', requires_grad=True)
    et = torch.tensor(eta, device='cuda', requires_grad=True)
    loss = adjoint.FCFitLoss.apply(Gt, et, prob)
    loss.sum().backward()
    prob2, *_ = problem(I=2, T=200)
    prob2.forward(G, eta)
    dG, deta = prob2.backward()
    np.testing.assert_allclose(Gt.grad.cpu().numpy(), dG.cpu().numpy(), rtol=1e-6)
    np.testing.assert_allclose(et.grad.cpu().numpy(), deta.cpu().numpy(), rtol=1e-6, atol=1e-12)


def test_fcfit_zgrad_kernel(cuda):
    "tvbg_fcfit_zgrad (dL/dZ = Z A, FP32) against an FP64 product, ragged sizes."
    import ctypes
    from tvb_hpc import _native as nat
    torch = cuda
    lib = nat.load()
    g = torch.Generator(device='cuda').manual_seed(0)
    for I, T, N in ((3, 130, 84), (1, 2000, 998), (5, 64, 17)):
        Z = torch.randn(I, T, N, device='cuda', generator=g) / np.sqrt(T)
        A = torch.randn(I, N, N, device='cuda', generator=g) / N
        out = torch.empty_like(Z)
        nat.check(lib.tvbg_fcfit_zgrad(Z.data_ptr(), A.data_ptr(), out.data_ptr(), I, T, N, None))
        ref = Z.double() @ A.double()
        assert rel_err(out.cpu().numpy(), ref.cpu().numpy()) < 1e-5
