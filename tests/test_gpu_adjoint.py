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


@pytest.mark.parametrize('layout,kernel', [('groups', 'groups'), ('groups', 'instances'),
                                           ('instances', 'instances')])
def test_adjoint_matches_fp64_oracle(cuda, layout, kernel):
    """Both sweep layouts of FCFit (the pipelined group kernel, default
    where the delays allow, and the per-instance step kernel) and both
    reverse-time kernels on the grouped layout (lane-interleaved groups,
    default, and per instance).  3 instances: one group with 5 idle lanes."""
    prob, conn, x0, eta, G, target = problem()
    assert prob.layout == 'groups' and prob.adjoint_kernel == 'groups'
    prob.layout = layout
    prob.adjoint_kernel = kernel
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


@pytest.mark.parametrize('I,N,K,pipe', [(11, 40, 8, False), (16, 84, 4, False), (9, 130, 8, False),
                                        (11, 40, 8, True), (16, 84, 4, True), (9, 130, 8, True)])
def test_adjoint_group_kernel_equals_per_instance(cuda, I, N, K, pipe):
    """tvbg_adjoint_mpr_groups (lane-interleaved, time-blocked, clusters
    where N needs them; one team or the two pipelined teams) against
    tvbg_adjoint_mpr on the same recomputed traces: the same per-step code
    and the same out-edge order, so equal results (checkpoints every 30
    steps: partial blocks at every segment edge)."""
    from tvb_hpc import adjoint
    torch = cuda
    prob, conn, x0, eta, G, target = problem(N=N, I=I, T=180, C=30, seed=N)
    assert prob.adjoint_kernel == 'groups' and prob.dmin >= 2 * K
    prob.adj_k = K
    prob.lognh_g = max(1, int(np.ceil(np.log2(prob.dmax + K))))
    prob.adjoint_shape = adjoint.adjoint_group_shape(N, pipelined=pipe)
    prob.forward(G, eta)
    dG_g, deta_g = (t.clone() for t in prob.backward())
    prob.adjoint_kernel = 'instances'
    dG_i, deta_i = prob.backward()
    assert torch.equal(dG_g, dG_i), (dG_g - dG_i).abs().max()
    assert torch.equal(deta_g, deta_i), (deta_g - deta_i).abs().max()


def test_adjoint_group_kernel_refuses_short_delays(cuda):
    """A record whose smallest delay is below the block length sets the
    status word (TVBG_EINVAL) and leaves the adjoint state untouched."""
    import ctypes
    from tvb_hpc import _native as nat
    torch = cuda
    lib = nat.load()
    tab = np.zeros(1, dtype=nat.ADJOINT_GROUP_DTYPE)
    lam = torch.ones(8 * 4 * 2, device='cuda')
    ring = torch.zeros(4 * 32 * 8, device='cuda')
    seg = torch.zeros(8 * 4 * 3 * 8, device='cuda')
    row = torch.zeros(5, dtype=torch.int32, device='cuda')
    edges = torch.zeros(2, dtype=torch.int32, device='cuda')
    t = tab[0]
    t['edges_t'], t['row_t'], t['seg'] = edges.data_ptr(), row.data_ptr(), seg.data_ptr()
    t['lam'], t['ring'] = lam.data_ptr(), ring.data_ptr()
    t['len'], t['N'], t['lognh'], t['lanes'], t['dmin'] = 8, 4, 4, 8, 3
    dev = torch.from_numpy(tab.view(np.uint8).copy()).cuda()
    status = torch.zeros(1, dtype=torch.int32, device='cuda')
    nat.check(lib.tvbg_adjoint_mpr_groups(dev.data_ptr(), 1, 32, 1, 8, 0, status.data_ptr(), None))
    torch.cuda.synchronize()
    assert int(status.item()) == nat.TVBG_EINVAL
    assert float(lam.min()) == 1.0 and float(lam.max()) == 1.0
    # the pipelined teams need every delay >= 2 K: dmin = 10 < 16 is refused
    status.zero_()
    t['dmin'] = 10
    dev = torch.from_numpy(tab.view(np.uint8).copy()).cuda()
    nat.check(lib.tvbg_adjoint_mpr_groups(dev.data_ptr(), 1, 64, 1, 8, 1, status.data_ptr(), None))
    torch.cuda.synchronize()
    assert int(status.item()) == nat.TVBG_EINVAL
    assert float(lam.min()) == 1.0 and float(lam.max()) == 1.0
    with pytest.raises(nat.TvbgError):
        nat.check(lib.tvbg_adjoint_mpr_groups(dev.data_ptr(), 1, 1024, 1, 8, 0, None, None))
    with pytest.raises(nat.TvbgError):   # pipelined CTAs: a multiple of 64 threads
        nat.check(lib.tvbg_adjoint_mpr_groups(dev.data_ptr(), 1, 96, 1, 8, 1, None, None))


def test_fcfit_reuse_matches_fresh(cuda):
    """FCFit keeps its group sets and buffers across calls: a second
    forward + backward with other couplings and eta gives the same bits as a
    fresh problem."""
    torch = cuda
    prob, conn, x0, eta, G, target = problem(N=40, I=11, T=250, C=50)
    prob.forward(G, eta)
    prob.backward()
    G2 = (G * 1.3).astype(np.float32)
    eta2 = (eta + 0.25).astype(np.float32)
    l1 = prob.forward(G2, eta2).clone()
    g1 = [t.clone() for t in prob.backward()]
    fresh, *_ = problem(N=40, I=11, T=250, C=50)
    l2 = fresh.forward(G2, eta2)
    g2 = fresh.backward()
    assert torch.equal(l1, l2)
    assert all(torch.equal(a, b) for a, b in zip(g1, g2))


def test_adjoint_recompute_windows(cuda):
    """The recomputation in windows of 1, 2 and 4 segments (several
    windows: two buffers, the next window recomputed while the reverse
    kernel reads the current one), with and without the eager start in
    forward, and a second backward after one forward: the same bits as one
    window of all segments."""
    torch = cuda
    prob, conn, x0, eta, G, target = problem(N=40, I=11, T=250, C=30)
    prob.forward(G, eta)
    ref = [t.clone() for t in prob.backward()]
    again = prob.backward()            # no eager window: from the checkpoints
    assert all(torch.equal(a, b) for a, b in zip(ref, again))
    for W, eager in ((1, True), (2, False), (4, True)):
        p2, *_ = problem(N=40, I=11, T=250, C=30)
        p2.recompute_window = W
        p2.eager_recompute = eager
        p2.forward(G, eta)
        assert len(p2._windows()[1]) == -(-9 // W)
        got = p2.backward()
        assert all(torch.equal(a, b) for a, b in zip(ref, got)), W


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


def fc_loss_torch(X, target):
    """The FC-fit loss path in plain torch FP64 (the reference for
    tvbg_fcfit_loss): Pearson FC, loss mean_{i<j}(FC - F*)^2, dL/dX."""
    import torch
    X = X.double().requires_grad_(True)
    I, T, N = X.shape
    Xc = X - X.mean(1, keepdim=True)
    Z = Xc / Xc.norm(dim=1, keepdim=True)
    FC = Z.transpose(1, 2) @ Z
    iu = torch.triu_indices(N, N, 1, device=X.device)
    loss = ((FC - target)[:, iu[0], iu[1]] ** 2).sum(1) / (N * (N - 1) / 2.0)
    loss.sum().backward()
    return loss.detach(), FC.detach(), X.grad


@pytest.mark.parametrize('I,T,N', [(3, 130, 84), (2, 700, 150), (4, 64, 17), (2, 90, 192),
                                   (2, 150, 260)])
def test_fcfit_loss_kernel(cuda, I, T, N):
    """tvbg_fcfit_loss (FP64 FC and loss, FP32 dL/dX, the series' last row
    from a separate array) against torch FP64 autograd of the same loss.
    N = 17, 84, 150, 192: the FP32 exact-triangle Gram (N <= 192, 192 with
    the shared-memory opt-in); 260: the FP64 tiles; dL/dX on whole rows for
    N <= 128, tiles above."""
    import ctypes
    from tvb_hpc import _native as nat
    torch = cuda
    lib = nat.load()
    g = torch.Generator(device='cuda').manual_seed(I * T + N)
    tr = torch.rand(I, T, N, device='cuda', generator=g) + 0.1     # trace rows 0..T-1
    last = torch.rand(I, N, 2, device='cuda', generator=g) + 0.1   # state (r, V); r is the last row
    X = torch.cat([tr[:, 1:], last[:, None, :, 0]], 1)
    target = torch.corrcoef(torch.rand(N, 40, device='cuda', generator=g).double())
    loss_ref, fc_ref, dx_ref = fc_loss_torch(X, target)
    nb = ctypes.c_int64()
    nat.check(lib.tvbg_fcfit_scratch_bytes(I, N, ctypes.byref(nb)))
    scratch = torch.empty(nb.value, dtype=torch.uint8, device='cuda')
    loss = torch.empty(I, dtype=torch.float64, device='cuda')
    fc = torch.empty(I, N, N, dtype=torch.float64, device='cuda')
    dr = torch.zeros(I, T + 1, N, device='cuda')
    nat.check(lib.tvbg_fcfit_loss(tr.data_ptr() + 4 * N, T * N, last.data_ptr(), 2 * N, 2, 1, I, T,
                                  N, target.data_ptr(), loss.data_ptr(), dr.data_ptr() + 4 * N,
                                  (T + 1) * N, fc.data_ptr(), scratch.data_ptr(), None))
    torch.cuda.synchronize()
    assert rel_err(fc.cpu().numpy(), fc_ref.cpu().numpy()) < 1e-12
    assert rel_err(loss.cpu().numpy(), loss_ref.cpu().numpy()) < 1e-10
    assert rel_err(dr[:, 1:].cpu().numpy(), dx_ref.cpu().numpy()) < 1e-5
    assert float(dr[:, 0].abs().max()) == 0.0
    # the same series lane-interleaved (groups of 8: [G][T][N][8], last [G][N][2][8])
    G = -(-I // 8)
    trg = torch.zeros(G * 8, T, N, device='cuda')
    trg[:I] = tr
    trg = trg.view(G, 8, T, N).permute(0, 2, 3, 1).contiguous()
    lg = torch.zeros(G * 8, N, 2, device='cuda')
    lg[:I] = last
    lg = lg.view(G, 8, N, 2).permute(0, 2, 3, 1).contiguous()
    dr2 = torch.zeros_like(dr)
    nat.check(lib.tvbg_fcfit_loss(trg.data_ptr() + 4 * N * 8, T * N * 8, lg.data_ptr(), N * 2 * 8,
                                  16, 8, I, T, N, target.data_ptr(), loss.data_ptr(),
                                  dr2.data_ptr() + 4 * N, (T + 1) * N, fc.data_ptr(),
                                  scratch.data_ptr(), None))
    torch.cuda.synchronize()
    assert torch.equal(dr2, dr)
    assert rel_err(loss.cpu().numpy(), loss_ref.cpu().numpy()) < 1e-10


def test_adjoint_at_benchmark_size(cuda):
    """The benchmark's adjoint fit: MPR, N = 84, 256 instances, 2000 steps of
    0.1 ms, checkpoints every 100 steps, deterministic.  Gradients through the
    torch.autograd.Function wrapper against the FP64 oracle's adjoint on 8
    sampled instances (1e-3) and against central differences (h = 1e-4) of
    the FP64 oracle loss for G and 8 eta components of 2 instances (1e-3)."""
    import os
    torch = cuda
    prob, conn, x0, eta, G, target = problem(N=84, I=256, T=2000, C=100, seed=5)
    Gt = torch.tensor(G, device='cuda', requires_grad=True)
    et = torch.tensor(eta, device='cuda', requires_grad=True)
    loss = adjoint.FCFitLoss.apply(Gt, et, prob)
    loss.sum().backward()
    loss = loss.detach().cpu().numpy()
    dG, deta = Gt.grad.cpu().numpy(), et.grad.cpu().numpy()
    d = conn.delays(4.0, 0.1, 'ceil')
    _, consts, _ = model.MPR().engine_spec()
    idx = np.linspace(0, 255, 8).astype(int)
    loss_o, dG_o, deta_o = orc.mpr_adjoint(conn.row, conn.col, conn.wnz, d,
                                           G[idx].astype(np.float64), eta[idx].astype(np.float64),
                                           x0[idx].astype(np.float64), 2000, 0.1, consts, target,
                                           nthreads=os.cpu_count() or 1)
    assert rel_err(loss[idx], loss_o) < 1e-4
    assert rel_err(dG[idx], dG_o) < 1e-3, (dG[idx], dG_o)
    assert rel_err(deta[idx], deta_o) < 1e-3
    print('adjoint at N=84, I=256, T=2000: rel err dG %.2e, deta %.2e vs FP64 oracle'
          % (rel_err(dG[idx], dG_o), rel_err(deta[idx], deta_o)))
    h = 1e-4
    for b in (int(idx[1]), int(idx[6])):
        f = lambda g, e: orc.mpr_loss(conn.row, conn.col, conn.wnz, d, g, e,  # noqa: E731
                                      x0[b].astype(np.float64), 2000, 0.1, consts, target)
        eb = eta[b].astype(np.float64)
        fd_G = (f(G[b] + h, eb) - f(G[b] - h, eb)) / (2 * h)
        assert abs(dG[b] - fd_G) / abs(fd_G) < 1e-3, (b, dG[b], fd_G)
        nodes = np.linspace(0, 83, 8).astype(int)
        fd_eta = []
        for i in nodes:
            ep, em = eb.copy(), eb.copy()
            ep[i] += h
            em[i] -= h
            fd_eta.append((f(G[b], ep) - f(G[b], em)) / (2 * h))
        assert rel_err(deta[b, nodes], np.array(fd_eta)) < 1e-3, b
