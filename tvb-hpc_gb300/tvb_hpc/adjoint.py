"""
Gradients of an FC-fit loss through the delayed network step (MPR with
linear coupling), by a hand-written adjoint.

Problem (one connectome, I instances, T steps, deterministic):
  x(t+1) = x(t) + dt f(x(t), G_b S(t), eta_b)   (Montbrio-Pazo-Roxin, r >= 0)
  S_i(t) = sum_e w_e r_{j_e}(t - d_e)           (zero history)
  X_b[s] = r_b(s + 1),  FC_b = Pearson(X_b),  loss_b = mean_{i<j}(FC_b,ij - F*_ij)^2

``FCFit.forward`` runs the sweep in chunks of `checkpoint_every` steps --
on the pipelined lane-interleaved group kernel where the delays allow
(every delay >= 2 K - 1), else on the per-instance step kernel -- keeping
the state and the history ring at every chunk start (checkpoints) and the
rate series for the FC; tvbg_fcfit_loss then takes
the FC (a symmetric FP64 Gram), the loss and dL/dr on the device in one
call, no library GEMM.  ``FCFit.backward`` walks the chunks backwards:
each chunk is recomputed from its checkpoint on the same kernel
(bit-identical to the forward) with the state and coupling sums traced
(the group kernel's TVBG_F_TRACE_CSUM column, read in place by the
adjoint), and the reverse-time recursion runs over it, carrying the adjoint
state and an adjoint ring of mu_V between chunks: on lane-interleaved
groups of 8 instances, time-blocked (tvbg_adjoint_mpr_groups), where every
delay is at least 4 steps and N <= 1024, else per instance
(tvbg_adjoint_mpr, through tvbg_adjoint.seg_lanes on a group trace);
dL/dG and dL/deta accumulate in FP64.

``FCFitLoss`` wraps it as a torch.autograd.Function of (G [I], eta [I, N]).
The reference builds only symbolic partials (tvb_hpc/model.py:61-65) and an
EM log-density (scheme.py:42-48); it has no gradient kernel.
"""

import ctypes

import numpy as np

from . import _native as nat
from . import model as mdl, coupling as cpl, scheme as sch
from .engine import InstanceSet, plan_ring, max_smem
from .utils import getLogger

LOG = getLogger(__name__)


def _transpose(row, col):
    """Out-edge order of a CSR of in-edges: by source j, then target i.
    Returns (order, target of each edge, row_t [N+1])."""
    row = np.asarray(row, np.int64)
    col = np.asarray(col, np.int64)
    N = row.size - 1
    tgt = np.repeat(np.arange(N), np.diff(row))
    order = np.lexsort((tgt, col))
    row_t = np.zeros(N + 1, np.int64)
    np.add.at(row_t, col[order] + 1, 1)
    return order, tgt, np.cumsum(row_t).astype(np.int32)


def transpose_edges(row, col, w, delays, lognh):
    """Out-edges of every source node j: (target i, delay d, weight), packed
    for the adjoint ring read of mu_V,i(t + d + 1): pk = (i << lognh) |
    ((i + d + 1) & mask).  Returns (row_t [N+1], packed [nnz])."""
    order, tgt, row_t = _transpose(row, col)
    mask = (1 << lognh) - 1
    i = tgt[order].astype(np.uint64)
    d = np.asarray(delays, np.int64)[order].astype(np.uint64)
    out = np.zeros(len(order), dtype=np.dtype([('pk', '<u4'), ('w', '<f4')]))
    out['pk'] = ((i << np.uint64(lognh)) | ((i + d + np.uint64(1)) & np.uint64(mask))).astype(np.uint32)
    out['w'] = np.asarray(w, np.float32)[order]
    return row_t, out


def transpose_edges_group(row, col, w, delays):
    """The same out-edges, same order, packed for tvbg_adjoint_mpr_groups:
    pk = (i << 16) | d.  Returns (row_t [N+1], packed [nnz])."""
    order, tgt, row_t = _transpose(row, col)
    d = np.asarray(delays, np.int64)[order]
    if row_t.size - 1 > 65535 or (d.size and int(d.max()) > 65535):
        raise ValueError('group adjoint edges: N and delays must be < 65536')
    out = np.zeros(len(order), dtype=np.dtype([('pk', '<u4'), ('w', '<f4')]))
    out['pk'] = ((tgt[order].astype(np.uint64) << np.uint64(16)) | d.astype(np.uint64)).astype(np.uint32)
    out['w'] = np.asarray(w, np.float32)[order]
    return row_t, out


def adjoint_group_shape(N, slots=16, max_threads=512, max_cluster=16):
    """(threads, cluster) of tvbg_adjoint_mpr_groups for N nodes: about
    `slots` node slots per CTA (measured at N = 84, 256 instances: 16 slots
    x 6 CTAs 9.15 ms per backward, 44 x 2 9.5 ms), as many CTAs as that
    takes up to max_cluster, node slots a multiple of 4 (threads a multiple
    of 32) and at most max_threads / 8; None when N does not fit."""
    c0 = min(max_cluster, max(-(-N // slots), -(-N // (max_threads // 8)), 1))
    for c in range(c0, max_cluster + 1):
        p = -(-N // c)
        p = -(-p // 4) * 4
        if 8 * p <= max_threads:
            return 8 * p, c
    return None


class FCFit:
    """
    FC-fit problem for I instances of deterministic MPR + linear coupling.

    conn : Connectivity;  dt : ms;  speed : mm/ms (delays ceil(len/speed/dt))
    x0 : [I, N, 2] initial (r, V);  target : [N, N] target FC;  T : steps
    """

    def __init__(self, conn, dt, speed, x0, target, T, checkpoint_every=100, rounding='ceil',
                 model=None):
        import torch
        self.torch = torch
        self.conn = conn
        self.dt = float(dt)
        self.speed = float(speed)
        self.x0 = np.asarray(x0, np.float32)
        self.I, self.N = self.x0.shape[0], conn.nnode
        self.T = int(T)
        self.C = int(checkpoint_every)
        self.model = model or mdl.MPR()
        self.cfun = cpl.Linear(self.model)
        self.cfun.param['b'] = 0.0
        self.scheme = sch.EulerStep(self.dt)
        self.target = torch.as_tensor(np.asarray(target), dtype=torch.float64, device='cuda')
        self.rounding = rounding
        d = conn.delays(speed, dt, rounding)
        self.lognh = plan_ring(int(d.min()), int(d.max()))[0]
        row_t, e_t = transpose_edges(conn.row, conn.col, conn.wnz, d, self.lognh)
        self.row_t = torch.from_numpy(row_t).cuda()
        self.edges_t = torch.from_numpy(e_t.view(np.uint8).copy()).cuda()
        _, consts, _ = self.model.engine_spec()
        self.consts = consts
        self.tpn = 1          # gather lanes per node of the per-instance sweeps
        self.adjoint_smem = 'auto'   # adjoint ring in shared memory: 'auto' or False
        # forward and recomputation sweeps: the pipelined lane-interleaved
        # group kernel where it applies (delays >= 2 K - 1, N <= 1024), else
        # the per-instance step kernel
        from .groups import plan_group, pipelined_threads
        k, _ = plan_group(int(d.min()), int(d.max()))
        self.layout = ('groups' if int(d.min()) >= 2 * k - 1 and pipelined_threads(self.N, 16)
                       else 'instances')
        # the reverse-time kernel on the grouped layout: lane-interleaved and
        # time-blocked (tvbg_adjoint_mpr_groups, blocks of K <= d_min steps)
        # where the delays and N allow, else per instance over the group trace
        self.dmin, self.dmax = int(d.min()), int(d.max())
        self.adj_k = 8 if self.dmin >= 8 else (4 if self.dmin >= 4 else 0)
        self.adjoint_shape = adjoint_group_shape(self.N) if self.adj_k else None
        self.adjoint_kernel = ('groups' if self.layout == 'groups' and self.adjoint_shape
                               else 'instances')
        # device buffers and group sets reused across calls (built on first use)
        self._fw_gs = self._rec_gs = None
        self._ck = None
        self._bufs = None
        self._adj_ring = None
        if self.adjoint_kernel == 'groups':
            self.lognh_g = max(1, int(np.ceil(np.log2(self.dmax + self.adj_k))))
            row_tg, e_tg = transpose_edges_group(conn.row, conn.col, conn.wnz, d)
            assert np.array_equal(row_tg, row_t)
            self.edges_tg = torch.from_numpy(e_tg.view(np.uint8).copy()).cuda()
            # slot positions by out-degree, largest first: the node slots of
            # a warp see similar edge counts
            outdeg = np.diff(row_t)
            self.nodes_t = torch.from_numpy(
                np.argsort(-outdeg, kind='stable').astype(np.int32)).cuda()

    def _set(self, G, eta, trace_len, trace_nobs, trace_csum):
        return InstanceSet(self.model, self.cfun, self.scheme, self.conn, dt=self.dt,
                           couplings=np.asarray(G, np.float32), speeds=self.speed,
                           state0=self.x0, nparam=np.asarray(eta, np.float32).reshape(self.I, self.N, 1),
                           rounding=self.rounding, blocked=False, trace_every=1,
                           trace_len=trace_len, trace_nobs=trace_nobs, trace_csum=trace_csum)

    @staticmethod
    def _sweep(iset, tpn=2):
        "A Sweep view of an InstanceSet (same device arrays)."
        from .engine import Sweep, DeviceStatus
        sw = Sweep.__new__(Sweep)
        sw.__dict__.update(iset.__dict__)
        sw.tpn = tpn
        sw.status = DeviceStatus()
        sw._uploaded = None
        return sw

    @staticmethod
    def _plan(sw, segs):
        """Launch tables of every segment (t0, n), built and uploaded up
        front so the segments then run back to back without host syncs."""
        plans = []
        for t0, n in segs:
            sw.t[:] = t0
            plans.append(sw.prepare(n))
        return plans

    def _groups(self, G, eta, trace_len, trace_nobs, trace_csum):
        "Lane-interleaved groups of the I instances on the pipelined kernel."
        from .groups import GroupSet, pipelined_shape, PIPELINED
        gs = GroupSet(self.model, self.cfun, self.scheme, self.conn, dt=self.dt,
                      couplings=np.asarray(G, np.float32), speeds=self.speed, state0=self.x0,
                      nparam=np.asarray(eta, np.float32).reshape(self.I, self.N, 1),
                      rounding=self.rounding, trace_every=1, trace_len=trace_len,
                      trace_nobs=trace_nobs, trace_csum=trace_csum)
        sms = self.torch.cuda.get_device_properties(
            self.torch.cuda.current_device()).multi_processor_count
        shape = pipelined_shape(gs, min_ctas=sms)
        assert shape[3] == PIPELINED
        gs.set_shape(*shape)
        return gs

    def forward(self, G, eta):
        "Loss [I] (FP64); keeps checkpoints and the rate series for backward."
        G = np.asarray(G, np.float32).reshape(self.I)
        eta = np.asarray(eta, np.float32).reshape(self.I, self.N)
        self.G, self.eta = G, eta
        if self.layout == 'groups':
            return self._forward_groups(G, eta)
        return self._forward_instances(G, eta)

    def _group_sets(self, G, eta):
        """The forward's and the recomputation's GroupSets (one-column r
        trace of T rows; r, V and the coupling sum over one segment), built
        on the first call and given this call's couplings, eta and initial
        state after that."""
        torch = self.torch
        if self._fw_gs is None:
            self._fw_gs = self._groups(G, eta, self.T, 1, False)
            # two recomputation sets: segment k - 1 is recomputed into one
            # while the reverse kernel reads segment k from the other
            self._rec_sets = [self._groups(G, eta, self.C, 2, True) for _ in range(2)]
            self._rec_gs = self._rec_sets[0]
            self._x0_dev = torch.from_numpy(self.x0).cuda()
            self._side = torch.cuda.Stream()
        else:
            for gs in [self._fw_gs] + self._rec_sets:
                gs.set_couplings(G)
                gs.set_nparam(eta)
            fw = self._fw_gs
            fw.set_state(self._x0_dev)
            fw.clear_history()
            fw.t[:] = 0
        return self._fw_gs, self._rec_gs

    def _forward_groups(self, G, eta):
        """Forward on the pipelined group kernel: segments of C steps, the
        group state and ring copied at each segment start, the r trace
        lane-interleaved ([G][T][N][1][8]); the loss path reads it in place."""
        torch = self.torch
        fw, _ = self._group_sets(G, eta)
        segs = [(t, min(self.C, self.T - t)) for t in range(0, self.T, self.C)]
        plans = fw.prepare_segments(segs)
        if self._ck is None:
            self._ck = (torch.empty((len(segs), ) + tuple(fw.gstate.shape), dtype=torch.float32,
                                    device='cuda'),
                        torch.empty((len(segs), fw.ring.numel()), dtype=torch.float32, device='cuda'))
        self.ckpt = []
        for s, ((t0, n), launches) in enumerate(zip(segs, plans)):
            self._ck[0][s].copy_(fw.gstate)
            self._ck[1][s].copy_(fw.ring)
            self.ckpt.append((t0, n, self._ck[0][s], self._ck[1][s]))
            fw.launch(launches)
        fw.t[:] = self.T
        self.fw = fw
        I, N, T = self.I, self.N, self.T
        L = 8
        loss = self._loss(fw.gtrace.data_ptr() + 4 * N * L, T * N * L, fw.gstate.data_ptr(),
                          N * 2 * L, 2 * L, L)
        torch.cuda.synchronize()
        fw.status.check()
        return loss

    def _loss(self, x, xs, last, ls, lns, lanes):
        """tvbg_fcfit_loss on the series at x (rows 1..T-1) and last (row T):
        FP64 FC and loss; dL/dr(t) = dL/dX[t-1] into self.dr[:, 1:]."""
        torch = self.torch
        I, N, T = self.I, self.N, self.T
        lib = nat.load()
        if self._bufs is None:
            nb = ctypes.c_int64()
            nat.check(lib.tvbg_fcfit_scratch_bytes(I, N, ctypes.byref(nb)))
            # dr row 0 stays zero; the loss path writes rows 1..T every call
            self._bufs = (torch.zeros((I, T + 1, N), dtype=torch.float32, device='cuda'),
                          torch.empty((I, N, N), dtype=torch.float64, device='cuda'),
                          torch.empty(int(nb.value), dtype=torch.uint8, device='cuda'))
        self.dr, self.fc, scratch = self._bufs
        loss = torch.empty(I, dtype=torch.float64, device='cuda')
        nat.check(lib.tvbg_fcfit_loss(x, xs, last, ls, lns, lanes, I, T, N, self.target.data_ptr(),
                                      loss.data_ptr(), self.dr.data_ptr() + 4 * N, (T + 1) * N,
                                      self.fc.data_ptr(), scratch.data_ptr(), nat.stream_handle()))
        return loss

    def _forward_instances(self, G, eta):
        "Forward on the per-instance step kernel (delays too short for the groups)."
        torch = self.torch
        fw = self._set(G, eta, self.T, 1, False)
        sw = self._sweep(fw)
        segs = [(t, min(self.C, self.T - t)) for t in range(0, self.T, self.C)]
        plans = self._plan(sw, segs)
        self.ckpt = []
        for (t0, n), pl in zip(segs, plans):
            self.ckpt.append((t0, n, fw.state.clone(), fw.ring.clone()))
            sw.launch(pl, self.tpn)
        fw.t[:] = self.T
        self.fw = fw
        # X[s] = r(s + 1): trace rows 1..T-1 (r(t), one column) and the
        # final state's r
        I, N, T = self.I, self.N, self.T
        assert fw.trace.shape[1:] == (T, N, 1)
        loss = self._loss(fw.trace.data_ptr() + 4 * N, T * N, fw.state.data_ptr(), 2 * N, 2, 1)
        torch.cuda.synchronize()
        sw.status.check()
        return loss

    def backward(self):
        "(dL/dG [I], dL/deta [I, N]) in FP64, by the adjoint over the checkpoints."
        return self._backward(self.layout == 'groups')

    def _backward(self, grouped):
        torch = self.torch
        lib = nat.load()
        I, N, T = self.I, self.N, self.T
        nh = 1 << self.lognh
        dr = self.dr                                   # dL/dr(t) = dL/dX[t-1], from forward
        lam = torch.zeros((I, N, 2), dtype=torch.float32, device='cuda')
        lam[:, :, 0] = dr[:, T]
        ring = torch.zeros((I, N * nh), dtype=torch.float32, device='cuda')
        deta = torch.zeros((I, N), dtype=torch.float64, device='cuda')
        dGn = torch.zeros((I, N), dtype=torch.float64, device='cuda')
        rev = list(reversed(self.ckpt))
        b = np.arange(I, dtype=np.int64)
        if grouped and self.adjoint_kernel == 'groups':
            return self._reverse_groups(rev, lam, deta, dGn)
        if grouped:
            # recomputation on the same pipelined group kernel (bit-identical
            # to the forward) with r, V and the coupling sum S traced,
            # lane-interleaved [G][C][N][3][8]; the adjoint reads it in place
            rec = self._rec_gs
            plans = rec.prepare_segments([(t0, n) for (t0, n, _, _) in rev])
            seg = rec.gtrace
            seg_ptr = seg.data_ptr() + 4 * ((b // 8) * self.C * N * 3 * 8 + b % 8)
            seg_lanes = 8
        else:
            rec = self._set(self.G, self.eta, self.C, 2, True)
            sw = self._sweep(rec)
            plans = self._plan(sw, [(t0, n) for (t0, n, _, _) in rev])
            seg = rec.trace                              # [I, C, N, 3]: r, V, S of a segment
            seg_ptr = seg.data_ptr() + 4 * b * seg.shape[1] * N * 3
            seg_lanes = 1
        threads = 32 * ((N + 31) // 32)
        tab = np.zeros((len(rev), I), dtype=nat.ADJOINT_DTYPE)
        for k, (t0, n, _, _) in enumerate(rev):
            tk = tab[k]
            tk['edges_t'] = self.edges_t.data_ptr()
            tk['row_t'] = self.row_t.data_ptr()
            tk['seg'] = seg_ptr
            tk['seg_lanes'] = seg_lanes
            tk['dr'] = dr.data_ptr() + 4 * (b * (T + 1) * N + t0 * N)
            tk['lam'] = lam.data_ptr() + 4 * b * N * 2
            tk['ring'] = ring.data_ptr() + 4 * b * N * nh
            tk['deta'] = deta.data_ptr() + 8 * b * N
            tk['dG'] = dGn.data_ptr() + 8 * b * N
            tk['t0'] = t0
            tk['len'] = n
            tk['N'] = N
            tk['lognh'] = self.lognh
            tk['dt'] = np.float32(self.dt)
            tk['G'] = self.G
            tk['consts'] = self.consts[:4]
        dev = torch.from_numpy(tab.view(np.uint8).reshape(-1).copy()).cuda()
        row_bytes = I * nat.ADJOINT_DTYPE.itemsize
        # segments last first: recompute from the checkpoint (bit-identical to
        # the forward), then the reverse-time kernel over it, back to back
        # the adjoint ring in shared memory when it fits one CTA and the
        # instances fit one wave of CTAs (with more, the CTAs the smaller
        # global-ring footprint keeps resident together win: measured)
        ring_b = 4 * N * nh
        sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
        smem = ring_b if (self.adjoint_smem == 'auto' and ring_b + 4096 <= max_smem()
                          and I <= sms) else 0
        for k, ((t0, n, st, rg), pl) in enumerate(zip(rev, plans)):
            if grouped:
                rec.gstate.copy_(st)
                rec.ring.copy_(rg)
                rec.launch(pl)
            else:
                rec.state.copy_(st)
                rec.ring.copy_(rg)
                sw.launch(pl, self.tpn)
            nat.check(lib.tvbg_adjoint_mpr_ex(dev.data_ptr() + k * row_bytes, I, threads, smem,
                                              nat.stream_handle()))
        torch.cuda.synchronize()
        (rec if grouped else sw).status.check()
        return dGn.sum(1), deta


    def _reverse_groups(self, rev, lam, deta, dGn):
        """Segments last first: recompute on the group kernel, then
        tvbg_adjoint_mpr_groups over the group trace in place (r, V, S
        lane-interleaved [G][C][N][3][8]), an adjoint ring per group.  The
        recomputation of segment k + 1 (in the list's order) runs on a side
        stream, into the other of two recomputation sets, while the reverse
        kernel works on segment k; events order each recomputation after the
        reverse kernel that last read its set, and each reverse kernel after
        its recomputation."""
        from .engine import DeviceStatus
        torch = self.torch
        lib = nat.load()
        recs = self._rec_sets
        S = len(rev)
        segs = [(t0, n) for (t0, n, _, _) in rev]
        plans = [None] * S
        for j in range(2):
            ks = list(range(j, S, 2))
            if ks:
                for k, pl in zip(ks, recs[j].prepare_segments([segs[k] for k in ks])):
                    plans[k] = pl
        I, N, T, K = self.I, self.N, self.T, self.adj_k
        Gn = (I + 7) // 8
        R = (1 << self.lognh_g) + K
        if self._adj_ring is None or tuple(self._adj_ring.shape) != (Gn, N, R, 8):
            self._adj_ring = torch.zeros((Gn, N, R, 8), dtype=torch.float32, device='cuda')
        else:
            self._adj_ring.zero_()
        ring = self._adj_ring
        threads, cluster = self.adjoint_shape
        g = np.arange(Gn, dtype=np.int64)[None, :]           # [1, Gn]
        t0s = np.array([r[0] for r in rev], np.int64)[:, None]
        lens = np.array([r[1] for r in rev], np.int64)[:, None]
        Gl = np.zeros(Gn * 8, np.float32)
        Gl[:I] = self.G
        tab = np.zeros((len(rev), Gn), dtype=nat.ADJOINT_GROUP_DTYPE)
        tab['edges_t'] = self.edges_tg.data_ptr()
        tab['row_t'] = self.row_t.data_ptr()
        tab['nodes'] = self.nodes_t.data_ptr()
        seg0 = np.array([recs[k % 2].gtrace.data_ptr() for k in range(S)], np.int64)[:, None]
        tab['seg'] = seg0 + 4 * g * self.C * N * 3 * 8
        tab['dr'] = self.dr.data_ptr() + 4 * (8 * g * (T + 1) * N + t0s * N)
        tab['lam'] = lam.data_ptr() + 4 * 8 * g * N * 2
        tab['ring'] = ring.data_ptr() + 4 * g * N * R * 8
        tab['deta'] = deta.data_ptr() + 8 * 8 * g * N
        tab['dG'] = dGn.data_ptr() + 8 * 8 * g * N
        tab['t0'] = t0s
        tab['dr_stride'] = (T + 1) * N
        tab['len'] = lens
        tab['N'] = N
        tab['lognh'] = self.lognh_g
        tab['lanes'] = np.minimum(8, I - 8 * g)
        tab['dmin'] = self.dmin
        tab['dt'] = np.float32(self.dt)
        tab['G'] = Gl.reshape(1, Gn, 8)
        tab['consts'] = self.consts[:4]
        dev = torch.from_numpy(tab.view(np.uint8).reshape(-1).copy()).cuda()
        row_bytes = Gn * nat.ADJOINT_GROUP_DTYPE.itemsize
        status = DeviceStatus()
        main, side = torch.cuda.current_stream(), self._side
        side.wait_stream(main)
        done = []
        for k, ((t0, n, st, rg), pl) in enumerate(zip(rev, plans)):
            rec = recs[k % 2]
            if k >= 2:
                side.wait_event(done[k - 2])
            with torch.cuda.stream(side):
                rec.gstate.copy_(st)
                rec.ring.copy_(rg)
            rec.launch(pl, stream=side)
            ready = torch.cuda.Event()
            ready.record(side)
            main.wait_event(ready)
            nat.check(lib.tvbg_adjoint_mpr_groups(dev.data_ptr() + k * row_bytes, Gn, threads,
                                                  cluster, K, status.t.data_ptr(),
                                                  main.cuda_stream))
            done.append(torch.cuda.Event())
            done[-1].record(main)
        main.wait_stream(side)
        torch.cuda.synchronize()
        for rec in recs:
            rec.status.check()
        status.check()
        return dGn.sum(1), deta


class FCFitLoss:
    """torch.autograd.Function: loss [I] = FCFitLoss.apply(G [I], eta [I, N], problem)."""

    _fn = None

    @classmethod
    def apply(cls, G, eta, problem):
        import torch

        if cls._fn is None:
            class _F(torch.autograd.Function):
                @staticmethod
                def forward(ctx, G_, eta_, prob):
                    ctx.prob = prob
                    return prob.forward(G_.detach().cpu().numpy(),
                                        eta_.detach().cpu().numpy()).to(G_.dtype)

                @staticmethod
                def backward(ctx, gl):
                    dG, deta = ctx.prob.backward()
                    gl = gl.to(torch.float64)
                    return ((gl * dG).to(torch.float32).to(gl.device),
                            (gl[:, None] * deta).to(torch.float32).to(gl.device), None)
            cls._fn = _F
        return cls._fn.apply(G, eta, problem)


_ = ctypes
