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
rate series for the FC; tvbg_fcfit_loss then takes the FC (FP64 means, a
centred upper-triangle Gram in FP32 error-free arithmetic), the loss and
dL/dr on the device in one call, no library GEMM.

``FCFit.backward`` walks the chunks backwards.  On the grouped layout the
chunks are recomputed in windows (as many as `trace_budget` holds, one
launch per window: every chunk from a working copy of its checkpoint, on
the forward's kernel, so bit-identical), the last window already at the end
of forward on a side stream; the recomputation traces the state and the
coupling sums (the group kernel's TVBG_F_TRACE_CSUM column).  The
reverse-time recursion then runs over each window in one launch, on
lane-interleaved groups of 8 instances, time-blocked, with two thread teams
where every delay is >= 2 K (tvbg_adjoint_mpr_groups), carrying the adjoint
state and an adjoint ring of mu_V between windows.  Elsewhere (delays under
4 steps, N > 1024, the per-instance layout) chunk by chunk per instance
(tvbg_adjoint_mpr; through tvbg_adjoint.seg_lanes on a group trace).
dL/dG and dL/deta accumulate in FP64, their partial sums grouped per chunk
in every form, so on the same traces the reverse kernels (per instance or
on groups, one team or two, any window) give the same bits.  Neither call
waits for the device: status words are checked at the next call (or by
check()).

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


def plan_windows(S, per_segment, budget, window=None):
    """Windows of the recomputation over S checkpoint segments, last
    first: (W, [(a, b), ...], buffers).  W segments per window, as many as
    `budget` bytes hold at `per_segment` bytes each (one buffer for a single
    window, two when the recomputation of the next window overlaps the
    reverse kernel of this one), or `window` when given."""
    S = int(S)
    W = max(1, min(S, int(budget) // int(per_segment)))
    if W < S:
        W = max(1, int(budget) // (2 * int(per_segment)))
    if window:
        W = max(1, min(S, int(window)))
    wins = []
    b = S
    while b > 0:
        wins.append((max(0, b - W), b))
        b -= W
    return W, wins, 1 if len(wins) == 1 else 2


def adjoint_group_shape(N, pipelined=False, slots=16, max_threads=512, max_cluster=16):
    """(threads, cluster, pipelined) of tvbg_adjoint_mpr_groups for N
    nodes: about `slots` node slots per CTA (measured at N = 84, 256
    instances: 16 slots x 6 CTAs 9.15 ms per backward, 44 x 2 9.5 ms), as
    many CTAs as that takes up to max_cluster, node slots a multiple of 4
    (each team's threads a multiple of 32); threads = 8 (16 with the two
    pipelined teams) per slot, at most max_threads; None when N does not
    fit."""
    per = 16 if pipelined else 8
    c0 = min(max_cluster, max(-(-N // slots), -(-N // (max_threads // per)), 1))
    for c in range(c0, max_cluster + 1):
        p = -(-N // c)
        p = -(-p // 4) * 4
        if per * p <= max_threads:
            return per * p, c, int(bool(pipelined))
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
        # the two-team reverse kernel where every delay is >= 2 K
        self.adjoint_shape = None
        if self.adj_k:
            self.adjoint_shape = (adjoint_group_shape(self.N, pipelined=True)
                                  if self.dmin >= 2 * self.adj_k else None) or \
                adjoint_group_shape(self.N)
        self.adjoint_kernel = ('groups' if self.layout == 'groups' and self.adjoint_shape
                               else 'instances')
        # device buffers and group sets reused across calls (built on first use)
        self._fw_gs = self._rec_gs = None
        self._ck = None
        self._bufs = None
        self._adj_ring = None
        self._win = None
        self._eager = None
        self._tables = []
        self._deferred = []      # status words of earlier calls, copied to the host
        # the recomputation on the grouped layout runs in windows of segments,
        # one launch per window, their traces (r, V, S) and working copies of
        # the checkpoints within trace_budget bytes; the last window is
        # recomputed at the end of forward() (side stream, overlapping the
        # loss path) when eager_recompute
        self.trace_budget = 2 << 30
        self.recompute_window = None   # segments per window (None: from trace_budget)
        self.eager_recompute = True
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

    def _defer(self, *statuses):
        """Copy device status words to pinned host memory without waiting
        (checked by check() or at the end of the next call, once that call's
        work is queued: the device never waits for the host)."""
        torch = self.torch
        for st in statuses:
            h = torch.empty(1, dtype=torch.int32, pin_memory=True)
            h.copy_(st.t, non_blocking=True)
            ev = torch.cuda.Event()
            ev.record()
            self._deferred.append((h, ev))

    def check(self, upto=None):
        """Raise if a kernel of an earlier forward/backward reported a
        device-side error (waits for those kernels)."""
        pend = self._deferred if upto is None else self._deferred[:upto]
        self._deferred = [] if upto is None else self._deferred[upto:]
        for h, ev in pend:
            ev.synchronize()
            if int(h[0]) != 0:
                raise nat.TvbgError(int(h[0]), 'device-side check failed in the adjoint')

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
        from .groups import pipelined_shape
        torch = self.torch
        if self._fw_gs is None:
            self._fw_gs = self._groups(G, eta, self.T, 1, False)
            # the recomputation set: its tables, flags and parameters serve the
            # windows (many groups per launch: the smallest pipelined cluster)
            self._rec_gs = self._groups(G, eta, self.C, 2, True)
            self._rec_gs.set_shape(*pipelined_shape(self._rec_gs))
            self._x0_dev = torch.from_numpy(self.x0).cuda()
            self._side = torch.cuda.Stream()
        else:
            for gs in (self._fw_gs, self._rec_gs):
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
        # an earlier call's recomputation (side stream) may still read the
        # checkpoints this forward overwrites
        torch.cuda.current_stream().wait_stream(self._side)
        self._tables = []
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
        self._eager = None
        if self.adjoint_kernel == 'groups' and self.eager_recompute:
            # the last window's recomputation overlaps the loss path
            self._windows()
            side = self._side
            side.wait_stream(torch.cuda.current_stream())
            self._eager = self._recompute_window(0, side)
        loss = self._loss(fw.gtrace.data_ptr() + 4 * N * L, T * N * L, fw.gstate.data_ptr(),
                          N * 2 * L, 2 * L, L)
        # this call's status copied without waiting; the earlier calls' checked
        # now that this call's work is queued behind theirs
        n_prev = len(self._deferred)
        self._defer(fw.status)
        self.check(n_prev)
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
            return self._reverse_windows(lam, deta, dGn)
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


    def _windows(self):
        """Windows of segments for the recomputation, last first: (a, b)
        segment ranges of at most W segments, W set by trace_budget (two
        buffers when there is more than one window); the buffers, allocated
        once: traces [G][W C][N][3][8] and working copies of W checkpoints."""
        torch = self.torch
        rec = self._rec_gs
        S = len(self.ckpt)
        G, N, C = rec.n_groups, self.N, self.C
        per = 4 * (G * C * N * 3 * 8 + rec.gstate.numel() + rec.ring.numel())
        W, wins, nbuf = plan_windows(S, per, self.trace_budget, self.recompute_window)
        if self._win is not None and self._win[0] == W and len(self._win[2]) == nbuf \
                and self._win[1] == wins:
            return self._win
        bufs = [(torch.empty((G, W * C, N, 3, 8), dtype=torch.float32, device='cuda'),
                 torch.empty((W, ) + tuple(rec.gstate.shape), dtype=torch.float32, device='cuda'),
                 torch.empty((W, rec.ring.numel()), dtype=torch.float32, device='cuda'))
                for _ in range(nbuf)]
        order = torch.arange(W * G, dtype=torch.int32, device='cuda')
        self._win = (W, wins, bufs, order)
        return self._win

    def _recompute_window(self, w, stream):
        """Recompute window w (of _windows) on `stream` in one launch of
        (segment, group) pairs, each group from a working copy of its
        segment's checkpoint, traces into the window's buffer (w % 2); the
        same kernel and tables as the forward's segments, so the same bits.
        Returns the event recorded after the launch."""
        torch = self.torch
        W, wins, bufs, order = self._windows()
        a, b = wins[w]
        tr, wst, wrg = bufs[w % len(bufs)]
        rec = self._rec_gs
        G, N, C = rec.n_groups, self.N, self.C
        with torch.cuda.stream(stream):
            wst[:b - a].copy_(self._ck[0][a:b])
            wrg[:b - a].copy_(self._ck[1][a:b])
        base, _ = rec.build_table(C)
        live = base['lanes']['nsteps'] > 0
        j = np.arange(b - a, dtype=np.int64)[:, None]        # [J, 1]
        g = np.arange(G, dtype=np.int64)[None, :]            # [1, G]
        ns = np.array([self.ckpt[a + k][1] for k in range(b - a)], np.int64)[:, None]
        tab = np.repeat(base[None], b - a, axis=0)           # [J, G]
        ns_g = rec.gstate[0].numel()
        tab['state'] = wst.data_ptr() + 4 * (j * G + g) * ns_g
        tab['ring'] = wrg.data_ptr() + 4 * (j * rec.ring.numel() + rec.ring_off[None, :])
        tab['trace'] = tr.data_ptr() + 4 * ((g * W + j) * C * N * 3 * 8)
        tab['t0'] = (a + j) * C
        tab['lanes']['nsteps'] = live[None] * ns[:, :, None]
        tab['nsteps'] = ns
        with torch.cuda.stream(stream):   # uploaded in the launch's stream order
            dev = torch.from_numpy(tab.view(np.uint8).reshape(-1).copy()).cuda()
        k = int(rec.block_k[0])
        if not (rec.block_k == k).all():
            raise ValueError('windowed recomputation: one block length')
        cfg = rec.launch_cfg(k, order, None, plain=False)
        rec._run_groups(dev.data_ptr(), (b - a) * G, cfg, stream.cuda_stream)
        ev = torch.cuda.Event()
        ev.record(stream)
        self._tables.append(dev)   # alive until the backward synchronises
        return ev

    def _reverse_windows(self, lam, deta, dGn):
        """Windows last first: each window recomputed in one launch (side
        stream; the last window at the end of forward when eager_recompute),
        then tvbg_adjoint_mpr_groups over the whole window in one launch,
        reading the window's traces in place.  The recomputation of window
        w + 1 overlaps the reverse kernel of window w; events order each
        recomputation after the reverse kernel that last read its buffer."""
        from .engine import DeviceStatus
        torch = self.torch
        lib = nat.load()
        I, N, T, K = self.I, self.N, self.T, self.adj_k
        Gn = (I + 7) // 8
        R = (1 << self.lognh_g) + K
        if self._adj_ring is None or tuple(self._adj_ring.shape) != (Gn, N, R, 8):
            self._adj_ring = torch.zeros((Gn, N, R, 8), dtype=torch.float32, device='cuda')
        else:
            self._adj_ring.zero_()
        ring = self._adj_ring
        threads, cluster, pipe = self.adjoint_shape
        if pipe and self.dmin < 2 * K:
            raise ValueError('pipelined reverse kernel: every delay >= 2 K')
        W, wins, bufs, _ = self._windows()
        nw = len(wins)
        g = np.arange(Gn, dtype=np.int64)[None, :]           # [1, Gn]
        t0s = np.array([wins[w][0] * self.C for w in range(nw)], np.int64)[:, None]
        lens = np.array([sum(self.ckpt[k][1] for k in range(*wins[w])) for w in range(nw)],
                        np.int64)[:, None]
        tr0 = np.array([bufs[w % len(bufs)][0].data_ptr() for w in range(nw)], np.int64)[:, None]
        Gl = np.zeros(Gn * 8, np.float32)
        Gl[:I] = self.G
        tab = np.zeros((nw, Gn), dtype=nat.ADJOINT_GROUP_DTYPE)
        tab['edges_t'] = self.edges_tg.data_ptr()
        tab['row_t'] = self.row_t.data_ptr()
        tab['nodes'] = self.nodes_t.data_ptr()
        tab['seg'] = tr0 + 4 * g * W * self.C * N * 3 * 8
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
        tab['flush_every'] = self.C      # partial sums grouped per segment
        tab['dt'] = np.float32(self.dt)
        tab['G'] = Gl.reshape(1, Gn, 8)
        tab['consts'] = self.consts[:4]
        dev = torch.from_numpy(tab.view(np.uint8).reshape(-1).copy()).cuda()
        row_bytes = Gn * nat.ADJOINT_GROUP_DTYPE.itemsize
        status = DeviceStatus()
        main, side = torch.cuda.current_stream(), self._side
        side.wait_stream(main)
        ready = [None] * nw
        done = [None] * nw
        ready[0], self._eager = self._eager, None
        if ready[0] is None:
            ready[0] = self._recompute_window(0, side)
        for w in range(nw):
            if w + 1 < nw:
                if w >= 1:
                    side.wait_event(done[w - 1])       # buffer (w + 1) % 2 last read by window w - 1
                ready[w + 1] = self._recompute_window(w + 1, side)
            main.wait_event(ready[w])
            nat.check(lib.tvbg_adjoint_mpr_groups(dev.data_ptr() + w * row_bytes, Gn, threads,
                                                  cluster, K, pipe, status.t.data_ptr(),
                                                  main.cuda_stream))
            done[w] = torch.cuda.Event()
            done[w].record(main)
        main.wait_stream(side)
        dG = dGn.sum(1)
        n_prev = len(self._deferred)
        self._defer(self._rec_gs.status, status)
        self.check(n_prev)
        return dG, deta


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
