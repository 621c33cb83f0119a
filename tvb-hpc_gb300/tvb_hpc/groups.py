"""
Lane-interleaved instance groups (tvbg_group_run): the sweep layout for many
instances of one connectome.

Instances that share a delay table (one conduction speed) are packed eight
to a group, one instance per lane of an 8-lane slice; every per-node array
of a group is interleaved over its eight instances (include/tvbg.h, "lane-
interleaved groups"), so a delayed read of one edge is one 32-byte sector
for the group and the edge record is read once for eight instances.  A
group runs on one CTA, or on a cluster of 2 to 16 CTAs that split its
nodes, with one barrier every K = 4 or 8 steps.  Where every delay is at
least 2K - 1 steps the pipelined kernel (tpn 2) overlaps the coupling
gather of block b + 1 with the steps of block b on two thread teams.

The step is the CUDA-order step of the per-instance kernels (same Philox
streams, same ring semantics); the coupling sums are taken in CSR order.
This is the layout of the reference's sweeps -- one parameter point per
GPU thread over a (coupling x speed) grid,
dsl/dsl_cuda/example/cuda_run.py:110-142 and
tvb_hpc/examples/hackathon.py:58-89 -- with the history interleaved by
instance so reads coalesce, CSR edges instead of the dense N x N scan, and
time blocking.
"""

import ctypes

import numpy as np

from . import _native as nat
from .engine import DeviceStatus, _device_ok, _torch
from .network import delays_f32
from .utils import next_pow2

L = nat.GROUP_LANES


def plan_group(dmin, dmax, block_k=None, ks=(8, 4)):
    """(K, lognh) for delays in [dmin, dmax]: K steps per barrier, the
    largest of `ks` with K <= dmin + 1 (the engine library builds K = 8, 4;
    the generated LEMS libraries also 2, 1), nh the smallest power of two
    >= dmax + 1 + K."""
    dmin, dmax = int(dmin), int(dmax)
    fits = [k for k in sorted(ks, reverse=True) if k <= dmin + 1]
    k = int(block_k) if block_k else (fits[0] if fits else 0)
    if k not in ks or k > dmin + 1:
        raise ValueError('group kernel needs K in %s and K <= d_min + 1 (d_min = %d)'
                         % (tuple(ks), dmin))
    nh = max(8, next_pow2(dmax + 1 + k))
    return k, int(np.log2(nh))


MAX_CLUSTER = 16   # CTAs per group; 9..16 are non-portable cluster sizes
PIPELINED = nat.GROUP_PIPELINED   # tvbg_launch.tpn of the pipelined kernel


def pipelined_threads(N, cluster):
    """CTA width of the pipelined kernel for N nodes on `cluster` CTAs: two
    teams of one node per 8-lane slot (0 when that exceeds 1024 threads)."""
    per = -(-N // int(cluster))
    thr = 2 * 32 * -(-(L * per) // 32)
    return thr if thr <= 1024 else 0


def pipelined_shape(gset, clusters=(1, 2, 3, 4, 6, 8, 12, 16), min_ctas=0):
    """(threads, cluster, 0, tpn) of gset on the pipelined kernel's smallest
    cluster that holds one node per slot and gives the set at least min_ctas
    CTAs (when some cluster does), or its plain default shape where the
    pipelined kernel does not apply (short delays, N > 1024).  With few
    groups, min_ctas = the SM count spreads them over the GPU (measured on
    32 groups of N = 84: 704 x 2 8.45 ms per adjoint forward, 256 x 6 8.02)."""
    if gset.can_pipeline:
        fits = [(pipelined_threads(gset.N, c), c) for c in clusters]
        fits = [(t, c) for t, c in fits if t]
        if fits:
            wide = [(t, c) for t, c in fits if gset.n_groups * c >= min_ctas]
            t, c = wide[0] if wide else fits[-1]
            return (t, c, 0, PIPELINED)
    return group_shape(gset.N) + (0, 1)


def group_shape(N, threads=None, cluster=None):
    """(threads, cluster) of a plain group launch: one node per 8-lane slot,
    on the smallest cluster (<= 8 CTAs) whose CTAs stay within 1024 threads;
    beyond 8 CTAs the slots take several nodes.  Measured on the uneven batch
    and the 64 x 64 grid, this beats packing more, smaller CTAs per SM when
    every connectome takes the same rule; the batch tuner
    (autotune.tune_group_batch) picks shapes per connectome by measurement."""
    if cluster is None:
        if threads is not None:
            cluster = min(8, -(-N // (int(threads) // L)))
        else:
            cluster = 1
            while L * -(-N // cluster) > 1024 and cluster < 8:
                cluster *= 2
    if not 1 <= int(cluster) <= MAX_CLUSTER:
        raise ValueError('group kernel: cluster in [1, %d]' % MAX_CLUSTER)
    if threads is None:
        per = -(-N // int(cluster))
        threads = min(1024, 32 * -(-(L * per) // 32))
    return int(threads), int(cluster)


def group_occupancy(cfg):
    lib = nat.load()
    per, sms = ctypes.c_int32(0), ctypes.c_int32(0)
    nat.check(lib.tvbg_group_occupancy(ctypes.byref(cfg), ctypes.byref(per), ctypes.byref(sms)))
    return int(per.value), int(sms.value)


def torch_stack_sc(x):
    "(sin x, cos x) stacked on a new axis before the last one."
    import torch
    return torch.stack([torch.sin(x), torch.cos(x)], dim=-2)


class GroupSet:
    """
    Device-resident instances of one connectome in lane-interleaved groups.

    Same parameters as engine.InstanceSet (model, cfun, scheme, conn, dt,
    couplings, speeds, state0, nparam, delays, rounding, seed, inst_ids,
    bold_period, bold_len, trace_every, trace_len, trace_nobs, flags, cf_b,
    t0); further:
      nsteps  : optional (I,) step counts, used to put instances of similar
                length into the same group (longest first);
      block_k : 4 or 8 steps per barrier (default: 8 when d_min >= 7);
      threads, cluster : launch shape (default: group_shape).
    Couplings must be separable (Linear, Diff, Sigmoidal), or the Kuramoto
    coupling with the Kuramoto model (whose ring keeps sin and cos of the
    phase); the Track-A order runs on the per-instance kernels.

    A lane that takes fewer steps than its group is finished after its run;
    the group's clock advances by the longest lane.
    """

    block_ks = (8, 4)     # block lengths the library's group kernels are built for

    def __init__(self, model, cfun, scheme, conn, dt, couplings, speeds=None, state0=None,
                 nparam=None, delays=None, rounding='ceil', seed=0, inst_ids=None,
                 bold_period=0, bold_len=0, trace_every=0, trace_len=0, trace_nobs=None,
                 trace_csum=False,
                 flags=0, cf_b=None, t0=0, nsteps=None, block_k=None, threads=None,
                 cluster=None, history='zero', delay_tables=None):
        _device_ok()
        torch = _torch()
        self.torch = torch
        lib = nat.load()
        self.model, self.cfun, self.scheme = model, cfun, scheme
        self.model_id, self.consts, self.sigma = model.engine_spec()
        self.cfun_id, cf_a0, cf_b0, self.cf_p = cfun.engine_spec()
        separable = self.cfun_id in (nat.CFUN_LINEAR, nat.CFUN_DIFF, nat.CFUN_SIGMOIDAL)
        kuramoto = (self.model_id, self.cfun_id) == (nat.MODEL_KURAMOTO, nat.CFUN_KURAMOTO)
        lems = self.model_id == nat.MODEL_LEMS and self.cfun_id in (nat.CFUN_LEMS, nat.CFUN_LEMS_SC,
                                                                    nat.CFUN_LEMS_2)
        if not (separable or kuramoto or lems):
            raise ValueError('group kernel: a separable coupling (Linear, Diff, Sigmoidal), or the '
                             'Kuramoto model with the Kuramoto coupling')
        # the Kuramoto coupling (and a LEMS sine coupling) keeps sin and cos of
        # the observable in the ring
        self.channels = 2 if self.cfun_id in (nat.CFUN_KURAMOTO, nat.CFUN_LEMS_SC,
                                              nat.CFUN_LEMS_2) else 1
        self.N = N = int(conn.nnode)
        if N > 65535:
            raise ValueError('group kernel: N < 65536')
        self.ns = model.nsvar
        self.nobs = model.nobs
        self.npar = len(model.param_sym)
        couplings = np.atleast_1d(np.asarray(couplings, np.float32))
        I = self.n = couplings.size
        self.dt = float(dt)
        row = np.asarray(conn.row, np.int64).astype(np.int32)
        col = np.asarray(conn.col, np.int64).astype(np.int32)
        w = np.asarray(conn.wnz, np.float32)
        self.nnz = int(col.size)
        self.row_np, self.col_np, self.w_np = row, col, w
        # delay tables, one per distinct speed
        if delay_tables is not None:
            tables = [np.asarray(d, np.int64).astype(np.int32) for d in delay_tables[0]]
            tab_of = np.broadcast_to(np.asarray(delay_tables[1], np.int64), (I, )).copy()
        elif delays is not None:
            tables = [np.asarray(delays, np.int64).astype(np.int32)]
            tab_of = np.zeros(I, np.int64)
        else:
            sp = np.broadcast_to(np.asarray(speeds, np.float32), (I, )).copy()
            uniq, tab_of = np.unique(sp, return_inverse=True)
            tables = [delays_f32(conn.lnz, s, dt, rounding) for s in uniq]
        self.delay_tables = tables
        plans = [plan_group(d.min() if d.size else 7, d.max() if d.size else 0, block_k,
                            self.block_ks) for d in tables]
        # the pipelined kernel needs d_min >= 2 K - 1 in a group's table; with
        # the pipelined shape, groups of tables that do not qualify take the
        # plain kernel on its default shape (their own launches)
        self.dmin_tab = np.array([int(d.min()) if d.size else 1 << 20 for d in tables], np.int64)
        self.pipe_tab = np.array([int(dm) >= 2 * k - 1 for dm, (k, _) in zip(self.dmin_tab, plans)])
        self.can_pipeline = bool(self.pipe_tab.any())
        # per-node constants shared by every table: in-edge weight sums and
        # the visiting order (in-degree, descending)
        deg = np.diff(row)
        wsum = np.zeros(N, np.float32)
        nz = deg > 0
        if col.size:
            wsum[nz] = np.add.reduceat(w, row[:-1][nz]).astype(np.float32)
        nodes = np.argsort(-deg, kind='stable').astype(np.int32)
        self.row = torch.from_numpy(row).cuda()
        self.wsum = torch.from_numpy(wsum).cuda()
        self.nodes = torch.from_numpy(nodes).cuda()
        eb = []
        for d, (k, lognh) in zip(tables, plans):
            out = np.zeros(max(1, col.size), dtype=np.dtype([('pk', '<u4'), ('w', '<f4')]))
            if col.size:
                nat.check(lib.tvbg_pack_edges_group(N, col.size, row.ctypes.data, col.ctypes.data,
                                                    w.ctypes.data, np.ascontiguousarray(d).ctypes.data,
                                                    lognh, out.ctypes.data))
            eb.append(out)
        self.edges = torch.from_numpy(np.concatenate(eb).view(np.uint8).copy()).cuda()
        self.edge_stride = max(1, col.size)
        # groups: per table, instances longest-first, eight per group
        order_key = (np.zeros(I) if nsteps is None
                     else -np.broadcast_to(np.asarray(nsteps, np.int64), (I, )).astype(np.float64))
        members, gtab = [], []
        for t in range(len(tables)):
            idx = np.nonzero(tab_of == t)[0]
            idx = idx[np.argsort(order_key[idx], kind='stable')]
            for g0 in range(0, idx.size, L):
                members.append(idx[g0:g0 + L])
                gtab.append(t)
        G = self.n_groups = len(members)
        self.members = members
        self.gtab = np.array(gtab, np.int64)
        self.grp_of = np.zeros(I, np.int64)
        self.lane_of = np.zeros(I, np.int64)
        for g, m in enumerate(members):
            self.grp_of[m] = g
            self.lane_of[m] = np.arange(m.size)
        self.block_k = np.array([plans[t][0] for t in self.gtab], np.int32)
        self.lognh = np.array([plans[t][1] for t in self.gtab], np.int32)
        R = (1 << self.lognh.astype(np.int64)) + 8
        ring_len = N * R * L * self.channels
        self.ring_off = np.concatenate([[0], np.cumsum(ring_len)[:-1]]).astype(np.int64)
        self.ring = torch.zeros(int(ring_len.sum()), dtype=torch.float32, device='cuda')
        self.R = R
        self.clear_history()
        self._gi = torch.from_numpy(self.grp_of).cuda()
        self._li = torch.from_numpy(self.lane_of).cuda()
        # state / parameters [G, N, ns, L]
        self.gstate = torch.zeros((G, N, self.ns, L), dtype=torch.float32, device='cuda')
        if state0 is not None:
            st = np.broadcast_to(np.asarray(state0, np.float32), (I, N, self.ns))
            self.set_state(torch.from_numpy(np.array(st, np.float32)).cuda())
        if nparam is None:
            npm = np.broadcast_to(model.node_params(N), (I, N, self.npar))
        else:
            npm = np.asarray(nparam, np.float32)
            if npm.ndim == 1:
                npm = npm.reshape(N, 1)
            if npm.ndim == 2 and npm.shape == (I, N) and self.npar == 1 and I != N:
                npm = npm[:, :, None]
            npm = np.broadcast_to(npm, (I, N, self.npar))
        self.gnparam = torch.zeros((G, N, self.npar, L), dtype=torch.float32, device='cuda')
        self.gnparam[self._gi, :, :, self._li] = torch.from_numpy(
            np.array(npm, np.float32)).cuda()
        if history == 'fill':
            self.fill_history()
        elif history != 'zero':
            raise ValueError("history must be 'zero' or 'fill'")
        # monitors
        fl = int(flags)
        self.bold_period, self.bold_len = int(bold_period), int(bold_len)
        self.gbold = self.gbold_out = None
        if self.bold_period > 0:
            self.gbold = torch.zeros((G, 4, N, L), dtype=torch.float32, device='cuda')
            self.gbold_out = torch.full((G, max(1, self.bold_len), N, L), float('nan'),
                                        dtype=torch.float32, device='cuda')
            fl |= nat.F_BOLD
        self.trace_every, self.trace_len = int(trace_every), int(trace_len)
        self.trace_nobs = int(trace_nobs if trace_nobs is not None else self.nobs)
        # trace_csum: one more trace column, the raw coupling sum of the step
        # (the adjoint's recomputation; pipelined kernel, one-channel couplings)
        self.trace_csum = bool(trace_csum)
        self.trace_cols = self.trace_nobs + (1 if self.trace_csum else 0)
        self.gtrace = None
        if self.trace_every > 0:
            self.gtrace = torch.zeros((G, max(1, self.trace_len), N, self.trace_cols, L),
                                      dtype=torch.float32, device='cuda')
            fl |= nat.F_TRACE
            if self.trace_csum:
                fl |= nat.F_TRACE_CSUM
        # an Euler-Maruyama scheme on a model whose diffusion is zero is Euler
        if getattr(scheme, 'noise', False) and np.any(self.sigma != 0):
            fl |= nat.F_NOISE
        self.flags = fl
        self.seed = int(seed) & ((1 << 64) - 1)
        self.inst_ids = (np.arange(I, dtype=np.uint32) if inst_ids is None
                         else np.asarray(inst_ids, np.uint32))
        self.cf_a = couplings
        self.cf_b = np.float32(cf_b if cf_b is not None else
                               (cf_b0 if isinstance(cf_b0, (int, float, np.number)) else 0.0))
        self.t = np.full(G, int(t0), np.int64)
        self.threads, self.cluster = group_shape(N, threads, cluster)
        self.priority = 0
        self.tpn = 1
        self.status = DeviceStatus()
        self._uploaded = None
        self._streams = None

    def bold_obs(self):
        """Observable feeding the balloon: sin(theta) for Kuramoto, V for G2DO
        (tvb_hpc order W, V), else obs 0 (as engine.InstanceSet)."""
        return 1 if self.model_id in (nat.MODEL_KURAMOTO, nat.MODEL_G2DO) else 0

    # -- per-instance views ------------------------------------------------------
    @property
    def state(self):
        "(I, N, nsvar) copy of the states."
        return self.gstate[self._gi, :, :, self._li]

    def set_state(self, x):
        self.gstate[self._gi, :, :, self._li] = x.to(self.gstate.dtype)

    @property
    def bold_out(self):
        "(I, bold_len, N) BOLD samples."
        return None if self.gbold_out is None else self.gbold_out[self._gi, :, :, self._li]

    @property
    def trace(self):
        "(I, trace_len, N, trace_cols) observable trace (+ coupling sum with trace_csum)."
        return None if self.gtrace is None else self.gtrace[self._gi, :, :, :, self._li]

    def reset(self, state=None):
        "Zero history and monitors; optionally set the state; clocks back to 0."
        self.clear_history()
        if self.gbold is not None:
            self.gbold.zero_()
        if state is not None:
            self.set_state(state)
        self.t[:] = 0

    def clear_history(self):
        """Zero history (every slot holds the observable 0): zeros, or with the
        Kuramoto coupling (sin 0, cos 0) = (0, 1) in every slot."""
        self.ring.zero_()
        if self.channels == 2:
            N = self.N
            for g in range(self.n_groups):
                R = int(self.R[g])
                o = int(self.ring_off[g])
                self.ring[o:o + N * R * L * 2].view(N, R, 2, L)[:, :, 1, :] = 1.0

    def fill_history(self):
        "Every ring slot of every lane holds obs0 of the current state."
        N, C = self.N, self.channels
        o0 = self.gstate[:, :, 0, :]                                  # [G, N, L]
        if C == 2:
            o0 = torch_stack_sc(o0)                                   # [G, N, 2, L]
        else:
            o0 = o0[:, :, None, :]
        for g in range(self.n_groups):
            R = int(self.R[g])
            o = int(self.ring_off[g])
            self.ring[o:o + N * R * L * C].view(N, R, C, L).copy_(
                o0[g][:, None, :, :].expand(N, R, C, L))

    def ring_plain(self, b):
        """Ring of instance b as numpy [nh, N] slot-major (the oracle's layout);
        with the Kuramoto coupling the phase is recovered from (sin, cos) into
        [0, 2 pi) (slots never written read 0)."""
        g, l = int(self.grp_of[b]), int(self.lane_of[b])
        R, C = int(self.R[g]), self.channels
        nh = 1 << int(self.lognh[g])
        o = int(self.ring_off[g])
        r = self.ring[o:o + self.N * R * L * C].view(self.N, R, C, L)[:, :nh, :, l]
        r = r.cpu().numpy()
        if C == 2:
            th = np.mod(np.arctan2(r[:, :, 0], r[:, :, 1]), 2 * np.pi)
            return np.ascontiguousarray(th.T.astype(np.float32))
        return np.ascontiguousarray(r[:, :, 0].T)

    # -- launches -------------------------------------------------------------------
    def set_couplings(self, couplings):
        "Per-instance coupling values (I,) for the following prepare() calls."
        a = np.atleast_1d(np.asarray(couplings, np.float32))
        if a.shape != (self.n, ):
            raise ValueError('couplings: one value per instance (%d)' % self.n)
        self.cf_a = a.copy()

    def set_nparam(self, nparam):
        "Per-instance node parameters, [I, N, npar] (or [I, N] with one parameter), on the device."
        torch = self.torch
        npm = np.asarray(nparam, np.float32).reshape(self.n, self.N, self.npar)
        self.gnparam[self._gi, :, :, self._li] = torch.from_numpy(np.array(npm, np.float32)).cuda()

    def build_table(self, nsteps):
        "Numpy tvbg_group table for the next nsteps (scalar or (I,))."
        G, N = self.n_groups, self.N
        steps = np.broadcast_to(np.asarray(nsteps, np.int64), (self.n, )).astype(np.int64)
        tab = np.zeros(G, dtype=nat.GROUP_DTYPE)
        gi = np.arange(G, dtype=np.int64)
        tab['edges'] = self.edges.data_ptr() + 8 * self.edge_stride * self.gtab
        tab['row'] = self.row.data_ptr()
        tab['wsum'] = self.wsum.data_ptr()
        tab['nodes'] = self.nodes.data_ptr()
        tab['ring'] = self.ring.data_ptr() + 4 * self.ring_off
        tab['state'] = self.gstate.data_ptr() + 4 * gi * N * self.ns * L
        tab['nparam'] = self.gnparam.data_ptr() + 4 * gi * N * self.npar * L
        if self.gbold is not None:
            tab['bold'] = self.gbold.data_ptr() + 4 * gi * 4 * N * L
            tab['bold_out'] = self.gbold_out.data_ptr() + 4 * gi * self.gbold_out.shape[1] * N * L
        if self.gtrace is not None:
            tab['trace'] = (self.gtrace.data_ptr()
                            + 4 * gi * self.gtrace.shape[1] * N * self.trace_cols * L)
        tab['t0'] = self.t
        tab['N'] = N
        tab['nnz'] = self.nnz
        tab['lognh'] = self.lognh
        tab['model'] = self.model_id
        tab['cfun'] = self.cfun_id
        tab['flags'] = self.flags
        tab['trace_every'] = max(1, self.trace_every)
        tab['trace_len'] = max(1, self.trace_len)
        tab['trace_nobs'] = self.trace_nobs
        tab['bold_period'] = max(1, self.bold_period)
        tab['bold_len'] = self.bold_len
        tab['bold_obs'] = self.bold_obs()
        tab['dmin'] = np.minimum(self.dmin_tab[self.gtab], 1 << 30)
        tab['seed_lo'] = self.seed & 0xffffffff
        tab['seed_hi'] = (self.seed >> 32) & 0xffffffff
        tab['dt'] = np.float32(self.dt)
        tab['sqrt_dt'] = np.sqrt(np.float32(self.dt)).astype(np.float32)
        tab['dt_bold'] = np.float32(self.dt / 1000.0)
        tab['cf_b'] = self.cf_b
        tab['cf_p'] = np.asarray(self.cf_p, np.float32)
        tab['sigma'] = self.sigma
        tab['consts'] = self.consts
        # lanes: instance b sits in group grp_of[b], lane lane_of[b]; padding
        # lanes keep nsteps = 0
        lanes = tab['lanes']
        gi_, li_ = self.grp_of, self.lane_of
        lanes['cf_a'][gi_, li_] = self.cf_a
        lanes['nsteps'][gi_, li_] = steps
        lanes['inst_id'][gi_, li_] = self.inst_ids
        gmax = lanes['nsteps'].max(axis=1).astype(np.int64)
        tab['nsteps'] = gmax
        return tab, gmax

    def set_shape(self, threads=None, cluster=None, priority=0, tpn=1):
        """Launch shape of the following prepare() calls: CTA width and
        cluster size (group_shape rules for what is left out), the launch
        priority (0 = the stream's; lower numbers are dispatched first) and
        tpn = 2 for the pipelined kernel (threads then count both teams;
        needs one node per slot and a table with d_min >= 2 K - 1; groups of
        the other tables keep the plain kernel on group_shape)."""
        tpn = int(tpn)
        if tpn == PIPELINED:
            if not self.can_pipeline:
                raise ValueError('pipelined group kernel needs d_min >= 2 K - 1')
            cluster = int(cluster or 1)
            thr = pipelined_threads(self.N, cluster) if threads is None else int(threads)
            if not thr or thr % 64 or thr > 1024 or cluster * (thr // (2 * L)) < self.N:
                raise ValueError('pipelined group kernel: two teams of one node per slot, '
                                 'a multiple of 64 threads <= 1024')
            if not 1 <= cluster <= MAX_CLUSTER:
                raise ValueError('group kernel: cluster in [1, %d]' % MAX_CLUSTER)
            self.threads, self.cluster = thr, cluster
        elif tpn in (0, 1):
            self.threads, self.cluster = group_shape(self.N, threads, cluster)
        else:
            raise ValueError('tpn: 1 (plain) or 2 (pipelined)')
        self.priority = int(priority)
        self.tpn = max(1, tpn)

    @property
    def shape(self):
        "(threads, cluster, priority, tpn) of the next launches."
        return (self.threads, self.cluster, self.priority, self.tpn)

    def launch_cfg(self, block_k, order=None, priority=None, plain=False):
        """Launch record of one block length; `plain` forces the plain kernel
        on its default shape (groups whose delays do not allow pipelining)."""
        cfg = nat.tvbg_launch()
        cfg.model, cfg.cfun = self.model_id, self.cfun_id
        if plain and self.tpn == PIPELINED:
            cfg.threads, cfg.cluster = group_shape(self.N)
            cfg.tpn = 1
        else:
            cfg.threads, cfg.cluster = self.threads, self.cluster
            cfg.tpn = self.tpn
        cfg.priority = self.priority if priority is None else int(priority)
        cfg.block_k = int(block_k)
        cfg.d_status = self.status.t.data_ptr()
        cfg.d_order = order.data_ptr() if order is not None else None
        return cfg

    def prepare(self, nsteps, priorities=None):
        """Upload the group tables for the next nsteps: one launch per block
        length, groups in longest-first order.  With `priorities` (one launch
        priority per group) the groups of each block length are split into
        one launch per priority, so that concurrent launches dispatch the
        CTAs of long groups first.  Returns the launch list."""
        torch = self.torch
        tab, gmax = self.build_table(nsteps)
        dev = torch.from_numpy(tab.view(np.uint8).copy()).cuda()
        prio = (np.full(self.n_groups, self.priority, np.int64) if priorities is None
                else np.asarray(priorities, np.int64))
        pipe = self.pipe_tab[self.gtab] if self.tpn == PIPELINED else np.ones(self.n_groups, bool)
        if self.trace_csum and (self.tpn != PIPELINED or not pipe.all()):
            raise ValueError('trace_csum: every group on the pipelined kernel (set_shape tpn=2, '
                             'delays >= 2 K - 1)')
        launches = []
        for k in sorted(set(self.block_k.tolist())):
            for pk in (True, False):
                sel = (self.block_k == k) & (pipe == pk)
                for pr in sorted(set(prio[sel].tolist())):
                    idx = np.nonzero(sel & (prio == pr))[0]
                    idx = idx[np.argsort(-gmax[idx], kind='stable')].astype(np.int32)
                    order = torch.from_numpy(idx).cuda()
                    launches.append((dev, order, int(idx.size),
                                     self.launch_cfg(k, order, pr, plain=not pk)))
        self._uploaded = (launches, gmax)
        return launches, gmax

    def prepare_segments(self, segs):
        """Launch lists of consecutive segments [(t0, nsteps), ...] of every
        instance, built together: one table per segment (t0 and step counts
        set), uploaded in one copy, and one order array per launch shared by
        all segments.  Each segment's launch list runs like prepare()'s; the
        caller runs them in order (the clocks are set from t0)."""
        torch = self.torch
        # one table, then t0 and the step counts of each segment set in bulk
        # (live lanes step, padding lanes keep 0)
        base, _ = self.build_table(1)
        live = base['lanes']['nsteps'] > 0                  # [G, L]
        t0s = np.array([t for t, _ in segs], np.int64)
        ns = np.array([n for _, n in segs], np.int64)
        allt = np.repeat(base[None], len(segs), axis=0)    # [S, G]
        allt['t0'] = t0s[:, None]
        allt['lanes']['nsteps'] = live[None] * ns[:, None, None]
        allt['nsteps'] = np.where(live.any(axis=1)[None], ns[:, None], 0)
        dev = torch.from_numpy(allt.view(np.uint8).reshape(-1).copy()).cuda()
        G = self.n_groups
        pipe = self.pipe_tab[self.gtab] if self.tpn == PIPELINED else np.ones(G, bool)
        if self.trace_csum and (self.tpn != PIPELINED or not pipe.all()):
            raise ValueError('trace_csum: every group on the pipelined kernel (set_shape tpn=2, '
                             'delays >= 2 K - 1)')
        shapes = []
        for k in sorted(set(self.block_k.tolist())):
            for pk in (True, False):
                idx = np.nonzero((self.block_k == k) & (pipe == pk))[0].astype(np.int32)
                if idx.size:
                    order = torch.from_numpy(idx).cuda()
                    shapes.append((order, int(idx.size), self.launch_cfg(k, order, None, plain=not pk)))
        row = G * nat.GROUP_DTYPE.itemsize
        out = []
        for s in range(len(segs)):
            view = dev[s * row:(s + 1) * row]
            out.append([(view, order, n, cfg) for order, n, cfg in shapes])
        self._segments_keep = dev
        return out

    def launch(self, launches=None, stream=None):
        """Enqueue the prepared launches on `stream` (a torch stream, default
        the current one); launches of different block lengths run
        concurrently on forked streams joined back into `stream`."""
        torch = self.torch
        launches = launches if launches is not None else self._uploaded[0]
        main = stream if stream is not None else torch.cuda.current_stream()
        if len(launches) == 1:
            dev, order, n, cfg = launches[0]
            self._run_groups(dev.data_ptr(), n, cfg, main.cuda_stream)
            return
        if self._streams is None or len(self._streams) < len(launches):
            self._streams = [torch.cuda.Stream() for _ in launches]
        for (dev, order, n, cfg), st in zip(launches, self._streams):
            st.wait_stream(main)
            self._run_groups(dev.data_ptr(), n, cfg, st.cuda_stream)
        for st in self._streams[:len(launches)]:
            main.wait_stream(st)

    def _run_groups(self, dev_ptr, n, cfg, stream):
        "One group launch through the engine library."
        nat.check(nat.load().tvbg_group_run(dev_ptr, n, ctypes.byref(cfg), stream))

    def advance(self, gmax):
        "Move the group clocks after a launch of the prepared tables."
        self.t += gmax

    def run(self, nsteps, stream=None, check=True):
        "Advance every instance by nsteps (scalar or per instance)."
        launches, gmax = self.prepare(nsteps)
        self.launch(launches, stream)
        self.advance(gmax)
        if check:
            self.torch.cuda.synchronize()
            self.status.check()

    @property
    def node_steps_per_step(self):
        return float(self.n * self.N)


class GroupBatch:
    """
    Several GroupSets (different connectomes, N and step counts) in one
    launch set: every set's launches go on their own forked stream and the
    whole batch can be captured into one CUDA graph.

    shapes: None (each set's current shape), 'tune' (autotune.tune_group_batch
    picks a launch shape per set, and whether to band the groups into launch
    priorities, by the batch's measured makespan), or a list of (threads,
    cluster[, priority[, tpn]]) per set (GroupSet.set_shape).
    step_ms: optional per-set time of one step of one group (ms); the groups
    are then banded by their estimated run time (steps x step_ms) into
    launch priorities, the longest groups of every set first, so the CTA
    dispatcher approximates a longest-first schedule over the whole batch
    instead of within each launch.
    """

    PRIORITY_LEVELS = 6   # CUDA stream priorities 0 (least) .. -5 (greatest)

    def __init__(self, sets, nsteps, shapes=None, step_ms=None, rank_priority=False):
        torch = _torch()
        self.torch = torch
        self.sets = list(sets)
        self.nsteps = [np.broadcast_to(np.asarray(n, np.int64), (s.n, )).astype(np.int64)
                       for s, n in zip(self.sets, nsteps)]
        self.tuning = None
        if isinstance(shapes, str):
            if shapes != 'tune':
                raise ValueError("shapes: None, 'tune' or one (threads, cluster[, priority[, tpn]]) "
                                 "per set")
            from .autotune import tune_group_batch
            self.tuning = tune_group_batch(self.sets, self.nsteps)
            shapes = self.tuning['shapes']
            if step_ms is None:
                step_ms = self.tuning.get('step_ms')
        if shapes is not None:
            if len(shapes) != len(self.sets):
                raise ValueError('shapes: one (threads, cluster[, priority[, tpn]]) per set')
            for s, sh in zip(self.sets, shapes):
                s.set_shape(*sh)
        self.shapes = [s.shape for s in self.sets]
        self.step_ms = step_ms
        self.status = DeviceStatus()
        self.plans = []
        prios = self.group_priorities(step_ms) if step_ms is not None else [None] * len(self.sets)
        for s, n, pr in zip(self.sets, self.nsteps, prios):
            launches, gmax = s.prepare(n, pr)
            for _, _, _, cfg in launches:
                cfg.d_status = self.status.t.data_ptr()
            self.plans.append((s, launches, gmax))
        # longest sets first (their streams are forked first)
        self.plans.sort(key=lambda p: -float(p[2].max(initial=0)) * p[0].N)
        if rank_priority:
            # launch priority by that rank (the longest set at the greatest
            # priority), so every replay of a captured graph dispatches the
            # CTAs of the long chains first whatever order its branches start in
            n = len(self.plans)
            for r, (s, launches, _) in enumerate(self.plans):
                for _, _, _, cfg in launches:
                    cfg.priority = -max(0, min(self.PRIORITY_LEVELS - 1, n - 1 - r))
        self.rank_priority = bool(rank_priority)
        self.streams = [torch.cuda.Stream() for _ in self.plans]
        self.graph = None

    def group_priorities(self, step_ms):
        """Launch priority per group of every set: estimated run time
        (longest lane's steps x the set's step time) in PRIORITY_LEVELS equal
        bands of the batch's longest, the longest band at the greatest
        priority (the most negative number)."""
        est = []
        for s, n, tau in zip(self.sets, self.nsteps, step_ms):
            gmax = np.array([n[m].max(initial=0) for m in s.members], np.float64)
            est.append(gmax * float(tau))
        top = max((e.max(initial=0.0) for e in est), default=0.0)
        levels = self.PRIORITY_LEVELS
        out = []
        for e in est:
            band = np.zeros(e.size, np.int64) if top <= 0 else np.minimum(
                levels - 1, np.floor(levels * e / top).astype(np.int64))
            out.append(-band)
        return out

    @property
    def node_steps(self):
        return float(sum((s.N * n).sum() for s, n in zip(self.sets, self.nsteps)))

    @property
    def n_launches(self):
        return sum(len(p[1]) for p in self.plans)

    def launch(self, stream=None):
        torch = self.torch
        main = stream or torch.cuda.current_stream()
        for (s, launches, _), st in zip(self.plans, self.streams):
            st.wait_stream(main)
            with torch.cuda.stream(st):
                s.launch(launches, st)
        for st in self.streams:
            main.wait_stream(st)

    def capture(self):
        torch = self.torch
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        cap = torch.cuda.Stream()
        with torch.cuda.stream(cap):
            with torch.cuda.graph(g, stream=cap):
                self.launch(cap)
        self.graph = g
        return g

    def replay(self):
        self.graph.replay()

    def run(self, check=True):
        if self.graph is not None:
            self.replay()
        else:
            self.launch()
        if check:
            self.torch.cuda.synchronize()
            self.status.check()
