"""
The GB300 network-step engine: instance tables, ring planning and launches.

An *instance* is one parameter point of a sweep (one (G, speed, per-node
parameters, seed) tuple) on one connectome.  The engine keeps for every
instance, resident in device memory:
  - its history ring (node-major, skewed, length nh = 2^k > max delay + 1),
  - its state [N][nsvar], per-node parameters, balloon state and outputs,
and describes it to the kernels with one ``tvbg_instance`` record
(include/tvbg.h).  Instances that share a speed share one packed edge table.

Launch planning:
  - a ring of N * nh * 4 bytes that fits the shared memory of one CTA is
    staged there by TMA bulk copies (flag F_SMEM_RING); otherwise the kernel
    works on the ring in global memory (L2-resident when it fits);
  - instances are grouped by (ring placement, nh) so each launch reserves
    only the shared memory its rings need;
  - sync_every = min(d_min + 1, nh - d_max - 1) block barriers (see
    tvbg_step.cuh) and the gather width tpn come from the planner/autotuner.

Reference behaviour mirrored: the per-instance time loop of
dsl/dsl_cuda/example/cuda_run.py:124-142 (one launch per chunk of steps,
state and history resident on the device between launches) and the
subject batch of examples/hcp100.py:65-118.
"""

import ctypes
import math

import numpy as np

from . import _native as nat
from .network import delays_f32
from .utils import getLogger, next_pow2

LOG = getLogger(__name__)

_SMEM_RESERVE = 1024  # static shared memory of the step kernel + slack


def _torch():
    import torch
    return torch


def _device_ok():
    torch = _torch()
    if not torch.cuda.is_available():
        raise RuntimeError('the GB300 engine needs a CUDA device; there is no CPU fallback')


def ring_index(N, lognh, node, slot):
    "Physical index of (node, time slot) in a skewed node-major ring."
    nh = 1 << lognh
    node = np.asarray(node, np.int64)
    slot = np.asarray(slot, np.int64)
    return node * nh + ((slot + node) & (nh - 1))


def unskew_ring(ring_flat, N, lognh):
    "Skewed node-major ring (N*nh,) -> plain slot-major [nh, N] (numpy)."
    nh = 1 << lognh
    r = np.asarray(ring_flat).reshape(N, nh)
    out = np.empty((nh, N), r.dtype)
    s = np.arange(nh)
    for j in range(N):
        out[:, j] = r[j, (s + j) & (nh - 1)]
    return out


def pack_edges(row, col, weights, delays, lognh):
    "tvbg_pack_edges through the C ABI (host helper) -> structured numpy array."
    lib = nat.load()
    row = np.ascontiguousarray(row, np.int32)
    col = np.ascontiguousarray(col, np.int32)
    w = np.ascontiguousarray(weights, np.float32)
    d = np.ascontiguousarray(delays, np.int32)
    N = row.size - 1
    out = np.zeros(col.size, dtype=np.dtype([('pk', '<u4'), ('w', '<f4')]))
    nat.check(lib.tvbg_pack_edges(N, col.size, row.ctypes.data, col.ctypes.data, w.ctypes.data,
                                  d.ctypes.data, int(lognh), out.ctypes.data if col.size else None))
    return out


def pack_edges_blocked(row, col, weights, delays, lognh):
    "tvbg_pack_edges_blocked (padded ring layout of the time-blocked kernel)."
    lib = nat.load()
    row = np.ascontiguousarray(row, np.int32)
    col = np.ascontiguousarray(col, np.int32)
    w = np.ascontiguousarray(weights, np.float32)
    d = np.ascontiguousarray(delays, np.int32)
    N = row.size - 1
    out = np.zeros(col.size, dtype=np.dtype([('pk', '<u4'), ('w', '<f4')]))
    nat.check(lib.tvbg_pack_edges_blocked(N, col.size, row.ctypes.data, col.ctypes.data,
                                          w.ctypes.data, d.ctypes.data, int(lognh),
                                          out.ctypes.data if col.size else None))
    return out


def plan_ring(dmin, dmax, extra=0, order='cuda'):
    """
    (lognh, sync_every, extra_flags) for delays in [dmin, dmax]: the smallest
    power-of-two ring with nh >= dmax + 2 (+ extra), then the largest barrier
    interval that keeps the read-after-write and overwrite constraints:
      CUDA order  : value of step t written to slot t+1, first read at
                    t + 1 + dmin  ->  sync <= dmin + 1, sync <= nh - dmax - 1;
      Track-A order: value of step t written to slot t after the gather,
                    first read at t + dmin -> sync <= dmin, sync <= nh - dmax;
                    with zero delays every step needs a barrier between the
                    gather and the update as well (F_MIDSYNC).
    """
    nh = max(4, next_pow2(int(dmax) + 2 + int(extra)))
    dmin, dmax = int(dmin), int(dmax)
    if order == 'cuda':
        return int(math.log2(nh)), max(1, min(dmin + 1, nh - dmax - 1)), 0
    if order != 'tracka':
        raise ValueError("order must be 'cuda' or 'tracka'")
    if dmin == 0:
        return int(math.log2(nh)), 1, nat.F_TRACKA | nat.F_MIDSYNC
    return int(math.log2(nh)), max(1, min(dmin, nh - dmax)), nat.F_TRACKA


def max_smem():
    lib = nat.load()
    v = ctypes.c_int32(0)
    nat.check(lib.tvbg_max_smem(ctypes.byref(v)))
    return int(v.value)


class DeviceStatus:
    "A device int the kernels set to their first error code."

    def __init__(self):
        torch = _torch()
        self.t = torch.zeros(1, dtype=torch.int32, device='cuda')

    def reset(self):
        self.t.zero_()

    def check(self):
        v = int(self.t.item())
        if v != 0:
            raise nat.TvbgError(v, 'device-side check failed in a step kernel')


class InstanceSet:
    """
    Device-resident instances sharing (model, coupling, scheme) and one
    connectome; the building block of Sweep, batch and serving.

    Parameters
    ----------
    model, cfun, scheme : tvb_hpc model / coupling / scheme objects
    conn : Connectivity (CSR, float32 weights and lengths)
    dt : float, ms
    speeds : (I,) conduction speeds (mm/ms), or None with ``delays`` given
    couplings : (I,) coupling `a` per instance (global coupling G)
    state0 : (I, N, nsvar) initial state, or (N, nsvar) shared
    nparam : (I, N, npar) or (N, npar) per-node parameters (default: const)
    delays : optional (nnz,) int delays shared by all instances
    delay_tables : optional (tables, table_of): a list of (nnz,) int delay
              arrays and, per instance, the index of its table
    rounding : 'ceil' | 'trunc' | 'dsl' delay rule (see network.delays_f32)
    seed : uint64 Philox seed; inst_ids : (I,) request-local ids (key word 1)
    history : 'zero' (zero history before t0) or 'fill' (state0 everywhere)
    order : 'cuda' (gather, drift, update, write slot t+1: the CUDA DSL
            kernels, dsl/dsl_cuda/CUDAmodels/kuramoto.c:85-139) or 'tracka'
            (the fused loopy kernel: gather reads slot t before the model
            writes obs(x_t) into it, tvb_hpc/transforms.py:30-42)
    bold_period, bold_len : BOLD sampling (steps) and rows to keep
    trace_every, trace_len, trace_nobs : observable trace sampling
    flags : extra TVBG_F_* bits (e.g. F_WRAP_FMOD)
    cf_b : coupling offset b (default from cfun.param)
    blocked : 'auto' | True | False -- use the time-blocked kernel (K steps
              per block, padded ring rows) where the coupling is separable,
              the order is 'cuda' and d_min + 1 >= 4
    warps : CTA width of the blocked kernel in warps (default: autotuned)
    """

    def __init__(self, model, cfun, scheme, conn, dt, couplings, speeds=None, state0=None,
                 nparam=None, delays=None, rounding='ceil', seed=0, inst_ids=None,
                 history='zero', bold_period=0, bold_len=0, trace_every=0, trace_len=0,
                 trace_nobs=None, flags=0, cf_b=None, nh_extra=0, t0=0, order='cuda',
                 sync_every=None, blocked='auto', warps=None, trace_csum=False,
                 pipeline=True, delay_tables=None):
        _device_ok()
        torch = _torch()
        self.torch = torch
        self.model, self.cfun, self.scheme = model, cfun, scheme
        self.model_id, self.consts, self.sigma = model.engine_spec()
        self.cfun_id, cf_a0, cf_b0, self.cf_p = cfun.engine_spec()
        self.N = N = int(conn.nnode)
        self.ns = model.nsvar
        self.nobs = model.nobs
        if N > 1024:
            raise ValueError('the step kernel holds one node per lane: N <= 1024')
        couplings = np.atleast_1d(np.asarray(couplings, np.float32))
        I = self.n = couplings.size
        self.dt = float(dt)
        row = np.asarray(conn.row, np.int64).astype(np.int32)
        col = np.asarray(conn.col, np.int64).astype(np.int32)
        w = np.asarray(conn.wnz, np.float32)
        self.row_np, self.col_np, self.w_np = row, col, w
        self.nnz = int(col.size)
        # delay tables: one per distinct speed
        if delay_tables is not None:
            tables = [np.asarray(d, np.int64).astype(np.int32) for d in delay_tables[0]]
            tab_of = np.broadcast_to(np.asarray(delay_tables[1], np.int64), (I, )).copy()
            if tab_of.min() < 0 or tab_of.max() >= len(tables):
                raise ValueError('delay table index out of range')
            self.speeds = None
        elif delays is not None:
            tables = [np.asarray(delays, np.int64).astype(np.int32)]
            tab_of = np.zeros(I, np.int64)
            self.speeds = None
        else:
            speeds = np.broadcast_to(np.asarray(speeds, np.float32), (I, )).copy()
            self.speeds = speeds
            uniq, tab_of = np.unique(speeds, return_inverse=True)
            tables = [delays_f32(conn.lnz, s, dt, rounding) for s in uniq]
        self.delay_tables = tables
        self.tab_of = tab_of
        # ring plan per table
        plans = []
        for d in tables:
            dmin = int(d.min()) if d.size else 0
            dmax = int(d.max()) if d.size else 0
            plans.append(plan_ring(dmin, dmax, nh_extra, order))
        self.order = order
        self.lognh = np.array([plans[t][0] for t in tab_of], np.int32)
        self.sync_every = np.array([plans[t][1] for t in tab_of], np.int32)
        self.order_flags = np.array([plans[t][2] for t in tab_of], np.uint32)
        if sync_every is not None:  # tighter barrier interval (never looser than planned)
            self.sync_every = np.minimum(self.sync_every, int(sync_every)).astype(np.int32)
        # time-blocked kernel where it applies (K steps per block)
        separable = self.cfun_id in (nat.CFUN_LINEAR, nat.CFUN_DIFF, nat.CFUN_SIGMOIDAL)
        can_block = (separable and order == 'cuda' and self.model_id in (
            nat.MODEL_G2DO, nat.MODEL_MPR, nat.MODEL_LINEAR, nat.MODEL_G2DOSC))
        tab_k, tab_pipe = [], []
        smem_total = max_smem() - _SMEM_RESERVE
        for t, d in enumerate(tables):
            dmin = int(d.min()) if d.size else 0
            # warp-specialised pipeline needs K <= (d_min + 1) / 2
            kp = 8 if (dmin + 1) // 2 >= 8 else (4 if (dmin + 1) // 2 >= 4 else 0)
            k = kp or (8 if dmin + 1 >= 8 else (4 if dmin + 1 >= 4 else 0))
            # the block's scratch (double-buffered sums, normals, BOLD inputs)
            # must fit one CTA's shared memory next to the descriptor
            while k and 4 * (2 * k * N * (2 + self.ns) + 4 * N) + 32 > smem_total:
                k, kp = k // 2 if k > 4 else 0, kp // 2 if kp > 4 else 0
            if blocked is False or not can_block or plans[t][0] > 16:
                k, kp = 0, 0
            elif blocked is True and k == 0:
                raise ValueError('blocked kernel needs d_min + 1 >= 4 (d_min = %d)' % dmin)
            tab_k.append(k)
            tab_pipe.append(bool(kp) and pipeline)
        self.block_k = np.array([tab_k[t] for t in tab_of], np.int32)
        self.pipe = np.array([tab_pipe[t] for t in tab_of], bool)
        self.warps = warps
        # packed edges per (table), device
        ebufs, eoff = [], []
        off = 0
        for t, d in enumerate(tables):
            if tab_k[t]:
                e = pack_edges_blocked(row, col, w, d, plans[t][0])
            else:
                e = pack_edges(row, col, w, d, plans[t][0])
            ebufs.append(e)
            eoff.append(off)
            off += max(1, e.size)
        edges = np.zeros(off, dtype=np.dtype([('pk', '<u4'), ('w', '<f4')]))
        for t, e in enumerate(ebufs):
            edges[eoff[t]:eoff[t] + e.size] = e
        self.edges = torch.from_numpy(edges.view(np.uint8).copy()).cuda()
        self.edge_off = eoff
        self.row = torch.from_numpy(row).cuda()
        # rings (16-byte aligned): N * stride floats, stride = nh (per-step
        # kernel) or nh + GHOST (time-blocked kernel)
        self.stride = ((1 << self.lognh.astype(np.int64))
                       + np.where(self.block_k > 0, nat.GHOST, 0)).astype(np.int64)
        ring_len = N * self.stride
        self.ring_off = np.concatenate([[0], np.cumsum(ring_len)[:-1]]).astype(np.int64)
        self.ring = torch.zeros(int(ring_len.sum()), dtype=torch.float32, device='cuda')
        # state and parameters
        if state0 is None:
            st = np.zeros((I, N, self.ns), np.float32)
        else:
            st = np.broadcast_to(np.asarray(state0, np.float32), (I, N, self.ns)).copy()
        self.state = torch.from_numpy(st).cuda()
        npar = len(model.param_sym)
        if nparam is None:
            npm = np.broadcast_to(model.node_params(N), (I, N, npar)).copy()
        else:
            npm = np.asarray(nparam, np.float32)
            if npm.ndim == 1:
                npm = npm.reshape(N, 1)
            if npm.ndim == 2 and npm.shape == (I, N) and npar == 1 and I != N:
                npm = npm[:, :, None]
            npm = np.broadcast_to(npm, (I, N, npar)).copy()
        self.nparam = torch.from_numpy(np.ascontiguousarray(npm, np.float32)).cuda()
        if history == 'fill':
            self.fill_history(st)
        elif history != 'zero':
            raise ValueError("history must be 'zero' or 'fill'")
        # monitors
        self.bold_period = int(bold_period)
        self.bold_len = int(bold_len)
        self.bold = None
        self.bold_out = None
        fl = int(flags)
        if self.bold_period > 0:
            # deviation state (s, f-1, v-1, q-1); rest is zero
            self.bold = torch.zeros((I, 4, N), dtype=torch.float32, device='cuda')
            self.bold_out = torch.full((I, max(1, self.bold_len), N), float('nan'),
                                       dtype=torch.float32, device='cuda')
            fl |= nat.F_BOLD
        self.trace_every = int(trace_every)
        self.trace_len = int(trace_len)
        self.trace_nobs = int(trace_nobs if trace_nobs is not None else self.nobs)
        # with trace_csum each trace row also carries the step's raw coupling sum
        self.trace_cols = self.trace_nobs + (1 if trace_csum else 0)
        self.trace = None
        if self.trace_every > 0:
            self.trace = torch.zeros((I, max(1, self.trace_len), N, self.trace_cols),
                                     dtype=torch.float32, device='cuda')
            fl |= nat.F_TRACE
            if trace_csum:
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
        self.t = np.full(I, int(t0), np.int64)
        # smem placement
        cap = max_smem()
        self.ring_bytes = N * self.stride * 4
        self.smem_cap = cap
        self.table = None
        self.table_dev = None

    # -- helpers ---------------------------------------------------------------
    def fill_history(self, st):
        "Fill every ring slot with obs0 of the initial state (history='fill')."
        torch = self.torch
        N = self.N
        obs0 = st[:, :, 0]
        for b in range(self.n):
            R = int(self.stride[b])
            o = int(self.ring_off[b])
            self.ring[o:o + N * R] = torch.from_numpy(
                np.repeat(obs0[b], R).astype(np.float32)).cuda()

    def threads(self, blocked_k=0):
        own = 32 * ((self.N + 31) // 32)
        if blocked_k and self.warps:
            return min(1024, max(own + 32, 32 * int(self.warps)))
        if blocked_k:
            return min(1024, max(own + 32, 256))
        return own

    def smem_ring_limit(self, threads, blocked_k=0):
        if blocked_k:
            ns = self.ns
            aux = 4 * (2 * blocked_k * self.N * (2 + ns) + 4 * self.N) + 32
            return self.smem_cap - aux - _SMEM_RESERVE
        return self.smem_cap - 4 * threads - 16 - _SMEM_RESERVE

    def build_table(self, nsteps, smem_allowed=True):
        "Fill the numpy instance table for the next `nsteps` steps (vectorised)."
        I, N = self.n, self.N
        tab = np.zeros(I, dtype=nat.INSTANCE_DTYPE)
        bidx = np.arange(I, dtype=np.int64)
        eoff = np.asarray(self.edge_off, np.int64)[self.tab_of]
        tab['edges'] = self.edges.data_ptr() + 8 * eoff
        tab['row'] = self.row.data_ptr()
        tab['ring'] = self.ring.data_ptr() + 4 * self.ring_off
        tab['state'] = self.state.data_ptr() + 4 * bidx * N * self.ns
        tab['nparam'] = self.nparam.data_ptr() + 4 * bidx * N * self.nparam.shape[2]
        if self.bold is not None:
            tab['bold'] = self.bold.data_ptr() + 4 * bidx * 4 * N
            tab['bold_out'] = self.bold_out.data_ptr() + 4 * bidx * self.bold_out.shape[1] * N
        if self.trace is not None:
            tab['trace'] = (self.trace.data_ptr()
                            + 4 * bidx * self.trace.shape[1] * N * self.trace_cols)
        tab['t0'] = self.t
        tab['trace_stride'] = N * self.trace_cols
        tab['nsteps'] = np.broadcast_to(np.asarray(nsteps, np.int64), (I, )).astype(np.int32)
        tab['N'] = N
        tab['nnz'] = self.nnz
        tab['lognh'] = self.lognh
        tab['model'] = self.model_id
        tab['cfun'] = self.cfun_id
        limit = np.array([self.smem_ring_limit(self.threads(k), k) for k in self.block_k])
        fits = (self.ring_bytes <= limit) if smem_allowed else np.zeros(I, bool)
        fl = (self.flags | self.order_flags).astype(np.uint32)
        fl = np.where(self.pipe, fl | nat.F_PIPELINE, fl).astype(np.uint32)
        tab['flags'] = np.where(fits, fl | nat.F_SMEM_RING, fl).astype(np.uint32)
        tab['sync_every'] = self.sync_every
        tab['trace_every'] = max(1, self.trace_every)
        tab['trace_len'] = max(1, self.trace_len)
        tab['trace_nobs'] = self.trace_nobs
        tab['bold_period'] = max(1, self.bold_period)
        tab['bold_len'] = self.bold_len
        tab['bold_obs'] = self.bold_obs()
        tab['seed_lo'] = self.seed & 0xffffffff
        tab['seed_hi'] = (self.seed >> 32) & 0xffffffff
        tab['inst_id'] = self.inst_ids
        tab['dt'] = np.float32(self.dt)
        tab['sqrt_dt'] = np.sqrt(np.float32(self.dt)).astype(np.float32)
        tab['dt_bold'] = np.float32(self.dt / 1000.0)
        tab['cf_a'] = self.cf_a
        tab['cf_b'] = self.cf_b
        tab['cf_p'] = np.asarray(self.cf_p, np.float32)
        tab['sigma'] = self.sigma
        tab['consts'] = self.consts
        return tab

    def bold_obs(self):
        """Observable feeding the balloon: sin(theta) for Kuramoto, V for the
        2-D oscillators, r for MPR, x for Linear."""
        if self.model_id in (nat.MODEL_KURAMOTO, nat.MODEL_G2DO):
            return 1
        return 0

    def groups(self, tab):
        """
        Launch groups: (indices, smem_ring) with indices sharing a ring
        placement and size, so each launch reserves only what it needs.
        """
        smem = (tab['flags'] & nat.F_SMEM_RING) != 0
        keys = {}
        for b in range(self.n):
            k = (int(self.block_k[b]), bool(smem[b]), int(tab['lognh'][b]) if smem[b] else -1)
            keys.setdefault(k, []).append(b)
        out = []
        for (bk, sm, lognh), idx in sorted(keys.items(), key=lambda kv: -len(kv[1])):
            ring = int(self.ring_bytes[idx[0]]) if sm else 0
            out.append((np.array(idx, np.int64), ring, bk))
        return out


class Sweep(InstanceSet):
    """
    The plain path: ``run(nsteps)`` advances every instance by nsteps with
    one tvbg_sweep launch per ring group (one CTA per instance).
    """

    def __init__(self, *args, tpn=None, **kwargs):
        super().__init__(*args, **kwargs)
        self.tpn = tpn
        self.status = DeviceStatus()
        self._uploaded = None

    def _launch_cfg(self, smem_ring, tpn, block_k=0):
        cfg = nat.tvbg_launch()
        cfg.model = self.model_id
        cfg.cfun = self.cfun_id
        cfg.threads = self.threads(block_k)
        cfg.tpn = int(tpn)
        if block_k and cfg.tpn < 2:
            cfg.tpn = 2
        cfg.smem_ring = int((smem_ring + 15) // 16 * 16)
        cfg.ctas = 0
        cfg.block_k = int(block_k)
        cfg.nmax = self.N if block_k else 0
        cfg.d_status = self.status.t.data_ptr()
        return cfg

    def prepare(self, nsteps):
        "Build and upload the instance tables of every launch group."
        torch = self.torch
        tab = self.build_table(nsteps)
        launches = []
        for idx, smem, bk in self.groups(tab):
            sub = np.ascontiguousarray(tab[idx])
            dev = torch.from_numpy(sub.view(np.uint8).copy()).cuda()
            launches.append((dev, len(idx), smem, bk))
        self._uploaded = launches
        return launches

    def pick_tpn(self):
        if self.tpn is None:
            from .autotune import tune_tpn
            self.tpn = tune_tpn(self)
        return self.tpn

    def launch(self, launches=None, tpn=None, stream=None):
        "Enqueue the prepared launches on `stream` (no host sync)."
        lib = nat.load()
        launches = launches if launches is not None else self._uploaded
        tpn = tpn if tpn is not None else (self.tpn or 2)
        sh = nat.stream_handle(stream)
        for dev, n, smem, bk in launches:
            cfg = self._launch_cfg(smem, tpn, bk)
            nat.check(lib.tvbg_sweep(dev.data_ptr(), n, ctypes.byref(cfg), sh))

    def run(self, nsteps, stream=None, check=True):
        "Advance all instances by nsteps (chunk boundaries are exact)."
        tpn = self.pick_tpn()
        launches = self.prepare(nsteps)
        self.launch(launches, tpn, stream)
        self.t += int(nsteps)
        if check:
            self.torch.cuda.synchronize()
            self.status.check()

    # -- results ----------------------------------------------------------------
    def ring_plain(self, b):
        "Ring of instance b as numpy [nh, N] slot-major (the oracle's layout)."
        R = int(self.stride[b])
        o = int(self.ring_off[b])
        rows = self.ring[o:o + self.N * R].cpu().numpy().reshape(self.N, R)
        nh = 1 << int(self.lognh[b])
        return unskew_ring(rows[:, :nh].reshape(-1), self.N, int(self.lognh[b]))


def occupancy(cfg):
    "Resident CTAs per SM and SM count for a launch configuration."
    lib = nat.load()
    per, sms = ctypes.c_int32(0), ctypes.c_int32(0)
    nat.check(lib.tvbg_occupancy(ctypes.byref(cfg), ctypes.byref(per), ctypes.byref(sms)))
    return int(per.value), int(sms.value)


class Batch:
    """
    Uneven batch: instances of several connectomes (different N, ring
    lengths and step counts) that share the model, coupling and scheme, run
    by persistent kernels (tvbg_batch_run).

    Instances are grouped by the CTA width they need; every group is one
    persistent launch whose CTAs pull instances from a device counter in
    longest-first order (cost = N x steps), and the groups run concurrently
    on forked streams with CTA counts proportional to their cost.  The whole
    batch can be captured into one CUDA graph (``capture()``), so a sweep of
    uneven instances is a single graph launch.

    This is the persistent counterpart of the subject batch of
    examples/hcp100.py:65-118 (OpenMP over subjects).
    """

    def __init__(self, sets, nsteps, tpn=None):
        import torch
        self.torch = torch
        self.sets = list(sets)
        m0 = self.sets[0]
        for s in self.sets:
            if (s.model_id, s.cfun_id) != (m0.model_id, m0.cfun_id):
                raise ValueError('a batch shares one model and coupling')
        self.nsteps = [np.broadcast_to(np.asarray(n, np.int64), (s.n, )).astype(np.int64)
                       for s, n in zip(self.sets, nsteps)]
        self.tpn = tpn
        self.status = DeviceStatus()
        self.graph = None
        self._build()

    @property
    def node_steps(self):
        return float(sum((s.N * n).sum() for s, n in zip(self.sets, self.nsteps)))

    def _build(self):
        torch = self.torch
        rows = []   # (threads, block_k, table record, cost, smem ring bytes or 0)
        for s, ns in zip(self.sets, self.nsteps):
            tab = s.build_table(ns)
            for b in range(s.n):
                bk = int(s.block_k[b])
                thr = s.threads(bk)
                smem = int(s.ring_bytes[b]) if tab['flags'][b] & nat.F_SMEM_RING else 0
                rows.append((thr, bk, tab[b], float(s.N * ns[b]), smem, s.N,
                             int(s.ring_bytes[b])))
        groups = {}
        for r in rows:
            groups.setdefault((r[0], r[1]), []).append(r)
        total = sum(r[3] for r in rows)
        self.launches = []
        m0 = self.sets[0]
        for (thr, bk), rs in sorted(groups.items(), key=lambda kv: -sum(r[3] for r in kv[1])):
            rs.sort(key=lambda r: -r[3])               # longest first
            nmax = max(r[5] for r in rs)
            # the CTA's scratch is sized by the group's largest N: re-check
            # which rings still fit shared memory next to it
            cap = m0.smem_cap - _SMEM_RESERVE - (
                4 * (2 * bk * nmax * (2 + m0.ns) + 4 * nmax) + 32 if bk else 4 * thr + 16)
            tab = np.array([r[2] for r in rs], dtype=nat.INSTANCE_DTYPE)
            ring_b = np.array([r[6] for r in rs], np.int64)
            smem_ok = ((tab['flags'] & nat.F_SMEM_RING) != 0) & (ring_b <= cap)
            tab['flags'] = np.where(smem_ok, tab['flags'] | nat.F_SMEM_RING,
                                    tab['flags'] & ~np.uint32(nat.F_SMEM_RING)).astype(np.uint32)
            smem_ring = int(ring_b[smem_ok].max()) if smem_ok.any() else 0
            dev = torch.from_numpy(tab.view(np.uint8).copy()).cuda()
            cfg = nat.tvbg_launch()
            cfg.model, cfg.cfun, cfg.threads = m0.model_id, m0.cfun_id, thr
            cfg.tpn = int(self.tpn or (4 if bk else 2))
            cfg.smem_ring = int((smem_ring + 15) // 16 * 16)
            cfg.block_k = bk
            cfg.nmax = nmax if bk else 0
            counter = torch.zeros(1, dtype=torch.int32, device='cuda')
            cfg.d_counter = counter.data_ptr()
            cfg.d_status = self.status.t.data_ptr()
            per_sm, sms = occupancy(cfg)
            cost = sum(r[3] for r in rs)
            cfg.ctas = int(max(1, min(len(rs), round(max(1, per_sm) * sms * cost / total))))
            self.launches.append(dict(dev=dev, n=len(rs), cfg=cfg, counter=counter, cost=cost,
                                      threads=thr, block_k=bk, per_sm=per_sm))
        self.streams = [torch.cuda.Stream() for _ in self.launches]

    def launch(self, stream=None):
        "Enqueue every group on forked streams joined back into `stream`."
        torch = self.torch
        lib = nat.load()
        main = stream or torch.cuda.current_stream()
        for L, s in zip(self.launches, self.streams):
            s.wait_stream(main)
            with torch.cuda.stream(s):
                nat.check(lib.tvbg_batch_run(L['dev'].data_ptr(), L['n'], ctypes.byref(L['cfg']),
                                             s.cuda_stream))
        for s in self.streams:
            main.wait_stream(s)

    def capture(self):
        """Capture the batch launch into one CUDA graph (replay with replay()).
        Nothing runs during capture; kernels were loaded by the planner."""
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


def shard(n, rank, world):
    """Instance range [lo, hi) of `rank` among `world` replicas: contiguous,
    balanced, covering 0..n-1 exactly once.  Instances are independent, so a
    sweep shards with no collective on the data path; only results are
    gathered (e.g. torch.distributed.all_gather_object on the host)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError('bad rank/world')
    base, extra = divmod(int(n), int(world))
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)
