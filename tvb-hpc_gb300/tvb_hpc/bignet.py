"""
One very large network, node-parallel (tvbg_net_run): the single-simulation
case of tvb_hpc/examples/sim515k.py (one G2DO network of 515 056 nodes with
linear coupling, CSR connectivity), where instances cannot fill the GPU and
the parallelism is over nodes.

The history ring is node-major ([N][nh + 8]) so the K slots an edge reads
in a block of K steps are contiguous; one kernel launch per block (the
launch boundary is the grid-wide barrier).  Either K lanes per node (lane k
gathers step k, one contiguous load per edge across the lanes; the default)
or one thread per node; both give bit-identical results.  The step is the
CUDA-order step of the other kernels, and the noise is instance 0's Philox
stream.
"""

import ctypes

import numpy as np

from . import _native as nat
from .engine import DeviceStatus, _device_ok, _torch
from .groups import plan_group
from .network import delays_f32


class SingleNetwork:
    """
    model, cfun, scheme : tvb_hpc objects (separable coupling: Linear, Diff,
        Sigmoidal; models G2DO, Generic2dOscillator, MPR, Linear)
    conn : Connectivity (CSR; see network.synthetic_sparse_connectome)
    dt : ms;  coupling : global coupling a;  speed : mm/ms (or delays)
    state0 : (N, nsvar);  nparam : (N, npar) or per-node scalar
    block_k : 4 or 8 steps per launch (default: 8 when d_min >= 7)
    threads : CTA width
    lanes : True (block_k lanes per node) or False (one thread per node)
    """

    def __init__(self, model, cfun, scheme, conn, dt, coupling=1.0, speed=None, delays=None,
                 rounding='ceil', state0=None, nparam=None, seed=0, block_k=None, threads=256,
                 cf_b=None, t0=0, lanes=True):
        _device_ok()
        torch = _torch()
        self.torch = torch
        self.model, self.cfun, self.scheme = model, cfun, scheme
        self.model_id, self.consts, self.sigma = model.engine_spec()
        self.cfun_id, cf_a0, cf_b0, self.cf_p = cfun.engine_spec()
        if self.cfun_id not in (nat.CFUN_LINEAR, nat.CFUN_DIFF, nat.CFUN_SIGMOIDAL):
            raise ValueError('the network kernel needs a separable coupling (Linear, Diff, Sigmoidal)')
        if self.model_id not in (nat.MODEL_G2DO, nat.MODEL_G2DOSC, nat.MODEL_MPR, nat.MODEL_LINEAR):
            raise ValueError('the network kernel is built for G2DO, Generic2dOscillator, MPR, Linear')
        N = self.N = int(conn.nnode)
        self.ns = model.nsvar
        self.npar = len(model.param_sym)
        self.dt = float(dt)
        row = np.asarray(conn.row, np.int64)
        if row[-1] >= 2 ** 31:
            raise ValueError('more than 2^31 edges')
        col = np.asarray(conn.col, np.int32)
        w = np.asarray(conn.wnz, np.float32)
        self.row_np, self.col_np, self.w_np = row.astype(np.int32), col, w
        d = (np.asarray(delays, np.int32) if delays is not None
             else delays_f32(conn.lnz, speed, dt, rounding))
        self.delays = d
        self.block_k, self.lognh = plan_group(d.min() if d.size else 7, d.max() if d.size else 0,
                                              block_k)
        nh = 1 << self.lognh
        off = ((nh - d.astype(np.int64)) & (nh - 1)).astype(np.uint16)
        deg = np.diff(row)
        wsum = np.zeros(N, np.float32)
        nz = deg > 0
        if col.size:
            wsum[nz] = np.add.reduceat(w, row[:-1][nz]).astype(np.float32)
        dev = 'cuda'
        self.row = torch.from_numpy(self.row_np).to(dev)
        self.col = torch.from_numpy(col).to(dev)
        self.w = torch.from_numpy(w).to(dev)
        self.off = torch.from_numpy(off.view(np.int16)).to(dev)
        self.wsum = torch.from_numpy(wsum).to(dev)
        self.R = nh + nat.GHOST
        self.ring = torch.zeros(N * self.R, dtype=torch.float32, device=dev)
        st = (np.zeros((N, self.ns), np.float32) if state0 is None
              else np.broadcast_to(np.asarray(state0, np.float32), (N, self.ns)))
        self.state = torch.from_numpy(np.array(st, np.float32)).to(dev)   # a writable copy
        npm = (model.node_params(N) if nparam is None
               else np.broadcast_to(np.asarray(nparam, np.float32).reshape(N, -1), (N, self.npar)))
        self.nparam = torch.from_numpy(np.array(npm, np.float32)).to(dev)
        fl = 0
        if getattr(scheme, 'noise', False) and np.any(self.sigma != 0):
            fl |= nat.F_NOISE
        self.flags = fl
        self.seed = int(seed) & ((1 << 64) - 1)
        self.cf_a = np.float32(coupling)
        self.cf_b = np.float32(cf_b if cf_b is not None else
                               (cf_b0 if isinstance(cf_b0, (int, float, np.number)) else 0.0))
        self.threads = int(threads)
        self.lanes = bool(lanes)
        self.t = int(t0)
        self.status = DeviceStatus()

    def descriptor(self):
        d = nat.tvbg_net()
        d.row, d.col, d.w, d.off = (self.row.data_ptr(), self.col.data_ptr(), self.w.data_ptr(),
                                    self.off.data_ptr())
        d.wsum = self.wsum.data_ptr()
        d.ring, d.state, d.nparam = self.ring.data_ptr(), self.state.data_ptr(), self.nparam.data_ptr()
        d.N, d.lognh, d.model, d.cfun, d.flags = self.N, self.lognh, self.model_id, self.cfun_id, self.flags
        d.seed_lo, d.seed_hi = self.seed & 0xffffffff, (self.seed >> 32) & 0xffffffff
        d.dt = np.float32(self.dt)
        d.sqrt_dt = float(np.sqrt(np.float32(self.dt)))
        d.cf_a, d.cf_b = float(self.cf_a), float(self.cf_b)
        d.cf_p[:] = [float(v) for v in np.asarray(self.cf_p, np.float32)]
        d.sigma[:] = [float(v) for v in self.sigma]
        d.consts[:] = [float(v) for v in self.consts]
        return d

    def launch(self, nsteps, stream=None):
        "Enqueue nsteps steps from the current clock (no host sync)."
        lib = nat.load()
        cfg = nat.tvbg_launch()
        cfg.model, cfg.cfun, cfg.threads, cfg.block_k = (self.model_id, self.cfun_id, self.threads,
                                                         self.block_k)
        cfg.tpn = self.block_k if self.lanes else 1
        cfg.d_status = self.status.t.data_ptr()
        d = self.descriptor()
        nat.check(lib.tvbg_net_run(ctypes.byref(d), self.t, int(nsteps), ctypes.byref(cfg),
                                   nat.stream_handle(stream)))
        self.t += int(nsteps)

    def run(self, nsteps, stream=None, check=True):
        self.launch(nsteps, stream)
        if check:
            self.torch.cuda.synchronize()
            self.status.check()

    def ring_plain(self):
        "Ring as numpy [nh, N] slot-major (the oracle's layout)."
        nh = 1 << self.lognh
        return self.ring.view(self.N, self.R)[:, :nh].t().contiguous().cpu().numpy()
