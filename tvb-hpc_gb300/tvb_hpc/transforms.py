"""
network_time_step: the drop-in for tvb_hpc/transforms.py:23-49.

The reference fuses the model, network and scheme loopy kernels, batches
them over `nstep` and returns an executor called with keyword arguments
(tvb_hpc/examples/hackathon.py:48-54):

    knl(nstep=10, nnode=N, ntime=T, state=state, input=input, param=param,
        drift=drift, diffs=diffs, obsrv=obsrv, nnz=nnz, delays=lnz, row=row,
        col=col, weights=wnz, a=coupling, i_step_0=i * 10)

Here the same call runs the hand-written sm_103a step kernel through the
C ABI (tvbg_sweep).  Semantics kept: obsrv is a time buffer of length ntime
indexed by (i_step + i_step_0) % ntime, row obsrv[t] holding obs(x_t);
delayed reads obsrv[t - d] of earlier rows; `state` and `obsrv` are updated
in place (host numpy arrays are copied to the device and back, torch CUDA
tensors are used in place).  A leading batch axis on state/param/obsrv
(examples/hcp100.py:75-80) runs one instance per batch entry.

Step order: by default the order of the fused loopy kernel (network, model,
scheme, transforms.py:30-42): the gather of step t reads obsrv[t] -- post
and zero-delay terms -- before the model overwrites it with obs(x_t).  This
is the order under which the reference's FC-SC known-answer test holds
(hackathon.py:88-89).  order='cuda' selects the CUDA DSL order instead
(kuramoto.c:85-139).  The returned Kuramoto state is wrapped into [0, 2 pi]
after the step, where tvb-hpc wraps it at the start of the next model call.  `input`, `drift` and `diffs` are
scratch of the fused kernel and are not written.  With EulerMaryuyamaStep
the Wiener increments are drawn in-kernel (Philox keyed by `seed` and the
batch index) instead of being read from a dWt array.
"""

import ctypes

import numpy as np

from . import _native as nat
from .coupling import symbolic_name
from .engine import plan_ring, pack_edges, max_smem, DeviceStatus, _device_ok
from .utils import getLogger

LOG = getLogger(__name__)


class NetworkTimeStep:
    "Executor returned by network_time_step (the fused loopy kernel's call)."

    def __init__(self, model, coupling, scheme, target=None, order='tracka'):
        self.model, self.coupling, self.scheme = model, coupling, scheme
        self.order = order
        self.model_id, self.consts, self.sigma = model.engine_spec()
        self.cfun_id, self.a, self.b, self.cf_p = coupling.engine_spec()
        self.name = '%s_and_Network_and_%s' % (type(model).__name__, type(scheme).__name__)
        self.tpn = 2
        self._status = None

    def __call__(self, nstep, nnode, ntime, state, input, param, drift, diffs, obsrv, nnz,
                 delays, row, col, weights, i_step_0=0, seed=0, **kwargs):
        import torch
        _device_ok()
        lib = nat.load()
        if self._status is None:
            self._status = DeviceStatus()
        host = not isinstance(state, torch.Tensor)

        def dev(a, dt):
            if isinstance(a, torch.Tensor):
                return a if a.is_cuda else a.cuda()
            return torch.from_numpy(np.ascontiguousarray(a, dt)).cuda()

        st = dev(state, np.float32)
        batched = st.dim() == 3
        if not batched:
            st = st[None]
        I, N, ns = st.shape
        if N != int(nnode):
            raise ValueError('state has %d nodes, nnode=%d' % (N, nnode))
        pa = dev(param, np.float32)
        if pa.dim() == 2:
            pa = pa[None].expand(I, -1, -1)
        pa = pa.contiguous()
        ob = dev(obsrv, np.float32)
        if not batched:
            ob = ob[:, None]
        if ob.shape[0] != int(ntime) or ob.shape[1] != I or ob.shape[2] != N:
            raise ValueError('obsrv must be [ntime, (nsubj,) nnode, nobs]')
        nobs = ob.shape[3]
        ob = ob.contiguous()
        dl = np.asarray(delays.cpu() if isinstance(delays, torch.Tensor) else delays).astype(np.int64)
        rw = np.asarray(row.cpu() if isinstance(row, torch.Tensor) else row).astype(np.int64)
        cl = np.asarray(col.cpu() if isinstance(col, torch.Tensor) else col).astype(np.int64)
        wt = np.asarray(weights.cpu() if isinstance(weights, torch.Tensor) else weights, np.float32)
        nnz = int(nnz)
        if dl.ndim == 2:
            raise NotImplementedError('per-subject delays: run one executor per delay table')
        dl, cl, wt = dl[:nnz], cl[:nnz], wt[:nnz]
        dmin = int(dl.min()) if nnz else 0
        dmax = int(dl.max()) if nnz else 0
        if dmax >= int(ntime):
            raise ValueError('delays must be shorter than ntime')
        tracka = self.order == 'tracka'
        # Track-A order reads the old rows t0..t0+nstep-1 (post, zero delays)
        # before overwriting them: the ring must hold them all at once
        lognh, sync, oflags = plan_ring(dmin, dmax, int(nstep) if tracka else 0, self.order)
        nh = 1 << lognh
        edges = torch.from_numpy(pack_edges(rw, cl, wt, dl, lognh).view(np.uint8).copy()).cuda()
        rowd = torch.from_numpy(rw.astype(np.int32)).cuda()
        t0 = int(i_step_0)
        # ring from the history rows obsrv[t0 - dmax .. t0] of observable 0
        ring = torch.zeros((I, N * nh), dtype=torch.float32, device='cuda')
        t_hi = t0 + int(nstep) if tracka else t0 + 1
        ts = torch.arange(t0 - dmax, t_hi, device='cuda', dtype=torch.int64)
        rows_ = torch.remainder(ts, int(ntime))
        vals = ob[rows_, :, :, 0]                                  # [T, I, N]
        j = torch.arange(N, device='cuda', dtype=torch.int64)
        idx = j[None, :] * nh + ((ts[:, None] + j[None, :]) & (nh - 1))  # [T, N]
        ring.view(I, N * nh)[:, idx.reshape(-1)] = vals.permute(1, 0, 2).reshape(I, -1)
        # coupling parameters: numbers or kernel arguments named by symbols
        a = self._param(self.a, kwargs, 'a')
        b = self._param(self.b, kwargs, 'b')
        dt = self.scheme.dt_value(kwargs)
        tab = np.zeros(I, dtype=nat.INSTANCE_DTYPE)
        bi = np.arange(I, dtype=np.int64)
        ring_bytes = N * nh * 4
        threads = 32 * ((N + 31) // 32)
        smem_ok = ring_bytes <= max_smem() - 4 * threads - 2048
        tab['edges'] = edges.data_ptr()
        tab['row'] = rowd.data_ptr()
        tab['ring'] = ring.data_ptr() + 4 * bi * N * nh
        st = st.contiguous()
        tab['state'] = st.data_ptr() + 4 * bi * N * ns
        tab['nparam'] = pa.data_ptr() + 4 * bi * N * pa.shape[2]
        tab['trace'] = ob.data_ptr() + 4 * bi * N * nobs
        tab['t0'] = t0
        tab['trace_stride'] = I * N * nobs
        tab['nsteps'] = int(nstep)
        tab['N'] = N
        tab['nnz'] = nnz
        tab['lognh'] = lognh
        tab['model'] = self.model_id
        tab['cfun'] = self.cfun_id
        fl = nat.F_TRACE | oflags | (nat.F_SMEM_RING if smem_ok else 0)
        if getattr(self.scheme, 'noise', False) and np.any(np.asarray(self.sigma) != 0):
            fl |= nat.F_NOISE
        tab['flags'] = fl
        tab['sync_every'] = sync
        tab['trace_every'] = 1
        tab['trace_len'] = int(ntime)
        tab['trace_nobs'] = nobs
        tab['bold_period'] = 1
        tab['seed_lo'] = int(seed) & 0xffffffff
        tab['seed_hi'] = (int(seed) >> 32) & 0xffffffff
        tab['inst_id'] = bi.astype(np.uint32)
        tab['dt'] = np.float32(dt)
        tab['sqrt_dt'] = np.sqrt(np.float32(dt))
        tab['cf_a'] = np.broadcast_to(np.asarray(a, np.float32), (I, ))
        tab['cf_b'] = np.broadcast_to(np.asarray(b, np.float32), (I, ))
        tab['cf_p'] = np.asarray(self._sig(kwargs), np.float32)
        tab['sigma'] = self.sigma
        tab['consts'] = self.consts
        tdev = torch.from_numpy(tab.view(np.uint8).copy()).cuda()
        cfg = nat.tvbg_launch()
        cfg.model, cfg.cfun, cfg.threads, cfg.tpn = self.model_id, self.cfun_id, threads, self.tpn
        cfg.smem_ring = (ring_bytes + 15) // 16 * 16 if smem_ok else 0
        cfg.d_status = self._status.t.data_ptr()
        nat.check(lib.tvbg_sweep(tdev.data_ptr(), I, ctypes.byref(cfg), nat.stream_handle()))
        torch.cuda.synchronize()
        self._status.check()
        out_state = st if batched else st[0]
        out_obs = ob if batched else ob[:, 0]
        if host:
            state[...] = out_state.cpu().numpy().reshape(np.shape(state))
            obsrv[...] = out_obs.cpu().numpy().reshape(np.shape(obsrv))
        else:
            if out_state.data_ptr() != state.data_ptr():
                state.copy_(out_state.reshape(state.shape))
            if out_obs.data_ptr() != obsrv.data_ptr():
                obsrv.copy_(out_obs.reshape(obsrv.shape))

    @staticmethod
    def _param(v, kwargs, default_name):
        "A number, or the kernel argument named by a symbolic parameter (scalar or per subject)."
        name = symbolic_name(v)
        if name is None:
            return float(v)
        if name not in kwargs:
            raise TypeError('coupling parameter %r is a kernel argument; pass %s=...' % (name, name))
        val = kwargs[name]
        if hasattr(val, 'cpu'):
            val = val.cpu().numpy()
        return np.asarray(val, np.float32)

    def _sig(self, kwargs):
        return [float(self._param(v, kwargs, '')) for v in self.cf_p]


def network_time_step(model, coupling, scheme, target=None, order='tracka'):
    """
    Fuse model, network and scheme into one GB300 step executor.  The default
    step order is the fused loopy kernel's ('tracka'): the network gather of
    step t reads obsrv[t] before the model writes it.  order='cuda' gives the
    order of the CUDA DSL kernels instead.
    """
    return NetworkTimeStep(model, coupling, scheme, target, order)
