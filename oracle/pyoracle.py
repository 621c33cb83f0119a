"""
ctypes wrapper of the CPU oracle (oracle/tvbg_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline / reference legs, never by the engine.  Builds
_build/liboracle.so with `make` on first use.
"""

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, '_build', 'liboracle.so')
REF_LIB = os.path.join(HERE, '_ref', 'libtvbref.so')

# the same bit values as include/tvbg.h's TVBG_F_*; F_BOLD_DEV is oracle-only
F_NOISE, F_BOLD, F_TRACE, F_WRAP_FMOD, F_NO_WRAP, F_TRACKA = 1, 2, 4, 8, 32, 64
F_BOLD_DEV = 256
_SEMANTIC = F_NOISE | F_WRAP_FMOD | F_NO_WRAP | F_TRACKA


class OrcCfg(ctypes.Structure):
    _fields_ = [
        ('model', ctypes.c_int32), ('cfun', ctypes.c_int32), ('N', ctypes.c_int32),
        ('nnz', ctypes.c_int32),
        ('row', ctypes.c_void_p), ('col', ctypes.c_void_p), ('weights', ctypes.c_void_p),
        ('nh', ctypes.c_int32), ('nsteps', ctypes.c_int32), ('t0', ctypes.c_int64),
        ('dt', ctypes.c_float), ('flags', ctypes.c_uint32),
        ('sigma', ctypes.c_float * 4), ('consts', ctypes.c_float * 16),
        ('cf_b', ctypes.c_float), ('cf_p', ctypes.c_float * 3),
        ('seed_lo', ctypes.c_uint32), ('seed_hi', ctypes.c_uint32),
        ('trace_every', ctypes.c_int32), ('trace_len', ctypes.c_int32),
        ('trace_nobs', ctypes.c_int32),
        ('bold_period', ctypes.c_int32), ('bold_len', ctypes.c_int32), ('bold_obs', ctypes.c_int32),
        ('dt_bold', ctypes.c_float), ('npar', ctypes.c_int32),
    ]


_lib = None


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            subprocess.run(['make', '-s', '-C', HERE], check=True)
        lib = ctypes.CDLL(LIB)
        vp = ctypes.c_void_p
        for name in ('orc_run_f32', 'orc_run_f64'):
            fn = getattr(lib, name)
            fn.restype = ctypes.c_int
            fn.argtypes = [ctypes.POINTER(OrcCfg), ctypes.c_int32] + [vp] * 9 + [ctypes.c_int32]
        lib.orc_philox_u32.argtypes = [ctypes.c_uint32] * 5 + [vp, ctypes.c_int64]
        lib.orc_philox_normal.argtypes = [ctypes.c_uint64, ctypes.c_uint32, vp, ctypes.c_int64]
        lib.orc_fc.argtypes = [vp, ctypes.c_int32, ctypes.c_int32, vp]
        lib.orc_fc_onepass_f32.argtypes = [vp, ctypes.c_int32, ctypes.c_int32, vp]
        i32, f64 = ctypes.c_int32, ctypes.c_double
        lib.orc_mpr_adjoint_f64.argtypes = [i32, vp, vp, vp, i32, i32, vp, vp, vp, vp, i32, f64,
                                            vp, vp, vp, vp, vp, i32]
        lib.orc_mpr_loss_f64.argtypes = [i32, vp, vp, vp, i32, vp, f64, vp, vp, i32, f64, vp, vp,
                                         vp]
        _lib = lib
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


def nstate(model):
    return {1: 2, 2: 2, 4: 2, 6: 6}.get(model, 1)


def run(model, cfun, row, col, weights, nh, nsteps, dt, delays, cf_a, nparam, state, ring=None,
        t0=0, flags=0, sigma=(0, 0, 0, 0), consts=None, cf_b=0.0, cf_p=(0, 0, 0), seed=0,
        inst_ids=None, trace_every=0, trace_len=0, trace_nobs=1, bold=None, bold_period=0,
        bold_len=0, bold_obs=0, real='f32', nthreads=1):
    """
    Run the oracle for I instances.  delays [I, nnz] int, cf_a [I],
    nparam [I, N] or [I, N, npar], state [I, N, ns], ring [I, nh, N] (plain slot-major),
    bold [I, 4, N].  Returns dict of the updated arrays.
    """
    lib = load()
    dtype = np.float32 if real == 'f32' else np.float64
    row = np.ascontiguousarray(row, np.int32)
    col = np.ascontiguousarray(col, np.int32)
    w = np.ascontiguousarray(weights, np.float32)
    N = row.size - 1
    state = np.array(state, dtype, copy=True).reshape(-1, N, nstate(model))
    I = state.shape[0]
    delays = np.ascontiguousarray(np.broadcast_to(np.asarray(delays, np.int32), (I, col.size)))
    cf_a = np.ascontiguousarray(np.broadcast_to(np.asarray(cf_a, dtype), (I, )))
    nparam = np.asarray(nparam, dtype)
    if nparam.ndim == 3:                       # [I, N, npar]
        npar = nparam.shape[2]
    else:                                      # [I, N] or [N]: one parameter per node
        npar = 1
        nparam = nparam.reshape(-1, N, 1)
    nparam = np.ascontiguousarray(np.broadcast_to(nparam, (I, N, npar)))
    ring = (np.zeros((I, nh, N), dtype) if ring is None
            else np.array(ring, dtype, copy=True).reshape(I, nh, N))
    cfg = OrcCfg()
    cfg.model, cfg.cfun, cfg.N, cfg.nnz = model, cfun, N, col.size
    cfg.row, cfg.col, cfg.weights = row.ctypes.data, col.ctypes.data, w.ctypes.data
    cfg.nh, cfg.nsteps, cfg.t0, cfg.dt, cfg.flags = nh, nsteps, t0, dt, flags
    cfg.npar = npar
    cfg.sigma[:] = list(np.asarray(sigma, np.float32))
    cfg.consts[:] = list(np.asarray(consts if consts is not None else np.zeros(16), np.float32))
    cfg.cf_b = cf_b
    cfg.cf_p[:] = list(np.asarray(cf_p, np.float32))
    cfg.seed_lo, cfg.seed_hi = int(seed) & 0xffffffff, (int(seed) >> 32) & 0xffffffff
    trace = None
    if trace_every > 0:
        cfg.flags |= F_TRACE
        trace = np.zeros((I, trace_len, N, trace_nobs), dtype)
    cfg.trace_every, cfg.trace_len, cfg.trace_nobs = max(1, trace_every), max(1, trace_len), trace_nobs
    bold_out = None
    if bold_period > 0:
        cfg.flags |= F_BOLD
        if bold is None:
            bold = np.zeros((I, 4, N), dtype)
            if not (flags & F_BOLD_DEV):
                bold[:, 1:] = 1
        bold = np.array(bold, dtype, copy=True)
        bold_out = np.full((I, max(1, bold_len), N), np.nan, dtype)
    cfg.bold_period, cfg.bold_len, cfg.bold_obs = max(1, bold_period), bold_len, bold_obs
    cfg.dt_bold = dt / 1000.0
    ids = np.ascontiguousarray(np.arange(I, dtype=np.uint32) if inst_ids is None
                               else np.asarray(inst_ids, np.uint32))
    fn = lib.orc_run_f32 if real == 'f32' else lib.orc_run_f64
    rc = fn(ctypes.byref(cfg), I, _p(delays), _p(cf_a), _p(nparam), _p(state), _p(ring),
            _p(bold) if bold_period > 0 else None, _p(bold_out), _p(trace), _p(ids), nthreads)
    if rc != 0:
        raise RuntimeError('oracle run failed (%d)' % rc)
    return dict(state=state, ring=ring, bold=bold, bold_out=bold_out, trace=trace)


def run_sweep_like(sw, state0, nsteps, real='f32', t0=0, rings=None, bold=None, nthreads=1):
    """Run the oracle on the configuration of an engine Sweep / InstanceSet:
    same delays, ring lengths, parameters, seeds, step order and monitors.
    Instances are grouped by ring length (one oracle call per group).
    Returns state [I,N,ns], rings (list of [nh, N]), bold, bold_out, trace."""
    I = sw.n
    state0 = np.broadcast_to(np.asarray(state0), (I, sw.N, sw.ns))
    nparam = sw.nparam.cpu().numpy()
    flags = (int(sw.flags) & _SEMANTIC) | F_BOLD_DEV
    res = dict(state=None, rings=[None] * I, bold=None, bold_out=None, trace=None)
    for lognh in sorted(set(int(x) for x in sw.lognh)):
        idx = np.nonzero(sw.lognh == lognh)[0]
        fl = flags | (int(sw.order_flags[idx[0]]) & F_TRACKA)
        delays = np.stack([sw.delay_tables[int(sw.tab_of[b])] for b in idx])
        ring = None if rings is None else np.stack([rings[b] for b in idx])
        bo = None if bold is None else np.asarray(bold)[idx]
        out = run(sw.model_id, sw.cfun_id, sw.row_np, sw.col_np, sw.w_np, 1 << lognh, nsteps,
                  sw.dt, delays, sw.cf_a[idx], nparam[idx], state0[idx], ring=ring, t0=t0,
                  flags=fl, sigma=sw.sigma, consts=sw.consts, cf_b=float(sw.cf_b),
                  cf_p=sw.cf_p, seed=sw.seed, inst_ids=sw.inst_ids[idx],
                  trace_every=sw.trace_every, trace_len=sw.trace_len, trace_nobs=sw.trace_nobs,
                  bold=bo, bold_period=sw.bold_period, bold_len=sw.bold_len,
                  bold_obs=sw.bold_obs(), real=real, nthreads=nthreads)
        for key in ('state', 'bold', 'bold_out', 'trace'):
            if out[key] is None:
                continue
            if res[key] is None:
                res[key] = np.zeros((I, ) + out[key].shape[1:], out[key].dtype)
            res[key][idx] = out[key]
        for k, b in enumerate(idx):
            res['rings'][b] = out['ring'][k]
    return res


def run_groups_like(gs, state0, nsteps, real='f32', nthreads=1):
    """Run the oracle on the configuration of a lane-interleaved GroupSet
    (CUDA step order): same delays, ring lengths, parameters, seeds and
    monitors; `nsteps` scalar or per instance.  Returns state [I,N,ns],
    rings (list of [nh, N]), bold_out [I,bold_len,N] and trace."""
    I = gs.n
    state0 = np.broadcast_to(np.asarray(state0), (I, gs.N, gs.ns))
    steps = np.broadcast_to(np.asarray(nsteps, np.int64), (I, ))
    nparam = gs.gnparam[gs._gi, :, :, gs._li].cpu().numpy()
    flags = (int(gs.flags) & _SEMANTIC) | F_BOLD_DEV
    lognh_i = gs.lognh[gs.grp_of]
    tab_i = gs.gtab[gs.grp_of]
    res = dict(state=None, rings=[None] * I, bold=None, bold_out=None, trace=None)
    keys = sorted(set(zip(lognh_i.tolist(), steps.tolist())))
    for lognh, n in keys:
        idx = np.nonzero((lognh_i == lognh) & (steps == n))[0]
        delays = np.stack([gs.delay_tables[int(tab_i[b])] for b in idx])
        out = run(gs.model_id, gs.cfun_id, gs.row_np, gs.col_np, gs.w_np, 1 << lognh, int(n),
                  gs.dt, delays, gs.cf_a[idx], nparam[idx], state0[idx], flags=flags,
                  sigma=gs.sigma, consts=gs.consts, cf_b=float(gs.cf_b), cf_p=gs.cf_p,
                  seed=gs.seed, inst_ids=gs.inst_ids[idx], trace_every=gs.trace_every,
                  trace_len=gs.trace_len, trace_nobs=gs.trace_nobs,
                  bold_period=gs.bold_period, bold_len=gs.bold_len, bold_obs=gs.bold_obs(),
                  real=real, nthreads=nthreads)
        for key in ('state', 'bold', 'bold_out', 'trace'):
            if out[key] is None:
                continue
            if res[key] is None:
                res[key] = np.zeros((I, ) + out[key].shape[1:], out[key].dtype)
            res[key][idx] = out[key]
        for k, b in enumerate(idx):
            res['rings'][b] = out['ring'][k]
    return res


def philox_u32(k0, k1, n_blocks, c1=0, c2=0, c3=0):
    lib = load()
    out = np.zeros(4 * n_blocks, np.uint32)
    lib.orc_philox_u32(k0, k1, c1, c2, c3, out.ctypes.data, n_blocks)
    return out.reshape(n_blocks, 4)


def philox_normal(seed, stream_id, n):
    lib = load()
    out = np.zeros(n, np.float32)
    lib.orc_philox_normal(int(seed), int(stream_id), out.ctypes.data, n)
    return out


def fc(x):
    "FP64 Pearson FC of x [T, N]."
    lib = load()
    x = np.ascontiguousarray(x, np.float32)
    T, N = x.shape
    out = np.zeros((N, N), np.float64)
    lib.orc_fc(x.ctypes.data, T, N, out.ctypes.data)
    return out


def fc_onepass_f32(x):
    "The reference's one-pass co-moment FC (covar.c) restated, float32."
    lib = load()
    x = np.ascontiguousarray(x, np.float32)
    T, N = x.shape
    out = np.zeros((N, N), np.float32)
    lib.orc_fc_onepass_f32(x.ctypes.data, T, N, out.ctypes.data)
    return out


def mpr_adjoint(row, col, w, delays, G, eta, x0, T, dt, consts, target, nthreads=1):
    """FP64 loss and gradients (dL/dG [I], dL/deta [I, N]) of the FC-fit loss
    of deterministic MPR + linear coupling (see orc_mpr_adjoint_f64)."""
    lib = load()
    row = np.ascontiguousarray(row, np.int32)
    col = np.ascontiguousarray(col, np.int32)
    w = np.ascontiguousarray(w, np.float32)
    N = row.size - 1
    G = np.ascontiguousarray(np.atleast_1d(G), np.float64)
    I = G.size
    delays = np.ascontiguousarray(np.broadcast_to(np.asarray(delays, np.int32), (I, col.size)))
    eta = np.ascontiguousarray(np.broadcast_to(np.asarray(eta, np.float64), (I, N)))
    x0 = np.ascontiguousarray(np.broadcast_to(np.asarray(x0, np.float64), (I, N, 2)))
    consts = np.ascontiguousarray(consts, np.float32)
    target = np.ascontiguousarray(target, np.float64)
    loss = np.zeros(I)
    dG = np.zeros(I)
    deta = np.zeros((I, N))
    rc = lib.orc_mpr_adjoint_f64(N, row.ctypes.data, col.ctypes.data, w.ctypes.data, col.size, I,
                                 delays.ctypes.data, G.ctypes.data, eta.ctypes.data,
                                 x0.ctypes.data, T, dt, consts.ctypes.data, target.ctypes.data,
                                 loss.ctypes.data, dG.ctypes.data, deta.ctypes.data, nthreads)
    if rc:
        raise RuntimeError('oracle adjoint failed')
    return loss, dG, deta


def mpr_loss(row, col, w, delays, G, eta, x0, T, dt, consts, target):
    "FP64 FC-fit loss of one instance (forward only)."
    lib = load()
    row = np.ascontiguousarray(row, np.int32)
    col = np.ascontiguousarray(col, np.int32)
    w = np.ascontiguousarray(w, np.float32)
    N = row.size - 1
    delays = np.ascontiguousarray(delays, np.int32)
    eta = np.ascontiguousarray(eta, np.float64)
    x0 = np.ascontiguousarray(x0, np.float64)
    consts = np.ascontiguousarray(consts, np.float32)
    target = np.ascontiguousarray(target, np.float64)
    out = ctypes.c_double(0.0)
    rc = lib.orc_mpr_loss_f64(N, row.ctypes.data, col.ctypes.data, w.ctypes.data, col.size,
                              delays.ctypes.data, float(G), eta.ctypes.data, x0.ctypes.data, T,
                              dt, consts.ctypes.data, target.ctypes.data, ctypes.byref(out))
    if rc:
        raise RuntimeError('oracle loss failed')
    return out.value


# ---- the reference's own kernels compiled for the host (oracle/_ref) --------
_ref = None


def load_ref():
    "libtvbref.so or None when the reference tree was not available to build it."
    global _ref
    if _ref is None:
        if not os.path.exists(REF_LIB):
            return None
        lib = ctypes.CDLL(REF_LIB)
        vp, u = ctypes.c_void_p, ctypes.c_uint
        lib.ref_kuramoto.argtypes = [u, u, u, u, ctypes.c_float, vp, vp, vp, vp, vp, u]
        lib.ref_bold_update.argtypes = [ctypes.c_int, ctypes.c_float, vp, vp, vp, u]
        lib.ref_update_cov.argtypes = [u, u, vp, vp, vp]
        lib.ref_cov_to_corr.argtypes = [u, u, vp, vp]
        _ref = lib
    return _ref
