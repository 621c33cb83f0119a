"""
ctypes binding of the engine's C ABI (include/tvbg.h).

The shared library ``_lib/libtvbg.so`` is built in-tree by
``__graft_entry__.build()`` (nvcc, sm_103a).  There is no fallback: every
compute call goes through this library, and loading fails loudly when it is
missing.  The binding style mirrors tvb_hpc/compiler.py:140-225
(CompiledKernel: ctypes pointers for arrays, scalars by value), with int
status returns turned into exceptions.
"""

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(HERE, '_lib')
LIB_PATH = os.path.join(LIB_DIR, 'libtvbg.so')

ABI_VERSION = 1

TVBG_OK = 0
TVBG_EINVAL = -1
TVBG_ECUDA = -2
TVBG_ETIMEOUT = -3
TVBG_EUNSUPPORTED = -4
TVBG_EDEVICE = -5

FC_NOALLOC_MAX_DOUBLES = 1048576

MODEL_KURAMOTO, MODEL_G2DO, MODEL_MPR, MODEL_LINEAR, MODEL_G2DOSC = 0, 1, 2, 3, 4
MODEL_RWW, MODEL_JANSENRIT = 5, 6
MODEL_LEMS = 64
CFUN_LINEAR, CFUN_DIFF, CFUN_KURAMOTO, CFUN_SIGMOIDAL = 0, 1, 2, 3
CFUN_LEMS, CFUN_LEMS_SC, CFUN_LEMS_2 = 64, 65, 66

F_NOISE = 1
F_BOLD = 2
F_TRACE = 4
F_WRAP_FMOD = 8
F_SMEM_RING = 16
F_NO_WRAP = 32
F_TRACKA = 64
F_MIDSYNC = 128
F_TRACE_CSUM = 256
F_PIPELINE = 512

GHOST = 8  # ghost slots per ring row of the time-blocked kernel


class tvbg_edge(ctypes.Structure):
    _fields_ = [('pk', ctypes.c_uint32), ('w', ctypes.c_float)]


class tvbg_instance(ctypes.Structure):
    _fields_ = [
        ('edges', ctypes.c_void_p),
        ('row', ctypes.c_void_p),
        ('ring', ctypes.c_void_p),
        ('state', ctypes.c_void_p),
        ('nparam', ctypes.c_void_p),
        ('bold', ctypes.c_void_p),
        ('bold_out', ctypes.c_void_p),
        ('trace', ctypes.c_void_p),
        ('t0', ctypes.c_int64),
        ('trace_stride', ctypes.c_int64),
        ('nsteps', ctypes.c_int32),
        ('N', ctypes.c_int32),
        ('nnz', ctypes.c_int32),
        ('lognh', ctypes.c_int32),
        ('model', ctypes.c_int32),
        ('cfun', ctypes.c_int32),
        ('flags', ctypes.c_uint32),
        ('sync_every', ctypes.c_int32),
        ('trace_every', ctypes.c_int32),
        ('trace_len', ctypes.c_int32),
        ('trace_nobs', ctypes.c_int32),
        ('bold_period', ctypes.c_int32),
        ('bold_len', ctypes.c_int32),
        ('bold_obs', ctypes.c_int32),
        ('seed_lo', ctypes.c_uint32),
        ('seed_hi', ctypes.c_uint32),
        ('inst_id', ctypes.c_uint32),
        ('reserved0', ctypes.c_int32),
        ('dt', ctypes.c_float),
        ('sqrt_dt', ctypes.c_float),
        ('dt_bold', ctypes.c_float),
        ('cf_a', ctypes.c_float),
        ('cf_b', ctypes.c_float),
        ('cf_p', ctypes.c_float * 3),
        ('sigma', ctypes.c_float * 4),
        ('consts', ctypes.c_float * 16),
    ]


class tvbg_launch(ctypes.Structure):
    _fields_ = [
        ('model', ctypes.c_int32),
        ('cfun', ctypes.c_int32),
        ('threads', ctypes.c_int32),
        ('tpn', ctypes.c_int32),
        ('smem_ring', ctypes.c_int32),
        ('ctas', ctypes.c_int32),
        ('block_k', ctypes.c_int32),
        ('nmax', ctypes.c_int32),
        ('cluster', ctypes.c_int32),
        ('priority', ctypes.c_int32),
        ('d_status', ctypes.c_void_p),
        ('d_counter', ctypes.c_void_p),
        ('d_order', ctypes.c_void_p),
    ]


GROUP_LANES = 8  # instances per lane-interleaved group (TVBG_GROUP_LANES)
GROUP_PIPELINED = 2  # tvbg_launch.tpn of the pipelined group kernel (TVBG_GROUP_PIPELINED)


class tvbg_lane(ctypes.Structure):
    _fields_ = [('cf_a', ctypes.c_float), ('nsteps', ctypes.c_int32),
                ('inst_id', ctypes.c_uint32), ('reserved0', ctypes.c_int32)]


class tvbg_group(ctypes.Structure):
    _fields_ = [
        ('edges', ctypes.c_void_p),
        ('row', ctypes.c_void_p),
        ('wsum', ctypes.c_void_p),
        ('nodes', ctypes.c_void_p),
        ('ring', ctypes.c_void_p),
        ('state', ctypes.c_void_p),
        ('nparam', ctypes.c_void_p),
        ('bold', ctypes.c_void_p),
        ('bold_out', ctypes.c_void_p),
        ('trace', ctypes.c_void_p),
        ('t0', ctypes.c_int64),
        ('nsteps', ctypes.c_int32),
        ('N', ctypes.c_int32),
        ('nnz', ctypes.c_int32),
        ('lognh', ctypes.c_int32),
        ('model', ctypes.c_int32),
        ('cfun', ctypes.c_int32),
        ('flags', ctypes.c_uint32),
        ('trace_every', ctypes.c_int32),
        ('trace_len', ctypes.c_int32),
        ('trace_nobs', ctypes.c_int32),
        ('bold_period', ctypes.c_int32),
        ('bold_len', ctypes.c_int32),
        ('bold_obs', ctypes.c_int32),
        ('seed_lo', ctypes.c_uint32),
        ('seed_hi', ctypes.c_uint32),
        ('dmin', ctypes.c_int32),
        ('dt', ctypes.c_float),
        ('sqrt_dt', ctypes.c_float),
        ('dt_bold', ctypes.c_float),
        ('cf_b', ctypes.c_float),
        ('cf_p', ctypes.c_float * 3),
        ('reserved1', ctypes.c_float),
        ('sigma', ctypes.c_float * 4),
        ('consts', ctypes.c_float * 16),
        ('lanes', tvbg_lane * GROUP_LANES),
    ]


class tvbg_net(ctypes.Structure):
    _fields_ = [
        ('row', ctypes.c_void_p), ('col', ctypes.c_void_p), ('w', ctypes.c_void_p),
        ('off', ctypes.c_void_p), ('wsum', ctypes.c_void_p), ('ring', ctypes.c_void_p),
        ('state', ctypes.c_void_p), ('nparam', ctypes.c_void_p),
        ('N', ctypes.c_int64), ('lognh', ctypes.c_int32), ('model', ctypes.c_int32),
        ('cfun', ctypes.c_int32), ('flags', ctypes.c_uint32), ('seed_lo', ctypes.c_uint32),
        ('seed_hi', ctypes.c_uint32), ('dt', ctypes.c_float), ('sqrt_dt', ctypes.c_float),
        ('cf_a', ctypes.c_float), ('cf_b', ctypes.c_float), ('cf_p', ctypes.c_float * 3),
        ('reserved0', ctypes.c_float), ('sigma', ctypes.c_float * 4),
        ('consts', ctypes.c_float * 16),
    ]


#: numpy view of tvbg_group (group tables are built in bulk)
GROUP_DTYPE = np.dtype(tvbg_group)


class tvbg_serve_request(ctypes.Structure):
    "include/tvbg.h tvbg_serve_request."
    _fields_ = [
        ('model', ctypes.c_int32), ('cfun', ctypes.c_int32), ('N', ctypes.c_int32),
        ('nnz', ctypes.c_int32), ('row', ctypes.c_void_p), ('col', ctypes.c_void_p),
        ('weights', ctypes.c_void_p), ('lengths', ctypes.c_void_p), ('n_inst', ctypes.c_int32),
        ('npar', ctypes.c_int32), ('couplings', ctypes.c_void_p), ('speeds', ctypes.c_void_p),
        ('state0', ctypes.c_void_p), ('nparam', ctypes.c_void_p), ('nsteps', ctypes.c_int64),
        ('dt', ctypes.c_float), ('rounding', ctypes.c_int32), ('seed', ctypes.c_uint64),
        ('flags', ctypes.c_uint32), ('cf_b', ctypes.c_float), ('cf_p', ctypes.c_float * 3),
        ('sigma', ctypes.c_float * 4), ('consts', ctypes.c_float * 16),
    ]


SERVE_QUEUED, SERVE_ACTIVE, SERVE_DONE, SERVE_CANCELLED = 0, 1, 2, 3


class tvbg_adjoint(ctypes.Structure):
    _fields_ = [
        ('edges_t', ctypes.c_void_p), ('row_t', ctypes.c_void_p), ('seg', ctypes.c_void_p),
        ('dr', ctypes.c_void_p), ('lam', ctypes.c_void_p), ('ring', ctypes.c_void_p),
        ('deta', ctypes.c_void_p), ('dG', ctypes.c_void_p), ('t0', ctypes.c_int64),
        ('len', ctypes.c_int32), ('N', ctypes.c_int32), ('lognh', ctypes.c_int32),
        ('seg_lanes', ctypes.c_int32), ('dt', ctypes.c_float), ('G', ctypes.c_float),
        ('consts', ctypes.c_float * 4),
    ]


ADJOINT_DTYPE = np.dtype(tvbg_adjoint)


class tvbg_adjoint_group(ctypes.Structure):
    _fields_ = [
        ('edges_t', ctypes.c_void_p), ('row_t', ctypes.c_void_p), ('nodes', ctypes.c_void_p),
        ('seg', ctypes.c_void_p), ('dr', ctypes.c_void_p), ('lam', ctypes.c_void_p),
        ('ring', ctypes.c_void_p), ('deta', ctypes.c_void_p), ('dG', ctypes.c_void_p),
        ('t0', ctypes.c_int64), ('dr_stride', ctypes.c_int64),
        ('len', ctypes.c_int32), ('N', ctypes.c_int32), ('lognh', ctypes.c_int32),
        ('lanes', ctypes.c_int32), ('dmin', ctypes.c_int32), ('flush_every', ctypes.c_int32),
        ('dt', ctypes.c_float), ('G', ctypes.c_float * 8), ('consts', ctypes.c_float * 4),
    ]


ADJOINT_GROUP_DTYPE = np.dtype(tvbg_adjoint_group)

#: numpy view of tvbg_instance (used to build instance tables in bulk)
INSTANCE_DTYPE = np.dtype(tvbg_instance)

_i32, _i64, _u32, _u64 = ctypes.c_int32, ctypes.c_int64, ctypes.c_uint32, ctypes.c_uint64
_vp, _sz = ctypes.c_void_p, ctypes.c_size_t
_fp = ctypes.POINTER(ctypes.c_float)
_ip = ctypes.POINTER(ctypes.c_int32)

# name -> (restype, argtypes); every entry point declared in include/tvbg.h
SIGNATURES = {
    'tvbg_abi_version': (ctypes.c_int, []),
    'tvbg_instance_size': (_sz, []),
    'tvbg_launch_size': (_sz, []),
    'tvbg_last_error': (ctypes.c_char_p, []),
    'tvbg_max_smem': (ctypes.c_int, [_ip]),
    'tvbg_occupancy': (ctypes.c_int, [ctypes.c_void_p, _ip, _ip]),
    'tvbg_pack_edges': (ctypes.c_int, [_i32, _i32, _vp, _vp, _vp, _vp, _i32, _vp]),
    'tvbg_delays': (ctypes.c_int, [_i32, _vp, ctypes.c_float, ctypes.c_float, _i32, _vp]),
    'tvbg_pack_edges_blocked': (ctypes.c_int, [_i32, _i32, _vp, _vp, _vp, _vp, _i32, _vp]),
    'tvbg_sweep': (ctypes.c_int, [_vp, _i32, ctypes.POINTER(tvbg_launch), _vp]),
    'tvbg_batch_run': (ctypes.c_int, [_vp, _i32, ctypes.POINTER(tvbg_launch), _vp]),
    'tvbg_fc': (ctypes.c_int, [_vp, _i32, _i32, _i32, _i64, _vp, _vp, _vp, _vp]),
    'tvbg_fc_ex': (ctypes.c_int, [_vp, _i32, _i32, _i32, _i64, _vp, _vp, _vp, _vp, _vp]),
    'tvbg_fc_scratch_bytes': (ctypes.c_int, [_i32, _i32, ctypes.POINTER(_i64)]),
    'tvbg_fc_noalloc': (ctypes.c_int, [_vp, _i32, _i32, _i32, _i64, _vp, _vp, _vp, _vp]),
    'tvbg_philox_normal': (ctypes.c_int, [_u64, _u32, _vp, _i64, _vp]),
    'tvbg_adjoint_mpr': (ctypes.c_int, [_vp, _i32, _i32, _vp]),
    'tvbg_adjoint_mpr_ex': (ctypes.c_int, [_vp, _i32, _i32, _i32, _vp]),
    'tvbg_adjoint_group_size': (_sz, []),
    'tvbg_adjoint_mpr_groups': (ctypes.c_int, [_vp, _i32, _i32, _i32, _i32, _i32, _vp, _vp]),
    'tvbg_philox_u32': (ctypes.c_int, [_u32, _u32, _u32, _u32, _u32, _vp, _i64, _vp]),
    'tvbg_group_size': (_sz, []),
    'tvbg_net_size': (_sz, []),
    'tvbg_net_run': (ctypes.c_int, [ctypes.POINTER(tvbg_net), _i64, _i32,
                                    ctypes.POINTER(tvbg_launch), _vp]),
    'tvbg_cov_update': (ctypes.c_int, [_vp, _i64, _i32, _i32, _i64, _vp, _vp, _vp]),
    'tvbg_cov_corr': (ctypes.c_int, [_vp, _i32, _i32, _vp, _vp]),
    'tvbg_pack_edges_group': (ctypes.c_int, [_i32, _i32, _vp, _vp, _vp, _vp, _i32, _vp]),
    'tvbg_group_run': (ctypes.c_int, [_vp, _i32, ctypes.POINTER(tvbg_launch), _vp]),
    'tvbg_group_occupancy': (ctypes.c_int, [ctypes.c_void_p, _ip, _ip]),
    'tvbg_group_max_clusters': (ctypes.c_int, [ctypes.c_void_p, _ip]),
    'tvbg_fcfit_zgrad': (ctypes.c_int, [_vp, _vp, _vp, _i32, _i32, _i32, _vp]),
    'tvbg_fcfit_scratch_bytes': (ctypes.c_int, [_i32, _i32, ctypes.POINTER(_i64)]),
    'tvbg_fcfit_loss': (ctypes.c_int, [_vp, _i64, _vp, _i64, _i64, _i32, _i32, _i32, _i32, _vp,
                                       _vp, _vp, _i64, _vp, _vp, _vp]),
    'tvbg_rmap_to_avg': (ctypes.c_int, [_i32, _i32, _i32, _vp, _vp, _vp, _vp]),
    'tvbg_rmap_from_avg': (ctypes.c_int, [_i32, _i32, _i32, _vp, _vp, _vp, _vp]),
    'tvbg_serve_create': (ctypes.c_int, [_i64, _i32, _vp, ctypes.POINTER(_vp)]),
    'tvbg_serve_destroy': (ctypes.c_int, [_vp]),
    'tvbg_serve_admit': (ctypes.c_int, [_vp, ctypes.POINTER(tvbg_serve_request),
                                        ctypes.POINTER(_i64)]),
    'tvbg_serve_tick': (ctypes.c_int, [_vp, _ip, _ip]),
    'tvbg_serve_finished': (ctypes.c_int, [_vp, _vp, _i32, _vp]),
    'tvbg_serve_issued': (ctypes.c_int, [_vp, _i64, _vp]),
    'tvbg_serve_poll': (ctypes.c_int, [_vp, _i64, _ip, _vp]),
    'tvbg_serve_cancel': (ctypes.c_int, [_vp, _i64]),
    'tvbg_serve_usage': (ctypes.c_int, [_vp, _i64, ctypes.POINTER(_i64), ctypes.POINTER(_i64)]),
    'tvbg_serve_set_budget': (ctypes.c_int, [_vp, _i64]),
    'tvbg_serve_progress': (ctypes.c_int, [_vp, _i64, ctypes.POINTER(_i64)]),
    'tvbg_serve_set_concurrency': (ctypes.c_int, [_vp, _i64]),
}


class TvbgError(RuntimeError):
    "A C-ABI call returned a negative status."

    def __init__(self, code, msg):
        super().__init__('%s (status %d)' % (msg, code))
        self.code = code


_lib = None


def load():
    "Load and type the library once; raise if it has not been built."
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            'tvb-hpc GB300 engine library missing at %s; build it with '
            '`python -c "import __graft_entry__ as g; g.build()"`' % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.tvbg_abi_version() != ABI_VERSION:
        raise RuntimeError('libtvbg ABI version mismatch')
    if lib.tvbg_instance_size() != ctypes.sizeof(tvbg_instance):
        raise RuntimeError('tvbg_instance layout mismatch: C %d vs ctypes %d' % (
            lib.tvbg_instance_size(), ctypes.sizeof(tvbg_instance)))
    if lib.tvbg_launch_size() != ctypes.sizeof(tvbg_launch):
        raise RuntimeError('tvbg_launch layout mismatch')
    if lib.tvbg_group_size() != ctypes.sizeof(tvbg_group):
        raise RuntimeError('tvbg_group layout mismatch')
    if lib.tvbg_net_size() != ctypes.sizeof(tvbg_net):
        raise RuntimeError('tvbg_net layout mismatch')
    _lib = lib
    return lib


def check(rc):
    "Turn a status code into an exception carrying tvbg_last_error()."
    if rc != TVBG_OK:
        msg = _lib.tvbg_last_error().decode(errors='replace') if _lib else 'libtvbg'
        raise TvbgError(rc, msg)
    return rc


def ptr(t):
    "Device (or host) address of a torch tensor / numpy array, or None."
    if t is None:
        return None
    if hasattr(t, 'data_ptr'):
        return t.data_ptr()
    return t.ctypes.data


def stream_handle(stream=None):
    "cudaStream_t of a torch stream (current stream by default) as int."
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream
