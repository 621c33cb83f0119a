"""
Host side of the native serving pool (tvbg_serve_*), no GPU needed: request
validation and the device footprint of the plan (delay tables, ring lengths,
lane-interleaved groups), which creating a pool and admitting requests
compute without touching a device.
"""

import ctypes

import numpy as np
import pytest

from tvb_hpc import _native as nat, network, model, coupling


def pool(budget=1 << 40):
    lib = nat.load()
    h = ctypes.c_void_p()
    nat.check(lib.tvbg_serve_create(int(budget), 1000, None, ctypes.byref(h)))
    return lib, h


def request(conn, I=10, speed=4.0, m=None, cf=None, nsteps=500):
    m = m or model.MPR()
    cf = cf or coupling.Linear(m)
    kid, consts, sigma = m.engine_spec()
    cid, _, cf_b, cf_p = cf.engine_spec()
    N = conn.nnode
    keep = dict(row=np.ascontiguousarray(conn.row, np.int32), col=np.ascontiguousarray(conn.col, np.int32),
                w=np.ascontiguousarray(conn.wnz, np.float32), ln=np.ascontiguousarray(conn.lnz, np.float32),
                G=np.linspace(0.1, 1, I).astype(np.float32), sp=np.full(I, speed, np.float32),
                x0=np.zeros((I, N, m.nsvar), np.float32),
                np=np.ascontiguousarray(np.broadcast_to(m.node_params(N), (I, N, len(m.param_sym)))))
    q = nat.tvbg_serve_request()
    q.model, q.cfun, q.N, q.nnz = kid, cid, N, conn.nnz
    q.row, q.col, q.weights, q.lengths = (keep[k].ctypes.data for k in ('row', 'col', 'w', 'ln'))
    q.n_inst, q.npar = I, len(m.param_sym)
    q.couplings, q.speeds = keep['G'].ctypes.data, keep['sp'].ctypes.data
    q.state0, q.nparam = keep['x0'].ctypes.data, keep['np'].ctypes.data
    q.nsteps, q.dt, q.rounding, q.seed = nsteps, 0.1, 1, 3
    q.cf_b = float(cf_b)
    q.sigma[:] = [float(v) for v in sigma[:4]]
    q.consts[:] = [float(v) for v in consts]
    return q, keep


def test_footprint_of_the_plan():
    w, ln = network.synthetic_connectome(68, 0.3, seed=0)
    conn = network.Connectivity.from_dense(w, ln)
    lib, h = pool()
    try:
        q, keep = request(conn, I=10)
        rid = ctypes.c_int64()
        nat.check(lib.tvbg_serve_admit(h, ctypes.byref(q), ctypes.byref(rid)))
        used, fp = ctypes.c_int64(), ctypes.c_int64()
        nat.check(lib.tvbg_serve_usage(h, rid.value, ctypes.byref(used), ctypes.byref(fp)))
        assert used.value == 0                      # nothing admitted to the device yet
        d = network.delays_f32(conn.lnz, 4.0, 0.1, 'ceil')
        K = 8 if d.min() + 1 >= 8 else 4
        nh = max(8, 1 << int(np.ceil(np.log2(d.max() + 1 + K))))
        G, N = 2, conn.nnode                        # 10 instances: two groups of eight lanes
        ring = G * N * (nh + 8) * 8 * 4
        state = G * N * 2 * 8 * 4
        assert ring + state < fp.value < ring + state + conn.nnz * 8 + 64 * 1024
        st = ctypes.c_int32()
        nat.check(lib.tvbg_serve_poll(h, rid.value, ctypes.byref(st), None))
        assert st.value == nat.SERVE_QUEUED
        nat.check(lib.tvbg_serve_cancel(h, rid.value))
        nat.check(lib.tvbg_serve_poll(h, rid.value, ctypes.byref(st), None))
        assert st.value == nat.SERVE_CANCELLED
    finally:
        lib.tvbg_serve_destroy(h)


def test_admission_rejects():
    w, ln = network.synthetic_connectome(30, 0.3, seed=1)
    conn = network.Connectivity.from_dense(w, ln)
    lib, h = pool(budget=1 << 20)
    try:
        rid = ctypes.c_int64()
        q, keep = request(conn, speed=200.0)         # delays < 3 steps: no group blocks
        assert lib.tvbg_serve_admit(h, ctypes.byref(q), ctypes.byref(rid)) == nat.TVBG_EUNSUPPORTED
        q, keep = request(conn, I=4000)              # alone larger than the budget
        assert lib.tvbg_serve_admit(h, ctypes.byref(q), ctypes.byref(rid)) == nat.TVBG_EINVAL
        m = model.G2DO()
        q, keep = request(conn, m=m, cf=coupling.Kuramoto(m))   # Kuramoto coupling on G2DO
        assert lib.tvbg_serve_admit(h, ctypes.byref(q), ctypes.byref(rid)) == nat.TVBG_EUNSUPPORTED
        q, keep = request(conn)
        q.npar = 3                                   # the model has one parameter per node
        assert lib.tvbg_serve_admit(h, ctypes.byref(q), ctypes.byref(rid)) == nat.TVBG_EINVAL
        st = ctypes.c_int32()
        assert lib.tvbg_serve_poll(h, 12345, ctypes.byref(st), None) == nat.TVBG_EINVAL
    finally:
        lib.tvbg_serve_destroy(h)


def test_set_budget():
    """tvbg_serve_set_budget lowers the admission budget of the next ticks
    (clamped to the creation budget); admitting a request is checked against
    the creation budget, so a request that fits the pool is queued even while
    the current budget is small."""
    w, ln = network.synthetic_connectome(30, 0.3, seed=1)
    conn = network.Connectivity.from_dense(w, ln)
    lib, h = pool(budget=1 << 24)
    try:
        assert lib.tvbg_serve_set_budget(h, -1) == nat.TVBG_EINVAL
        assert lib.tvbg_serve_set_budget(None, 10) == nat.TVBG_EINVAL
        nat.check(lib.tvbg_serve_set_budget(h, 16))
        q, keep = request(conn, I=4)
        rid = ctypes.c_int64()
        nat.check(lib.tvbg_serve_admit(h, ctypes.byref(q), ctypes.byref(rid)))
        nat.check(lib.tvbg_serve_set_budget(h, 1 << 40))   # clamped to the creation budget
    finally:
        lib.tvbg_serve_destroy(h)


def test_adjoint_footprint_counts_recompute_windows():
    """A gradient request's adjoint memory counts the recomputation windows:
    all segments when trace_budget holds them, else trace_budget, and at
    least one segment (traces r, V, S and a working copy of its checkpoint)."""
    from tvb_hpc import serve
    I, N, T, nh = 256, 84, 2000, 512
    per_seg = I * 100 * N * 3 * 4 + I * N * (nh + 8 + 2) * 4
    full = serve.adjoint_bytes(I, N, T, nh)                      # 2 GiB: all 20 segments
    small = serve.adjoint_bytes(I, N, T, nh, trace_budget=1 << 28)
    tiny = serve.adjoint_bytes(I, N, T, nh, trace_budget=1)
    assert 20 * per_seg < (2 << 30)
    assert full - small == 20 * per_seg - (1 << 28)
    assert small - tiny == (1 << 28) - per_seg
