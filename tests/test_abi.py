"""
The C-ABI library (no GPU needed): it loads, exports every entry point that
include/tvbg.h declares, agrees with the ctypes struct layouts, and its host
helpers (delay rule, edge packing) give the specified integers.
"""

import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT

from tvb_hpc import _native as nat
from tvb_hpc import engine, network

HEADER = os.path.join(ROOT, 'include', 'tvbg.h')


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r'/\*.*?\*/', '', text, flags=re.S)
    return sorted(set(re.findall(r'\b(tvbg_[a-z0-9_]+)\s*\(', text)))


def test_library_exports_every_declared_symbol():
    lib = nat.load()
    syms = declared_symbols()
    assert len(syms) >= 12
    out = subprocess.run(['nm', '-D', '--defined-only', nat.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = set(line.split()[-1] for line in out.splitlines() if ' T ' in line)
    missing = [s for s in syms if s not in exported]
    assert not missing, missing
    for s in syms:
        assert hasattr(lib, s)
    assert set(nat.SIGNATURES) <= set(syms)


def test_struct_layouts_match():
    lib = nat.load()
    assert lib.tvbg_abi_version() == nat.ABI_VERSION
    assert lib.tvbg_instance_size() == ctypes.sizeof(nat.tvbg_instance) == nat.INSTANCE_DTYPE.itemsize
    assert lib.tvbg_launch_size() == ctypes.sizeof(nat.tvbg_launch)
    assert lib.tvbg_group_size() == ctypes.sizeof(nat.tvbg_group) == nat.GROUP_DTYPE.itemsize
    assert ctypes.sizeof(nat.tvbg_lane) == 16 and nat.GROUP_LANES == 8
    assert (lib.tvbg_adjoint_group_size() == ctypes.sizeof(nat.tvbg_adjoint_group)
            == nat.ADJOINT_GROUP_DTYPE.itemsize == 168)


def test_adjoint_recompute_windows_plan():
    """plan_windows: windows of at most W segments, last first, covering
    every segment once; one buffer for one window, two otherwise."""
    from tvb_hpc.adjoint import plan_windows
    for S in (1, 7, 20):
        for per, budget, win in ((10, 1000, None), (10, 60, None), (10, 15, None), (10, 1000, 3)):
            W, wins, nbuf = plan_windows(S, per, budget, win)
            covered = [k for a, b in wins for k in range(a, b)]
            assert sorted(covered) == list(range(S))
            assert all(0 < b - a <= W for a, b in wins)
            assert [a for a, _ in wins] == sorted([a for a, _ in wins], reverse=True)
            assert nbuf == (1 if len(wins) == 1 else 2)
            if win is None:
                assert nbuf * W * per <= max(budget, nbuf * per)
    assert plan_windows(20, 71, 2000) == (20, [(0, 20)], 1)
    # 15 segments fit the budget, not all 20: two buffers of 7
    assert plan_windows(20, 100, 1500) == (7, [(13, 20), (6, 13), (0, 6)], 2)


def test_adjoint_group_edges_and_shapes():
    """Group packing of the transposed CSR: same out-edge order as the
    per-instance packing, pk = (i << 16) | d; launch shapes hold N."""
    from tvb_hpc import adjoint, network
    w, ln = network.synthetic_connectome(50, 0.3, seed=3)
    conn = network.Connectivity.from_dense(w, ln)
    d = conn.delays(4.0, 0.1, 'ceil')
    lognh = 9
    row_t, e = adjoint.transpose_edges(conn.row, conn.col, conn.wnz, d, lognh)
    row_tg, eg = adjoint.transpose_edges_group(conn.row, conn.col, conn.wnz, d)
    assert np.array_equal(row_t, row_tg)
    assert np.array_equal(e['w'], eg['w'])
    i = eg['pk'] >> 16
    dd = eg['pk'] & 0xffff
    assert np.array_equal(e['pk'] >> lognh, i)
    assert np.array_equal(e['pk'] & ((1 << lognh) - 1), (i + dd + 1) & ((1 << lognh) - 1))
    # every out-edge (j -> i) of the in-edge CSR appears once, in row j
    tgt = np.repeat(np.arange(50), np.diff(conn.row))
    pairs = sorted(zip(conn.col.tolist(), tgt.tolist(), d.tolist()))
    src = np.repeat(np.arange(50), np.diff(row_tg))
    assert sorted(zip(src.tolist(), i.tolist(), dd.tolist())) == pairs
    for N in (1, 17, 84, 400, 998, 1024):
        th, c, pipe = adjoint.adjoint_group_shape(N)
        assert th % 32 == 0 and th <= 512 and 1 <= c <= 16 and c * th // 8 >= N and pipe == 0
    for N in (1, 17, 84, 400, 512):
        th, c, pipe = adjoint.adjoint_group_shape(N, pipelined=True)
        assert th % 64 == 0 and th <= 512 and 1 <= c <= 16 and c * th // 16 >= N and pipe == 1
    assert adjoint.adjoint_group_shape(1025) is None
    assert adjoint.adjoint_group_shape(513, pipelined=True) is None


@pytest.mark.parametrize('rounding', ['trunc', 'ceil', 'dsl'])
def test_delay_rule_host_helper_matches_numpy(rounding):
    lib = nat.load()
    rng = np.random.default_rng(0)
    lengths = rng.uniform(0, 250, 5000).astype(np.float32)
    # include exact multiples, where trunc and ceil agree and rounding bites
    lengths[:100] = (np.arange(100) * 0.4).astype(np.float32)
    for speed, dt in [(4.0, 0.1), (1.0, 0.1), (3.7, 0.1), (10 ** 0.5, 1.0), (100.0, 1.0)]:
        out = np.zeros(lengths.size, np.int32)
        nat.check(lib.tvbg_delays(lengths.size, lengths.ctypes.data, speed, dt,
                                  network.ROUNDING[rounding], out.ctypes.data))
        np.testing.assert_array_equal(out, network.delays_f32(lengths, speed, dt, rounding))


def test_delay_rule_is_the_float32_reference_rule():
    "hackathon.py:44 under numpy 1.15 casting: f32(f32(len / speed) / dt)."
    ln = np.array([10.0, 200.0, 123.4567, 0.4, 0.30000001], np.float32)
    speed, dt = np.float64(4.0), 0.1
    q = (ln / np.float32(speed)).astype(np.float32) / np.float32(dt)
    np.testing.assert_array_equal(network.delays_f32(ln, speed, dt, 'trunc'),
                                  np.trunc(q.astype(np.float32)).astype(np.int32))
    np.testing.assert_array_equal(network.delays_f32(ln, speed, dt, 'ceil'),
                                  np.ceil(q.astype(np.float32)).astype(np.int32))
    # ceil(len/speed/dt) of the benchmark configurations
    assert network.delays_f32(np.float32([10.0]), 4.0, 0.1, 'ceil')[0] == 25
    assert network.delays_f32(np.float32([200.0]), 4.0, 0.1, 'ceil')[0] == 500


def test_pack_edges_ring_addressing_is_bit_exact():
    """pk = (col << lognh) | ((col - d) & mask) reproduces the reference ring
    address (t - d + nh) % nh (kuramoto.c:108) in the skewed layout."""
    rng = np.random.default_rng(3)
    N, lognh = 37, 7
    nh = 1 << lognh
    nnz = 300
    row = np.sort(rng.integers(0, nnz + 1, N - 1))
    row = np.concatenate([[0], row, [nnz]]).astype(np.int32)
    col = rng.integers(0, N, nnz).astype(np.int32)
    d = rng.integers(0, nh - 1, nnz).astype(np.int32)
    w = rng.random(nnz).astype(np.float32)
    pk = engine.pack_edges(row, col, w, d, lognh)['pk'].astype(np.int64)
    mask = nh - 1
    for t in [0, 1, 5, nh - 1, nh, 3 * nh + 17, 123456789]:
        tm = t & mask
        idx = ((tm + pk) & mask) | (pk & ~mask)
        slot = (t - d.astype(np.int64) + nh) % nh
        np.testing.assert_array_equal(idx, engine.ring_index(N, lognh, col, slot))
    # unskew(ring_index) is the identity layout
    ring = np.zeros(N * nh, np.float32)
    slots = np.arange(nh)
    for j in range(N):
        ring[engine.ring_index(N, lognh, j, slots)] = j * 1000 + slots
    plain = engine.unskew_ring(ring, N, lognh)
    assert np.array_equal(plain, (np.arange(N)[None, :] * 1000 + slots[:, None]).astype(np.float32))


def test_pack_edges_rejects_bad_input():
    lib = nat.load()
    row = np.array([0, 1], np.int32)
    col = np.array([0], np.int32)
    w = np.array([1.0], np.float32)
    out = np.zeros(1, np.dtype([('pk', '<u4'), ('w', '<f4')]))
    for d, lognh in [(4, 2), (-1, 4), (0, 1), (0, 25)]:
        dd = np.array([d], np.int32)
        rc = lib.tvbg_pack_edges(1, 1, row.ctypes.data, col.ctypes.data, w.ctypes.data,
                                 dd.ctypes.data, lognh, out.ctypes.data)
        assert rc == nat.TVBG_EINVAL
        assert lib.tvbg_last_error()
    bad_col = np.array([3], np.int32)
    dd = np.array([0], np.int32)
    assert lib.tvbg_pack_edges(1, 1, row.ctypes.data, bad_col.ctypes.data, w.ctypes.data,
                               dd.ctypes.data, 4, out.ctypes.data) == nat.TVBG_EINVAL


def test_pack_edges_group_addressing_is_bit_exact():
    """Group layout: pk = (col << 16) | ((nh - d) & mask); the read of slot
    t - d of node col at ring position (tm + lo) & mask is the reference's
    (t - d + nh) % nh (kuramoto.c:108)."""
    lib = nat.load()
    rng = np.random.default_rng(5)
    N, lognh, nnz = 300, 9, 2000
    nh = 1 << lognh
    row = np.concatenate([[0], np.sort(rng.integers(0, nnz + 1, N - 1)), [nnz]]).astype(np.int32)
    col = rng.integers(0, N, nnz).astype(np.int32)
    d = rng.integers(0, nh, nnz).astype(np.int32)
    w = rng.random(nnz).astype(np.float32)
    out = np.zeros(nnz, np.dtype([('pk', '<u4'), ('w', '<f4')]))
    nat.check(lib.tvbg_pack_edges_group(N, nnz, row.ctypes.data, col.ctypes.data, w.ctypes.data,
                                        d.ctypes.data, lognh, out.ctypes.data))
    pk = out['pk'].astype(np.int64)
    np.testing.assert_array_equal(pk >> 16, col)
    np.testing.assert_array_equal(out['w'], w)
    for t in [0, 1, 7, nh - 1, nh, 5 * nh + 3, 987654321]:
        pos = ((t & (nh - 1)) + (pk & 0xffff)) & (nh - 1)
        np.testing.assert_array_equal(pos, (t - d.astype(np.int64) + nh) % nh)


def test_pack_edges_group_rejects_bad_input():
    lib = nat.load()
    row = np.array([0, 1], np.int32)
    col = np.array([0], np.int32)
    w = np.array([1.0], np.float32)
    out = np.zeros(1, np.dtype([('pk', '<u4'), ('w', '<f4')]))
    for d, lognh in [(8, 3), (-1, 4), (0, 2), (0, 17)]:
        dd = np.array([d], np.int32)
        assert lib.tvbg_pack_edges_group(1, 1, row.ctypes.data, col.ctypes.data, w.ctypes.data,
                                         dd.ctypes.data, lognh, out.ctypes.data) == nat.TVBG_EINVAL
        assert lib.tvbg_last_error()
    bad_col = np.array([1], np.int32)
    dd = np.array([0], np.int32)
    assert lib.tvbg_pack_edges_group(1, 1, row.ctypes.data, bad_col.ctypes.data, w.ctypes.data,
                                     dd.ctypes.data, 4, out.ctypes.data) == nat.TVBG_EINVAL
    big = np.zeros(65538, np.int32)
    assert lib.tvbg_pack_edges_group(65537, 0, big.ctypes.data, None, None, None, 4,
                                     None) == nat.TVBG_EINVAL


def test_group_plan_and_shape():
    from tvb_hpc import groups
    for dmin, dmax in [(3, 3), (7, 500), (25, 500), (5, 2000), (100, 100)]:
        k, lognh = groups.plan_group(dmin, dmax)
        nh = 1 << lognh
        assert k in (4, 8) and k <= dmin + 1 and nh >= dmax + 1 + k
    with pytest.raises(ValueError):
        groups.plan_group(2, 10)
    with pytest.raises(ValueError):
        groups.plan_group(5, 10, block_k=8)
    for N in (1, 4, 20, 68, 84, 128, 192, 300, 400, 998):
        thr, cl = groups.group_shape(N)
        assert thr % 32 == 0 and 32 <= thr <= 1024 and 1 <= cl <= 8
        assert cl * (thr // 8) >= N or thr == 1024
    for N, shape in [(68, (544, 1)), (84, (672, 1)), (128, (1024, 1)),
                     (192, (768, 2)), (400, (800, 4)), (998, (1024, 8))]:
        assert groups.group_shape(N) == shape
    assert groups.group_shape(84, threads=672) == (672, 1)
    assert groups.group_shape(84, threads=128) == (128, 6)


def test_fc_pair_count_is_64_bit():
    """N (N + 1) overflows 32 bits from N = 46341: the scratch size and the
    allocation-free entry point's limit check count it in 64 bits (both
    return before any device call)."""
    lib = nat.load()
    out = ctypes.c_int64(0)
    for n_inst, N in [(1, 46341), (3, 50000), (2, 65535)]:
        assert lib.tvbg_fc_scratch_bytes(n_inst, N, ctypes.byref(out)) == nat.TVBG_OK
        assert out.value == n_inst * N * (N + 1) * 8
    assert lib.tvbg_fc_scratch_bytes(4, 126, ctypes.byref(out)) == nat.TVBG_OK and out.value == 0
    rc = lib.tvbg_fc_noalloc(None, 1, 16, 46341, 16 * 46341, None, None, None, None)
    assert rc == nat.TVBG_EINVAL
    assert b'TVBG_FC_NOALLOC_MAX_DOUBLES' in lib.tvbg_last_error()


def test_pipelined_shapes_and_priority_bands():
    """Host rules of the pipelined group kernel: two teams of one node per
    8-lane slot in at most 1024 threads; the batch tuner's candidates;
    priority bands of a batch (no device needed for the rules)."""
    from tvb_hpc import autotune, groups
    assert groups.pipelined_threads(998, 16) == 1024 and groups.pipelined_threads(998, 12) == 0
    assert groups.pipelined_threads(68, 2) == 576 and groups.pipelined_threads(68, 1) == 0
    for N in (20, 68, 84, 192, 400, 998):
        for thr, c, pr, tpn in autotune.group_shapes(N, pipelined=True):
            assert thr % 32 == 0 and thr <= 1024 and 1 <= c <= groups.MAX_CLUSTER and pr == 0
            per = thr // 8 if tpn == 1 else thr // 16
            assert c * per >= N
            if tpn == nat.GROUP_PIPELINED:
                assert thr % 64 == 0

    class FakeSet:
        def __init__(self, steps):
            self.members = [np.arange(i, min(i + 8, len(steps))) for i in range(0, len(steps), 8)]

    b = groups.GroupBatch.__new__(groups.GroupBatch)
    steps = [np.array([100] * 8 + [50] * 8), np.array([400] * 8)]
    b.sets = [FakeSet(n) for n in steps]
    b.nsteps = steps
    pr = b.group_priorities([1.0, 1.0])
    assert list(pr[1]) == [-5] and list(pr[0]) == [-1, 0]


def test_plan_ring_constraints():
    for order in ('cuda', 'tracka'):
        for dmin, dmax in [(0, 0), (0, 5), (1, 1), (25, 500), (100, 2000), (5, 6), (3, 250)]:
            lognh, sync, fl = engine.plan_ring(dmin, dmax, order=order)
            nh = 1 << lognh
            assert nh >= dmax + 2
            if order == 'cuda':
                assert 1 <= sync <= max(1, dmin + 1) and sync <= nh - dmax - 1
            else:
                assert fl & nat.F_TRACKA
                if dmin == 0:
                    assert sync == 1 and fl & nat.F_MIDSYNC
                else:
                    assert 1 <= sync <= dmin and sync <= nh - dmax


def test_oracle_flag_values_match_the_abi():
    "The oracle reads engine flags directly: the bit values must agree with tvbg.h."
    import pyoracle as orc
    text = open(HEADER).read()
    for name in ('NOISE', 'BOLD', 'TRACE', 'WRAP_FMOD', 'NO_WRAP', 'TRACKA'):
        m = re.search(r'#define TVBG_F_%s (\d+)u' % name, text)
        assert m, name
        assert int(m.group(1)) == getattr(orc, 'F_' + name) == getattr(nat, 'F_' + name)
    src = open(os.path.join(ROOT, 'oracle', 'tvbg_oracle.c')).read()
    for name in ('NOISE', 'BOLD', 'TRACE', 'WRAP_FMOD', 'NO_WRAP', 'TRACKA'):
        m = re.search(r'#define ORC_F_%s (\d+)u' % name, src)
        assert int(m.group(1)) == getattr(nat, 'F_' + name)


def test_pipelined_shape_min_ctas():
    """pipelined_shape: the smallest cluster holding one node per slot, or,
    with min_ctas, the smallest that also gives the set that many CTAs
    (the adjoint's 32 groups of N = 84 on 152 SMs: 256 threads x 6)."""
    from types import SimpleNamespace
    from tvb_hpc import groups
    gs = SimpleNamespace(can_pipeline=True, N=84, n_groups=32)
    assert groups.pipelined_shape(gs) == (704, 2, 0, groups.PIPELINED)
    assert groups.pipelined_shape(gs, min_ctas=152) == (256, 6, 0, groups.PIPELINED)
    assert groups.pipelined_shape(gs, min_ctas=10 ** 6)[1] == 16      # the largest cluster
    for t, c, _, tpn in [groups.pipelined_shape(SimpleNamespace(can_pipeline=True, N=n, n_groups=g),
                                                min_ctas=152) for n in (17, 68, 400, 998) for g in (1, 32)]:
        assert t % 64 == 0 and t <= 1024 and tpn == groups.PIPELINED
    # no pipelining: the plain default shape
    assert groups.pipelined_shape(SimpleNamespace(can_pipeline=False, N=84, n_groups=32))[3] == 1
