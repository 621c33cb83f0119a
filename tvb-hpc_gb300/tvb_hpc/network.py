"""
Sparse delayed connectivity, with the interface of tvb_hpc/network.py.

``Connectivity.from_dense`` builds the same CSR arrays as the reference
(network.py:66-78: rows = target node i, columns = source node j,
non-zeros in row-major order).  ``delays`` turns tract lengths into integer
delays with the reference's float32 rule (hackathon.py:44 under numpy 1.15
casting, or the CUDA DSL rule of kuramoto.c:65,105), rounding up by default
as the benchmark configurations ask.

``Network(model, cfun)`` describes the coupling step
  input[i, k] = post_k( sum_j w_ij pre_k(obsrv[t - d_ij, j, k], obsrv[t, i, k]) )
(network.py:96-171); the GB300 kernel implements it, so the class keeps only
the description.  ``RMapToAvg`` / ``RMapFromAvg`` are the region-mapping
kernels of network.py:174-202, run with torch on the device of their inputs.
"""

import numpy as np
from scipy import sparse

from .utils import getLogger

LOG = getLogger(__name__)

ROUNDING = {'trunc': 0, 'ceil': 1, 'dsl': 2}


def delays_f32(lengths, speed, dt, rounding='ceil'):
    """
    Integer delays from tract lengths, evaluated in float32 exactly as the
    reference does (bit-exact delay indices):
      'trunc': trunc(f32(f32(len / speed) / dt))   hackathon.py:44
      'ceil' : ceil (same quotient)                 benchmark configurations
      'dsl'  : trunc(len * f32(f32(1 / speed) / dt)) kuramoto.c:65,105
    """
    lengths = np.asarray(lengths, np.float32)
    s = np.float32(speed)
    d = np.float32(dt)
    if rounding == 'dsl':
        rec = np.float32(np.float32(np.float32(1.0) / s) / d)
        q = (lengths * rec).astype(np.float32)
        out = np.trunc(q)
    else:
        q = (lengths / s).astype(np.float32)
        q = (q / d).astype(np.float32)
        out = np.ceil(q) if rounding == 'ceil' else np.trunc(q)
    if np.any(out < 0) or np.any(~np.isfinite(out)):
        raise ValueError('negative or non-finite delay')
    return out.astype(np.int32)


class Connectivity:
    """
    Data class managing sparse connectivity (network.py:40-93).
    """

    def __init__(self, nnode: int, nz, nnz, col, row, wnz, lnz):
        self.nnode = nnode
        self.nz = nz
        self.nnz = nnz
        self.col = col
        self.row = row
        self.wnz = wnz
        self.lnz = lnz

    @classmethod
    def from_dense(cls, weights, lengths):
        weights = np.asarray(weights)
        lengths = np.asarray(lengths)
        nnode = weights.shape[0]
        nz = ~(weights == 0)
        nnz = nz.sum()
        wnz = weights[nz]
        lnz = lengths[nz]
        sw = sparse.csr_matrix(weights)
        col = sw.indices.astype(np.uintc)
        row = sw.indptr.astype(np.uintc)
        obj = cls(nnode, nz, nnz, col, row, wnz, lnz)
        obj.weights = weights
        obj.lengths = lengths
        return obj

    @classmethod
    def from_npz(cls, fname, weights_key='weights', lengths_key='lengths'):
        npz = np.load(fname)
        return cls.from_dense(npz[weights_key], npz[lengths_key])

    @classmethod
    def hcp0(cls, fname='data/hcp0.npz'):
        "The 84-node HCP connectome shipped with tvb-hpc (network.py:91-93)."
        return cls.from_npz(fname)

    def delays(self, speed, dt, rounding='ceil'):
        "Integer delay per non-zero (see delays_f32)."
        return delays_f32(self.lnz, speed, dt, rounding)

    @property
    def in_degree(self):
        return np.diff(self.row.astype(np.int64))


def synthetic_connectome(N, density, seed, mu=-1.0, sigma=1.0, len_lo=10.0, len_hi=200.0):
    """
    Seeded synthetic connectome of the benchmark configurations: symmetric,
    zero diagonal, upper triangle Bernoulli(density), log-normal(mu, sigma)
    weights normalised to max 1, tract lengths U(len_lo, len_hi) mm,
    symmetric.  Returns float32 (weights, lengths).
    """
    rng = np.random.default_rng(seed)
    iu = np.triu_indices(N, 1)
    mask = rng.random(iu[0].size) < density
    w = np.zeros((N, N), np.float64)
    w[iu] = np.where(mask, rng.lognormal(mu, sigma, iu[0].size), 0.0)
    w = w + w.T
    if w.max() > 0:
        w /= w.max()
    ln = np.zeros((N, N), np.float64)
    ln[iu] = rng.uniform(len_lo, len_hi, iu[0].size)
    ln = ln + ln.T
    ln[w == 0] = 0.0
    return w.astype(np.float32), ln.astype(np.float32)


def synthetic_sparse_connectome(N, mean_degree, seed, mu=-1.0, sigma=1.0, len_lo=10.0,
                                len_hi=200.0):
    """
    Seeded synthetic sparse connectivity for networks too large for a dense
    matrix (the 515 056-node case of tvb_hpc/examples/sim515k.py, whose data
    file is not available): every node gets Poisson(mean_degree) in-edges
    from uniformly drawn distinct sources (no self-edges), log-normal(mu,
    sigma) weights normalised to max 1, tract lengths U(len_lo, len_hi) mm.
    Returns a Connectivity (CSR, columns sorted within each row).
    """
    rng = np.random.default_rng(seed)
    deg = np.minimum(rng.poisson(mean_degree, N), N - 1).astype(np.int64)
    # sorted sources per row without a global sort: the normalised cumulative
    # sums of d + 1 exponential gaps are d sorted uniforms on (0, 1)
    seg = np.repeat(np.arange(N, dtype=np.int64), deg + 1)
    cs = np.cumsum(rng.exponential(1.0, seg.size))
    ends = np.cumsum(deg + 1) - 1                       # last element of each segment
    base = np.concatenate([[0.0], cs[ends[:-1]]])
    total = cs[ends] - base
    keep = np.ones(seg.size, bool)
    keep[ends] = False
    tgt = seg[keep]
    u = (cs[keep] - base[tgt]) / total[tgt]
    src = np.minimum((u * (N - 1)).astype(np.int64), N - 2)
    src = src + (src >= tgt)                            # skip the diagonal (order kept)
    dup = np.zeros(src.size, bool)
    dup[1:] = (src[1:] == src[:-1]) & (tgt[1:] == tgt[:-1])
    tgt, src = tgt[~dup], src[~dup]
    row = np.concatenate([[0], np.cumsum(np.bincount(tgt, minlength=N))]).astype(np.int32)
    w = rng.lognormal(mu, sigma, src.size)
    w = (w / w.max()).astype(np.float32)
    ln = rng.uniform(len_lo, len_hi, src.size).astype(np.float32)
    return Connectivity(N, None, int(src.size), src.astype(np.int32), row, w, ln)


class Network:
    """
    Network implementing sparse time-delay coupling with pre/post summation
    (network.py:96-171).
    """

    def __init__(self, model, cfun):
        self.model = model
        self.cfun = cfun

    def kernel_isns(self):
        yield '<> j_node_lo = row[i_node]'
        yield '<> j_node_hi = row[i_node + 1]'
        for k, (_, pre, post, _) in enumerate(self.cfun.io):
            yield 'input[i_node, %d] = %s <- sum(j_node, weights[j_node] * %s)' % (k, post, pre)


class RegionMappingMix:
    domains = '{[i,j,k]: 0<=i<nroi and 0<=j<nvar and 0<=k<nnode}'
    dtypes = {'roi,node': 'f', 'rmap,nroi,nvar,nnode': 'i'}


def _rmap_call(fn, nroi, nvar, nnode, rmap, src, dst):
    """Run a region-mapping kernel on the device: numpy or CUDA-tensor
    arguments, the result written into `dst` (numpy or tensor) in place."""
    import torch
    from . import _native as nat
    from .engine import _device_ok
    _device_ok()
    lib = nat.load()

    np_of = {torch.int32: np.int32, torch.float32: np.float32}

    def dev(a, dtype):
        if isinstance(a, torch.Tensor):
            return a.to(device='cuda', dtype=dtype).contiguous()
        return torch.from_numpy(np.ascontiguousarray(np.asarray(a), dtype=np_of[dtype])).cuda()

    rm = dev(rmap, torch.int32).reshape(-1)[:nnode].contiguous()
    s = dev(src, torch.float32)
    if isinstance(dst, torch.Tensor) and dst.is_cuda and dst.dtype == torch.float32 and dst.is_contiguous():
        d = dst
    else:
        d = dev(dst, torch.float32)
    nat.check(getattr(lib, fn)(int(nroi), int(nvar), int(nnode), rm.data_ptr(), s.data_ptr(),
                               d.data_ptr(), nat.stream_handle()))
    if d is not dst:
        if isinstance(dst, np.ndarray):
            dst[...] = d.cpu().numpy().reshape(dst.shape)
        else:
            dst.copy_(d.reshape(dst.shape))


class RMapToAvg(RegionMappingMix):
    """roi[i, j] = sum of node[k, j] over rmap[k] == i (network.py:179-191:
    roi is zeroed, then accumulated), on the device (tvbg_rmap_to_avg)."""

    def kernel(self, target=None):
        def knl(nroi, nvar, nnode, rmap, node, roi):
            _rmap_call('tvbg_rmap_to_avg', nroi, nvar, nnode, rmap, node, roi)
        return knl


class RMapFromAvg(RegionMappingMix):
    "node[k, j] = roi[rmap[k], j] (network.py:194-202), on the device (tvbg_rmap_from_avg)."

    def kernel(self, target=None):
        def knl(nroi, nvar, nnode, rmap, node, roi):
            _rmap_call('tvbg_rmap_from_avg', nroi, nvar, nnode, rmap, roi, node)
        return knl
