"""
Functional-connectivity metrics with the names of tvb_hpc/metric.py.

``fc(x)`` computes the Pearson correlation matrix of every instance's time
series with an FP64 reduction on the GPU (tvbg_fc), replacing the one-pass
co-moment kernels Covar / CovToCorr (metric.py:18-139) and
dsl/dsl_cuda/CUDAmodels/refs/covar.c; ``fc_error`` is the FC-SC squared
error of tvb_hpc/examples/hackathon.py:73-87.
"""

import ctypes

import numpy as np

from . import _native as nat


def fc(x, target=None):
    """
    x: torch CUDA float32 [I, T, N] (or [T, N]).  Returns fc [I, N, N] float32
    and, with target [N, N], the per-instance error sum_{i<j}(fc - target)^2
    as float64 [I].
    """
    import torch
    lib = nat.load()
    squeeze = x.dim() == 2
    if squeeze:
        x = x[None]
    x = x.contiguous()
    I, T, N = x.shape
    out = torch.empty((I, N, N), dtype=torch.float32, device=x.device)
    err = None
    tg = None
    if target is not None:
        tg = torch.as_tensor(target, dtype=torch.float32, device=x.device).contiguous()
        err = torch.empty(I, dtype=torch.float64, device=x.device)
    nbytes = ctypes.c_int64(0)
    nat.check(lib.tvbg_fc_scratch_bytes(I, N, ctypes.byref(nbytes)))
    scratch = None
    if nbytes.value:
        scratch = torch.empty(nbytes.value // 8, dtype=torch.float64, device=x.device)
    nat.check(lib.tvbg_fc_ex(x.data_ptr(), I, T, N, T * N, out.data_ptr(),
                             nat.ptr(tg), nat.ptr(err), nat.ptr(scratch), nat.stream_handle()))
    if squeeze:
        out = out[0]
    return (out, err) if target is not None else out


def fc_error(fc_mat, target):
    "Sum over the upper triangle of (fc - target)^2 (hackathon.py:73-87)."
    fc_mat = np.asarray(fc_mat)
    r, c = np.triu_indices(fc_mat.shape[-1], 1)
    return ((fc_mat[..., r, c] - np.asarray(target)[r, c]) ** 2).sum(axis=-1)


class Covar:
    "Name kept from metric.py:18; use fc()."


class CovToCorr:
    "Name kept from metric.py:111; use fc()."


class BatchCov:
    "Batch covariance (metric.py:71-84) of x [m, n] as float64."

    def __call__(self, x):
        x = np.asarray(x, np.float64)
        u = x.mean(axis=0)
        return (x - u).T @ (x - u)


class OnlineCov:
    """
    One-pass co-moment update (metric.py:87-108) in float64 on the host,
    with the Welford weight 1/n for the n-th sample (the reference's
    1/i_sample with a 0-based i_sample, covar.c:101, biases the mean).
    """

    def __init__(self, n):
        self.t = 0
        self.u = np.zeros(n)
        self.cov = np.zeros((n, n))

    def update(self, x):
        x = np.asarray(x, np.float64)
        if self.t == 0:
            self.u = x.copy()
            self.t = 1
            return
        u1 = self.u + (x - self.u) / (self.t + 1)
        self.cov += np.outer(x - u1, x - self.u)
        self.u = u1
        self.t += 1


class StreamingFC:
    """
    Device-resident streaming covariance / FC of many instances for long
    runs (tvbg_cov_update, tvbg_cov_corr): fold one sample per instance at a
    time -- e.g. each new BOLD row -- with FP64 Welford updates, read the
    Pearson FC at any point; the time series itself need not be kept.  The
    GPU counterpart of OnlineCov (metric.py:87-108) and
    dsl/dsl_cuda/CUDAmodels/refs/covar.c:9-109.
    """

    def __init__(self, n_inst, N, device='cuda'):
        import torch
        self.torch = torch
        self.n_inst, self.N = int(n_inst), int(N)
        self.n = 0
        self.mean = torch.empty((n_inst, N), dtype=torch.float64, device=device)
        self.m2 = torch.empty((n_inst, N, N), dtype=torch.float64, device=device)

    def update(self, x, stream=None):
        "x: float32 CUDA [n_inst, N] (rows may be strided); one sample per instance."
        lib = nat.load()
        torch = self.torch
        if x.dtype != torch.float32:
            x = x.float()
        if x.shape != (self.n_inst, self.N):
            raise ValueError('sample shape %s, expected %s' % (tuple(x.shape), (self.n_inst, self.N)))
        if x.stride(1) != 1 or x.stride(0) < self.N:
            x = x.contiguous()
        nat.check(lib.tvbg_cov_update(x.data_ptr(), x.stride(0), self.n_inst, self.N, self.n,
                                      self.mean.data_ptr(), self.m2.data_ptr(),
                                      nat.stream_handle(stream)))
        self.n += 1

    def update_rows(self, xs, rows, stream=None):
        "Fold rows `rows` of xs [n_inst, T, N] in order."
        for r in rows:
            self.update(xs[:, r, :], stream)

    def corr(self, stream=None):
        "Pearson FC [n_inst, N, N] float32 of the samples folded so far."
        lib = nat.load()
        out = self.torch.empty((self.n_inst, self.N, self.N), dtype=self.torch.float32,
                               device=self.m2.device)
        nat.check(lib.tvbg_cov_corr(self.m2.data_ptr(), self.n_inst, self.N, out.data_ptr(),
                                    nat.stream_handle(stream)))
        return out
