"""
tvbg_fc_noalloc, the FC entry point for callers that cannot call cudaMalloc
(their device memory belongs to a host framework's pool or budget, or their
loop may not take cudaMalloc's implicit synchronisation).  Its FP64 scratch
is a file-scope device array inside the library, so this test checks it
against tvbg_fc_ex -- the same computation with caller-provided scratch --
through the C ABI, on two calls in a row (the second call reuses the array
the first one left behind), and checks that sizes beyond the array's limit
are rejected.  Collected last; passes alone and after the other tests.
"""

import ctypes

import numpy as np
import pytest

from tvb_hpc import _native as nat

pytestmark = pytest.mark.gpu

ATOL = 1e-6  # the FC tolerance of tests/test_gpu_rng_fc.py


def _fc_ex(lib, torch, x, target, I, T, N):
    fc = torch.empty((I, N, N), dtype=torch.float32, device='cuda')
    err = torch.empty(I, dtype=torch.float64, device='cuda')
    nbytes = ctypes.c_int64(0)
    nat.check(lib.tvbg_fc_scratch_bytes(I, N, ctypes.byref(nbytes)))
    scratch = torch.empty(max(1, nbytes.value // 8), dtype=torch.float64, device='cuda')
    nat.check(lib.tvbg_fc_ex(x.data_ptr(), I, T, N, T * N, fc.data_ptr(), target.data_ptr(),
                             err.data_ptr(), scratch.data_ptr(), nat.stream_handle()))
    return fc, err


def _fc_noalloc(lib, torch, x, target, I, T, N):
    fc = torch.empty((I, N, N), dtype=torch.float32, device='cuda')
    err = torch.empty(I, dtype=torch.float64, device='cuda')
    nat.check(lib.tvbg_fc_noalloc(x.data_ptr(), I, T, N, T * N, fc.data_ptr(), target.data_ptr(),
                                  err.data_ptr(), nat.stream_handle()))
    return fc, err


@pytest.mark.parametrize('I,T,N', [(6, 80, 192), (2, 40, 84)])
def test_fc_noalloc_matches_fc_ex_twice(cuda, I, T, N):
    torch = cuda
    lib = nat.load()
    rng = np.random.default_rng(N)
    x = torch.from_numpy((rng.normal(size=(I, T, N)) + rng.normal(size=(I, 1, N)))
                         .astype(np.float32)).cuda()
    target = torch.from_numpy(np.corrcoef(rng.normal(size=(N, 30))).astype(np.float32)).cuda()
    fc_ref, err_ref = _fc_ex(lib, torch, x, target, I, T, N)
    for _ in range(2):
        fc, err = _fc_noalloc(lib, torch, x, target, I, T, N)
        torch.cuda.synchronize()
        np.testing.assert_allclose(fc.cpu().numpy(), fc_ref.cpu().numpy(), atol=ATOL)
        np.testing.assert_allclose(err.cpu().numpy(), err_ref.cpu().numpy(), rtol=1e-9)
    # a different problem in between must not leak into the next call
    x2 = torch.from_numpy(rng.normal(size=(3, 50, N)).astype(np.float32)).cuda()
    _fc_noalloc(lib, torch, x2, target, 3, 50, N)
    fc, err = _fc_noalloc(lib, torch, x, target, I, T, N)
    np.testing.assert_allclose(fc.cpu().numpy(), fc_ref.cpu().numpy(), atol=ATOL)


def test_fc_noalloc_rejects_oversize(cuda):
    "Rejected on the host before any launch: the buffers are never touched."
    torch = cuda
    lib = nat.load()
    N = 998
    I = nat.FC_NOALLOC_MAX_DOUBLES // (N * (N + 1)) + 1
    x = torch.zeros(16, dtype=torch.float32, device='cuda')
    fc = torch.zeros(16, dtype=torch.float32, device='cuda')
    rc = lib.tvbg_fc_noalloc(x.data_ptr(), I, 10, N, 10 * N, fc.data_ptr(), None, None,
                             nat.stream_handle())
    assert rc == nat.TVBG_EINVAL
    assert b'TVBG_FC_NOALLOC_MAX_DOUBLES' in lib.tvbg_last_error()
