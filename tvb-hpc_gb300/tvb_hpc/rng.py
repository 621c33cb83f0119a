"""
Counter-based normal generator with the interface of tvb_hpc/rng.py.

``RNG().build(spec)`` / ``RNG.fill(array, seed)`` fill a float32 array with
N(0, 1) samples from Philox4x32-10 + Box-Muller, computed on the GPU by
tvbg_philox_normal.  Where tvb-hpc leaves the Philox key uninitialised
(rng.py:40-48), here key = (seed_lo, stream) and counter = (i/4, 0,
seed_hi, 0), so a fill is reproducible.  numpy arrays are filled through a
device buffer; torch CUDA tensors in place.
"""

import numpy as np

from . import _native as nat


class RNG:

    def __init__(self, comp=None):
        self.comp = comp

    def generate_c(self, spec=None):
        "The kernel is prebuilt (tvb-hpc_gb300/csrc/tvbg_abi.cu)."
        return ''

    def build(self, spec=None):
        self.lib = nat.load()
        return self

    def fill(self, array, seed=42, stream_id=0):
        import torch
        lib = nat.load()
        if isinstance(array, torch.Tensor):
            if array.dtype != torch.float32 or not array.is_cuda or not array.is_contiguous():
                raise ValueError('fill needs a contiguous float32 CUDA tensor')
            nat.check(lib.tvbg_philox_normal(int(seed) & (2**64 - 1), int(stream_id),
                                             array.data_ptr(), array.numel(),
                                             nat.stream_handle()))
            return array
        assert array.dtype == np.float32
        buf = torch.empty(array.size, dtype=torch.float32, device='cuda')
        nat.check(lib.tvbg_philox_normal(int(seed) & (2**64 - 1), int(stream_id), buf.data_ptr(),
                                         array.size, nat.stream_handle()))
        array.reshape(-1)[:] = buf.cpu().numpy()
        return array


def philox_u32(k0, k1, n_blocks, c1=0, c2=0, c3=0):
    "Raw Philox4x32-10 words [n_blocks, 4] for counter (i, c1, c2, c3), key (k0, k1)."
    import torch
    lib = nat.load()
    out = torch.empty(4 * n_blocks, dtype=torch.int32, device='cuda')
    nat.check(lib.tvbg_philox_u32(k0, k1, c1, c2, c3, out.data_ptr(), n_blocks,
                                  nat.stream_handle()))
    return out.cpu().numpy().view(np.uint32).reshape(n_blocks, 4)
