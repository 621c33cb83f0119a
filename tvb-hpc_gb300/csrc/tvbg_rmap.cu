// Region mapping between node and region (roi) arrays, tvb_hpc/network.py:
// RMapToAvg (179-191): roi[i, j] = sum over k with rmap[k] == i of node[k, j]
// (the reference zeroes roi and accumulates, so it is a sum);
// RMapFromAvg (194-202): node[k, j] = roi[rmap[k], j].
//
// to_avg: one CTA per region; its threads take the nodes in a strided
// pattern and the partial sums meet in a fixed-shape tree in shared memory,
// so the result is deterministic (its summation order differs from the
// reference's sequential one by rounding only).  Entries of rmap outside
// [0, nroi) contribute to no region, and from_avg leaves their node rows
// unchanged.
#include <algorithm>

#include "tvbg_abi_internal.h"

namespace {

constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads)
    rmap_to_avg_kernel(int nroi, int nvar, int nnode, const int32_t* __restrict__ rmap,
                       const float* __restrict__ node, float* __restrict__ roi) {
    __shared__ float part[kThreads];
    const int i = blockIdx.x;
    for (int j = 0; j < nvar; ++j) {
        float s = 0.0f;
        for (int k = threadIdx.x; k < nnode; k += kThreads)
            if (__ldg(rmap + k) == i) s += __ldg(node + static_cast<size_t>(k) * nvar + j);
        part[threadIdx.x] = s;
        __syncthreads();
        for (int w = kThreads / 2; w > 0; w >>= 1) {
            if (threadIdx.x < w) part[threadIdx.x] += part[threadIdx.x + w];
            __syncthreads();
        }
        if (threadIdx.x == 0) roi[static_cast<size_t>(i) * nvar + j] = part[0];
        __syncthreads();
    }
    (void)nroi;
}

__global__ void rmap_from_avg_kernel(int nroi, int nvar, long long n, const int32_t* __restrict__ rmap,
                                     const float* __restrict__ roi, float* __restrict__ node) {
    for (long long e = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; e < n;
         e += static_cast<long long>(gridDim.x) * blockDim.x) {
        const long long k = e / nvar;
        const int j = static_cast<int>(e - k * nvar);
        const int i = __ldg(rmap + k);
        if (i >= 0 && i < nroi) node[e] = __ldg(roi + static_cast<size_t>(i) * nvar + j);
    }
}

}  // namespace

extern "C" {

int tvbg_rmap_to_avg(int32_t nroi, int32_t nvar, int32_t nnode, const int32_t* d_rmap,
                     const float* d_node, float* d_roi, void* stream) {
    if (nroi < 0 || nvar < 0 || nnode < 0 || (nnode > 0 && (!d_rmap || !d_node)) ||
        (nroi > 0 && nvar > 0 && !d_roi))
        return tvbg::set_error(TVBG_EINVAL, "tvbg_rmap_to_avg: bad arguments");
    if (nroi == 0 || nvar == 0) return TVBG_OK;
    rmap_to_avg_kernel<<<nroi, kThreads, 0, static_cast<cudaStream_t>(stream)>>>(nroi, nvar, nnode, d_rmap,
                                                                                 d_node, d_roi);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? TVBG_OK : tvbg::set_cuda_error(e, "tvbg_rmap_to_avg launch");
}

int tvbg_rmap_from_avg(int32_t nroi, int32_t nvar, int32_t nnode, const int32_t* d_rmap,
                       const float* d_roi, float* d_node, void* stream) {
    if (nroi < 0 || nvar < 0 || nnode < 0 || (nnode > 0 && nvar > 0 && (!d_rmap || !d_node)) ||
        (nroi > 0 && nvar > 0 && !d_roi))
        return tvbg::set_error(TVBG_EINVAL, "tvbg_rmap_from_avg: bad arguments");
    const long long n = static_cast<long long>(nnode) * nvar;
    if (n == 0) return TVBG_OK;
    const long long blocks = std::min<long long>((n + 255) / 256, 65536);
    rmap_from_avg_kernel<<<static_cast<unsigned>(blocks), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        nroi, nvar, n, d_rmap, d_roi, d_node);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? TVBG_OK : tvbg::set_cuda_error(e, "tvbg_rmap_from_avg launch");
}

}  // extern "C"
