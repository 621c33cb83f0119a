// Pearson functional connectivity per instance with an FP64 reduction, and
// the FC-fit error against a target matrix.
//
// Restates tvb_hpc/metric.py:18-139 (Covar one-pass co-moment + CovToCorr)
// and dsl/dsl_cuda/CUDAmodels/refs/covar.c:9-109 as a two-pass FP64 method:
// means, then the centred Gram  C_ij = sum_t (x_ti - m_i)(x_tj - m_j),
// corr_ij = C_ij / sqrt(C_ii C_jj).  (The 1/n normalisation of covar.c:155-159
// cancels in the ratio.)  One CTA per instance; samples are staged through
// shared memory in tiles of kTile time points.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "tvbg_abi_internal.h"

namespace tvbg {

constexpr int kFcThreads = 512;
constexpr int kTile = 32;
constexpr int kMaxPairsPerThread = 16;  // N(N+1)/2 <= 512*16  ->  N <= 127

// Each thread owns a fixed list of (i <= j) pairs of the upper triangle.
__global__ void __launch_bounds__(kFcThreads)
    fc_small_kernel(const float* __restrict__ x, int T, int N, long long inst_stride,
                    float* __restrict__ fc, const float* __restrict__ target,
                    double* __restrict__ err) {
    extern __shared__ double sh[];  // mean[N] | tile[kTile][N] | err partials
    double* mean = sh;
    double* tile = sh + N;
    double* part = tile + kTile * N;
    const float* xb = x + blockIdx.x * inst_stride;
    const int tid = threadIdx.x;

    // pass 1: means in FP64
    for (int i = tid; i < N; i += blockDim.x) {
        double s = 0.0;
        for (int t = 0; t < T; ++t) s += static_cast<double>(xb[static_cast<long long>(t) * N + i]);
        mean[i] = s / static_cast<double>(T);
    }
    __syncthreads();

    const int npairs = N * (N + 1) / 2;  // small path only: N (N + 1) / 2 <= kFcThreads * kMaxPairsPerThread
    double acc[kMaxPairsPerThread];
    int pi[kMaxPairsPerThread], pj[kMaxPairsPerThread];
#pragma unroll
    for (int q = 0; q < kMaxPairsPerThread; ++q) {
        acc[q] = 0.0;
        const int pidx = tid + q * kFcThreads;
        int i = 0, j = 0;
        if (pidx < npairs) {
            // row-major upper triangle: pairs (i, j>=i)
            int rem = pidx;
            i = 0;
            while (rem >= N - i) {
                rem -= N - i;
                ++i;
            }
            j = i + rem;
        }
        pi[q] = i;
        pj[q] = j;
    }

    // pass 2: centred Gram over tiles of time points
    for (int t0 = 0; t0 < T; t0 += kTile) {
        const int nt = (T - t0) < kTile ? (T - t0) : kTile;
        __syncthreads();
        for (int e = tid; e < nt * N; e += blockDim.x) {
            const int tt = e / N, i = e - tt * N;
            tile[tt * N + i] =
                static_cast<double>(xb[static_cast<long long>(t0 + tt) * N + i]) - mean[i];
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < kMaxPairsPerThread; ++q) {
            if (tid + q * kFcThreads < npairs) {
                const int i = pi[q], j = pj[q];
                double a = acc[q];
                for (int tt = 0; tt < nt; ++tt) a = fma(tile[tt * N + i], tile[tt * N + j], a);
                acc[q] = a;
            }
        }
    }
    __syncthreads();
    // diagonal to shared for normalisation
    double* var = tile;  // reuse
#pragma unroll
    for (int q = 0; q < kMaxPairsPerThread; ++q)
        if (tid + q * kFcThreads < npairs && pi[q] == pj[q]) var[pi[q]] = acc[q];
    __syncthreads();
    double e_local = 0.0;
    float* fcb = fc + static_cast<long long>(blockIdx.x) * N * N;
#pragma unroll
    for (int q = 0; q < kMaxPairsPerThread; ++q) {
        if (tid + q * kFcThreads < npairs) {
            const int i = pi[q], j = pj[q];
            const double r = acc[q] / sqrt(var[i] * var[j]);
            const float rf = static_cast<float>(r);
            fcb[i * N + j] = rf;
            fcb[j * N + i] = rf;
            if (target && i < j) {
                const double dd = r - static_cast<double>(target[i * N + j]);
                e_local = fma(dd, dd, e_local);
            }
        }
    }
    if (err) {
        part[tid] = e_local;
        __syncthreads();
        for (int off = blockDim.x / 2; off > 0; off >>= 1) {
            if (tid < off) part[tid] += part[tid + off];
            __syncthreads();
        }
        if (tid == 0) err[blockIdx.x] = part[0];
    }
}

// Large-N path: one thread per output entry (i, j), rows of a 16x16 tile.
__global__ void fc_large_kernel(const float* __restrict__ x, int T, int N, long long inst_stride,
                                const double* __restrict__ mean, double* __restrict__ gram) {
    const int b = blockIdx.z;
    const int i = blockIdx.y * 16 + threadIdx.y;
    const int j = blockIdx.x * 16 + threadIdx.x;
    __shared__ double ti[kTile][16], tj[kTile][16];
    const float* xb = x + b * inst_stride;
    const double* mb = mean + static_cast<long long>(b) * N;
    double a = 0.0;
    for (int t0 = 0; t0 < T; t0 += kTile) {
        const int nt = (T - t0) < kTile ? (T - t0) : kTile;
        for (int tt = threadIdx.y; tt < kTile; tt += 16) {
            const int ii = blockIdx.y * 16 + threadIdx.x;
            const int jj = blockIdx.x * 16 + threadIdx.x;
            ti[tt][threadIdx.x] = (tt < nt && ii < N)
                                      ? static_cast<double>(xb[static_cast<long long>(t0 + tt) * N + ii]) - mb[ii]
                                      : 0.0;
            tj[tt][threadIdx.x] = (tt < nt && jj < N)
                                      ? static_cast<double>(xb[static_cast<long long>(t0 + tt) * N + jj]) - mb[jj]
                                      : 0.0;
        }
        __syncthreads();
        for (int tt = 0; tt < nt; ++tt) a = fma(ti[tt][threadIdx.y], tj[tt][threadIdx.x], a);
        __syncthreads();
    }
    if (i < N && j < N) gram[(static_cast<long long>(b) * N + i) * N + j] = a;
}

__global__ void fc_mean_kernel(const float* __restrict__ x, int T, int N, long long inst_stride,
                               double* __restrict__ mean) {
    const int b = blockIdx.y;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const float* xb = x + b * inst_stride;
    double s = 0.0;
    for (int t = 0; t < T; ++t) s += static_cast<double>(xb[static_cast<long long>(t) * N + i]);
    mean[static_cast<long long>(b) * N + i] = s / static_cast<double>(T);
}

__global__ void fc_norm_kernel(const double* __restrict__ gram, int N, float* __restrict__ fc,
                               const float* __restrict__ target, double* __restrict__ err) {
    const int b = blockIdx.x;
    const double* g = gram + static_cast<long long>(b) * N * N;
    __shared__ double part[256];
    double e = 0.0;
    for (int q = threadIdx.x; q < N * N; q += blockDim.x) {
        const int i = q / N, j = q - i * N;
        const double r = g[q] / sqrt(g[i * N + i] * g[j * N + j]);
        fc[static_cast<long long>(b) * N * N + q] = static_cast<float>(r);
        if (target && i < j) {
            const double dd = r - static_cast<double>(target[q]);
            e = fma(dd, dd, e);
        }
    }
    if (err) {
        part[threadIdx.x] = e;
        __syncthreads();
        for (int off = blockDim.x / 2; off > 0; off >>= 1) {
            if (threadIdx.x < off) part[threadIdx.x] += part[threadIdx.x + off];
            __syncthreads();
        }
        if (threadIdx.x == 0) err[b] = part[0];
    }
}

}  // namespace tvbg

using namespace tvbg;

namespace {
// Whether N nodes take the one-CTA small path: N (N + 1) / 2 pairs, counted
// in 64 bits (the product overflows 32 bits from N = 46341).
bool fc_small_path(int32_t N) {
    return static_cast<int64_t>(N) * (N + 1) / 2 <= static_cast<int64_t>(kFcThreads) * kMaxPairsPerThread;
}
}  // namespace

extern "C" int tvbg_fc_scratch_bytes(int32_t n_inst, int32_t N, int64_t* bytes) {
    if (!bytes || n_inst <= 0 || N <= 0) return set_error(TVBG_EINVAL, "tvbg_fc_scratch_bytes: bad args");
    if (fc_small_path(N)) {
        *bytes = 0;
    } else {
        *bytes = static_cast<int64_t>(n_inst) * N * (static_cast<int64_t>(N) + 1) *
                 static_cast<int64_t>(sizeof(double));
    }
    return TVBG_OK;
}

// Large-N FC needs caller scratch of tvbg_fc_scratch_bytes() (FP64 means and Gram).
extern "C" int tvbg_fc_ex(const float* d_x, int32_t n_inst, int32_t T, int32_t N,
                          int64_t inst_stride, float* d_fc, const float* d_target, double* d_err,
                          double* d_scratch, void* stream) {
    if (!d_x || !d_fc || n_inst <= 0 || T < 2 || N <= 0 || inst_stride < static_cast<int64_t>(T) * N)
        return set_error(TVBG_EINVAL, "tvbg_fc: bad arguments (need T >= 2, inst_stride >= T*N)");
    if ((d_target == nullptr) != (d_err == nullptr))
        return set_error(TVBG_EINVAL, "tvbg_fc: d_target and d_err go together");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (fc_small_path(N)) {
        const size_t smem = sizeof(double) * (static_cast<size_t>(N) + static_cast<size_t>(kTile) * N + kFcThreads);
        if (smem > 200 * 1024) return set_error(TVBG_EINVAL, "tvbg_fc: N too large for the small path");
        if (smem > 48 * 1024) {
            cudaError_t e = cudaFuncSetAttribute(fc_small_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 static_cast<int>(smem));
            if (e != cudaSuccess) return set_cuda_error(e, "tvbg_fc: smem attribute");
        }
        fc_small_kernel<<<n_inst, kFcThreads, smem, st>>>(d_x, T, N, inst_stride, d_fc, d_target, d_err);
    } else {
        if (!d_scratch) return set_error(TVBG_EINVAL, "tvbg_fc: N > 126 needs d_scratch (tvbg_fc_scratch_bytes)");
        double* mean = d_scratch;
        double* gram = d_scratch + static_cast<long long>(n_inst) * N;
        dim3 gm((N + 127) / 128, n_inst);
        fc_mean_kernel<<<gm, 128, 0, st>>>(d_x, T, N, inst_stride, mean);
        dim3 g((N + 15) / 16, (N + 15) / 16, n_inst), b(16, 16);
        fc_large_kernel<<<g, b, 0, st>>>(d_x, T, N, inst_stride, mean, gram);
        fc_norm_kernel<<<n_inst, 256, 0, st>>>(gram, N, d_fc, d_target, d_err);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_cuda_error(e, "tvbg_fc launch");
    return TVBG_OK;
}

extern "C" int tvbg_fc(const float* d_x, int32_t n_inst, int32_t T, int32_t N, int64_t inst_stride,
                       float* d_fc, const float* d_target, double* d_err, void* stream) {
    return tvbg_fc_ex(d_x, n_inst, T, N, inst_stride, d_fc, d_target, d_err, nullptr, stream);
}

// ---- allocation-free variant (tvbg_fc_noalloc) ------------------------------
// Scratch for callers that cannot allocate device memory: a file-scope device
// array, one instance per device that loads this library.  Host code must not
// pass `g_fc_noalloc_scratch` itself to a kernel (in host code the name is a
// host-side stand-in); its device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) double g_fc_noalloc_scratch[TVBG_FC_NOALLOC_MAX_DOUBLES];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
double* g_noalloc_addr[kMaxDevices] = {};

// Device address of the scratch array on `dev` (the current device), looked
// up once per device on first use.
int noalloc_scratch(int dev, double** out) {
    if (dev < 0 || dev >= kMaxDevices) return set_error(TVBG_EINVAL, "tvbg_fc_noalloc: device index out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_fc_noalloc_scratch);
        if (e != cudaSuccess) return set_cuda_error(e, "tvbg_fc_noalloc: cudaGetSymbolAddress");
        g_noalloc_addr[dev] = static_cast<double*>(p);
    }
    *out = g_noalloc_addr[dev];
    return TVBG_OK;
}
}  // namespace

extern "C" int tvbg_fc_noalloc(const float* d_x, int32_t n_inst, int32_t T, int32_t N,
                               int64_t inst_stride, float* d_fc, const float* d_target,
                               double* d_err, void* stream) {
    if (n_inst <= 0 || N <= 0) return set_error(TVBG_EINVAL, "tvbg_fc_noalloc: bad arguments");
    int64_t need = 0;
    int rc = tvbg_fc_scratch_bytes(n_inst, N, &need);
    if (rc) return rc;
    need /= static_cast<int64_t>(sizeof(double));
    if (need > TVBG_FC_NOALLOC_MAX_DOUBLES)
        return set_error(TVBG_EINVAL,
                         "tvbg_fc_noalloc: n_inst * N * (N + 1) exceeds TVBG_FC_NOALLOC_MAX_DOUBLES; "
                         "split the instances over several calls or use tvbg_fc_ex");
    double* scratch = nullptr;
    if (need > 0) {
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e != cudaSuccess) return set_cuda_error(e, "tvbg_fc_noalloc: cudaGetDevice");
        rc = noalloc_scratch(dev, &scratch);
        if (rc) return rc;
    }
    // the mean and Gram kernels write every scratch entry they later read,
    // so the previous call's contents need no clearing
    return tvbg_fc_ex(d_x, n_inst, T, N, inst_stride, d_fc, d_target, d_err, scratch, stream);
}
