// Streaming (online) covariance per instance with FP64 Welford updates, and
// its Pearson correlation.
//
// Restates the online co-moment of tvb_hpc/metric.py:87-108 (OnlineCov) and
// dsl/dsl_cuda/CUDAmodels/refs/covar.c:9-68 (update_cov), in FP64 and with
// the Welford form of the update: for the (n+1)-th sample x,
//   d_i    = x_i - mean_i
//   mean_i += d_i / (n + 1)
//   m2_ij  += d_i (x_j - mean_j')          (mean' the updated mean)
// so after n samples m2 is the co-moment sum_s (x_si - m_i)(x_sj - m_j) and
// corr_ij = m2_ij / sqrt(m2_ii m2_jj) (covar.c:73-109, whose 1/n
// normalisation cancels in the ratio).  One CTA per instance; the instance's
// sample and means are staged in shared memory.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "tvbg_abi_internal.h"

namespace tvbg {

constexpr int kCovThreads = 256;

__global__ void __launch_bounds__(kCovThreads)
    cov_update_kernel(const float* __restrict__ x, long long x_stride, int N, long long n,
                      double* __restrict__ mean, double* __restrict__ m2) {
    extern __shared__ double sh[];  // d[N] | x[N] - mean'[N]
    double* d = sh;
    double* e = sh + N;
    const long long b = blockIdx.x;
    const float* xb = x + b * x_stride;
    double* mb = mean + b * N;
    double* cb = m2 + b * static_cast<long long>(N) * N;
    const double rn = 1.0 / static_cast<double>(n + 1);
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        const double xi = static_cast<double>(xb[i]);
        const double m_old = n == 0 ? 0.0 : mb[i];
        const double di = xi - m_old;
        const double m_new = m_old + di * rn;
        d[i] = di;
        e[i] = xi - m_new;
        mb[i] = m_new;
    }
    __syncthreads();
    const long long NN = static_cast<long long>(N) * N;
    for (long long q = threadIdx.x; q < NN; q += blockDim.x) {
        const int i = static_cast<int>(q / N), j = static_cast<int>(q % N);
        const double inc = d[i] * e[j];
        cb[q] = n == 0 ? inc : cb[q] + inc;   // n == 0 starts the co-moment (inc is 0)
    }
}

__global__ void __launch_bounds__(kCovThreads)
    cov_corr_kernel(const double* __restrict__ m2, int N, float* __restrict__ corr) {
    const long long b = blockIdx.x;
    const double* cb = m2 + b * static_cast<long long>(N) * N;
    float* ob = corr + b * static_cast<long long>(N) * N;
    const long long NN = static_cast<long long>(N) * N;
    for (long long q = threadIdx.x; q < NN; q += blockDim.x) {
        const int i = static_cast<int>(q / N), j = static_cast<int>(q % N);
        const double den = sqrt(cb[static_cast<long long>(i) * N + i] * cb[static_cast<long long>(j) * N + j]);
        ob[q] = static_cast<float>(cb[q] / den);
    }
}

}  // namespace tvbg

using namespace tvbg;

extern "C" int tvbg_cov_update(const float* d_x, int64_t x_stride, int32_t n_inst, int32_t N,
                               int64_t n, double* d_mean, double* d_m2, void* stream) {
    if (n_inst < 0 || N <= 0 || n < 0 || x_stride < N || (n_inst > 0 && (!d_x || !d_mean || !d_m2)))
        return set_error(TVBG_EINVAL, "tvbg_cov_update: bad arguments");
    if (N > 3000) return set_error(TVBG_EINVAL, "tvbg_cov_update: N above 3000");
    if (n_inst == 0) return TVBG_OK;
    const size_t smem = 2u * sizeof(double) * static_cast<size_t>(N);
    cov_update_kernel<<<n_inst, kCovThreads, smem, static_cast<cudaStream_t>(stream)>>>(
        d_x, x_stride, N, n, d_mean, d_m2);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_cuda_error(e, "tvbg_cov_update launch");
    return TVBG_OK;
}

extern "C" int tvbg_cov_corr(const double* d_m2, int32_t n_inst, int32_t N, float* d_corr,
                             void* stream) {
    if (n_inst < 0 || N <= 0 || (n_inst > 0 && (!d_m2 || !d_corr)))
        return set_error(TVBG_EINVAL, "tvbg_cov_corr: bad arguments");
    if (n_inst == 0) return TVBG_OK;
    cov_corr_kernel<<<n_inst, kCovThreads, 0, static_cast<cudaStream_t>(stream)>>>(d_m2, N, d_corr);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_cuda_error(e, "tvbg_cov_corr launch");
    return TVBG_OK;
}
