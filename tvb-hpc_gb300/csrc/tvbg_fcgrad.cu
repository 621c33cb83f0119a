// dL/dZ = Z A of the FC-fit loss, per instance: Z [T][N] (the normalised,
// centred series), A [N][N] (2 (FC - target) / P with a zero diagonal),
// FP32.  A batched tiled product on the CUDA cores: one CTA per 64 x 64
// output tile of one instance, 256 threads of 4 x 4 outputs each, the A and
// Z panels staged through shared memory 16 columns at a time.  It is a sum
// over the N nodes per sample (the loss's reductions over time, the FC
// itself, stay FP64 in the caller).
#include "tvbg_abi_internal.h"

namespace {

constexpr int kTM = 64, kTN = 64, kTK = 16;

__global__ void __launch_bounds__(256)
    fcgrad_kernel(const float* __restrict__ Z, const float* __restrict__ A, float* __restrict__ out,
                  int T, int N) {
    __shared__ float sZ[kTK][kTM + 4];  // [k][t]
    __shared__ float sA[kTK][kTN];      // [k][j]
    const int b = blockIdx.z;
    const int t0 = blockIdx.y * kTM, j0 = blockIdx.x * kTN;
    const float* Zb = Z + static_cast<size_t>(b) * T * N;
    const float* Ab = A + static_cast<size_t>(b) * N * N;
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;  // 16 x 16 threads, 4 x 4 outputs each
    float acc[4][4] = {};
    for (int k0 = 0; k0 < N; k0 += kTK) {
        // Z panel: 64 rows (t) x 16 columns (k); A panel: 16 rows (k) x 64 columns (j)
        for (int i = threadIdx.x; i < kTM * kTK; i += 256) {
            const int r = i / kTK, c = i % kTK;
            const int t = t0 + r, k = k0 + c;
            sZ[c][r] = (t < T && k < N) ? __ldg(Zb + static_cast<size_t>(t) * N + k) : 0.0f;
        }
        for (int i = threadIdx.x; i < kTK * kTN; i += 256) {
            const int r = i / kTN, c = i % kTN;
            const int k = k0 + r, j = j0 + c;
            sA[r][c] = (k < N && j < N) ? __ldg(Ab + static_cast<size_t>(k) * N + j) : 0.0f;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kTK; ++k) {
            float z[4], a[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                z[u] = sZ[k][ty * 4 + u];
                a[u] = sA[k][tx * 4 + u];
            }
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v) acc[u][v] = fmaf(z[u], a[v], acc[u][v]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int t = t0 + ty * 4 + u;
        if (t >= T) continue;
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int j = j0 + tx * 4 + v;
            if (j < N) out[static_cast<size_t>(b) * T * N + static_cast<size_t>(t) * N + j] = acc[u][v];
        }
    }
}

}  // namespace

extern "C" int tvbg_fcfit_zgrad(const float* d_z, const float* d_a, float* d_out, int32_t n_inst,
                               int32_t T, int32_t N, void* stream) {
    if (n_inst < 0 || T < 0 || N < 0 || n_inst > 65535 ||
        (static_cast<long long>(n_inst) * T * N > 0 && (!d_z || !d_a || !d_out)))
        return tvbg::set_error(TVBG_EINVAL, "tvbg_fcfit_zgrad: bad arguments");
    if (n_inst == 0 || T == 0 || N == 0) return TVBG_OK;
    const dim3 grid((N + kTN - 1) / kTN, (T + kTM - 1) / kTM, n_inst);
    if (grid.y > 65535u) return tvbg::set_error(TVBG_EINVAL, "tvbg_fcfit_zgrad: T too large");
    fcgrad_kernel<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(d_z, d_a, d_out, T, N);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? TVBG_OK : tvbg::set_cuda_error(e, "tvbg_fcfit_zgrad launch");
}
