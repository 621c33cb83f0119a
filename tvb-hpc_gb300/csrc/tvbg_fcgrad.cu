// The FC-fit loss path of the adjoint (tvbg_fcfit_loss, below) and its
// product dL/dZ = Z A alone (tvbg_fcfit_zgrad).
//
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

// ---------------------------------------------------------------------------
// The whole FC-fit loss path (tvbg_fcfit_loss): for instance b, the series
// X_b [T][N] (rows 0..T-2 from x, row T-1 from `last` when given), its
// Pearson FC in FP64, the loss mean_{i<j} (FC_ij - F*_ij)^2 and
// dL/dX = (Z A - Z diag(FC A)) / nrm, Z = (X - mean) / nrm, A = 2 (FC - F*) / P
// with a zero diagonal (P = N (N - 1) / 2).  Kernels: FP64 means; the
// centred Gram, upper triangle only (FP32 error-free transformations for
// N <= 192, FP64 tiles above); per instance the norms from the Gram's
// diagonal, FC, loss, A and diag(FC A) (the chain rule's time reduction
// sum_t Z_ti (Z A)_ti, taken from FC in FP64); dL/dX in FP32 (Z A is a sum
// over N nodes per sample, the precision of the backward).  The Pearson FC
// restates refs/covar.c:70-109 / metric.py:111-139 as a two-pass sum
// (centred Gram of the centred series) accurate to FP64 level.
// ---------------------------------------------------------------------------

namespace {

// Instance b of a series lives in block b / lanes at lane b % lanes:
// lanes = 1 for per-instance arrays, 8 for lane-interleaved groups.
struct SeriesView {
    const float* x;      // row s (s < T - 1, or every row without `last`):
    int64_t xs;          //   x + (b / lanes) xs + b % lanes + (s N + i) lanes
    const float* last;   // row T - 1: last + (b / lanes) ls + b % lanes + i lns, or NULL
    int64_t ls, lns;
    int T, N, lanes;
    __device__ __forceinline__ float at(int b, int s, int i) const {
        const int g = b / lanes, l = b % lanes;
        if (last && s == T - 1) return __ldg(last + g * ls + l + static_cast<int64_t>(i) * lns);
        return __ldg(x + g * xs + l + (static_cast<int64_t>(s) * N + i) * lanes);
    }
};

// FP64 mean of every (instance, node): the samples split into kMS slices
// of consecutive samples, one thread each, the slices' sums added in slice
// order.  CTA = 32 nodes x kMS slices of one instance (blockIdx.y).
constexpr int kMS = 8;
__global__ void __launch_bounds__(256) fcfit_mean_kernel(SeriesView v, double* mean) {
    __shared__ double part[kMS][32];
    const int b = blockIdx.y;
    const int i = blockIdx.x * 32 + static_cast<int>(threadIdx.x);
    const int per = (v.T + kMS - 1) / kMS;
    const int t0 = static_cast<int>(threadIdx.y) * per;
    const int t1 = t0 + per < v.T ? t0 + per : v.T;
    double s = 0.0;
    if (i < v.N)
        for (int t = t0; t < t1; ++t) s += static_cast<double>(v.at(b, t, i));
    part[threadIdx.y][threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.y == 0 && i < v.N) {
        double m = 0.0;
#pragma unroll
        for (int k = 0; k < kMS; ++k) m += part[k][threadIdx.x];
        mean[static_cast<int64_t>(b) * v.N + i] = m / static_cast<double>(v.T);
    }
}

// Error-free transformations in FP32 (Knuth's TwoSum and TwoProduct by FMA,
// as used in Ogita, Rump and Oishi, "Accurate sum and dot
// product", SIAM J. Sci. Comput. 26(6), 2005).  Every operation is an
// explicitly rounded intrinsic: nothing is contracted or reordered.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Centred Gram G_ij = sum_t c_ti c_tj, c = x - mean, for N <= kTriMaxN,
// all in FP32 arithmetic with error-free transformations (GB300 runs FP32
// at about 64 times its FP64 rate; one DFMA per product took 4.2 ms per
// adjoint pass at N = 84, 256 instances, 2000 samples).
//
// Work split: the exact upper triangle of 2 x 2 pair blocks (ceil(N/2)
// (ceil(N/2) + 1) / 2 of them, row-major), kSplitBPT blocks per thread,
// CTA = (instance blockIdx.x, part blockIdx.y), instances fastest so that
// the lanes of a lane-interleaved group read the same sectors together.
//
// Centring: each mean (FP64) is split once into mh + ml (FP32 words); a
// sample x becomes c = (x - mh) - ml as (hi, lo) with hi + lo = c up to
// about 2^-48 (|c| + 2 |mean|): TwoSum(x, -mh) = (d, de), then
// TwoSum(d, de - ml).  kTriL samples of every node staged per pass.
//
// Products: per pair and sample hi_i hi_j = p + e exactly (TwoProduct);
// p is summed by TwoSum (rounding errors collected in a second word),
// e + hi_i lo_j + lo_i hi_j (2^-24 of the product) in a third word; lo_i lo_j
// (2^-48) is dropped.  Every kTriL samples the three words are added into
// the pair's double-FP32 sum (TwoSum, then the small words, then TwoSum
// again), converted to FP64 at the end.  The error is bounded by about kTriL^2 2^-48 sum_t |c_ti c_tj| (the
// collected rounding errors of a pass summed in FP32), below 4e-12 of
// ||c_i|| ||c_j||; typical errors are near 1e-14.  Both triangles of G
// written.
constexpr int kTriL = 32;
constexpr int kTriMaxN = 192;   // staging (kTriL + 1) x N float2 <= 50.7 KB
constexpr int kSplitBPT = 2;
__global__ void __launch_bounds__(256) fcfit_gram_split_kernel(SeriesView v,
                                                               const double* __restrict__ mean,
                                                               double* G) {
    extern __shared__ float2 sh[];  // [kTriL][Np] (hi, lo); then [Np] (mh, ml)
    const int b = blockIdx.x;
    const int N = v.N;
    const int nb = (N + 1) / 2;
    const int Np = 2 * nb;
    float2* smean = sh + kTriL * Np;
    const long long nblk = static_cast<long long>(nb) * (nb + 1) / 2;
    int i0[kSplitBPT], j0[kSplitBPT];
    bool act[kSplitBPT];
#pragma unroll
    for (int q = 0; q < kSplitBPT; ++q) {
        const long long k =
            (static_cast<long long>(blockIdx.y) * kSplitBPT + q) * blockDim.x + threadIdx.x;
        act[q] = k < nblk;
        int bi = 0, bj = 0;
        if (act[q]) {
            long long rem = k;
            while (rem >= nb - bi) {
                rem -= nb - bi;
                ++bi;
            }
            bj = bi + static_cast<int>(rem);
        }
        i0[q] = 2 * bi;
        j0[q] = 2 * bj;
    }
    const double* mb = mean + static_cast<int64_t>(b) * N;
    for (int c = threadIdx.x; c < N; c += blockDim.x) {
        const double m = mb[c];
        const float mh = __double2float_rn(m);
        smean[c] = make_float2(mh, __double2float_rn(m - static_cast<double>(mh)));
    }
    float ah[kSplitBPT][4], al[kSplitBPT][4];  // double-FP32 sums
#pragma unroll
    for (int q = 0; q < kSplitBPT; ++q)
#pragma unroll
        for (int m = 0; m < 4; ++m) ah[q][m] = al[q][m] = 0.0f;
    __syncthreads();
    for (int t0 = 0; t0 < v.T; t0 += kTriL) {
        for (int e = threadIdx.x; e < kTriL * Np; e += blockDim.x) {
            const int r = e / Np, c = e % Np;
            const int t = t0 + r;
            float2 hl = make_float2(0.0f, 0.0f);
            if (t < v.T && c < N) {
                const float2 m = smean[c];
                float d, de;
                two_sum(v.at(b, t, c), -m.x, d, de);
                two_sum(d, __fsub_rn(de, m.y), hl.x, hl.y);
            }
            sh[e] = hl;
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < kSplitBPT; ++q) {
            if (!act[q]) continue;
            float s[4] = {0.0f, 0.0f, 0.0f, 0.0f}, cp[4] = {0.0f, 0.0f, 0.0f, 0.0f};
            float sm[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll 4
            for (int r = 0; r < kTriL; ++r) {
                const float2* row = sh + r * Np;
                const float2 x[2] = {row[i0[q]], row[i0[q] + 1]};
                const float2 y[2] = {row[j0[q]], row[j0[q] + 1]};
#pragma unroll
                for (int u = 0; u < 2; ++u)
#pragma unroll
                    for (int w = 0; w < 2; ++w) {
                        const int m = 2 * u + w;
                        const float p = __fmul_rn(x[u].x, y[w].x);
                        const float e = __fmaf_rn(x[u].x, y[w].x, -p);  // hi hi - p, exact
                        sm[m] = __fadd_rn(sm[m], __fmaf_rn(x[u].x, y[w].y, __fmaf_rn(x[u].y, y[w].x, e)));
                        float t, err;
                        two_sum(s[m], p, t, err);
                        s[m] = t;
                        cp[m] = __fadd_rn(cp[m], err);
                    }
            }
#pragma unroll
            for (int m = 0; m < 4; ++m) {  // (ah, al) += s + (cp + sm)
                float hi, lo;
                two_sum(ah[q][m], s[m], hi, lo);
                lo = __fadd_rn(lo, __fadd_rn(al[q][m], __fadd_rn(cp[m], sm[m])));
                two_sum(hi, lo, ah[q][m], al[q][m]);
            }
        }
        __syncthreads();
    }
    double* gb = G + static_cast<int64_t>(b) * N * N;
#pragma unroll
    for (int q = 0; q < kSplitBPT; ++q) {
        if (!act[q]) continue;
#pragma unroll
        for (int u = 0; u < 2; ++u)
#pragma unroll
            for (int w = 0; w < 2; ++w) {
                const int i = i0[q] + u, j = j0[q] + w;
                if (i < N && j < N && j >= i) {
                    const double g = static_cast<double>(ah[q][2 * u + w]) +
                                     static_cast<double>(al[q][2 * u + w]);
                    gb[static_cast<int64_t>(i) * N + j] = g;
                    gb[static_cast<int64_t>(j) * N + i] = g;
                }
            }
    }
}

constexpr int kGT = 32;   // Gram tile: 32 x 32 node pairs, 32 samples per stage

// The centred Gram for larger N: one CTA per upper-triangle 32 x 32 tile
// (blockIdx.y enumerates tiles with jt >= it; instance blockIdx.x), 256
// threads of 2 x 2 pairs, samples in order; both triangles written.
__global__ void __launch_bounds__(256) fcfit_gram_kernel(SeriesView v, const double* __restrict__ mean,
                                                         double* G) {
    __shared__ double sI[kGT][kGT + 1];
    __shared__ double sJ[kGT][kGT + 1];
    const int b = blockIdx.x;
    const int N = v.N;
    const int nt = (N + kGT - 1) / kGT;
    int it = 0, rem = blockIdx.y;
    while (rem >= nt - it) {
        rem -= nt - it;
        ++it;
    }
    const int jt = it + rem;
    const int i0 = it * kGT, j0 = jt * kGT;
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const double* mb = mean + static_cast<int64_t>(b) * N;
    double acc[2][2] = {{0.0, 0.0}, {0.0, 0.0}};
    for (int t0 = 0; t0 < v.T; t0 += kGT) {
        for (int k = threadIdx.x; k < kGT * kGT; k += 256) {
            const int r = k / kGT, c = k % kGT;   // r: sample, c: node within the tile
            const int t = t0 + r;
            const int ii = i0 + c, jj = j0 + c;
            sI[r][c] = (t < v.T && ii < N) ? static_cast<double>(v.at(b, t, ii)) - mb[ii] : 0.0;
            sJ[r][c] = (t < v.T && jj < N) ? static_cast<double>(v.at(b, t, jj)) - mb[jj] : 0.0;
        }
        __syncthreads();
#pragma unroll 8
        for (int r = 0; r < kGT; ++r) {
            const double a0 = sI[r][2 * ty], a1 = sI[r][2 * ty + 1];
            const double c0 = sJ[r][2 * tx], c1 = sJ[r][2 * tx + 1];
            acc[0][0] = fma(a0, c0, acc[0][0]);
            acc[0][1] = fma(a0, c1, acc[0][1]);
            acc[1][0] = fma(a1, c0, acc[1][0]);
            acc[1][1] = fma(a1, c1, acc[1][1]);
        }
        __syncthreads();
    }
    double* gb = G + static_cast<int64_t>(b) * N * N;
#pragma unroll
    for (int u = 0; u < 2; ++u)
#pragma unroll
        for (int w = 0; w < 2; ++w) {
            const int i = i0 + 2 * ty + u, j = j0 + 2 * tx + w;
            if (i < N && j < N && j >= i) {
                gb[static_cast<int64_t>(i) * N + j] = acc[u][w];
                gb[static_cast<int64_t>(j) * N + i] = acc[u][w];
            }
        }
}

// Per instance (one CTA): nrm_i = sqrt(G_ii) (the centred sum of squares);
// FC_ij = G_ij / (nrm_i nrm_j) in place; loss_b = sum_{i<j} (FC - F*)^2 / P;
// A = 2 (FC - F*) / P with a zero diagonal (FP32 copy for Z A);
// zg_i = sum_j FC_ij A_ij (FP64); and the FP32 factors of the dL/dX
// epilogue per node: mean, 1 / nrm, zg / nrm (rounded once from FP64).
__global__ void __launch_bounds__(256) fcfit_loss_kernel(double* fc, const double* __restrict__ target,
                                                         int N, const double* __restrict__ mean,
                                                         double* nrm, double* loss, float* a32,
                                                         double* zg, float* fs) {
    __shared__ double red[256];
    const int b = blockIdx.x;
    const double P = 0.5 * static_cast<double>(N) * (N - 1);
    double* fb = fc + static_cast<int64_t>(b) * N * N;
    double* nb = nrm + static_cast<int64_t>(b) * N;
    float* ab = a32 + static_cast<int64_t>(b) * N * N;
    for (int i = threadIdx.x; i < N; i += blockDim.x) nb[i] = sqrt(fb[static_cast<int64_t>(i) * N + i]);
    __syncthreads();
    double part = 0.0;
    for (int64_t k = threadIdx.x; k < static_cast<int64_t>(N) * N; k += blockDim.x) {
        const int i = static_cast<int>(k / N), j = static_cast<int>(k % N);
        const double r = fb[k] / (nb[i] * nb[j]);
        fb[k] = r;
        const double d = r - target[k];
        if (j > i) part = fma(d, d, part);
        ab[k] = i == j ? 0.0f : static_cast<float>(2.0 * d / P);
    }
    red[threadIdx.x] = part;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (static_cast<int>(threadIdx.x) < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) loss[b] = red[0] / P;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        double s = 0.0;
        for (int j = 0; j < N; ++j) {
            if (j == i) continue;
            const double d = fb[static_cast<int64_t>(i) * N + j] - target[static_cast<int64_t>(i) * N + j];
            s = fma(fb[static_cast<int64_t>(i) * N + j], 2.0 * d / P, s);
        }
        const int64_t bi = static_cast<int64_t>(b) * N + i;
        zg[bi] = s;
        fs[3 * bi] = static_cast<float>(mean[bi]);
        fs[3 * bi + 1] = static_cast<float>(1.0 / nb[i]);
        fs[3 * bi + 2] = static_cast<float>(s / nb[i]);
    }
}

// dL/dX_tj = ((Z A)_tj - Z_tj zg_j) / nrm_j with Z = (x - mean) / nrm formed
// on the fly in FP32 (the backward's precision); the tiled FP32 product of
// fcgrad_kernel with that epilogue.
// Grid (instance, sample tile, node tile), instances fastest.
__global__ void __launch_bounds__(256)
    fcfit_dx_kernel(SeriesView v, const float* __restrict__ fs, const float* __restrict__ A,
                    float* __restrict__ dx, int64_t dxs) {
    __shared__ float sZ[kTK][kTM + 4];  // [k][t]
    __shared__ float sA[kTK][kTN];      // [k][j]
    const int b = blockIdx.x;
    const int T = v.T, N = v.N;
    const int t0 = blockIdx.y * kTM, j0 = blockIdx.z * kTN;
    const float* fb = fs + static_cast<int64_t>(b) * N * 3;   // [N][mean, 1/nrm, zg/nrm]
    const float* Ab = A + static_cast<size_t>(b) * N * N;
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    float acc[4][4] = {};
    for (int k0 = 0; k0 < N; k0 += kTK) {
        for (int i = threadIdx.x; i < kTM * kTK; i += 256) {
            const int r = i / kTK, c = i % kTK;
            const int t = t0 + r, k = k0 + c;
            sZ[c][r] = (t < T && k < N) ? (v.at(b, t, k) - fb[3 * k]) * fb[3 * k + 1] : 0.0f;
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
                for (int w = 0; w < 4; ++w) acc[u][w] = fmaf(z[u], a[w], acc[u][w]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int t = t0 + ty * 4 + u;
        if (t >= T) continue;
#pragma unroll
        for (int w = 0; w < 4; ++w) {
            const int j = j0 + tx * 4 + w;
            if (j >= N) continue;
            const float z = (v.at(b, t, j) - fb[3 * j]) * fb[3 * j + 1];
            dx[b * dxs + static_cast<int64_t>(t) * N + j] =
                fmaf(-z, fb[3 * j + 2], acc[u][w] * fb[3 * j + 1]);
        }
    }
}

// The same product for N <= 16 WN, whole rows: CTA = (instance blockIdx.x,
// 64 samples blockIdx.y), A_b [N][16 WN] and the Z tile [64][N + 1] staged
// in shared memory once; thread (tx, ty) of 16 x 16 owns samples 4 ty .. +3
// and nodes tx + 16 w.  Sums over k in order, as fcfit_dx_kernel: the same
// results.
template <int WN>
__global__ void __launch_bounds__(256)
    fcfit_dx_rows_kernel(SeriesView v, const float* __restrict__ fs, const float* __restrict__ A,
                         float* __restrict__ dx, int64_t dxs) {
    extern __shared__ float sm[];
    constexpr int NP = 16 * WN;
    const int b = blockIdx.x;
    const int T = v.T, N = v.N;
    const int t0 = blockIdx.y * 64;
    float* sA = sm;             // [N][NP]
    float* sZ = sm + N * NP;    // [64][N + 1]
    const int zs = N + 1;
    const float* fb = fs + static_cast<int64_t>(b) * N * 3;
    const float* Ab = A + static_cast<size_t>(b) * N * N;
    for (int e = threadIdx.x; e < N * NP; e += 256) {
        const int k = e / NP, j = e % NP;
        sA[e] = j < N ? __ldg(Ab + static_cast<size_t>(k) * N + j) : 0.0f;
    }
    for (int e = threadIdx.x; e < 64 * N; e += 256) {
        const int r = e / N, k = e % N;
        const int t = t0 + r;
        sZ[r * zs + k] = t < T ? (v.at(b, t, k) - fb[3 * k]) * fb[3 * k + 1] : 0.0f;
    }
    __syncthreads();
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    float acc[4][WN] = {};
    for (int k = 0; k < N; ++k) {
        float z[4], a[WN];
#pragma unroll
        for (int u = 0; u < 4; ++u) z[u] = sZ[(ty * 4 + u) * zs + k];
#pragma unroll
        for (int w = 0; w < WN; ++w) a[w] = sA[k * NP + tx + 16 * w];
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int w = 0; w < WN; ++w) acc[u][w] = fmaf(z[u], a[w], acc[u][w]);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int t = t0 + ty * 4 + u;
        if (t >= T) continue;
#pragma unroll
        for (int w = 0; w < WN; ++w) {
            const int j = tx + 16 * w;
            if (j >= N) continue;
            const float z = sZ[(ty * 4 + u) * zs + j];
            dx[b * dxs + static_cast<int64_t>(t) * N + j] =
                fmaf(-z, fb[3 * j + 2], acc[u][w] * fb[3 * j + 1]);
        }
    }
}

template <int WN>
int launch_dx_rows(SeriesView v, const float* fs, const float* A, float* dx, int64_t dxs, int n_inst,
                   cudaStream_t st) {
    const size_t smem = 4u * (static_cast<size_t>(v.N) * 16 * WN + 64u * (v.N + 1));
    if (smem > 48u * 1024u) {
        const cudaError_t e = cudaFuncSetAttribute(reinterpret_cast<const void*>(fcfit_dx_rows_kernel<WN>),
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   static_cast<int>(smem));
        if (e != cudaSuccess) return tvbg::set_cuda_error(e, "tvbg_fcfit_loss: smem attribute");
    }
    const dim3 grid(static_cast<unsigned>(n_inst), static_cast<unsigned>((v.T + 63) / 64));
    fcfit_dx_rows_kernel<WN><<<grid, 256, smem, st>>>(v, fs, A, dx, dxs);
    return TVBG_OK;
}

}  // namespace

extern "C" int tvbg_fcfit_scratch_bytes(int32_t n_inst, int32_t N, int64_t* bytes) {
    if (!bytes || n_inst <= 0 || N <= 0) return tvbg::set_error(TVBG_EINVAL, "tvbg_fcfit_scratch_bytes: bad args");
    const int64_t nn = static_cast<int64_t>(N) * N, in = static_cast<int64_t>(n_inst);
    // mean, nrm, zg [I][N] FP64; FC [I][N][N] FP64; A [I][N][N] FP32; the
    // epilogue factors [I][N][3] FP32 (each 256-byte aligned)
    auto al = [](int64_t x) { return (x + 255) & ~static_cast<int64_t>(255); };
    *bytes = 3 * al(in * N * 8) + al(in * nn * 8) + al(in * nn * 4) + al(in * N * 12);
    return TVBG_OK;
}

extern "C" int tvbg_fcfit_loss(const float* d_x, int64_t x_inst_stride, const float* d_last,
                               int64_t last_inst_stride, int64_t last_node_stride, int32_t lanes,
                               int32_t n_inst, int32_t T, int32_t N, const double* d_target,
                               double* d_loss, float* d_dx, int64_t dx_inst_stride, double* d_fc,
                               void* d_scratch, void* stream) {
    if (!d_x || !d_target || !d_loss || !d_scratch || n_inst <= 0 || n_inst > 65535 || T < 2 ||
        N < 2 || x_inst_stride < 0 || lanes < 1 || lanes > 8 ||
        (d_dx && dx_inst_stride < static_cast<int64_t>(T) * N))
        return tvbg::set_error(TVBG_EINVAL, "tvbg_fcfit_loss: bad arguments (need T >= 2, N >= 2)");
    const int64_t nn = static_cast<int64_t>(N) * N, in = static_cast<int64_t>(n_inst);
    auto al = [](int64_t x) { return (x + 255) & ~static_cast<int64_t>(255); };
    char* s = static_cast<char*>(d_scratch);
    double* mean = reinterpret_cast<double*>(s);
    double* nrm = reinterpret_cast<double*>(s + al(in * N * 8));
    double* zg = reinterpret_cast<double*>(s + 2 * al(in * N * 8));
    double* fc = d_fc ? d_fc : reinterpret_cast<double*>(s + 3 * al(in * N * 8));
    float* a32 = reinterpret_cast<float*>(s + 3 * al(in * N * 8) + al(in * nn * 8));
    float* fsc = reinterpret_cast<float*>(s + 3 * al(in * N * 8) + al(in * nn * 8) + al(in * nn * 4));
    SeriesView v{d_x, x_inst_stride, d_last, last_inst_stride, last_node_stride, T, N, lanes};
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if ((T + 63) / 64 > 65535) return tvbg::set_error(TVBG_EINVAL, "tvbg_fcfit_loss: T too large");
    const int nt = (N + kGT - 1) / kGT;
    if (N > kTriMaxN && nt * (nt + 1) / 2 > 65535)
        return tvbg::set_error(TVBG_EINVAL, "tvbg_fcfit_loss: N too large");
    fcfit_mean_kernel<<<dim3((N + 31) / 32, n_inst), dim3(32, kMS), 0, st>>>(v, mean);
    if (N <= kTriMaxN) {
        const int nb = (N + 1) / 2;
        const long long nblk = static_cast<long long>(nb) * (nb + 1) / 2;
        const unsigned parts = static_cast<unsigned>((nblk + 256 * kSplitBPT - 1) / (256 * kSplitBPT));
        const size_t smem = 8u * (kTriL + 1) * 2u * static_cast<size_t>(nb);
        if (smem > 48u * 1024u) {
            const cudaError_t e = cudaFuncSetAttribute(reinterpret_cast<const void*>(fcfit_gram_split_kernel),
                                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                       static_cast<int>(smem));
            if (e != cudaSuccess) return tvbg::set_cuda_error(e, "tvbg_fcfit_loss: smem attribute");
        }
        fcfit_gram_split_kernel<<<dim3(n_inst, parts), 256, smem, st>>>(v, mean, fc);
    } else {
        fcfit_gram_kernel<<<dim3(n_inst, nt * (nt + 1) / 2), 256, 0, st>>>(v, mean, fc);
    }
    fcfit_loss_kernel<<<n_inst, 256, 0, st>>>(fc, d_target, N, mean, nrm, d_loss, a32, zg, fsc);
    if (d_dx) {
        int rc = TVBG_OK;
        if (N <= 32) rc = launch_dx_rows<2>(v, fsc, a32, d_dx, dx_inst_stride, n_inst, st);
        else if (N <= 64) rc = launch_dx_rows<4>(v, fsc, a32, d_dx, dx_inst_stride, n_inst, st);
        else if (N <= 96) rc = launch_dx_rows<6>(v, fsc, a32, d_dx, dx_inst_stride, n_inst, st);
        else if (N <= 128) rc = launch_dx_rows<8>(v, fsc, a32, d_dx, dx_inst_stride, n_inst, st);
        else {
            const dim3 grid(n_inst, (T + kTM - 1) / kTM, (N + kTN - 1) / kTN);
            if (grid.z > 65535u) return tvbg::set_error(TVBG_EINVAL, "tvbg_fcfit_loss: N too large");
            fcfit_dx_kernel<<<grid, 256, 0, st>>>(v, fsc, a32, d_dx, dx_inst_stride);
        }
        if (rc != TVBG_OK) return rc;
    }
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? TVBG_OK : tvbg::set_cuda_error(e, "tvbg_fcfit_loss launch");
}
