// Reverse-time adjoint of the delayed Euler scheme (Montbrio-Pazo-Roxin,
// linear coupling), one CTA per instance, one thread per node.  The
// recursion and its terms are documented at tvbg_adjoint_mpr in tvbg.h.
#include <cuda_runtime.h>

#include "tvbg_abi_internal.h"
#include "tvbg_device.cuh"

namespace tvbg {

// The adjoint ring of mu_V: global memory, or staged in shared memory for
// the kernel's run (loaded at the start, stored at the end: it carries mu_V
// across segments).
template <bool SMEM>
struct AdjRing;
template <>
struct AdjRing<false> {
    float* p;
    __device__ __forceinline__ float ld(uint32_t i) const { return p[i]; }
    __device__ __forceinline__ void st(uint32_t i, float v) const { p[i] = v; }
};
template <>
struct AdjRing<true> {
    float* p;  // shared
    __device__ __forceinline__ float ld(uint32_t i) const { return p[i]; }
    __device__ __forceinline__ void st(uint32_t i, float v) const { p[i] = v; }
};

template <bool SMEM>
__device__ __forceinline__ void adjoint_segment(const tvbg_adjoint& a, AdjRing<SMEM> ring) {
    const int j = threadIdx.x;
    const int N = a.N;
    const bool own = j < N;
    const uint32_t lognh = static_cast<uint32_t>(a.lognh);
    const uint32_t mask = (1u << lognh) - 1u;
    const float Delta = a.consts[0], J = a.consts[1], tau = a.consts[2];
    const float pi = 3.14159265358979323846f;
    const float dt = a.dt;
    const float cG = dt * a.G / tau;
    float lr = 0.f, lv = 0.f;
    double deta = 0.0, dG = 0.0;
    int lo = 0, hi = 0;
    if (own) {
        lr = a.lam[2 * j];
        lv = a.lam[2 * j + 1];
        lo = __ldg(a.row_t + j);
        hi = __ldg(a.row_t + j + 1);
    }
    const uint32_t my_row = static_cast<uint32_t>(j) << lognh;
    const uint2* __restrict__ edges = reinterpret_cast<const uint2*>(a.edges_t);
    for (int k = a.len - 1; k >= 0; --k) {
        const long long t = a.t0 + k;
        const uint32_t tm = static_cast<uint32_t>(t) & mask;
        float r = 0.f, V = 0.f, S = 0.f, mr = 0.f, mv = 0.f;
        if (own) {
            const long long sl = a.seg_lanes > 1 ? a.seg_lanes : 1;
            const float* x = a.seg + (static_cast<long long>(k) * N + j) * 3 * sl;
            r = x[0];
            V = x[sl];
            S = x[2 * sl];
            // the rate update of step t was clamped at 0 where it went negative
            const float fr = (Delta / (pi * tau) + 2.0f * r * V) * (1.0f / tau);  // as MPR::drift
            const float rpre = fmaf(dt, fr, r);
            mr = rpre >= 0.0f ? lr : 0.0f;
            mv = lv;
            ring.st(my_row | ((tm + 1u + static_cast<uint32_t>(j)) & mask), mv);
        }
        __syncthreads();
        if (own) {
            // out-edges in order, four loads in flight
            float coup = 0.0f;
            int e = lo;
            for (; e + 4 <= hi; e += 4) {
                float v[4], w[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const uint2 ew = __ldg(edges + e + u);
                    v[u] = ring.ld(((tm + ew.x) & mask) | (ew.x & ~mask));
                    w[u] = __uint_as_float(ew.y);
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) coup = fmaf(w[u], v[u], coup);
            }
            for (; e < hi; ++e) {
                const uint2 ew = __ldg(edges + e);
                coup = fmaf(__uint_as_float(ew.y), ring.ld(((tm + ew.x) & mask) | (ew.x & ~mask)), coup);
            }
            const float dfr_dr = 2.0f * V / tau, dfr_dV = 2.0f * r / tau;
            const float dfV_dr = (J * tau - 2.0f * pi * pi * tau * tau * r) / tau;
            const float dfV_dV = 2.0f * V / tau;
            float nlr = mr + dt * (mr * dfr_dr + mv * dfV_dr) + cG * coup;
            const float nlv = mv + dt * (mr * dfr_dV + mv * dfV_dV);
            nlr += a.dr[static_cast<long long>(k) * N + j];
            deta += static_cast<double>(dt / tau) * static_cast<double>(mv);
            dG += static_cast<double>(dt / tau) * static_cast<double>(mv) * static_cast<double>(S);
            lr = nlr;
            lv = nlv;
        }
        __syncthreads();
    }
    if (own) {
        a.lam[2 * j] = lr;
        a.lam[2 * j + 1] = lv;
        a.deta[j] += deta;
        a.dG[j] += dG;
    }
}

// smem_ring: bytes of shared memory for the ring (0 = global); an instance
// whose ring does not fit uses the global ring.
__global__ void __launch_bounds__(1024, 1)
    adjoint_mpr_kernel(const tvbg_adjoint* __restrict__ adj, int32_t n_inst, uint32_t smem_ring) {
    extern __shared__ __align__(16) float s_ring[];
    if (static_cast<int>(blockIdx.x) >= n_inst) return;
    const tvbg_adjoint a = adj[blockIdx.x];
    const uint32_t floats = static_cast<uint32_t>(a.N) << a.lognh;
    if (smem_ring >= 4u * floats && a.N > 0) {
        for (uint32_t i = threadIdx.x; i < floats; i += blockDim.x) s_ring[i] = a.ring[i];
        __syncthreads();
        adjoint_segment<true>(a, AdjRing<true>{s_ring});
        for (uint32_t i = threadIdx.x; i < floats; i += blockDim.x) a.ring[i] = s_ring[i];
    } else {
        adjoint_segment<false>(a, AdjRing<false>{a.ring});
    }
}

}  // namespace tvbg

using namespace tvbg;

static int adjoint_launch(const tvbg_adjoint* d_adj, int32_t n_inst, int32_t threads,
                          int32_t smem_ring, void* stream) {
    if (!d_adj || n_inst < 0 || threads < 32 || threads > 1024 || (threads & 31) || smem_ring < 0)
        return set_error(TVBG_EINVAL, "tvbg_adjoint_mpr: bad arguments");
    if (n_inst == 0) return TVBG_OK;
    const size_t smem = static_cast<size_t>(smem_ring);
    if (smem > 48u * 1024u) {
        int dev = 0, optin = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e == cudaSuccess)
            e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        if (e != cudaSuccess) return set_cuda_error(e, "tvbg_adjoint_mpr: device attributes");
        if (smem > static_cast<size_t>(optin))
            return set_error(TVBG_EINVAL, "tvbg_adjoint_mpr: ring exceeds the shared memory of one CTA");
        e = cudaFuncSetAttribute(reinterpret_cast<const void*>(adjoint_mpr_kernel),
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        if (e != cudaSuccess) return set_cuda_error(e, "tvbg_adjoint_mpr: smem attribute");
    }
    adjoint_mpr_kernel<<<n_inst, threads, smem, static_cast<cudaStream_t>(stream)>>>(
        d_adj, n_inst, static_cast<uint32_t>(smem_ring));
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_cuda_error(e, "tvbg_adjoint_mpr launch");
    return TVBG_OK;
}

extern "C" int tvbg_adjoint_mpr(const tvbg_adjoint* d_adj, int32_t n_inst, int32_t threads,
                                void* stream) {
    return adjoint_launch(d_adj, n_inst, threads, 0, stream);
}

extern "C" int tvbg_adjoint_mpr_ex(const tvbg_adjoint* d_adj, int32_t n_inst, int32_t threads,
                                   int32_t smem_ring, void* stream) {
    return adjoint_launch(d_adj, n_inst, threads, smem_ring, stream);
}
