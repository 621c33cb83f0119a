// Reverse-time adjoint of the delayed Euler scheme (Montbrio-Pazo-Roxin,
// linear coupling): one CTA per instance and one thread per node
// (adjoint_mpr_kernel), or lane-interleaved groups of 8 instances,
// time-blocked (adjoint_group_kernel).  The recursion and its terms are
// documented at tvbg_adjoint_mpr in tvbg.h.
#include <cuda_runtime.h>

#include <cstring>

#include "tvbg_abi_internal.h"
#include "tvbg_device.cuh"
#include "tvbg_lanes.cuh"

namespace tvbg {

// One reverse step of one node, shared by both kernels so that they compute
// the same numbers.  adj_mu_r: mu_r(t+1) = lambda_r(t+1), masked where the
// rate update of step t was clamped at 0 (rpre as MPR::drift computes it).
struct AdjMpr {
    float Delta, J, tau, dt;

    __device__ __forceinline__ float mu_r(float r, float V, float lr) const {
        const float pi = 3.14159265358979323846f;
        const float fr = (Delta / (pi * tau) + 2.0f * r * V) * (1.0f / tau);  // as MPR::drift
        const float rpre = fmaf(dt, fr, r);
        return rpre >= 0.0f ? lr : 0.0f;
    }

    // lambda(t) from mu(t+1) = (mr, mv), the coupling gather and dL/dr(t).
    // Every rounding is spelled out (no contraction left to the compiler), so
    // both kernels produce the same bits.
    __device__ __forceinline__ void update(float r, float V, float S, float mr, float mv, float coup,
                                           float cG, float drt, float& lr, float& lv, double& deta,
                                           double& dG) const {
        const float pi = 3.14159265358979323846f;
        const float dfr_dr = __fdiv_rn(__fmul_rn(2.0f, V), tau);  // = dfV_dV
        const float dfr_dV = __fdiv_rn(__fmul_rn(2.0f, r), tau);
        const float c2 = __fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(2.0f, pi), pi), tau), tau);
        const float dfV_dr = __fdiv_rn(__fsub_rn(__fmul_rn(J, tau), __fmul_rn(c2, r)), tau);
        float nlr = __fmaf_rn(dt, __fmaf_rn(mv, dfV_dr, __fmul_rn(mr, dfr_dr)), mr);
        nlr = __fmaf_rn(cG, coup, nlr);
        const float nlv = __fmaf_rn(dt, __fmaf_rn(mv, dfr_dr, __fmul_rn(mr, dfr_dV)), mv);
        const double c = static_cast<double>(__fdiv_rn(dt, tau));
        const double cm = __dmul_rn(c, static_cast<double>(mv));
        deta = __dadd_rn(deta, cm);
        dG = __fma_rn(cm, static_cast<double>(S), dG);
        lr = __fadd_rn(nlr, drt);
        lv = nlv;
    }
};

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
    const AdjMpr m{a.consts[0], a.consts[1], a.consts[2], a.dt};
    const float cG = a.dt * a.G / a.consts[2];
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
            mr = m.mu_r(r, V, lr);
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
            m.update(r, V, S, mr, mv, coup, cG, a.dr[static_cast<long long>(k) * N + j], lr, lv, deta,
                     dG);
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

// ---------------------------------------------------------------------------
// Lane-interleaved groups, time-blocked
// ---------------------------------------------------------------------------

// Out-edge sums of node slot (lanes l = 0..7) for the K reverse steps of a
// block: lane l loads ring positions tm + d + (l % K) of NI instances
// (32 contiguous bytes for K = 8) and accumulates pairs of instances with
// the packed FMA (each half rounded as fmaf), edges in out-edge order.  The
// sum of step ks, instance m lands at cs[ks * stride + m] (cs: the slot's
// first thread).  U edges per iteration: 8 loads of 16 bytes in flight.
template <int K>
__device__ __forceinline__ void adj_gather(const float* __restrict__ ring_g,
                                           const uint2* __restrict__ edges, int lo, int hi,
                                           uint32_t tm, uint32_t mask, uint32_t R, int l, float* cs,
                                           int stride) {
    static_assert(K == 4 || K == 8, "adjoint group gather: K = 4 or 8");
    constexpr int NI = K == 8 ? 8 : 4;  // instances per lane
    constexpr int NV = NI / 4;          // 16-byte loads per edge
    constexpr int U = 8 / NV;
    const int ks = l % K;
    const int m0 = (l / K) * NI;
    const float* __restrict__ ring = ring_g + m0;
    float2 acc[NI / 2];
#pragma unroll
    for (int i = 0; i < NI / 2; ++i) acc[i] = make_float2(0.0f, 0.0f);
    for (int e = lo; e < hi; e += U) {
        float4 v[U][NV];
        float w[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (e + u < hi) {
                const uint2 ed = __ldg(edges + e + u);
                const float4* p = reinterpret_cast<const float4*>(
                    ring + (static_cast<size_t>(ed.x >> 16) * R + (((tm + (ed.x & 0xffffu)) & mask) + ks)) * kLanes);
                w[u] = __uint_as_float(ed.y);
#pragma unroll
                for (int j = 0; j < NV; ++j) v[u][j] = __ldcg(p + j);
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (e + u < hi) {
                const float2 ww = make_float2(w[u], w[u]);
#pragma unroll
                for (int j = 0; j < NV; ++j) {
                    acc[2 * j] = __ffma2_rn(ww, make_float2(v[u][j].x, v[u][j].y), acc[2 * j]);
                    acc[2 * j + 1] = __ffma2_rn(ww, make_float2(v[u][j].z, v[u][j].w), acc[2 * j + 1]);
                }
            }
        }
    }
#pragma unroll
    for (int i = 0; i < NI / 2; ++i) {
        cs[ks * stride + m0 + 2 * i] = acc[i].x;
        cs[ks * stride + m0 + 2 * i + 1] = acc[i].y;
    }
}

// One group per CTA (or cluster of C CTAs): thread t of CTA r is lane
// l = t % 8 of node slot q = (t / 8) C + r.  Per block of K reverse steps
// (tb, tb - 1, ..., tb - K + 1): the gather of all K steps (reads slots
// t + 1 + d >= tb + 2, written by earlier blocks since d >= K), then the K
// updates from registers, each writing mu_V(t + 1) to slot t + 1, then one
// barrier.  A slot written in a block aliases slot + nh, which no read of
// the block reaches (nh >= d_max + K).
//
// PIPE: two thread teams of blockDim / 2 on the same (node slot, lane)
// pairs; the update team runs block b from one coupling-sum buffer while
// the gather team sums block b + 1 into the other, and the cluster meets at
// one barrier per block.  Block b + 1 reads slots >= tb - 2K + 2 + d_min,
// all written before block b started when d_min >= 2K; the slots block b
// writes ([tb - K + 2, tb + 1]) alias none of them (nh > d_max - 1).  Each
// team runs its own loop; both meet at the same number of barriers.  Same
// per-step code and gather order: the same results.
template <int K, bool PIPE>
__global__ void __launch_bounds__(512, 1)
    adjoint_group_kernel(const tvbg_adjoint_group* __restrict__ adj, int32_t n_groups,
                         int32_t* __restrict__ status) {
    __shared__ __align__(16) tvbg_adjoint_group s;
    extern __shared__ float csum[];  // [(PIPE ? 2 : 1)][K][team threads]: out-edge sums
    const int cid = static_cast<int>(cluster_id_x());
    if (cid >= n_groups) return;  // uniform over the cluster
    {
        static_assert(sizeof(tvbg_adjoint_group) % 4 == 0, "record size");
        const uint32_t* src = reinterpret_cast<const uint32_t*>(adj + cid);
        uint32_t* dst = reinterpret_cast<uint32_t*>(&s);
        for (int i = threadIdx.x; i < static_cast<int>(sizeof(tvbg_adjoint_group) / 4); i += blockDim.x)
            dst[i] = __ldg(src + i);
        __syncthreads();
    }
    const uint32_t C = cluster_nranks();
    const uint32_t rank = cluster_rank();
    const bool cluster = C > 1;
    const int N = s.N;
    const int H = PIPE ? static_cast<int>(blockDim.x) / 2 : static_cast<int>(blockDim.x);
    const int P = H / kLanes;
    if (N < 1 || N > 65535 || static_cast<int>(C) * P < N || s.lognh < 1 || s.lognh > 16 ||
        (1 << s.lognh) < K || s.dmin < (PIPE ? 2 * K : K) || (H & 31) || s.len < 0 || s.lanes < 1 ||
        s.lanes > kLanes || !s.ring || !s.seg || !s.edges_t || !s.row_t ||
        (reinterpret_cast<uintptr_t>(s.ring) & 15u) != 0) {
        if (threadIdx.x == 0) report(status, TVBG_EINVAL);
        return;  // uniform over the cluster: same record, same launch shape
    }
    const bool gather_team = PIPE && static_cast<int>(threadIdx.x) >= H;
    const int tid = static_cast<int>(threadIdx.x) - (gather_team ? H : 0);
    const int l = tid % kLanes;
    const int q = (tid / kLanes) * static_cast<int>(C) + static_cast<int>(rank);
    const bool valid = q < N;
    const int n = valid ? (s.nodes ? __ldg(s.nodes + q) : q) : 0;
    const bool live = valid && l < s.lanes;
    const uint32_t nh = 1u << s.lognh;
    const uint32_t mask = nh - 1u;
    const uint32_t R = nh + K;
    float* cs = csum + (tid - l);
    const int bufsz = K * H;
    const uint2* __restrict__ edges = reinterpret_cast<const uint2*>(s.edges_t);
    const long long t0 = s.t0;
    const long long top = t0 + s.len - 1;
    int lo = 0, hi = 0;
    if (!PIPE || gather_team) {
        lo = valid ? __ldg(s.row_t + n) : 0;
        hi = valid ? __ldg(s.row_t + n + 1) : 0;
    }
    if (gather_team) {
        if (s.len > 0)
            adj_gather<K>(s.ring, edges, lo, hi, static_cast<uint32_t>(top - K + 2) & mask, mask, R, l, cs,
                          H);
        group_barrier(cluster);
        int buf = 1;
        for (long long tb = top; tb >= t0; tb -= K) {
            if (tb - K >= t0)
                adj_gather<K>(s.ring, edges, lo, hi, static_cast<uint32_t>(tb - 2 * K + 2) & mask, mask, R,
                              l, cs + buf * bufsz, H);
            buf ^= 1;
            group_barrier(cluster);
        }
        return;
    }
    const AdjMpr m{s.consts[0], s.consts[1], s.consts[2], s.dt};
    const float cG = s.dt * s.G[l] / s.consts[2];
    float lr = 0.0f, lv = 0.0f;
    if (live) {
        lr = s.lam[2LL * N * l + 2 * n];
        lv = s.lam[2LL * N * l + 2 * n + 1];
    }
    double deta = 0.0, dG = 0.0;
    float* __restrict__ ring_n = s.ring + static_cast<size_t>(n) * R * kLanes + l;
    const float* __restrict__ seg_n = s.seg + static_cast<size_t>(n) * 3 * kLanes + l;
    const float* __restrict__ dr_n = s.dr + s.dr_stride * l + n;
    if (PIPE) group_barrier(cluster);  // block 0's sums
    // partial sums of deta and dG go to memory after each step t with
    // t % flush_every == 0 (the grouping of one launch per segment)
    const long long fe = s.flush_every > 0 ? s.flush_every : 0;
    long long next_flush = fe ? top - (top % fe) : t0 - 1;
    bool pending = false;
    int buf = 0;
    for (long long tb = top; tb >= t0; tb -= K) {
        const int cnt = (tb - t0 + 1) < K ? static_cast<int>(tb - t0 + 1) : K;
        if (!PIPE) {
            adj_gather<K>(s.ring, edges, lo, hi, static_cast<uint32_t>(tb - K + 2) & mask, mask, R, l, cs,
                          H);
            __syncwarp();
        }
        const float* csb = cs + buf * bufsz;
#pragma unroll
        for (int i = 0; i < K; ++i) {
            if (i < cnt) {
                const long long k = tb - i - t0;
                const float* x = seg_n + static_cast<size_t>(k) * N * 3 * kLanes;
                const float r = x[0], V = x[kLanes], S = x[2 * kLanes];
                const float drt = live ? dr_n[k * N] : 0.0f;
                const float mr = m.mu_r(r, V, lr);
                const float mv = lv;
                if (valid) {
                    const uint32_t pos = static_cast<uint32_t>(tb - i + 1) & mask;
                    ring_n[pos * kLanes] = mv;
                    if (pos < static_cast<uint32_t>(K)) ring_n[(pos + nh) * kLanes] = mv;
                }
                m.update(r, V, S, mr, mv, csb[(K - 1 - i) * H + l], cG, drt, lr, lv, deta, dG);
                pending = true;
                if (tb - i == next_flush) {
                    if (live) {
                        s.deta[static_cast<long long>(N) * l + n] += deta;
                        s.dG[static_cast<long long>(N) * l + n] += dG;
                    }
                    deta = dG = 0.0;
                    pending = false;
                    next_flush -= fe;
                }
            }
        }
        if (PIPE) buf ^= 1;
        group_barrier(cluster);
    }
    if (live) {
        s.lam[2LL * N * l + 2 * n] = lr;
        s.lam[2LL * N * l + 2 * n + 1] = lv;
        if (pending) {
            s.deta[static_cast<long long>(N) * l + n] += deta;
            s.dG[static_cast<long long>(N) * l + n] += dG;
        }
    }
}

}  // namespace tvbg

using namespace tvbg;

extern "C" size_t tvbg_adjoint_group_size(void) { return sizeof(tvbg_adjoint_group); }

extern "C" int tvbg_adjoint_mpr_groups(const tvbg_adjoint_group* d_adj, int32_t n_groups,
                                       int32_t threads, int32_t cluster, int32_t block_k,
                                       int32_t pipelined, int32_t* d_status, void* stream) {
    if (n_groups < 0 || (n_groups > 0 && !d_adj) || threads < 32 || threads > 512 || (threads & 31) ||
        cluster < 1 || cluster > 16 || (block_k != 4 && block_k != 8) || pipelined < 0 ||
        pipelined > 1 || (pipelined && (threads & 63)))
        return set_error(TVBG_EINVAL, "tvbg_adjoint_mpr_groups: bad arguments");
    if (n_groups == 0) return TVBG_OK;
    using Fn = void (*)(const tvbg_adjoint_group*, int32_t, int32_t*);
    const Fn kfn = pipelined ? (block_k == 8 ? adjoint_group_kernel<8, true> : adjoint_group_kernel<4, true>)
                             : (block_k == 8 ? adjoint_group_kernel<8, false> : adjoint_group_kernel<4, false>);
    const size_t smem = 4u * static_cast<size_t>(block_k) * static_cast<size_t>(threads);
    cudaError_t e = cudaSuccess;
    if (cluster > 8) {
        e = cudaFuncSetAttribute(reinterpret_cast<const void*>(kfn),
                                 cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        if (e != cudaSuccess) return set_cuda_error(e, "tvbg_adjoint_mpr_groups: cluster attribute");
    }
    cudaLaunchConfig_t lc;
    std::memset(&lc, 0, sizeof(lc));
    lc.gridDim = dim3(static_cast<unsigned>(n_groups) * static_cast<unsigned>(cluster), 1, 1);
    lc.blockDim = dim3(static_cast<unsigned>(threads), 1, 1);
    lc.dynamicSmemBytes = smem;
    lc.stream = static_cast<cudaStream_t>(stream);
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = static_cast<unsigned>(cluster);
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    lc.attrs = attr;
    lc.numAttrs = cluster > 1 ? 1 : 0;
    e = cudaLaunchKernelEx(&lc, kfn, d_adj, n_groups, d_status);
    if (e != cudaSuccess) return set_cuda_error(e, "tvbg_adjoint_mpr_groups launch");
    return TVBG_OK;
}

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
