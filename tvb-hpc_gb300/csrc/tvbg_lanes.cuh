// Lane-interleaved group kernel: TVBG_GROUP_LANES (8) instances that share a
// connectome, a delay table, the model constants and t0 run together, one
// instance per lane of an 8-lane slice of a warp.
//
// Canonical step (CUDA order, the same as tvbg_step.cuh and
// tvbg_step_blocked.cuh; tvb_hpc/network.py:115-143, coupling.py:103-116,
// model.py:131-155, scheme.py:88-107, ring addressing of
// dsl/dsl_cuda/CUDAmodels/kuramoto.c:92,108,128):
//   S     = sum_e w_e pre(ring[t - d_e][col_e])          (CSR order)
//   c     = post(S, obs0(x_i), sum_e w_e)
//   x'    = limit(x + dt f(x, c, p) + sqrt(dt) sigma z)   z: Philox(seed_lo, inst; node, t/SPC, seed_hi)
//           (Box-Muller with CUDA's fast intrinsics, box_muller_fast)
//   ring[t+1][i] = obs0(x')
//
// Layout.  Every per-node quantity is interleaved over the 8 instances of
// the group, so a lane slice reading "node j, slot s" reads 32 contiguous
// bytes -- one DRAM/L2 sector -- and the edge record (column, delay,
// weight) is the same for the 8 lanes:
//   ring   [N][R][8], R = nh + 8: slot s of node j at (j R + (s & (nh-1))) 8 + l,
//          positions < 8 mirrored at +nh so a run of K <= 8 slots never wraps;
//          with the Kuramoto coupling [N][R][2][8]: sin and cos of the observable
//   state  [N][NS][8], nparam [N][NP][8], bold [4][N][8],
//   bold_out [bold_len][N][8], trace [trace_len][N][trace_nobs][8].
//
// Thread mapping.  Thread t of CTA r (cluster of C CTAs) is lane l = t % 8
// of node slot q = t / 8; node slot q of CTA r serves the node positions
// q C + r, q C + r + C P, ... (P = blockDim / 8) of the group's node order
// (the host sorts nodes by in-degree, so the slots of a warp see similar
// edge counts and the C CTAs of a cluster the same work).
//
// Time blocking.  A value written at step t is first read at t + 1 + d_min,
// so the K <= d_min + 1 steps of a block read only slots that exist when the
// block starts; with nh >= d_max + 1 + K no slot written in a block aliases
// one read in it.  The cluster meets at one barrier per block.
//
// Gather.  Each thread sums its node's in-edges for the K steps of the
// block: one edge record and one address per K steps, K sector loads per
// edge (cache-global, __ldcg: with C > 1 the values come from other SMs,
// ordered by the cluster barrier's release/acquire), 16 independent loads
// in flight per thread.  The sums are parked in shared memory and the
// node's K updates run from registers.  (Staging the edges' K-slot runs in
// shared memory with cp.async.bulk instead was measured slower on the
// benchmark workloads: the kernel is bound by instruction issue and latency,
// not by bytes in flight.)
#pragma once

#include "tvbg_step_blocked.cuh"

namespace tvbg {

constexpr int kLanes = TVBG_GROUP_LANES;

// steps of the pipelined kernel's update loop unrolled (update_node)
#ifndef TVBG_UPDATE_UNROLL
#define TVBG_UPDATE_UNROLL 1
#endif
constexpr int kUpdateUnroll = TVBG_UPDATE_UNROLL;

// 16-byte loads in flight per thread in the transposed gather (lane_gather_t)
#ifndef TVBG_GATHER_LOADS
#define TVBG_GATHER_LOADS 8
#endif

__device__ __forceinline__ uint32_t cluster_nranks() {
    uint32_t n;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(n));
    return n;
}
__device__ __forceinline__ uint32_t cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ uint32_t cluster_id_x() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
    return r;
}

// Block barrier of the group: the CTA, or every CTA of the cluster.
__device__ __forceinline__ void group_barrier(bool cluster) {
    if (cluster) {
        asm volatile("barrier.cluster.arrive.release.aligned;\n\t"
                     "barrier.cluster.wait.acquire.aligned;" ::: "memory");
    } else {
        __syncthreads();
    }
}

// Copy a group descriptor into shared memory (word-parallel).
__device__ __forceinline__ void stage_group(const tvbg_group* src, tvbg_group* dst) {
    static_assert(sizeof(tvbg_group) % 4 == 0, "descriptor size");
    const uint32_t* s = reinterpret_cast<const uint32_t*>(src);
    uint32_t* d = reinterpret_cast<uint32_t*>(dst);
    for (int i = threadIdx.x; i < static_cast<int>(sizeof(tvbg_group) / 4); i += blockDim.x)
        d[i] = __ldg(s + i);
    __syncthreads();
}

// Normal number r (0..3) of one Philox call, without dynamic indexing.
__device__ __forceinline__ float pick4(const float z[4], int r) {
    const float a = (r & 1) ? z[1] : z[0];
    const float b = (r & 1) ? z[3] : z[2];
    return (r & 2) ? b : a;
}

template <int CF>
__device__ __forceinline__ float lane_pre(float xj, const float* cf_p) {
    if constexpr (CF == TVBG_CFUN_SIGMOIDAL) {
        return cf_p[0] / (1.0f + expf(cf_p[2] * (cf_p[1] - xj)));
    } else {
        return xj;
    }
}

template <int CF>
__device__ __forceinline__ float lane_post(float S, float xi, float wsum, float a, float b) {
    if constexpr (CF == TVBG_CFUN_DIFF) {
        return a * (S - xi * wsum) + b;
    } else if constexpr (CF == TVBG_CFUN_SIGMOIDAL) {
        return a * S;
    } else {
        return a * S + b;
    }
}

// Coupling sums of node n (in-edges [lo, hi)) for the K steps of the block
// starting at ring position tm, accumulated in CSR order.  U = 16 / K edges
// per iteration: 16 independent sector loads in flight per thread.
template <int CF, int K>
__device__ __forceinline__ void lane_gather(const tvbg_group& g, int lo, int hi, uint32_t tm,
                                            uint32_t mask, uint32_t R, int l, float acc[K]) {
    constexpr int U = 16 / K;
    const float* __restrict__ ring = g.ring + l;
    const uint2* __restrict__ edges = reinterpret_cast<const uint2*>(g.edges);
#pragma unroll
    for (int k = 0; k < K; ++k) acc[k] = 0.0f;
    auto addr = [&](uint32_t pk) {
        return ring + (static_cast<size_t>(pk >> 16) * R + ((tm + (pk & 0xffffu)) & mask)) * kLanes;
    };
    int e = lo;
    for (; e + U <= hi; e += U) {
        float v[U][K];
        float w[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint2 ed = __ldg(edges + e + u);
            const float* p = addr(ed.x);
            w[u] = __uint_as_float(ed.y);
#pragma unroll
            for (int k = 0; k < K; ++k) v[u][k] = __ldcg(p + k * kLanes);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
#pragma unroll
            for (int k = 0; k < K; ++k) acc[k] = fmaf(w[u], lane_pre<CF>(v[u][k], g.cf_p), acc[k]);
        }
    }
    if (e < hi) {  // fewer than U edges left, loads still issued together
        float v[U][K];
        float w[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (e + u < hi) {
                const uint2 ed = __ldg(edges + e + u);
                const float* p = addr(ed.x);
                w[u] = __uint_as_float(ed.y);
#pragma unroll
                for (int k = 0; k < K; ++k) v[u][k] = __ldcg(p + k * kLanes);
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (e + u < hi) {
#pragma unroll
                for (int k = 0; k < K; ++k) acc[k] = fmaf(w[u], lane_pre<CF>(v[u][k], g.cf_p), acc[k]);
            }
        }
    }
}

// Kuramoto coupling, sum_e w_e sin(x_j - x_i) = cos x_i sum_e w_e sin x_j
// - sin x_i sum_e w_e cos x_j: the ring carries two channels, sin and cos
// of the observable ([N][R][2][8]), and the gather sums both for the K steps
// (16 independent loads in flight per thread, CSR order).
template <int K>
__device__ __forceinline__ void lane_gather_sc(const tvbg_group& g, int lo, int hi, uint32_t tm,
                                               uint32_t mask, uint32_t R, int l, float accs[K],
                                               float accc[K]) {
    constexpr int RL = 2 * kLanes;
    constexpr int U = 8 / K;
    const float* __restrict__ ring = g.ring + l;
    const uint2* __restrict__ edges = reinterpret_cast<const uint2*>(g.edges);
#pragma unroll
    for (int k = 0; k < K; ++k) accs[k] = accc[k] = 0.0f;
    auto addr = [&](uint32_t pk) {
        return ring + (static_cast<size_t>(pk >> 16) * R + ((tm + (pk & 0xffffu)) & mask)) * RL;
    };
    int e = lo;
    for (; e < hi; e += U) {
        float vs[U][K], vc[U][K];
        float w[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (e + u < hi) {
                const uint2 ed = __ldg(edges + e + u);
                const float* p = addr(ed.x);
                w[u] = __uint_as_float(ed.y);
#pragma unroll
                for (int k = 0; k < K; ++k) {
                    vs[u][k] = __ldcg(p + k * RL);
                    vc[u][k] = __ldcg(p + k * RL + kLanes);
                }
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (e + u < hi) {
#pragma unroll
                for (int k = 0; k < K; ++k) {
                    accs[k] = fmaf(w[u], vs[u][k], accs[k]);
                    accc[k] = fmaf(w[u], vc[u][k], accc[k]);
                }
            }
        }
    }
}

// Ring channels per (node, slot): 2 (sin, cos) for the Kuramoto coupling and
// the LEMS sine coupling, 2 for a LEMS model's two couplings, else 1.
template <int CF>
__host__ __device__ constexpr int ring_channels() {
    return (CF == TVBG_CFUN_KURAMOTO || CF == TVBG_CFUN_LEMS_SC || CF == TVBG_CFUN_LEMS_2) ? 2 : 1;
}

// Value a one-channel ring slot holds for observable o: o itself, or for a
// LEMS model its separable pre-synaptic term pre(o), so the gather sums
// w_e * pre(x_j) without evaluating pre per edge.
template <class M, int CF>
__device__ __forceinline__ float ring_val(float o, const float* p) {
    if constexpr (CF == TVBG_CFUN_LEMS) {
        return M::ring_value(o, p);
    } else {
        return o;
    }
}

// Dynamic shared memory of a group CTA: the K coupling sums (per ring
// channel) of every thread.
__host__ __device__ constexpr uint32_t group_smem_bytes(int K, int threads, int nc) {
    return static_cast<uint32_t>(4 * K * threads * nc);
}

template <class M, int CF, int K>
__device__ __forceinline__ void run_group(const tvbg_group& g, float* csum, int32_t* status) {
    constexpr int NS = M::NS;
    constexpr int NP = M::NP;
    constexpr int SPC = Noise<M>::SPC;
    constexpr int NC = ring_channels<CF>();
    constexpr int RL = kLanes * NC;  // floats per (node, slot)
    const int N = g.N;
    const uint32_t C = cluster_nranks();
    const uint32_t rank = cluster_rank();
    const bool cluster = C > 1;
    if (N <= 0 || N > 65535 || g.lognh < 3 || g.lognh > 16 || g.model != M::ID || g.cfun != CF ||
        g.nsteps < 0 || (g.flags & (TVBG_F_TRACKA | TVBG_F_MIDSYNC | TVBG_F_TRACE_CSUM)) ||
        (!Noise<M>::kOK && !WideNoise<M>::value && (g.flags & TVBG_F_NOISE))) {
        if (threadIdx.x == 0) report(status, TVBG_EINVAL);
        return;  // every CTA of the cluster reads the same descriptor and leaves here
    }
    const int l = threadIdx.x % kLanes;
    const int slot = threadIdx.x / kLanes;
    const int P = blockDim.x / kLanes;
    const int stride = static_cast<int>(C) * P;
    const int rounds = (N + stride - 1) / stride;       // warp-uniform node loop
    const uint32_t nh = 1u << g.lognh;
    const uint32_t mask = nh - 1u;
    const uint32_t R = nh + kGhost;
    const uint32_t flags = g.flags;
    const bool noise = (flags & TVBG_F_NOISE) != 0;
    const bool bold = (flags & TVBG_F_BOLD) != 0 && g.bold != nullptr && g.bold_out != nullptr;
    const bool trace = (flags & TVBG_F_TRACE) != 0 && g.trace != nullptr;
    const float dt = g.dt, sqrt_dt = g.sqrt_dt;
    const float cf_a = g.lanes[l].cf_a;
    const int my_steps = g.lanes[l].nsteps < g.nsteps ? g.lanes[l].nsteps : g.nsteps;
    const uint32_t inst_id = g.lanes[l].inst_id;
    const long long t0 = g.t0;
    const long long t_end = t0 + my_steps;  // this lane updates while t < t_end
    float* __restrict__ ring = g.ring;
    float* __restrict__ state = g.state;
    const int q0 = slot * static_cast<int>(C) + static_cast<int>(rank);

    // seed: slot t0 holds obs0 of the state at t0
    {
        const uint32_t pos = static_cast<uint32_t>(t0) & mask;
        for (int q = q0; q < N; q += stride) {
            const int n = g.nodes ? __ldg(g.nodes + q) : q;
            float x[NS];
#pragma unroll
            for (int v = 0; v < NS; ++v) x[v] = state[(n * NS + v) * kLanes + l];
            const size_t idx = (static_cast<size_t>(n) * R + pos) * RL + l;
            const float o = M::obs(x, 0);
            float p[NP];
#pragma unroll
            for (int v = 0; v < NP; ++v) p[v] = __ldg(g.nparam + (n * NP + v) * kLanes + l);
            if constexpr (NC == 2) {
                float sn, cs;
                if constexpr (CF == TVBG_CFUN_LEMS_2) {
                    sn = M::ring_value(o, p);
                    cs = M::ring_value2(x[M::CVAR2], p);
                } else {
                    sincosf(o, &sn, &cs);
                }
                ring[idx] = sn;
                ring[idx + kLanes] = cs;
                if (pos < kGhost) {
                    ring[idx + static_cast<size_t>(nh) * RL] = sn;
                    ring[idx + static_cast<size_t>(nh) * RL + kLanes] = cs;
                }
            } else {
                const float rv = ring_val<M, CF>(o, p);
                ring[idx] = rv;
                if (pos < kGhost) ring[idx + static_cast<size_t>(nh) * kLanes] = rv;
            }
        }
    }
    group_barrier(cluster);

    // monitor schedule as 32-bit counters carried across blocks (the 64-bit
    // divisions run once per kernel): BOLD sample after step t when
    // (t + 1) % bold_period == 0, trace row before step t when
    // t % trace_every == 0
    const int bper = g.bold_period > 0 ? g.bold_period : 1;
    const int tev = g.trace_every > 0 ? g.trace_every : 1;
    int b_until = bold ? static_cast<int>((bper - 1) - t0 % bper) : 0;  // steps to the next sample
    int b_row = bold ? static_cast<int>((t0 + b_until + 1) / bper - 1) : 0;
    int tr_until = trace ? static_cast<int>((tev - t0 % tev) % tev) : 0;
    int tr_row = trace ? static_cast<int>(((t0 + tr_until) / tev) % g.trace_len) : 0;
    for (long long tb = t0; tb < t0 + g.nsteps; tb += K) {
        const int cnt = (t0 + g.nsteps - tb) < K ? static_cast<int>(t0 + g.nsteps - tb) : K;
        const uint32_t tm = static_cast<uint32_t>(tb) & mask;
        for (int r = 0; r < rounds; ++r) {
            const int q = q0 + r * stride;
            const bool valid = q < N;
            const int n = valid ? (g.nodes ? __ldg(g.nodes + q) : q) : 0;
            {
                const int lo = valid ? __ldg(g.row + n) : 0;
                const int hi = valid ? __ldg(g.row + n + 1) : 0;
                if constexpr (NC == 2) {
                    float accs[K], accc[K];
                    lane_gather_sc<K>(g, lo, hi, tm, mask, R, l, accs, accc);
#pragma unroll
                    for (int k = 0; k < K; ++k) {
                        csum[k * blockDim.x + threadIdx.x] = accs[k];
                        csum[(K + k) * blockDim.x + threadIdx.x] = accc[k];
                    }
                } else {
                    float acc[K];
                    lane_gather<CF, K>(g, lo, hi, tm, mask, R, l, acc);
#pragma unroll
                    for (int k = 0; k < K; ++k) csum[k * blockDim.x + threadIdx.x] = acc[k];
                }
            }
            if (!valid) continue;
            float x[NS], p[NP];
#pragma unroll
            for (int v = 0; v < NS; ++v) x[v] = state[(n * NS + v) * kLanes + l];
#pragma unroll
            for (int v = 0; v < NP; ++v) p[v] = __ldg(g.nparam + (n * NP + v) * kLanes + l);
            const float wsum = (CF == TVBG_CFUN_DIFF && g.wsum) ? __ldg(g.wsum + n) : 0.0f;
            float bs = 0.0f, bF = 0.0f, bV = 0.0f, bQ = 0.0f;
            if (bold) {
                bs = g.bold[(0 * N + n) * kLanes + l];
                bF = g.bold[(1 * N + n) * kLanes + l];
                bV = g.bold[(2 * N + n) * kLanes + l];
                bQ = g.bold[(3 * N + n) * kLanes + l];
            }
            float obs0 = M::obs(x, 0);
            float sn0 = 0.0f, cs0 = 0.0f;  // sin, cos of obs0 (Kuramoto coupling)
            if constexpr (NC == 2 && CF != TVBG_CFUN_LEMS_2) sincosf(obs0, &sn0, &cs0);
            float zz[4] = {0.0f, 0.0f, 0.0f, 0.0f};
            int b_next = b_until, tr_next = tr_until;
            int brow = b_row, trow = tr_row;
#pragma unroll 1
            for (int k = 0; k < cnt; ++k) {
                const long long t = tb + k;
                if (t >= t_end) break;
                if (trace && k == tr_next) {
                    float* dst = g.trace + ((static_cast<size_t>(trow) * N + n) * g.trace_nobs) * kLanes + l;
                    for (int o = 0; o < g.trace_nobs; ++o) dst[o * kLanes] = M::obs(x, o);
                    tr_next += tev;
                    trow = trow + 1 == g.trace_len ? 0 : trow + 1;
                }
                const float xbold = bold ? M::obs(x, g.bold_obs) : 0.0f;
                float c, c2 = 0.0f;
                if constexpr (CF == TVBG_CFUN_LEMS_2) {
                    c = M::coupling(csum[k * blockDim.x + threadIdx.x], x, p);
                    c2 = M::coupling2(csum[(K + k) * blockDim.x + threadIdx.x], x, p);
                } else if constexpr (NC == 2) {
                    // sum_e w sin(x_j - x_i); Kuramoto: post = a * mean (coupling.py:119-121)
                    const float S = cs0 * csum[k * blockDim.x + threadIdx.x] -
                                    sn0 * csum[(K + k) * blockDim.x + threadIdx.x];
                    if constexpr (CF == TVBG_CFUN_LEMS_SC) {
                        c = M::coupling(S, x, p);
                    } else {
                        c = cf_a * (S / static_cast<float>(N));
                    }
                } else if constexpr (CF == TVBG_CFUN_LEMS) {
                    c = M::coupling(csum[k * blockDim.x + threadIdx.x], x, p);
                } else {
                    c = lane_post<CF>(csum[k * blockDim.x + threadIdx.x], obs0, wsum, cf_a, g.cf_b);
                }
                float f[NS];
                if constexpr (CF == TVBG_CFUN_LEMS_2) {
                    M::drift2(x, c, c2, p, g.consts, f);
                } else {
                    M::drift(x, c, p, g.consts, f);
                }
#pragma unroll
                for (int v = 0; v < NS; ++v) x[v] = fmaf(dt, f[v], x[v]);
                if constexpr (Noise<M>::kOK) {
                    if (noise) {
                        const int r0 = static_cast<int>(t & (SPC - 1));
                        if (k == 0 || r0 == 0) {
                            const u32x4 w = philox4x32_10(static_cast<uint32_t>(n),
                                                          static_cast<uint32_t>(t / SPC), g.seed_hi, 0u,
                                                          g.seed_lo, inst_id);
                            box_muller_fast(w.v[0], w.v[1], zz[0], zz[1]);
                            box_muller_fast(w.v[2], w.v[3], zz[2], zz[3]);
                        }
#pragma unroll
                        for (int v = 0; v < NS; ++v)
                            x[v] = fmaf(sqrt_dt * pick4(zz, r0 * NS + v), g.sigma[v], x[v]);
                    }
                } else if constexpr (WideNoise<M>::value) {
                    if (noise) {
                        float z8[8];
#pragma unroll
                        for (int b = 0; b < 2; ++b) {
                            const u32x4 w = philox4x32_10(static_cast<uint32_t>(n),
                                                          static_cast<uint32_t>(t), g.seed_hi,
                                                          static_cast<uint32_t>(b), g.seed_lo, inst_id);
                            box_muller_fast(w.v[0], w.v[1], z8[4 * b], z8[4 * b + 1]);
                            box_muller_fast(w.v[2], w.v[3], z8[4 * b + 2], z8[4 * b + 3]);
                        }
#pragma unroll
                        for (int v = 0; v < NS; ++v)
                            x[v] = fmaf(sqrt_dt * z8[v], g.sigma[0] * NoiseScale<M>::at(v), x[v]);
                    }
                }
                M::limit(x, flags);
                obs0 = M::obs(x, 0);
                const uint32_t pos = (static_cast<uint32_t>(t) + 1u) & mask;
                const size_t idx = (static_cast<size_t>(n) * R + pos) * RL + l;
                if constexpr (NC == 2) {
                    if constexpr (CF == TVBG_CFUN_LEMS_2) {
                        sn0 = M::ring_value(obs0, p);
                        cs0 = M::ring_value2(x[M::CVAR2], p);
                    } else {
                        sincosf(obs0, &sn0, &cs0);
                    }
                    ring[idx] = sn0;
                    ring[idx + kLanes] = cs0;
                    if (pos < kGhost) {
                        ring[idx + static_cast<size_t>(nh) * RL] = sn0;
                        ring[idx + static_cast<size_t>(nh) * RL + kLanes] = cs0;
                    }
                } else {
                    const float rv = ring_val<M, CF>(obs0, p);
                    ring[idx] = rv;
                    if (pos < kGhost) ring[idx + static_cast<size_t>(nh) * kLanes] = rv;
                }
                if (bold) {
                    Balloon::step(bs, bF, bV, bQ, xbold, g.dt_bold);
                    if (k == b_next) {
                        if (brow >= 0 && brow < g.bold_len)
                            g.bold_out[(static_cast<size_t>(brow) * N + n) * kLanes + l] =
                                Balloon::signal(bV, bQ);
                        b_next += bper;
                        brow += 1;
                    }
                }
            }
#pragma unroll
            for (int v = 0; v < NS; ++v) state[(n * NS + v) * kLanes + l] = x[v];
            if (bold) {
                g.bold[(0 * N + n) * kLanes + l] = bs;
                g.bold[(1 * N + n) * kLanes + l] = bF;
                g.bold[(2 * N + n) * kLanes + l] = bV;
                g.bold[(3 * N + n) * kLanes + l] = bQ;
            }
        }
        // advance the monitor counters past this block
        if (bold) {
            while (b_until < cnt) {
                b_until += bper;
                b_row += 1;
            }
            b_until -= cnt;
        }
        if (trace) {
            while (tr_until < cnt) {
                tr_until += tev;
                tr_row = tr_row + 1 == g.trace_len ? 0 : tr_row + 1;
            }
            tr_until -= cnt;
        }
        group_barrier(cluster);
    }
}

// ---------------------------------------------------------------------------
// Pipelined group kernel (group_kernel_pipelined).  The per-node pieces of
// run_group as functions; run_group itself keeps its own inline body (its
// register allocation and instruction schedule were tuned as written).
// ---------------------------------------------------------------------------

// Transposed gather of one node for the K steps of the block at ring
// position tm.  The 8 lanes of a node slot share the edge records; lane l
// reads, per edge, ring position t + (l mod K) for NI = 64 / K consecutive
// instances m0 = (l / K) NI .. m0 + NI - 1 -- 4 NI contiguous bytes, two
// (K = 8) or one (K = 4) 16-byte loads -- and accumulates, in CSR order,
// acc[i] = sum_e w_e pre(v_e[m0 + i]), the sum of step (l mod K) of
// instance m0 + i.  Pairs of accumulators take one packed FP32 FMA
// (__ffma2_rn: each half rounded as fmaf), so every sum equals
// lane_gather's.  The sums are written transposed: cs_slot[k * stride + m]
// holds step k of instance m, where the node's lane m reads them.  Needs the
// ring 16-byte aligned and K in {4, 8}.
template <int CF, int K>
__device__ __forceinline__ void lane_gather_t(const tvbg_group& g, int lo, int hi, uint32_t tm,
                                              uint32_t mask, uint32_t R, int l, float* cs_slot,
                                              int stride) {
    static_assert(K == 4 || K == 8, "transposed gather: K = 4 or 8");
    constexpr int NI = K == 8 ? 8 : 4;   // instances per lane
    constexpr int NV = NI / 4;           // 16-byte loads per edge
    constexpr int U = TVBG_GATHER_LOADS / NV;  // edges per iteration (loads in flight / loads per edge)
    const int ks = l % K;
    const int m0 = (l / K) * NI;
    const float* __restrict__ ring = g.ring + m0;
    const uint2* __restrict__ edges = reinterpret_cast<const uint2*>(g.edges);
    float2 acc[NI / 2];
#pragma unroll
    for (int i = 0; i < NI / 2; ++i) acc[i] = make_float2(0.0f, 0.0f);
    auto addr = [&](uint32_t pk) {
        return ring + (static_cast<size_t>(pk >> 16) * R + (((tm + (pk & 0xffffu)) & mask) + ks)) * kLanes;
    };
    for (int e = lo; e < hi; e += U) {
        float4 v[U][NV];
        float w[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (e + u < hi) {
                const uint2 ed = __ldg(edges + e + u);
                const float4* p = reinterpret_cast<const float4*>(addr(ed.x));
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
                    const float2 a = make_float2(lane_pre<CF>(v[u][j].x, g.cf_p), lane_pre<CF>(v[u][j].y, g.cf_p));
                    const float2 b = make_float2(lane_pre<CF>(v[u][j].z, g.cf_p), lane_pre<CF>(v[u][j].w, g.cf_p));
                    acc[2 * j] = __ffma2_rn(ww, a, acc[2 * j]);
                    acc[2 * j + 1] = __ffma2_rn(ww, b, acc[2 * j + 1]);
                }
            }
        }
    }
#pragma unroll
    for (int i = 0; i < NI / 2; ++i) {
        cs_slot[ks * stride + m0 + 2 * i] = acc[i].x;
        cs_slot[ks * stride + m0 + 2 * i + 1] = acc[i].y;
    }
}

// Per-thread constants of a group run (lane l of one node slot).
struct GroupLane {
    int l;                  // lane = instance of the group
    uint32_t nh, mask, R;   // ring length, mask, row length (nh + ghost slots)
    uint32_t flags;
    bool noise, bold, trace;
    float cf_a;
    long long t0, t_end;    // this lane updates while t < t_end
    uint32_t inst_id;
};

// allow_csum: the pipelined kernel's one-channel couplings can write the
// raw coupling sum into the trace (TVBG_F_TRACE_CSUM).
template <class M, int CF>
__device__ __forceinline__ bool group_descriptor_ok(const tvbg_group& g, bool allow_csum = false) {
    const int N = g.N;
    const uint32_t bad = TVBG_F_TRACKA | TVBG_F_MIDSYNC |
                         ((allow_csum && ring_channels<CF>() == 1) ? 0u : TVBG_F_TRACE_CSUM);
    return !(N <= 0 || N > 65535 || g.lognh < 3 || g.lognh > 16 || g.model != M::ID || g.cfun != CF ||
             g.nsteps < 0 || (g.flags & bad) ||
             (!Noise<M>::kOK && !WideNoise<M>::value && (g.flags & TVBG_F_NOISE)));
}

template <class M>
__device__ __forceinline__ GroupLane make_lane(const tvbg_group& g, int l) {
    GroupLane c;
    c.l = l;
    c.nh = 1u << g.lognh;
    c.mask = c.nh - 1u;
    c.R = c.nh + kGhost;
    c.flags = g.flags;
    c.noise = (g.flags & TVBG_F_NOISE) != 0;
    c.bold = (g.flags & TVBG_F_BOLD) != 0 && g.bold != nullptr && g.bold_out != nullptr;
    c.trace = (g.flags & TVBG_F_TRACE) != 0 && g.trace != nullptr;
    c.cf_a = g.lanes[l].cf_a;
    const int my_steps = g.lanes[l].nsteps < g.nsteps ? g.lanes[l].nsteps : g.nsteps;
    c.inst_id = g.lanes[l].inst_id;
    c.t0 = g.t0;
    c.t_end = g.t0 + my_steps;
    return c;
}

// Seed: ring slot t0 of node n holds obs0 (or the ring channels) of the
// state at t0.
template <class M, int CF>
__device__ __forceinline__ void seed_node(const tvbg_group& g, const GroupLane& c, int n) {
    constexpr int NS = M::NS;
    constexpr int NP = M::NP;
    constexpr int NC = ring_channels<CF>();
    constexpr int RL = kLanes * NC;
    const int l = c.l;
    const uint32_t pos = static_cast<uint32_t>(c.t0) & c.mask;
    float x[NS];
#pragma unroll
    for (int v = 0; v < NS; ++v) x[v] = g.state[(n * NS + v) * kLanes + l];
    const size_t idx = (static_cast<size_t>(n) * c.R + pos) * RL + l;
    const float o = M::obs(x, 0);
    float p[NP];
#pragma unroll
    for (int v = 0; v < NP; ++v) p[v] = __ldg(g.nparam + (n * NP + v) * kLanes + l);
    float* __restrict__ ring = g.ring;
    if constexpr (NC == 2) {
        float sn, cs;
        if constexpr (CF == TVBG_CFUN_LEMS_2) {
            sn = M::ring_value(o, p);
            cs = M::ring_value2(x[M::CVAR2], p);
        } else {
            sincosf(o, &sn, &cs);
        }
        ring[idx] = sn;
        ring[idx + kLanes] = cs;
        if (pos < kGhost) {
            ring[idx + static_cast<size_t>(c.nh) * RL] = sn;
            ring[idx + static_cast<size_t>(c.nh) * RL + kLanes] = cs;
        }
    } else {
        const float rv = ring_val<M, CF>(o, p);
        ring[idx] = rv;
        if (pos < kGhost) ring[idx + static_cast<size_t>(c.nh) * kLanes] = rv;
    }
}

// Coupling sums of node n (an invalid slot gathers nothing) for the K steps
// of the block at ring position tm, written to cs[k * stride] (and
// cs[(K + k) * stride] for the second ring channel); cs points at this
// thread's own sums.  One-channel couplings take the transposed gather (the
// caller has checked the ring's 16-byte alignment).
template <class M, int CF, int K>
__device__ __forceinline__ void gather_node(const tvbg_group& g, const GroupLane& c, bool valid, int n,
                                            uint32_t tm, float* cs, int stride) {
    constexpr int NC = ring_channels<CF>();
    const int lo = valid ? __ldg(g.row + n) : 0;
    const int hi = valid ? __ldg(g.row + n + 1) : 0;
    if constexpr (NC == 2) {
        float accs[K], accc[K];
        lane_gather_sc<K>(g, lo, hi, tm, c.mask, c.R, c.l, accs, accc);
#pragma unroll
        for (int k = 0; k < K; ++k) {
            cs[k * stride] = accs[k];
            cs[(K + k) * stride] = accc[k];
        }
    } else {
        lane_gather_t<CF, K>(g, lo, hi, tm, c.mask, c.R, c.l, cs - c.l, stride);
    }
}

// Monitor schedule as 32-bit counters carried across blocks (the 64-bit
// divisions run once per kernel): BOLD sample after step t when
// (t + 1) % bold_period == 0, trace row before step t when
// t % trace_every == 0.
struct MonitorClock {
    int bper, tev;
    int b_until, b_row, tr_until, tr_row;

    __device__ __forceinline__ void init(const tvbg_group& g, const GroupLane& c) {
        bper = g.bold_period > 0 ? g.bold_period : 1;
        tev = g.trace_every > 0 ? g.trace_every : 1;
        const long long t0 = c.t0;
        b_until = c.bold ? static_cast<int>((bper - 1) - t0 % bper) : 0;  // steps to the next sample
        b_row = c.bold ? static_cast<int>((t0 + b_until + 1) / bper - 1) : 0;
        tr_until = c.trace ? static_cast<int>((tev - t0 % tev) % tev) : 0;
        tr_row = c.trace ? static_cast<int>(((t0 + tr_until) / tev) % g.trace_len) : 0;
    }
    // advance the counters past a block of cnt steps
    __device__ __forceinline__ void advance(const tvbg_group& g, const GroupLane& c, int cnt) {
        if (c.bold) {
            while (b_until < cnt) {
                b_until += bper;
                b_row += 1;
            }
            b_until -= cnt;
        }
        if (c.trace) {
            while (tr_until < cnt) {
                tr_until += tev;
                tr_row = tr_row + 1 == g.trace_len ? 0 : tr_row + 1;
            }
            tr_until -= cnt;
        }
    }
};

// The cnt (<= K) updates of node n for the block starting at step tb, from
// the coupling sums cs[k * stride] (second channel cs[(K + k) * stride]):
// drift, Euler-Maruyama, limit, ring write, balloon/BOLD and trace -- the
// update of run_group, in the same order.
template <class M, int CF, int K>
__device__ __forceinline__ void update_node(const tvbg_group& g, const GroupLane& c, int n, long long tb,
                                            int cnt, const float* cs, int stride, const MonitorClock& mc) {
    constexpr int NS = M::NS;
    constexpr int NP = M::NP;
    constexpr int SPC = Noise<M>::SPC;
    constexpr int NC = ring_channels<CF>();
    constexpr int RL = kLanes * NC;  // floats per (node, slot)
    const int N = g.N;
    const int l = c.l;
    const uint32_t mask = c.mask, R = c.R, nh = c.nh;
    const bool noise = c.noise, bold = c.bold, trace = c.trace;
    const float dt = g.dt, sqrt_dt = g.sqrt_dt;
    float* __restrict__ ring = g.ring;
    float* __restrict__ state = g.state;
    float x[NS], p[NP];
#pragma unroll
    for (int v = 0; v < NS; ++v) x[v] = state[(n * NS + v) * kLanes + l];
#pragma unroll
    for (int v = 0; v < NP; ++v) p[v] = __ldg(g.nparam + (n * NP + v) * kLanes + l);
    const float wsum = (CF == TVBG_CFUN_DIFF && g.wsum) ? __ldg(g.wsum + n) : 0.0f;
    float bs = 0.0f, bF = 0.0f, bV = 0.0f, bQ = 0.0f;
    if (bold) {
        bs = g.bold[(0 * N + n) * kLanes + l];
        bF = g.bold[(1 * N + n) * kLanes + l];
        bV = g.bold[(2 * N + n) * kLanes + l];
        bQ = g.bold[(3 * N + n) * kLanes + l];
    }
    float obs0 = M::obs(x, 0);
    float sn0 = 0.0f, cs0 = 0.0f;  // sin, cos of obs0 (Kuramoto coupling)
    if constexpr (NC == 2 && CF != TVBG_CFUN_LEMS_2) sincosf(obs0, &sn0, &cs0);
    float zz[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    int b_next = mc.b_until, tr_next = mc.tr_until;
    int brow = mc.b_row, trow = mc.tr_row;
#pragma unroll kUpdateUnroll
    for (int k = 0; k < cnt; ++k) {
        const long long t = tb + k;
        if (t >= c.t_end) break;
        if (trace && k == tr_next) {
            // a trace row holds the observables, then with TVBG_F_TRACE_CSUM
            // the raw coupling sum of the step (one-channel couplings)
            const bool csum = (c.flags & TVBG_F_TRACE_CSUM) != 0;
            const int tw = g.trace_nobs + (csum ? 1 : 0);
            float* dst = g.trace + ((static_cast<size_t>(trow) * N + n) * tw) * kLanes + l;
            for (int o = 0; o < g.trace_nobs; ++o) dst[o * kLanes] = M::obs(x, o);
            if constexpr (NC == 1) {
                if (csum) dst[g.trace_nobs * kLanes] = cs[k * stride];
            }
            tr_next += mc.tev;
            trow = trow + 1 == g.trace_len ? 0 : trow + 1;
        }
        const float xbold = bold ? M::obs(x, g.bold_obs) : 0.0f;
        float cc, c2 = 0.0f;
        if constexpr (CF == TVBG_CFUN_LEMS_2) {
            cc = M::coupling(cs[k * stride], x, p);
            c2 = M::coupling2(cs[(K + k) * stride], x, p);
        } else if constexpr (NC == 2) {
            // sum_e w sin(x_j - x_i); Kuramoto: post = a * mean (coupling.py:119-121)
            const float S = cs0 * cs[k * stride] - sn0 * cs[(K + k) * stride];
            if constexpr (CF == TVBG_CFUN_LEMS_SC) {
                cc = M::coupling(S, x, p);
            } else {
                cc = c.cf_a * (S / static_cast<float>(N));
            }
        } else if constexpr (CF == TVBG_CFUN_LEMS) {
            cc = M::coupling(cs[k * stride], x, p);
        } else {
            cc = lane_post<CF>(cs[k * stride], obs0, wsum, c.cf_a, g.cf_b);
        }
        float f[NS];
        if constexpr (CF == TVBG_CFUN_LEMS_2) {
            M::drift2(x, cc, c2, p, g.consts, f);
        } else {
            M::drift(x, cc, p, g.consts, f);
        }
#pragma unroll
        for (int v = 0; v < NS; ++v) x[v] = fmaf(dt, f[v], x[v]);
        if constexpr (Noise<M>::kOK) {
            if (noise) {
                const int r0 = static_cast<int>(t & (SPC - 1));
                if (k == 0 || r0 == 0) {
                    const u32x4 w = philox4x32_10(static_cast<uint32_t>(n), static_cast<uint32_t>(t / SPC),
                                                  g.seed_hi, 0u, g.seed_lo, c.inst_id);
                    box_muller_fast(w.v[0], w.v[1], zz[0], zz[1]);
                    box_muller_fast(w.v[2], w.v[3], zz[2], zz[3]);
                }
#pragma unroll
                for (int v = 0; v < NS; ++v) x[v] = fmaf(sqrt_dt * pick4(zz, r0 * NS + v), g.sigma[v], x[v]);
            }
        } else if constexpr (WideNoise<M>::value) {
            if (noise) {
                float z8[8];
#pragma unroll
                for (int b = 0; b < 2; ++b) {
                    const u32x4 w = philox4x32_10(static_cast<uint32_t>(n), static_cast<uint32_t>(t), g.seed_hi,
                                                  static_cast<uint32_t>(b), g.seed_lo, c.inst_id);
                    box_muller_fast(w.v[0], w.v[1], z8[4 * b], z8[4 * b + 1]);
                    box_muller_fast(w.v[2], w.v[3], z8[4 * b + 2], z8[4 * b + 3]);
                }
#pragma unroll
                for (int v = 0; v < NS; ++v)
                    x[v] = fmaf(sqrt_dt * z8[v], g.sigma[0] * NoiseScale<M>::at(v), x[v]);
            }
        }
        M::limit(x, c.flags);
        obs0 = M::obs(x, 0);
        const uint32_t pos = (static_cast<uint32_t>(t) + 1u) & mask;
        const size_t idx = (static_cast<size_t>(n) * R + pos) * RL + l;
        if constexpr (NC == 2) {
            if constexpr (CF == TVBG_CFUN_LEMS_2) {
                sn0 = M::ring_value(obs0, p);
                cs0 = M::ring_value2(x[M::CVAR2], p);
            } else {
                sincosf(obs0, &sn0, &cs0);
            }
            ring[idx] = sn0;
            ring[idx + kLanes] = cs0;
            if (pos < kGhost) {
                ring[idx + static_cast<size_t>(nh) * RL] = sn0;
                ring[idx + static_cast<size_t>(nh) * RL + kLanes] = cs0;
            }
        } else {
            const float rv = ring_val<M, CF>(obs0, p);
            ring[idx] = rv;
            if (pos < kGhost) ring[idx + static_cast<size_t>(nh) * kLanes] = rv;
        }
        if (bold) {
            Balloon::step(bs, bF, bV, bQ, xbold, g.dt_bold);
            if (k == b_next) {
                if (brow >= 0 && brow < g.bold_len)
                    g.bold_out[(static_cast<size_t>(brow) * N + n) * kLanes + l] = Balloon::signal(bV, bQ);
                b_next += mc.bper;
                brow += 1;
            }
        }
    }
#pragma unroll
    for (int v = 0; v < NS; ++v) state[(n * NS + v) * kLanes + l] = x[v];
    if (bold) {
        g.bold[(0 * N + n) * kLanes + l] = bs;
        g.bold[(1 * N + n) * kLanes + l] = bF;
        g.bold[(2 * N + n) * kLanes + l] = bV;
        g.bold[(3 * N + n) * kLanes + l] = bQ;
    }
}

// Pipelined group run: the CTA's warps form two teams of H = blockDim / 2
// threads, both mapped onto the same (node, lane) pairs.  While the update
// team runs the K steps of block b from the coupling sums in one shared
// buffer, the gather team sums block b + 1 into the other; one (cluster)
// barrier per block.  Block b + 1 reads ring slots up to
// tb + 2K - 1 - d_min, so with d_min >= 2K - 1 every slot it reads was
// written before block b started (ordered by the previous barrier), and
// the newest slot written in block b (tb + K) is at most d_max < nh slots
// ahead of the oldest read, so no read aliases a write.  Same arithmetic in
// the same order as run_group, so the results are identical.  Needs one
// node per slot (C * H / 8 >= N), K in {4, 8} and a 16-byte aligned ring.
template <class M, int CF, int K>
__device__ __forceinline__ void run_group_pipelined(const tvbg_group& g, float* csum, int32_t* status) {
    constexpr int NC = ring_channels<CF>();
    const int N = g.N;
    const uint32_t C = cluster_nranks();
    const uint32_t rank = cluster_rank();
    const bool cluster = C > 1;
    const int H = static_cast<int>(blockDim.x) / 2;
    const int P = H / kLanes;
    if (!group_descriptor_ok<M, CF>(g, true) || g.dmin < 2 * K - 1 || (H & 31) ||
        static_cast<int>(C) * P < N || (reinterpret_cast<uintptr_t>(g.ring) & 15u) != 0) {
        if (threadIdx.x == 0) report(status, TVBG_EINVAL);
        return;  // uniform over the cluster: same descriptor, same launch shape
    }
    const bool gather_team = static_cast<int>(threadIdx.x) >= H;
    const int tid = static_cast<int>(threadIdx.x) - (gather_team ? H : 0);
    const int l = tid % kLanes;
    const int q = (tid / kLanes) * static_cast<int>(C) + static_cast<int>(rank);
    const bool valid = q < N;
    const int n = valid ? (g.nodes ? __ldg(g.nodes + q) : q) : 0;
    const GroupLane c = make_lane<M>(g, l);
    const int bufsz = NC * K * H;  // floats per coupling-sum buffer

    if (!gather_team && valid) seed_node<M, CF>(g, c, n);
    group_barrier(cluster);
    // each team runs its own loop (disjoint live ranges); both meet at the
    // same number of barriers: one after block 0's gather, one per block
    const long long t_stop = c.t0 + g.nsteps;
    if (gather_team) {
        if (g.nsteps > 0)
            gather_node<M, CF, K>(g, c, valid, n, static_cast<uint32_t>(c.t0) & c.mask, csum + tid, H);
        group_barrier(cluster);
        int buf = 1;
        for (long long tb = c.t0; tb < t_stop; tb += K) {
            if (tb + K < t_stop)
                gather_node<M, CF, K>(g, c, valid, n, static_cast<uint32_t>(tb + K) & c.mask,
                                      csum + buf * bufsz + tid, H);
            buf ^= 1;
            group_barrier(cluster);
        }
    } else {
        group_barrier(cluster);
        MonitorClock mc;
        mc.init(g, c);
        int buf = 0;
        for (long long tb = c.t0; tb < t_stop; tb += K) {
            const int cnt = (t_stop - tb) < K ? static_cast<int>(t_stop - tb) : K;
            if (valid) update_node<M, CF, K>(g, c, n, tb, cnt, csum + buf * bufsz + tid, H, mc);
            mc.advance(g, c, cnt);
            buf ^= 1;
            group_barrier(cluster);
        }
    }
}

// Dynamic shared memory of a pipelined group CTA: two coupling-sum buffers
// of half the CTA each.
__host__ __device__ constexpr uint32_t group_pipelined_smem_bytes(int K, int threads, int nc) {
    return static_cast<uint32_t>(4 * 2 * K * (threads / 2) * nc);
}

// One group per CTA (or per cluster of CTAs): group index = order[cluster id].
template <class M, int CF, int K>
__global__ void __launch_bounds__(1024, 1)
    group_kernel(const tvbg_group* __restrict__ groups, int32_t n_groups,
                 const int32_t* __restrict__ order, int32_t* __restrict__ status) {
    __shared__ __align__(16) tvbg_group s_grp;
    extern __shared__ float csum[];  // [channels][K][blockDim]: the block's coupling sums
    const int cid = static_cast<int>(cluster_id_x());
    if (cid >= n_groups) return;  // uniform over the cluster
    const int idx = order ? __ldg(order + cid) : cid;
    stage_group(groups + idx, &s_grp);
    run_group<M, CF, K>(s_grp, csum, status);
}

// Pipelined variant (run_group_pipelined): blockDim = 2 teams x 8 lanes x
// node slots; same tables and results as group_kernel.
template <class M, int CF, int K>
__global__ void __launch_bounds__(1024, 1)
    group_kernel_pipelined(const tvbg_group* __restrict__ groups, int32_t n_groups,
                           const int32_t* __restrict__ order, int32_t* __restrict__ status) {
    __shared__ __align__(16) tvbg_group s_grp;
    extern __shared__ float csum[];  // [2][channels][K][blockDim / 2]
    const int cid = static_cast<int>(cluster_id_x());
    if (cid >= n_groups) return;  // uniform over the cluster
    const int idx = order ? __ldg(order + cid) : cid;
    stage_group(groups + idx, &s_grp);
    run_group_pipelined<M, CF, K>(s_grp, csum, status);
}

}  // namespace tvbg
