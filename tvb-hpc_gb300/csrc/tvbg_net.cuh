// Node-parallel kernel for one very large network (one instance, N up to
// millions of nodes): the single-simulation case of
// tvb_hpc/examples/sim515k.py (515 056 nodes, CSR connectivity, one G2DO
// network with linear coupling).
//
// Canonical step: the CUDA-order step of the other kernels (tvbg_step.cuh);
// coupling sums in CSR order; Philox streams keyed (seed_lo, 0) with counter
// (node, t / SPC, seed_hi, 0), as for instance 0 of a sweep.
//
// Layout.  Node-major ring [N][R], R = nh + 8: slot s of node j at
// j R + (s & (nh-1)), positions < 8 mirrored at +nh, so the K slots an edge
// reads in a block are K contiguous floats (one or two sectors).  Edges in
// three CSR arrays: col (int32), w (float) and off = (nh - d) & (nh-1)
// (uint16).  State [N][nsvar], parameters [N][npar].
//
// Time blocking.  One launch runs one block of K <= d_min + 1 steps (with
// nh >= d_max + 1 + K no slot written in the block aliases one read in it):
// thread n gathers the K coupling sums of node n, runs its K updates and
// writes K ring slots; the launch boundary is the grid-wide barrier.  The
// network descriptor travels as a kernel parameter (constant bank).
#pragma once

#include "tvbg_lanes.cuh"

namespace tvbg {

template <class M, int CF, int K>
__global__ void __launch_bounds__(256)
    net_kernel(const tvbg_net g, long long tb, int cnt, int32_t* __restrict__ status) {
    constexpr int NS = M::NS;
    constexpr int NP = M::NP;
    constexpr int SPC = Noise<M>::SPC;
    constexpr int U = K >= 8 ? 2 : 4;
    const long long n = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (n >= g.N) return;
    const uint32_t nh = 1u << g.lognh;
    const uint32_t mask = nh - 1u;
    const uint32_t R = nh + kGhost;
    const uint32_t tm = static_cast<uint32_t>(tb) & mask;
    const bool noise = (g.flags & TVBG_F_NOISE) != 0;
    // gather: K sums per node, U edges per iteration (U K independent loads)
    float acc[K];
#pragma unroll
    for (int k = 0; k < K; ++k) acc[k] = 0.0f;
    const long long lo = __ldg(g.row + n), hi = __ldg(g.row + n + 1);
    long long e = lo;
    for (; e + U <= hi; e += U) {
        float v[U][K], w[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const float* p = g.ring + static_cast<size_t>(__ldg(g.col + e + u)) * R +
                             ((tm + __ldg(g.off + e + u)) & mask);
            w[u] = __ldg(g.w + e + u);
#pragma unroll
            for (int k = 0; k < K; ++k) v[u][k] = __ldcg(p + k);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
#pragma unroll
            for (int k = 0; k < K; ++k) acc[k] = fmaf(w[u], lane_pre<CF>(v[u][k], g.cf_p), acc[k]);
        }
    }
    for (; e < hi; ++e) {
        const float* p = g.ring + static_cast<size_t>(__ldg(g.col + e)) * R +
                         ((tm + __ldg(g.off + e)) & mask);
        const float w = __ldg(g.w + e);
#pragma unroll
        for (int k = 0; k < K; ++k) acc[k] = fmaf(w, lane_pre<CF>(__ldcg(p + k), g.cf_p), acc[k]);
    }
    // K updates
    float x[NS], p[NP];
#pragma unroll
    for (int v = 0; v < NS; ++v) x[v] = g.state[n * NS + v];
#pragma unroll
    for (int v = 0; v < NP; ++v) p[v] = __ldg(g.nparam + n * NP + v);
    const float wsum = (CF == TVBG_CFUN_DIFF && g.wsum) ? __ldg(g.wsum + n) : 0.0f;
    float obs0 = M::obs(x, 0);
    float zz[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    float* rrow = g.ring + static_cast<size_t>(n) * R;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        if (k < cnt) {
            const long long t = tb + k;
            const float c = lane_post<CF>(acc[k], obs0, wsum, g.cf_a, g.cf_b);
            float f[NS];
            M::drift(x, c, p, g.consts, f);
#pragma unroll
            for (int v = 0; v < NS; ++v) x[v] = fmaf(g.dt, f[v], x[v]);
            if constexpr (Noise<M>::kOK) {
                if (noise) {
                    const int r0 = static_cast<int>(t & (SPC - 1));
                    if (k == 0 || r0 == 0) {
                        const u32x4 w = philox4x32_10(static_cast<uint32_t>(n),
                                                      static_cast<uint32_t>(t / SPC), g.seed_hi, 0u,
                                                      g.seed_lo, 0u);
                        box_muller_fast(w.v[0], w.v[1], zz[0], zz[1]);
                        box_muller_fast(w.v[2], w.v[3], zz[2], zz[3]);
                    }
#pragma unroll
                    for (int v = 0; v < NS; ++v)
                        x[v] = fmaf(g.sqrt_dt * pick4(zz, r0 * NS + v), g.sigma[v], x[v]);
                }
            }
            M::limit(x, g.flags);
            obs0 = M::obs(x, 0);
            const uint32_t pos = (static_cast<uint32_t>(t) + 1u) & mask;
            rrow[pos] = obs0;
            if (pos < kGhost) rrow[pos + nh] = obs0;
        }
    }
#pragma unroll
    for (int v = 0; v < NS; ++v) g.state[n * NS + v] = x[v];
    (void)status;
}

// Seed slot t0 of every node with obs0 of its state.
template <class M>
__global__ void net_seed_kernel(const tvbg_net g, long long t0) {
    const long long n = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (n >= g.N) return;
    float x[M::NS];
#pragma unroll
    for (int v = 0; v < M::NS; ++v) x[v] = g.state[n * M::NS + v];
    const uint32_t nh = 1u << g.lognh;
    const uint32_t pos = static_cast<uint32_t>(t0) & (nh - 1u);
    float* rrow = g.ring + static_cast<size_t>(n) * (nh + kGhost);
    const float o = M::obs(x, 0);
    rrow[pos] = o;
    if (pos < kGhost) rrow[pos + nh] = o;
}

}  // namespace tvbg
