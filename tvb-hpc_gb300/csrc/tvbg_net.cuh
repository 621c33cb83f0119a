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
// the K coupling sums of node n are gathered, its K updates run and K ring
// slots are written; the launch boundary is the grid-wide barrier.  Slots
// read in a launch are never written by it, so ring reads may go through
// the non-coherent L1 path.  The network descriptor travels as a kernel
// parameter (constant bank).
//
// Two thread mappings:
//   net_kernel       one thread per node, K sums in registers;
//   net_kernel_lanes K lanes per node, lane k sums step k: the K slots an
//                    edge reads are one contiguous 4K-byte load across the
//                    node's lanes, and the K updates run redundantly on every
//                    lane from sums and normals broadcast by shuffles.
// Both sum each node's in-edges in CSR order and take the same arithmetic
// per update, so they give bit-identical results.
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
            for (int k = 0; k < K; ++k) v[u][k] = __ldg(p + k);
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
        for (int k = 0; k < K; ++k) acc[k] = fmaf(w, lane_pre<CF>(__ldg(p + k), g.cf_p), acc[k]);
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

template <class M, int CF, int K>
__global__ void __launch_bounds__(256)
    net_kernel_lanes(const tvbg_net g, long long tb, int cnt, int32_t* __restrict__ status) {
    constexpr int NS = M::NS;
    constexpr int NP = M::NP;
    constexpr int SPC = Noise<M>::SPC;
    constexpr int U = 8;  // edges in flight per lane
    const long long gid = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    const long long n = gid / K;
    const int k = static_cast<int>(threadIdx.x & (K - 1));
    // blockDim is a multiple of 32, so a node's K lanes leave together
    if (n >= g.N) return;
    const unsigned gmask = ((1u << K) - 1u) << ((threadIdx.x & 31u) & ~static_cast<unsigned>(K - 1));
    const uint32_t nh = 1u << g.lognh;
    const uint32_t mask = nh - 1u;
    const uint32_t R = nh + kGhost;
    const uint32_t tm = static_cast<uint32_t>(tb) & mask;
    const bool noise = (g.flags & TVBG_F_NOISE) != 0;
    // gather: this lane sums slot k of every in-edge (step tb + k)
    float acc = 0.0f;
    const long long lo = __ldg(g.row + n), hi = __ldg(g.row + n + 1);
    long long e = lo;
    for (; e + U <= hi; e += U) {
        float v[U], w[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const size_t c = static_cast<size_t>(__ldg(g.col + e + u));
            const uint32_t o = __ldg(g.off + e + u);
            w[u] = __ldg(g.w + e + u);
            v[u] = __ldg(g.ring + c * R + ((tm + o) & mask) + k);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) acc = fmaf(w[u], lane_pre<CF>(v[u], g.cf_p), acc);
    }
    for (; e < hi; ++e) {
        const size_t c = static_cast<size_t>(__ldg(g.col + e));
        const float v = __ldg(g.ring + c * R + ((tm + __ldg(g.off + e)) & mask) + k);
        acc = fmaf(__ldg(g.w + e), lane_pre<CF>(v, g.cf_p), acc);
    }
    // K updates, run by every lane of the node
    float x[NS], p[NP];
#pragma unroll
    for (int v = 0; v < NS; ++v) x[v] = g.state[n * NS + v];
#pragma unroll
    for (int v = 0; v < NP; ++v) p[v] = __ldg(g.nparam + n * NP + v);
    const float wsum = (CF == TVBG_CFUN_DIFF && g.wsum) ? __ldg(g.wsum + n) : 0.0f;
    // the normals of step tb + k, drawn by lane k
    float zk[NS];
#pragma unroll
    for (int v = 0; v < NS; ++v) zk[v] = 0.0f;
    if constexpr (Noise<M>::kOK) {
        if (noise && k < cnt) {
            const long long t = tb + k;
            const int r0 = static_cast<int>(t & (SPC - 1));
            const u32x4 w = philox4x32_10(static_cast<uint32_t>(n), static_cast<uint32_t>(t / SPC),
                                          g.seed_hi, 0u, g.seed_lo, 0u);
            float zz[4];
            box_muller_fast(w.v[0], w.v[1], zz[0], zz[1]);
            box_muller_fast(w.v[2], w.v[3], zz[2], zz[3]);
#pragma unroll
            for (int v = 0; v < NS; ++v) zk[v] = pick4(zz, r0 * NS + v);
        }
    }
    float obs0 = M::obs(x, 0);
    float mine = 0.0f;
#pragma unroll
    for (int s = 0; s < K; ++s) {
        if (s < cnt) {
            const float S = __shfl_sync(gmask, acc, s, K);
            const float c = lane_post<CF>(S, obs0, wsum, g.cf_a, g.cf_b);
            float f[NS];
            M::drift(x, c, p, g.consts, f);
#pragma unroll
            for (int v = 0; v < NS; ++v) x[v] = fmaf(g.dt, f[v], x[v]);
            if constexpr (Noise<M>::kOK) {
                if (noise) {
#pragma unroll
                    for (int v = 0; v < NS; ++v) {
                        const float zv = __shfl_sync(gmask, zk[v], s, K);
                        x[v] = fmaf(g.sqrt_dt * zv, g.sigma[v], x[v]);
                    }
                }
            }
            M::limit(x, g.flags);
            obs0 = M::obs(x, 0);
            if (k == s) mine = obs0;
        }
    }
    if (k < cnt) {
        float* rrow = g.ring + static_cast<size_t>(n) * R;
        const uint32_t pos = (static_cast<uint32_t>(tb + k) + 1u) & mask;
        rrow[pos] = mine;
        if (pos < kGhost) rrow[pos + nh] = mine;
    }
    if (k == 0) {
#pragma unroll
        for (int v = 0; v < NS; ++v) g.state[n * NS + v] = x[v];
    }
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
