// Time-blocked step kernel for couplings whose pre-summation term depends
// only on the source node (Linear, Diff, Sigmoidal: tvb_hpc/coupling.py:103-116).
//
// The canonical step is the one of tvbg_step.cuh (CUDA order).  Because a
// value written at step t is first read at step t + 1 + d_min, the coupling
// sums of K <= d_min + 1 consecutive steps only read ring slots that exist
// when the block starts.  Each block of K steps therefore runs as
//
//   phase A (all warps of the CTA):
//     - gather: for every node, K sums  S_k = sum_e w_e pre(ring[t+k-d_e][col_e])
//       -- one edge load and one address per K steps, K shared loads at
//       consecutive addresses (ring rows carry KG ghost slots so a run of K
//       slots never wraps);
//     - noise: the Philox4x32-10 normals of the K steps of every node;
//     - BOLD: the balloon steps of the previous block, from the inputs the
//       owners stored (the monitor lags the state by one block);
//   phase B (one owner lane per node): K model updates from the sums and
//     normals (Diff: post = a (S - x_i sum_e w_e) + b), ring writes, trace.
//
// Two block barriers per K steps.  The node update -- the serial part --
// is cut to the drift, the Euler-Maruyama update and the ring write, and
// the CTA may have more warps than owner lanes so the gather, the generator
// and the monitor use the whole CTA.
#pragma once

#include "tvbg_step.cuh"

namespace tvbg {

constexpr int kGhost = 8;  // ghost slots per ring row (>= the largest K)

// Pre-summation term of a separable coupling (source value only).
template <int CF>
__device__ __forceinline__ float pre_src(float xj, const tvbg_instance& d) {
    if constexpr (CF == TVBG_CFUN_SIGMOIDAL) {
        return d.cf_p[0] / (1.0f + expf(d.cf_p[2] * (d.cf_p[1] - xj)));
    } else {
        return xj;
    }
}

// Post-summation of a separable coupling: Diff subtracts x_i * sum_e w_e.
template <int CF>
__device__ __forceinline__ float post_sep(float S, float xi, float wsum, const tvbg_instance& d) {
    if constexpr (CF == TVBG_CFUN_DIFF) {
        return d.cf_a * (S - xi * wsum) + d.cf_b;
    } else if constexpr (CF == TVBG_CFUN_SIGMOIDAL) {
        return d.cf_a * S;
    } else {
        return d.cf_a * S + d.cf_b;
    }
}

struct BlockedSmem {
    uint32_t ring;   // shared address of the ring (TMA copies)
    uint32_t mbar;   // 8-byte mbarrier
    float* sring;    // N * R floats (shared-memory ring) -- 0 bytes if global
    float* csum;     // K * N floats
    float* z;        // K * NS * N floats
    float* xb;       // K * N floats (BOLD inputs of the block)
    float* bs;       // 4 * N floats (balloon state)
};

// Integrate the balloon of node n over `cnt` stored inputs starting at step tb.
__device__ __forceinline__ void bold_steps(const tvbg_instance& d, int n, int N, long long tb,
                                           int cnt, const float* xb, float* bsm) {
    float s = bsm[0 * N + n], F = bsm[1 * N + n], V = bsm[2 * N + n], Q = bsm[3 * N + n];
    for (int k = 0; k < cnt; ++k) {
        const long long t = tb + k;
        Balloon::step(s, F, V, Q, xb[k * N + n], d.dt_bold);
        if ((t + 1) % d.bold_period == 0) {
            const long long row = (t + 1) / d.bold_period - 1;
            if (row >= 0 && row < d.bold_len) d.bold_out[row * N + n] = Balloon::signal(V, Q);
        }
    }
    bsm[0 * N + n] = s;
    bsm[1 * N + n] = F;
    bsm[2 * N + n] = V;
    bsm[3 * N + n] = Q;
}

// Phase-A work of one block on the threads [first, first + nthr): the K
// coupling sums of every node into csum, and the block's Philox normals into z.
template <class M, int CF, int TPN, int K, bool SMEM>
__device__ __forceinline__ void gather_block(const tvbg_instance& d, const float* __restrict__ rsrc,
                                             float* csum, float* z, long long t0b, int cnt,
                                             int first, int nthr) {
    constexpr int NS = M::NS;
    constexpr int SPC = 4 / NS;
    const int N = d.N;
    const uint32_t nh = 1u << d.lognh;
    const uint32_t mask = nh - 1u;
    const uint32_t R = nh + kGhost;
    const uint32_t tm = static_cast<uint32_t>(t0b) & mask;
    const int tid = threadIdx.x - first;
    const int ngroups = nthr / TPN;
    const int gid = tid / TPN, lig = tid % TPN;
    const tvbg_edge* __restrict__ edges = d.edges;
    const int rounds = (N + ngroups - 1) / ngroups;
    for (int r = 0; r < rounds; ++r) {
        const int n = gid + r * ngroups;
        const bool valid = n < N;
        float acc[K];
#pragma unroll
        for (int k = 0; k < K; ++k) acc[k] = 0.0f;
        const int lo = valid ? __ldg(d.row + n) : 0;
        const int hi = valid ? __ldg(d.row + n + 1) : 0;
        int e = lo + lig;
        for (; e + TPN < hi; e += 2 * TPN) {
            const uint2 e0 = __ldg(reinterpret_cast<const uint2*>(edges) + e);
            const uint2 e1 = __ldg(reinterpret_cast<const uint2*>(edges) + e + TPN);
            const uint32_t i0 = (e0.x >> 16) * R + ((tm + (e0.x & 0xffffu)) & mask);
            const uint32_t i1 = (e1.x >> 16) * R + ((tm + (e1.x & 0xffffu)) & mask);
            const float w0 = __uint_as_float(e0.y), w1 = __uint_as_float(e1.y);
#pragma unroll
            for (int k = 0; k < K; ++k) {
                const float v0 = rsrc[i0 + k], v1 = rsrc[i1 + k];
                acc[k] = fmaf(w0, pre_src<CF>(v0, d), acc[k]);
                acc[k] = fmaf(w1, pre_src<CF>(v1, d), acc[k]);
            }
        }
        if (e < hi) {
            const uint2 e0 = __ldg(reinterpret_cast<const uint2*>(edges) + e);
            const uint32_t i0 = (e0.x >> 16) * R + ((tm + (e0.x & 0xffffu)) & mask);
            const float w0 = __uint_as_float(e0.y);
#pragma unroll
            for (int k = 0; k < K; ++k) acc[k] = fmaf(w0, pre_src<CF>(rsrc[i0 + k], d), acc[k]);
        }
#pragma unroll
        for (int k = 0; k < K; ++k) {
#pragma unroll
            for (int off = TPN / 2; off > 0; off >>= 1)
                acc[k] += __shfl_xor_sync(kFullMask, acc[k], off);
        }
        if (valid && lig == 0) {
#pragma unroll
            for (int k = 0; k < K; ++k)
                if (k < cnt) csum[k * N + n] = acc[k];
        }
    }
    if (d.flags & TVBG_F_NOISE) {
        const long long c0 = t0b / SPC, c1 = (t0b + cnt - 1) / SPC;
        const int ncall = static_cast<int>(c1 - c0) + 1;
        for (int q = tid; q < N * ncall; q += nthr) {
            const int n = q % N;
            const long long tc = c0 + q / N;
            float zz[4];
            philox_normals4(static_cast<uint32_t>(n), static_cast<uint32_t>(tc), d.seed_hi,
                            d.seed_lo, d.inst_id, zz);
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const long long ts = tc * SPC + r / NS;
                const int v = r % NS;
                if (ts >= t0b && ts < t0b + cnt) z[(static_cast<int>(ts - t0b) * NS + v) * N + n] = zz[r];
            }
        }
    }
}

// Phase-B work of one block on the owner thread of node `tid`.
template <class M, int CF, int K, bool SMEM>
__device__ __forceinline__ void update_block(const tvbg_instance& d, float* rdst, const float* csum,
                                             const float* z, float* xb, long long t0b, int cnt,
                                             float* x, const float* p, float wsum, float& obs0) {
    constexpr int NS = M::NS;
    const int tid = threadIdx.x;
    const int N = d.N;
    const uint32_t nh = 1u << d.lognh;
    const uint32_t mask = nh - 1u;
    const uint32_t R = nh + kGhost;
    const uint32_t flags = d.flags;
    const bool noise = (flags & TVBG_F_NOISE) != 0;
    const bool bold = (flags & TVBG_F_BOLD) != 0 && d.bold_out != nullptr;
    const bool trace = (flags & TVBG_F_TRACE) != 0 && d.trace != nullptr;
    const float dt = d.dt, sqrt_dt = d.sqrt_dt;
    const float* K_ = d.consts;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        if (k < cnt) {
            const long long t = t0b + k;
            if (trace && t % d.trace_every == 0) {
                const long long row = (t / d.trace_every) % d.trace_len;
                float* dst = d.trace + row * d.trace_stride + static_cast<long long>(tid) * d.trace_nobs;
                for (int o = 0; o < d.trace_nobs; ++o) dst[o] = M::obs(x, o);
            }
            if (bold) xb[k * N + tid] = M::obs(x, d.bold_obs);
            const float c = post_sep<CF>(csum[k * N + tid], obs0, wsum, d);
            float f[NS];
            M::drift(x, c, p, K_, f);
#pragma unroll
            for (int v = 0; v < NS; ++v) x[v] = fmaf(dt, f[v], x[v]);
            if (noise) {
#pragma unroll
                for (int v = 0; v < NS; ++v)
                    x[v] = fmaf(sqrt_dt * z[(k * NS + v) * N + tid], d.sigma[v], x[v]);
            }
            M::limit(x, flags);
            obs0 = M::obs(x, 0);
            const uint32_t pos = (static_cast<uint32_t>(t) + 1u + static_cast<uint32_t>(tid)) & mask;
            const uint32_t idx = static_cast<uint32_t>(tid) * R + pos;
            rdst[idx] = obs0;
            if (pos < kGhost) rdst[idx + nh] = obs0;
        }
    }
}

// Warp-specialised loop: owners (threads < N rounded to warps) update block
// i while the other warps gather block i+1 and integrate the balloon of
// block i-1.  csum, z and xb are double-buffered (two halves); one block
// barrier per block.  Valid when K <= (d_min + 1) / 2: block i+1 then reads
// only ring slots written by block i-1 or earlier.
template <class M, int CF, int TPN, int K, bool SMEM>
__device__ __forceinline__ void run_pipelined(const tvbg_instance& d, const BlockedSmem& sm,
                                              float* x, const float* p, float wsum) {
    constexpr int NS = M::NS;
    const int N = d.N;
    const int tid = threadIdx.x;
    const int nthr = blockDim.x;
    const int owners = ((N + 31) / 32) * 32;
    const int workers = nthr - owners;
    const bool is_owner = tid < owners;
    const bool own = tid < N;
    const bool bold = (d.flags & TVBG_F_BOLD) != 0 && d.bold_out != nullptr;
    float* ring = SMEM ? sm.sring : d.ring;
    // half h of each double buffer: base + h * (K * N [* NS])
    auto csum = [&](int h) { return sm.csum + h * K * N; };
    auto z = [&](int h) { return sm.z + h * K * NS * N; };
    auto xb = [&](int h) { return sm.xb + h * K * N; };
    const long long t0 = d.t0;
    const int nsteps = d.nsteps;
    const int nblk = (nsteps + K - 1) / K;
    float obs0 = own ? M::obs(x, 0) : 0.0f;
    if (nblk == 0) return;
    // prologue: gather block 0
    if (!is_owner) gather_block<M, CF, TPN, K, SMEM>(d, ring, csum(0), z(0), t0, nsteps < K ? nsteps : K, owners, workers);
    __syncthreads();
    for (int i = 0; i < nblk; ++i) {
        const long long tb = t0 + static_cast<long long>(i) * K;
        const int cnt = (nsteps - i * K) < K ? (nsteps - i * K) : K;
        if (is_owner) {
            if (own) update_block<M, CF, K, SMEM>(d, ring, csum(i & 1), z(i & 1), xb(i & 1), tb, cnt,
                                                  x, p, wsum, obs0);
        } else {
            if (i + 1 < nblk) {
                const int cn = (nsteps - (i + 1) * K) < K ? (nsteps - (i + 1) * K) : K;
                gather_block<M, CF, TPN, K, SMEM>(d, ring, csum((i + 1) & 1), z((i + 1) & 1),
                                                  tb + K, cn, owners, workers);
            }
            if (bold && i > 0) {
                for (int n = tid - owners; n < N; n += workers)
                    bold_steps(d, n, N, tb - K, K, xb((i - 1) & 1), sm.bs);
            }
        }
        __syncthreads();
    }
    // epilogue: the balloon of the last block
    if (bold && !is_owner) {
        const int last = nblk - 1;
        const int cnt = nsteps - last * K;
        for (int n = tid - owners; n < N; n += workers)
            bold_steps(d, n, N, t0 + static_cast<long long>(last) * K, cnt, xb(last & 1), sm.bs);
    }
    __syncthreads();
}

template <class M, int CF, int TPN, int K, bool SMEM>
__device__ __forceinline__ void run_blocked(const tvbg_instance& d, const BlockedSmem& sm,
                                            float* x, const float* p, float wsum) {
    constexpr int NS = M::NS;
    constexpr int SPC = 4 / NS;
    const int tid = threadIdx.x;
    const int nthr = blockDim.x;
    const int N = d.N;
    const bool own = tid < N;
    const int lognh = d.lognh;
    const uint32_t nh = 1u << lognh;
    const uint32_t mask = nh - 1u;
    const uint32_t R = nh + kGhost;
    const uint32_t flags = d.flags;
    const bool noise = (flags & TVBG_F_NOISE) != 0;
    const bool bold = (flags & TVBG_F_BOLD) != 0 && d.bold_out != nullptr;
    const bool trace = (flags & TVBG_F_TRACE) != 0 && d.trace != nullptr;
    const tvbg_edge* __restrict__ edges = d.edges;
    const float dt = d.dt, sqrt_dt = d.sqrt_dt;
    const int ngroups = nthr / TPN;
    const int gid = tid / TPN, lig = tid % TPN;
    float* gring = d.ring;
    const float* K_ = d.consts;

    long long t0b = d.t0;
    int left = d.nsteps;
    int prev_cnt = 0;          // BOLD inputs waiting from the previous block
    long long prev_t0 = 0;
    float obs0 = own ? M::obs(x, 0) : 0.0f;

    while (left > 0 || prev_cnt > 0) {
        const int cnt = left < K ? left : K;
        const uint32_t tm = static_cast<uint32_t>(t0b) & mask;
        // ---------------- phase A: gather, noise, lagged BOLD ----------------
        if (cnt > 0) {
            // warp-uniform rounds: every lane takes part in every shuffle
            const int rounds = (N + ngroups - 1) / ngroups;
            for (int r = 0; r < rounds; ++r) {
                const int n = gid + r * ngroups;
                const bool valid = n < N;
                float acc[K];
#pragma unroll
                for (int k = 0; k < K; ++k) acc[k] = 0.0f;
                const int lo = valid ? __ldg(d.row + n) : 0;
                const int hi = valid ? __ldg(d.row + n + 1) : 0;
                const float* __restrict__ rsrc = SMEM ? sm.sring : gring;
                int e = lo + lig;
                // two edges per iteration: independent loads in flight
                for (; e + TPN < hi; e += 2 * TPN) {
                    const uint2 e0 = __ldg(reinterpret_cast<const uint2*>(edges) + e);
                    const uint2 e1 = __ldg(reinterpret_cast<const uint2*>(edges) + e + TPN);
                    const uint32_t i0 = (e0.x >> 16) * R + ((tm + (e0.x & 0xffffu)) & mask);
                    const uint32_t i1 = (e1.x >> 16) * R + ((tm + (e1.x & 0xffffu)) & mask);
                    const float w0 = __uint_as_float(e0.y), w1 = __uint_as_float(e1.y);
#pragma unroll
                    for (int k = 0; k < K; ++k) {
                        const float v0 = rsrc[i0 + k], v1 = rsrc[i1 + k];
                        acc[k] = fmaf(w0, pre_src<CF>(v0, d), acc[k]);
                        acc[k] = fmaf(w1, pre_src<CF>(v1, d), acc[k]);
                    }
                }
                if (e < hi) {
                    const uint2 e0 = __ldg(reinterpret_cast<const uint2*>(edges) + e);
                    const uint32_t i0 = (e0.x >> 16) * R + ((tm + (e0.x & 0xffffu)) & mask);
                    const float w0 = __uint_as_float(e0.y);
#pragma unroll
                    for (int k = 0; k < K; ++k) acc[k] = fmaf(w0, pre_src<CF>(rsrc[i0 + k], d), acc[k]);
                }
#pragma unroll
                for (int k = 0; k < K; ++k) {
#pragma unroll
                    for (int off = TPN / 2; off > 0; off >>= 1)
                        acc[k] += __shfl_xor_sync(kFullMask, acc[k], off);
                }
                if (valid && lig == 0) {
#pragma unroll
                    for (int k = 0; k < K; ++k)
                        if (k < cnt) sm.csum[k * N + n] = acc[k];
                }
            }
            if (noise) {
                // Philox calls covering the steps [t0b, t0b + cnt) of every node
                const long long c0 = t0b / SPC, c1 = (t0b + cnt - 1) / SPC;
                const int ncall = static_cast<int>(c1 - c0) + 1;
                for (int q = tid; q < N * ncall; q += nthr) {
                    const int n = q % N;
                    const long long tc = c0 + q / N;
                    float zz[4];
                    philox_normals4(static_cast<uint32_t>(n), static_cast<uint32_t>(tc), d.seed_hi,
                                    d.seed_lo, d.inst_id, zz);
#pragma unroll
                    for (int r = 0; r < 4; ++r) {
                        const long long ts = tc * SPC + r / NS;
                        const int v = r % NS;
                        if (ts >= t0b && ts < t0b + cnt)
                            sm.z[(static_cast<int>(ts - t0b) * NS + v) * N + n] = zz[r];
                    }
                }
            }
        }
        if (bold && prev_cnt > 0) {
            // node n's balloon runs on thread nthr-1-n: the last warps, which
            // own no node in phase B when the CTA is wider than N
            const int n = nthr - 1 - tid;
            if (n < N) bold_steps(d, n, N, prev_t0, prev_cnt, sm.xb, sm.bs);
        }
        __syncthreads();
        if (cnt == 0) break;
        // ---------------- phase B: node updates ----------------
        if (own) {
#pragma unroll
            for (int k = 0; k < K; ++k) {
                if (k < cnt) {
                    const long long t = t0b + k;
                    if (trace && t % d.trace_every == 0) {
                        const long long row = (t / d.trace_every) % d.trace_len;
                        float* dst = d.trace + row * d.trace_stride +
                                     static_cast<long long>(tid) * d.trace_nobs;
                        for (int o = 0; o < d.trace_nobs; ++o) dst[o] = M::obs(x, o);
                    }
                    if (bold) sm.xb[k * N + tid] = M::obs(x, d.bold_obs);
                    const float S = sm.csum[k * N + tid];
                    const float c = post_sep<CF>(S, obs0, wsum, d);
                    float f[NS];
                    M::drift(x, c, p, K_, f);
#pragma unroll
                    for (int v = 0; v < NS; ++v) x[v] = fmaf(dt, f[v], x[v]);
                    if (noise) {
#pragma unroll
                        for (int v = 0; v < NS; ++v)
                            x[v] = fmaf(sqrt_dt * sm.z[(k * NS + v) * N + tid], d.sigma[v], x[v]);
                    }
                    M::limit(x, flags);
                    obs0 = M::obs(x, 0);
                    const uint32_t pos =
                        (static_cast<uint32_t>(t) + 1u + static_cast<uint32_t>(tid)) & mask;
                    const uint32_t idx = static_cast<uint32_t>(tid) * R + pos;
                    float* rdst = SMEM ? sm.sring : gring;
                    rdst[idx] = obs0;
                    if (pos < kGhost) rdst[idx + nh] = obs0;
                }
            }
        }
        prev_cnt = bold ? cnt : 0;
        prev_t0 = t0b;
        t0b += cnt;
        left -= cnt;
        __syncthreads();
    }
}

template <class M, int CF, int TPN, int K>
__device__ __forceinline__ void run_instance_blocked(const tvbg_instance& d, const BlockedSmem& sp,
                                                     uint32_t smem_ring_cap, uint32_t& phase,
                                                     int32_t* status) {
    const int N = d.N;
    const int tid = threadIdx.x;
    const bool own = tid < N;
    if (N > static_cast<int>(blockDim.x) || N <= 0 || d.lognh < 3 || d.lognh > 16 ||
        d.model != M::ID || d.cfun != CF || (d.flags & TVBG_F_TRACKA)) {
        if (tid == 0) report(status, TVBG_EINVAL);
        return;
    }
    const uint32_t nh = 1u << d.lognh;
    const uint32_t R = nh + kGhost;
    const uint32_t ring_bytes = static_cast<uint32_t>(N) * R * 4u;
    const bool smem = (d.flags & TVBG_F_SMEM_RING) && ring_bytes <= smem_ring_cap &&
                      ((reinterpret_cast<uintptr_t>(d.ring) & 15u) == 0);
    // the pipelined loop needs at least one worker warp beyond the owners
    const bool pipe = (d.flags & TVBG_F_PIPELINE) &&
                      static_cast<int>(blockDim.x) >= ((N + 31) / 32) * 32 + 32;
    float x[M::NS], p[M::NP];
#pragma unroll
    for (int v = 0; v < M::NS; ++v) x[v] = own ? d.state[tid * M::NS + v] : 0.0f;
#pragma unroll
    for (int k = 0; k < M::NP; ++k) p[k] = own ? __ldg(d.nparam + tid * M::NP + k) : 0.0f;
    float wsum = 0.0f;
    if (own) {
        const int lo = __ldg(d.row + tid), hi = __ldg(d.row + tid + 1);
        for (int e = lo; e < hi; ++e) wsum += __uint_as_float(__ldg(&d.edges[e].pk + 1));
    }
    const bool bold = (d.flags & TVBG_F_BOLD) && d.bold;
    for (int q = tid; q < 4 * N; q += blockDim.x) sp.bs[q] = bold ? d.bold[q] : 0.0f;
    const uint32_t mask = nh - 1u;
    const uint32_t pos0 = (static_cast<uint32_t>(d.t0) + static_cast<uint32_t>(tid)) & mask;
    const uint32_t seed_idx = static_cast<uint32_t>(tid) * R + pos0;
    __syncthreads();
    if (smem) {
        const bool ok = tma_load(sp.ring, d.ring, ring_bytes, sp.mbar, phase);
        if (!ok) {
            if (tid == 0) report(status, TVBG_ETIMEOUT);
            return;
        }
        if (own) {
            sp.sring[seed_idx] = M::obs(x, 0);
            if (pos0 < kGhost) sp.sring[seed_idx + nh] = M::obs(x, 0);
        }
        __syncthreads();
        if (pipe)
            run_pipelined<M, CF, TPN, K, true>(d, sp, x, p, wsum);
        else
            run_blocked<M, CF, TPN, K, true>(d, sp, x, p, wsum);
        __syncthreads();
        tma_store(d.ring, sp.ring, ring_bytes);
    } else {
        if (own) {
            d.ring[seed_idx] = M::obs(x, 0);
            if (pos0 < kGhost) d.ring[seed_idx + nh] = M::obs(x, 0);
        }
        __syncthreads();
        if (pipe)
            run_pipelined<M, CF, TPN, K, false>(d, sp, x, p, wsum);
        else
            run_blocked<M, CF, TPN, K, false>(d, sp, x, p, wsum);
    }
    if (own) {
#pragma unroll
        for (int v = 0; v < M::NS; ++v) d.state[tid * M::NS + v] = x[v];
    }
    if (bold)
        for (int q = tid; q < 4 * N; q += blockDim.x) d.bold[q] = sp.bs[q];
    __syncthreads();
}

// Shared memory of a blocked launch: ring | csum | z | xb | bs | mbarrier.
__host__ __device__ constexpr uint32_t blocked_aux_floats(int K, int NS, int nmax) {
    return static_cast<uint32_t>(K * nmax + K * NS * nmax + K * nmax + 4 * nmax);
}

template <class M, int CF, int TPN, int K>
__global__ void __launch_bounds__(1024, 1)
    blocked_kernel(const tvbg_instance* __restrict__ insts, int32_t n_inst,
                   const int32_t* __restrict__ order, int32_t* __restrict__ counter,
                   int32_t* __restrict__ status, uint32_t smem_ring_cap, int32_t nmax) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ int32_t next_idx;
    __shared__ tvbg_instance s_inst;
    BlockedSmem sp;
    sp.ring = smem_addr(smem);
    sp.sring = reinterpret_cast<float*>(smem);
    sp.csum = reinterpret_cast<float*>(smem + smem_ring_cap);
    sp.z = sp.csum + 2 * K * nmax;
    sp.xb = sp.z + 2 * K * M::NS * nmax;
    sp.bs = sp.xb + 2 * K * nmax;
    sp.mbar = (smem_addr(sp.bs + 4 * nmax) + 15u) & ~15u;
    uint32_t phase = 0;
    if (threadIdx.x == 0) {
        mbar_init(sp.mbar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (counter == nullptr) {
        if (static_cast<int>(blockIdx.x) < n_inst) {
            stage_instance(insts + blockIdx.x, &s_inst);
            if (s_inst.N <= nmax) run_instance_blocked<M, CF, TPN, K>(s_inst, sp, smem_ring_cap, phase, status);
            else if (threadIdx.x == 0) report(status, TVBG_EINVAL);
        }
        return;
    }
    for (;;) {
        if (threadIdx.x == 0) next_idx = atomicAdd(counter, 1);
        __syncthreads();
        const int k = next_idx;
        if (k >= n_inst) break;
        const int idx = order ? __ldg(order + k) : k;
        stage_instance(insts + idx, &s_inst);
        if (s_inst.N <= nmax) run_instance_blocked<M, CF, TPN, K>(s_inst, sp, smem_ring_cap, phase, status);
        else if (threadIdx.x == 0) report(status, TVBG_EINVAL);
    }
}

}  // namespace tvbg
