// The fused network step kernel: delayed gather from the history ring,
// coupling, neural-mass drift, Euler-Maruyama with Philox noise, limit/wrap,
// ring write, trace and Balloon-Windkessel monitor -- for one instance per
// CTA at a time.
//
// Canonical step for instance b, node i, step t (tvb_hpc/network.py:115-143,
// coupling.py:103-121, model.py:131-155, scheme.py:88-107, and the ring
// addressing of dsl/dsl_cuda/CUDAmodels/kuramoto.c:92,108,128):
//   post = obs0(x_i(t))                  ring slot t
//   S    = sum_e w_e pre(ring[t - d_e][col_e], post)
//   c    = post_fn(S)
//   x'   = x + dt f(x, c, p_i) + sqrt(dt) sigma z      z ~ Philox/Box-Muller
//   x'   = limit(x')
//   ring slot t+1 <- obs0(x')
//
// Thread mapping.  Warp w owns nodes [32w, 32w+32): lane L updates node
// 32w+L (state in registers).  The gather for those 32 nodes is done by
// groups of TPN consecutive lanes, each group summing the in-edges of TPN
// nodes with coalesced CSR loads and a shuffle reduction; the sums reach the
// owning lanes through a 32-float shared slot per warp.
//
// Ring.  Node-major and skewed (see tvbg.h): either staged in shared memory
// by TMA bulk copies (cp.async.bulk + mbarrier) when it fits, or used in
// place in global memory.  Block barriers are needed only every sync_every
// steps: a value written at step t is first read at step t + 1 + d_min, and a
// slot is overwritten nh - d_max - 1 steps after its last read, so any
// sync_every <= min(d_min + 1, nh - d_max - 1) keeps every read correct.
#pragma once

#include "tvbg_device.cuh"

namespace tvbg {

constexpr uint32_t kFullMask = 0xffffffffu;
constexpr long long kWaitLimit = 1LL << 24;  // bounded mbarrier polls

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ float lds(uint32_t addr) {
    float v;
    asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(addr));
    return v;
}
__device__ __forceinline__ void sts(uint32_t addr, float v) {
    asm volatile("st.shared.f32 [%0], %1;" ::"r"(addr), "f"(v) : "memory");
}

// ---- TMA bulk copies (non-tensor, 16-byte granules) -----------------------
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes,
                                         uint32_t bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            dst),
        "l"(src), "r"(bytes), "r"(bar)
        : "memory");
}
__device__ __forceinline__ void bulk_s2g(void* dst, uint32_t src, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(src),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() {
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
__device__ __forceinline__ void bulk_wait_all() {
    asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void report(int32_t* status, int32_t code) {
    if (status) atomicCAS(status, 0, code);
}

// Shared-memory layout of a CTA: [ring capacity][csum: nwarps*32 floats][mbarrier].
struct SmemPlan {
    uint32_t ring;   // shared address of the ring
    uint32_t csum;   // shared address of the per-warp sums
    uint32_t mbar;   // shared address of the 8-byte mbarrier
};

// Stage `bytes` from global `src` into shared `dst` with bulk copies, waiting
// on the mbarrier with a bounded poll.  Returns false on timeout.
__device__ __forceinline__ bool tma_load(uint32_t dst, const void* src, uint32_t bytes,
                                         uint32_t bar, uint32_t& phase) {
    if (threadIdx.x == 0) {
        mbar_expect_tx(bar, bytes);
        constexpr uint32_t kChunk = 32768;
        for (uint32_t off = 0; off < bytes; off += kChunk) {
            const uint32_t n = (bytes - off) < kChunk ? (bytes - off) : kChunk;
            bulk_g2s(dst + off, static_cast<const char*>(src) + off, n, bar);
        }
    }
    bool ok = false;
    for (long long it = 0; it < kWaitLimit; ++it) {
        if (mbar_try_wait(bar, phase)) {
            ok = true;
            break;
        }
    }
    if (__syncthreads_or(!ok)) {
        // give the copy in flight a second bounded chance before leaving
        for (long long it = 0; it < kWaitLimit && !ok; ++it) ok = mbar_try_wait(bar, phase);
        __syncthreads();
        return false;
    }
    phase ^= 1u;
    return true;
}

__device__ __forceinline__ void tma_store(void* dst, uint32_t src, uint32_t bytes) {
    if (threadIdx.x == 0) {
        fence_proxy_async();
        constexpr uint32_t kChunk = 32768;
        for (uint32_t off = 0; off < bytes; off += kChunk) {
            const uint32_t n = (bytes - off) < kChunk ? (bytes - off) : kChunk;
            bulk_s2g(static_cast<char*>(dst) + off, src + off, n);
        }
        bulk_commit();
        bulk_wait_all();
    }
}

// Ring accessor: shared (explicit ld/st.shared) or global.
template <bool SMEM>
struct Ring;
template <>
struct Ring<true> {
    uint32_t base;
    __device__ __forceinline__ float ld(uint32_t i) const { return lds(base + 4u * i); }
    __device__ __forceinline__ void st(uint32_t i, float v) const { sts(base + 4u * i, v); }
};
template <>
struct Ring<false> {
    float* base;
    __device__ __forceinline__ float ld(uint32_t i) const { return base[i]; }
    __device__ __forceinline__ void st(uint32_t i, float v) const { base[i] = v; }
};

// The time loop of one instance.  All threads of the CTA call it.
template <class M, int CF, int TPN, bool SMEM>
__device__ __forceinline__ void run_steps(const tvbg_instance& d, const Ring<SMEM> ring,
                                          uint32_t csum_base, float* x, const float* p,
                                          float* bs) {
    using C = Cfun<CF>;
    constexpr int G = 32 / TPN;
    constexpr int SPC = Noise<M>::SPC;  // steps served by one Philox call
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int N = d.N;
    const int base = warp * 32;
    const int my = base + lane;
    const bool own = my < N;
    const bool active_warp = base < N;
    const uint32_t lognh = static_cast<uint32_t>(d.lognh);
    const uint32_t mask = (1u << lognh) - 1u;
    const uint32_t lo_mask = mask;
    const uint32_t hi_mask = ~mask;
    const uint32_t flags = d.flags;
    const bool noise = (flags & TVBG_F_NOISE) != 0;
    const bool bold = (flags & TVBG_F_BOLD) != 0 && d.bold_out != nullptr;
    const bool trace = (flags & TVBG_F_TRACE) != 0 && d.trace != nullptr;
    const bool tracka = (flags & TVBG_F_TRACKA) != 0;
    const bool midsync = (flags & TVBG_F_MIDSYNC) != 0;
    const bool trace_csum = trace && (flags & TVBG_F_TRACE_CSUM) != 0;
    const int trace_cols = d.trace_nobs + (trace_csum ? 1 : 0);
    const tvbg_edge* __restrict__ edges = d.edges;
    const float dt = d.dt, sqrt_dt = d.sqrt_dt;
    const int g = lane / TPN, lig = lane % TPN;
    const uint32_t my_ring_row = static_cast<uint32_t>(my) << lognh;

    // cached CSR bounds of the TPN nodes this lane gathers for
    int lo[TPN], hi[TPN];
#pragma unroll
    for (int k = 0; k < TPN; ++k) {
        const int n = base + g + G * k;
        lo[k] = (n < N) ? __ldg(d.row + n) : 0;
        hi[k] = (n < N) ? __ldg(d.row + n + 1) : 0;
    }

    const float* K = d.consts;

    long long t = d.t0;
    uint32_t tm = static_cast<uint32_t>(t) & mask;
    int since_sync = 0;
    const int sync_every = d.sync_every > 0 ? d.sync_every : 1;
    // countdowns to the next trace sample / BOLD sample
    int trace_cd = 0, bold_cd = 0;
    if (trace) {
        const long long r = t % d.trace_every;
        trace_cd = r == 0 ? 0 : static_cast<int>(d.trace_every - r);
    }
    if (bold) {
        const long long r = (t + 1) % d.bold_period;
        bold_cd = r == 0 ? 0 : static_cast<int>(d.bold_period - r);
    }
    float z[4] = {0.f, 0.f, 0.f, 0.f};

    float obs0 = own ? M::obs(x, 0) : 0.0f;

    for (int s = 0; s < d.nsteps; ++s, ++t) {
        // ---- trace of obs(x_t) at the start of the step (Track-A obsrv[t])
        if (trace) {
            if (trace_cd == 0) {
                if (own) {
                    const long long row = (t / d.trace_every) % d.trace_len;
                    float* dst = d.trace + row * d.trace_stride +
                                 static_cast<long long>(my) * trace_cols;
                    for (int o = 0; o < d.trace_nobs; ++o) dst[o] = M::obs(x, o);
                }
                trace_cd = d.trace_every;
            }
            --trace_cd;
        }
        // ---- phase 1: gather and reduce the coupling sums of this warp's nodes
        if (active_warp) {
#pragma unroll
            for (int k = 0; k < TPN; ++k) {
                const int L = g + G * k;
                const int n = base + L;
                float post = 0.0f;
                if (C::kNeedsPost) {
                    if (tracka) {
                        if (n < N)
                            post = ring.ld((static_cast<uint32_t>(n) << lognh) |
                                           ((tm + static_cast<uint32_t>(n)) & mask));
                    } else {
                        post = __shfl_sync(kFullMask, obs0, L);
                    }
                }
                float acc = 0.0f;
                for (int e = lo[k] + lig; e < hi[k]; e += TPN) {
                    const uint2 ew = __ldg(reinterpret_cast<const uint2*>(edges) + e);
                    const uint32_t idx = ((tm + ew.x) & lo_mask) | (ew.x & hi_mask);
                    const float pre = ring.ld(idx);
                    acc = fmaf(__uint_as_float(ew.y), C::pre(pre, post, d), acc);
                }
#pragma unroll
                for (int off = TPN / 2; off > 0; off >>= 1)
                    acc += __shfl_xor_sync(kFullMask, acc, off);
                if (lig == 0) sts(csum_base + 4u * static_cast<uint32_t>(L), acc);
            }
            __syncwarp();
        }
        if (midsync) __syncthreads();
        // ---- phase 2: update the node owned by this lane
        if (active_warp) {
            if (own) {
                const float S = lds(csum_base + 4u * static_cast<uint32_t>(lane));
                const float c = C::post(S, d);
                if (trace_csum && t % d.trace_every == 0) {
                    const long long row = (t / d.trace_every) % d.trace_len;
                    d.trace[row * d.trace_stride + static_cast<long long>(my) * trace_cols +
                            d.trace_nobs] = S;
                }
                if (tracka)  // the model writes obsrv[t] after the gather read it
                    ring.st(my_ring_row | ((tm + static_cast<uint32_t>(my)) & mask), obs0);
                if (bold) {
                    const float xb = M::obs(x, d.bold_obs);
                    Balloon::step(bs[0], bs[1], bs[2], bs[3], xb, d.dt_bold);
                    if (bold_cd == 0) {
                        const long long row = (t + 1) / d.bold_period - 1;
                        if (row >= 0 && row < d.bold_len)
                            d.bold_out[row * N + my] = Balloon::signal(bs[2], bs[3]);
                    }
                }
                float f[M::NS];
                M::drift(x, c, p, K, f);
#pragma unroll
                for (int v = 0; v < M::NS; ++v) x[v] = fmaf(dt, f[v], x[v]);
                if constexpr (Noise<M>::kOK) {
                    if (noise) {
                        const uint32_t tt = static_cast<uint32_t>(t);
                        const uint32_t ph = tt % SPC;
                        if (ph == 0 || s == 0)
                            philox_normals4(static_cast<uint32_t>(my), tt / SPC, d.seed_hi,
                                            d.seed_lo, d.inst_id, z);
#pragma unroll
                        for (int v = 0; v < M::NS; ++v) {
                            float zv = z[0];
#pragma unroll
                            for (int q = 0; q < 4; ++q)
                                if (q == static_cast<int>(ph) * M::NS + v) zv = z[q];
                            x[v] = fmaf(sqrt_dt * zv, d.sigma[v], x[v]);
                        }
                    }
                } else if constexpr (WideNoise<M>::value) {
                    if (noise) {
                        float z8[8];
                        const uint32_t tt = static_cast<uint32_t>(t);
                        philox_normals4(static_cast<uint32_t>(my), tt, d.seed_hi, d.seed_lo,
                                        d.inst_id, z8, 0u);
                        philox_normals4(static_cast<uint32_t>(my), tt, d.seed_hi, d.seed_lo,
                                        d.inst_id, z8 + 4, 1u);
#pragma unroll
                        for (int v = 0; v < M::NS; ++v)
                            x[v] = fmaf(sqrt_dt * z8[v], d.sigma[0] * NoiseScale<M>::at(v), x[v]);
                    }
                }
                M::limit(x, flags);
                obs0 = M::obs(x, 0);
                if (!tracka)
                    ring.st(my_ring_row | ((tm + 1u + static_cast<uint32_t>(my)) & mask), obs0);
            }
            __syncwarp();
        }
        if (bold) bold_cd = (bold_cd == 0) ? d.bold_period - 1 : bold_cd - 1;
        tm = (tm + 1u) & mask;
        if (++since_sync == sync_every) {
            __syncthreads();
            since_sync = 0;
        }
    }
}

// Run one instance on the calling CTA: stage, step, write back.
template <class M, int CF, int TPN>
__device__ __forceinline__ void run_instance(const tvbg_instance& d, const SmemPlan& sp,
                                             uint32_t smem_ring_cap, uint32_t& phase,
                                             int32_t* status) {
    const int N = d.N;
    const int my = threadIdx.x;
    const bool own = my < N;
    if (N > static_cast<int>(blockDim.x) || N <= 0 || d.lognh < 2 || d.lognh > 24 ||
        d.model != M::ID || d.cfun != CF ||
        (!Noise<M>::kOK && !WideNoise<M>::value && (d.flags & TVBG_F_NOISE))) {
        if (threadIdx.x == 0) report(status, TVBG_EINVAL);
        return;
    }
    const uint32_t nh = 1u << d.lognh;
    const uint32_t ring_bytes = static_cast<uint32_t>(N) * nh * 4u;
    const bool smem = (d.flags & TVBG_F_SMEM_RING) && ring_bytes <= smem_ring_cap &&
                      ((reinterpret_cast<uintptr_t>(d.ring) & 15u) == 0);

    float x[M::NS], p[M::NP], bs[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int v = 0; v < M::NS; ++v) x[v] = own ? d.state[my * M::NS + v] : 0.0f;
#pragma unroll
    for (int k = 0; k < M::NP; ++k) p[k] = own ? __ldg(d.nparam + my * M::NP + k) : 0.0f;
    if ((d.flags & TVBG_F_BOLD) && d.bold && own) {
#pragma unroll
        for (int k = 0; k < 4; ++k) bs[k] = d.bold[k * N + my];
    }
    const uint32_t mask = nh - 1u;
    const uint32_t tm0 = static_cast<uint32_t>(d.t0) & mask;
    const uint32_t seed_idx = (static_cast<uint32_t>(my) << d.lognh) |
                              ((tm0 + static_cast<uint32_t>(my)) & mask);

    const uint32_t csum = sp.csum + 4u * 32u * (threadIdx.x >> 5);
    if (smem) {
        __syncthreads();  // previous instance finished with shared memory
        const bool ok = tma_load(sp.ring, d.ring, ring_bytes, sp.mbar, phase);
        if (!ok) {
            if (threadIdx.x == 0) report(status, TVBG_ETIMEOUT);
            return;
        }
        // slot t0 holds obs0 of the state being resumed (CUDA order only)
        if (own && !(d.flags & TVBG_F_TRACKA)) sts(sp.ring + 4u * seed_idx, M::obs(x, 0));
        __syncthreads();
        Ring<true> r{sp.ring};
        run_steps<M, CF, TPN, true>(d, r, csum, x, p, bs);
        __syncthreads();
        tma_store(d.ring, sp.ring, ring_bytes);
    } else {
        if (own && !(d.flags & TVBG_F_TRACKA)) d.ring[seed_idx] = M::obs(x, 0);
        __syncthreads();
        Ring<false> r{d.ring};
        run_steps<M, CF, TPN, false>(d, r, csum, x, p, bs);
    }
    if (own) {
#pragma unroll
        for (int v = 0; v < M::NS; ++v) d.state[my * M::NS + v] = x[v];
        if ((d.flags & TVBG_F_BOLD) && d.bold) {
#pragma unroll
            for (int k = 0; k < 4; ++k) d.bold[k * N + my] = bs[k];
        }
    }
    __syncthreads();
}

// Copy one instance descriptor into shared memory (8-byte words).
__device__ __forceinline__ void stage_instance(const tvbg_instance* src, tvbg_instance* dst) {
    static_assert(sizeof(tvbg_instance) % 8 == 0, "descriptor size");
    constexpr int kWords = sizeof(tvbg_instance) / 8;
    const unsigned long long* s = reinterpret_cast<const unsigned long long*>(src);
    unsigned long long* d = reinterpret_cast<unsigned long long*>(dst);
    for (int i = threadIdx.x; i < kWords; i += blockDim.x) d[i] = s[i];
    __syncthreads();
}

// Sweep (counter == nullptr: CTA b runs instance b) or persistent batch
// (CTAs pull instance indices from *counter in `order`).
template <class M, int CF, int TPN>
__global__ void __launch_bounds__(1024, 1)
    step_kernel(const tvbg_instance* __restrict__ insts, int32_t n_inst,
                const int32_t* __restrict__ order, int32_t* __restrict__ counter,
                int32_t* __restrict__ status, uint32_t smem_ring_cap) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ int32_t next_idx;
    __shared__ tvbg_instance s_inst;
    SmemPlan sp;
    sp.ring = smem_addr(smem);
    sp.csum = sp.ring + smem_ring_cap;
    sp.mbar = sp.csum + 4u * blockDim.x;  // nwarps * 32 floats = blockDim floats
    uint32_t phase = 0;
    if (threadIdx.x == 0) {
        mbar_init(sp.mbar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (counter == nullptr) {
        if (static_cast<int>(blockIdx.x) < n_inst) {
            stage_instance(insts + blockIdx.x, &s_inst);
            run_instance<M, CF, TPN>(s_inst, sp, smem_ring_cap, phase, status);
        }
        return;
    }
    for (;;) {
        if (threadIdx.x == 0) next_idx = atomicAdd(counter, 1);
        __syncthreads();
        const int k = next_idx;
        if (k >= n_inst) break;
        const int idx = order ? __ldg(order + k) : k;
        stage_instance(insts + idx, &s_inst);  // ends with a barrier
        run_instance<M, CF, TPN>(s_inst, sp, smem_ring_cap, phase, status);
    }
}

}  // namespace tvbg
