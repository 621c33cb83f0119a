// C ABI of the engine: argument checks, kernel dispatch, host helpers and
// the Philox generator kernels.  Declarations and reference citations are in
// include/tvbg.h.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "tvbg_abi_internal.h"
#include "tvbg_device.cuh"
#include "tvbg_step_launch.cuh"

namespace tvbg {

static thread_local char g_last_error[512] = "";

int set_error(int code, const char* msg) {
    std::snprintf(g_last_error, sizeof(g_last_error), "%s", msg);
    return code;
}

int set_cuda_error(cudaError_t e, const char* where) {
    std::snprintf(g_last_error, sizeof(g_last_error), "%s: %s (%s)", where, cudaGetErrorName(e),
                  cudaGetErrorString(e));
    return TVBG_ECUDA;
}

static StepKernel lookup(int model, int cfun, int tpn) {
    switch (model) {
        case TVBG_MODEL_KURAMOTO: return step_kernel_kuramoto(cfun, tpn);
        case TVBG_MODEL_G2DO: return step_kernel_g2do(cfun, tpn);
        case TVBG_MODEL_MPR: return step_kernel_mpr(cfun, tpn);
        case TVBG_MODEL_LINEAR: return step_kernel_linear(cfun, tpn);
        case TVBG_MODEL_G2DOSC: return step_kernel_g2dosc(cfun, tpn);
        case TVBG_MODEL_RWW: return step_kernel_rww(cfun, tpn);
        case TVBG_MODEL_JANSENRIT: return step_kernel_jansenrit(cfun, tpn);
        default: return nullptr;
    }
}

static BlockedKernel lookup_blocked(int model, int cfun, int tpn, int k) {
    switch (model) {
        case TVBG_MODEL_G2DO: return blocked_kernel_g2do(cfun, tpn, k);
        case TVBG_MODEL_MPR: return blocked_kernel_mpr(cfun, tpn, k);
        case TVBG_MODEL_LINEAR: return blocked_kernel_linear(cfun, tpn, k);
        case TVBG_MODEL_G2DOSC: return blocked_kernel_g2dosc(cfun, tpn, k);
        default: return nullptr;
    }
}

uint32_t blocked_aux_bytes(int model, int k, int nmax) {
    const int ns = (model == TVBG_MODEL_G2DO || model == TVBG_MODEL_MPR || model == TVBG_MODEL_G2DOSC) ? 2 : 1;
    // csum, z and xb are double-buffered for the pipelined loop
    return 4u * static_cast<uint32_t>(2 * k * nmax * (2 + ns) + 4 * nmax) + 32u;
}

static const ErrSink kSink{set_error, set_cuda_error};

static int check_launch(const tvbg_launch* cfg, const tvbg_instance* d_inst, int32_t n_inst) {
    return check_step_launch(cfg, d_inst, n_inst, kSink);
}

static int launch_step(int model, int cfun, const tvbg_instance* d_inst, int32_t n_inst,
                       const tvbg_launch* cfg, bool persistent, void* stream) {
    const bool blocked = cfg->block_k > 1;
    const int nmax = cfg->nmax > 0 ? cfg->nmax : cfg->threads;
    const void* kfn = nullptr;
    StepKernel k1 = nullptr;
    BlockedKernel kb = nullptr;
    size_t smem = 0;
    if (blocked) {
        kb = lookup_blocked(model, cfun, cfg->tpn, cfg->block_k);
        if (!kb)
            return set_error(TVBG_EUNSUPPORTED,
                             "time-blocked kernel not built for this model/coupling/tpn/block_k");
        kfn = reinterpret_cast<const void*>(kb);
        smem = static_cast<size_t>(cfg->smem_ring) + blocked_aux_bytes(model, cfg->block_k, nmax);
    } else {
        k1 = lookup(model, cfun, cfg->tpn);
        if (!k1) return set_error(TVBG_EUNSUPPORTED, "model/coupling pair not built into the library");
        kfn = reinterpret_cast<const void*>(k1);
        smem = step_smem_bytes(cfg->threads, cfg->smem_ring);
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int grid = 0;
    int rc = prepare_step_launch(kfn, smem, n_inst, cfg, persistent, st, kSink, &grid);
    if (rc) return rc;
    if (grid == 0) return TVBG_OK;
    const int32_t* order = persistent ? cfg->d_order : nullptr;
    int32_t* counter = persistent ? cfg->d_counter : nullptr;
    if (blocked)
        kb<<<grid, cfg->threads, smem, st>>>(d_inst, n_inst, order, counter, cfg->d_status,
                                             static_cast<uint32_t>(cfg->smem_ring), nmax);
    else
        k1<<<grid, cfg->threads, smem, st>>>(d_inst, n_inst, order, counter, cfg->d_status,
                                             static_cast<uint32_t>(cfg->smem_ring));
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_cuda_error(e, "step kernel launch");
    return TVBG_OK;
}

// ---- Philox fill kernels ---------------------------------------------------
__global__ void philox_normal_kernel(uint32_t k0, uint32_t k1, uint32_t c2, float* __restrict__ out,
                                     long long n) {
    const long long nb = (n + 3) / 4;
    for (long long b = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; b < nb;
         b += static_cast<long long>(gridDim.x) * blockDim.x) {
        float z[4];
        philox_normals4(static_cast<uint32_t>(b), static_cast<uint32_t>(b >> 32), c2, k0, k1, z);
        const long long i = 4 * b;
#pragma unroll
        for (int q = 0; q < 4; ++q)
            if (i + q < n) out[i + q] = z[q];
    }
}

__global__ void philox_u32_kernel(uint32_t k0, uint32_t k1, uint32_t c1, uint32_t c2, uint32_t c3,
                                  uint32_t* __restrict__ out, long long nb) {
    for (long long b = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; b < nb;
         b += static_cast<long long>(gridDim.x) * blockDim.x) {
        const u32x4 w = philox4x32_10(static_cast<uint32_t>(b), c1, c2, c3, k0, k1);
        reinterpret_cast<uint4*>(out)[b] = make_uint4(w.v[0], w.v[1], w.v[2], w.v[3]);
    }
}

}  // namespace tvbg

using namespace tvbg;

extern "C" {

int tvbg_abi_version(void) { return TVBG_ABI_VERSION; }
size_t tvbg_instance_size(void) { return sizeof(tvbg_instance); }
size_t tvbg_launch_size(void) { return sizeof(tvbg_launch); }
const char* tvbg_last_error(void) { return g_last_error; }

int tvbg_max_smem(int32_t* bytes) {
    if (!bytes) return set_error(TVBG_EINVAL, "tvbg_max_smem: null");
    int dev = 0, optin = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_cuda_error(e, "cudaGetDevice");
    e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e != cudaSuccess) return set_cuda_error(e, "cudaDeviceGetAttribute");
    *bytes = optin;
    return TVBG_OK;
}

int tvbg_occupancy(const tvbg_launch* cfg, int32_t* ctas_per_sm, int32_t* sms) {
    if (!cfg || !ctas_per_sm || !sms) return set_error(TVBG_EINVAL, "tvbg_occupancy: null");
    const tvbg_instance dummy{};
    int rc = check_launch(cfg, &dummy, 0);
    if (rc) return rc;
    const bool blocked = cfg->block_k > 1;
    const int nmax = cfg->nmax > 0 ? cfg->nmax : cfg->threads;
    const void* kfn = nullptr;
    size_t smem = 0;
    if (blocked) {
        BlockedKernel kb = lookup_blocked(cfg->model, cfg->cfun, cfg->tpn, cfg->block_k);
        if (!kb) return set_error(TVBG_EUNSUPPORTED, "time-blocked kernel not built");
        kfn = reinterpret_cast<const void*>(kb);
        smem = static_cast<size_t>(cfg->smem_ring) + blocked_aux_bytes(cfg->model, cfg->block_k, nmax);
    } else {
        StepKernel k1 = lookup(cfg->model, cfg->cfun, cfg->tpn);
        if (!k1) return set_error(TVBG_EUNSUPPORTED, "model/coupling pair not built");
        kfn = reinterpret_cast<const void*>(k1);
        smem = step_smem_bytes(cfg->threads, cfg->smem_ring);
    }
    cudaError_t e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
    if (e != cudaSuccess) return set_cuda_error(e, "tvbg_occupancy: smem attribute");
    int n = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kfn, cfg->threads, smem);
    if (e != cudaSuccess) return set_cuda_error(e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    int dev = 0, nsm = 0;
    e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return set_cuda_error(e, "tvbg_occupancy: SM count");
    *ctas_per_sm = n;
    *sms = nsm;
    return TVBG_OK;
}

int tvbg_pack_edges(int32_t N, int32_t nnz, const int32_t* row, const int32_t* col,
                    const float* weights, const int32_t* delays, int32_t lognh, tvbg_edge* out) {
    if (N <= 0 || nnz < 0 || !row || (nnz > 0 && (!col || !weights || !delays || !out)))
        return set_error(TVBG_EINVAL, "tvbg_pack_edges: bad arguments");
    if (lognh < 2 || lognh > 24) return set_error(TVBG_EINVAL, "tvbg_pack_edges: lognh out of [2, 24]");
    const uint64_t nh = 1ull << lognh;
    if (static_cast<uint64_t>(N) * nh > (1ull << 32))
        return set_error(TVBG_EINVAL, "tvbg_pack_edges: N * nh overflows 32-bit ring indices");
    if (row[0] != 0 || row[N] != nnz) return set_error(TVBG_EINVAL, "tvbg_pack_edges: row[0] != 0 or row[N] != nnz");
    for (int32_t i = 0; i < N; ++i)
        if (row[i + 1] < row[i]) return set_error(TVBG_EINVAL, "tvbg_pack_edges: row not monotone");
    const uint32_t mask = static_cast<uint32_t>(nh - 1);
    for (int32_t e = 0; e < nnz; ++e) {
        const int32_t c = col[e];
        const int32_t d = delays[e];
        if (c < 0 || c >= N) return set_error(TVBG_EINVAL, "tvbg_pack_edges: column out of range");
        if (d < 0 || static_cast<uint64_t>(d) >= nh)
            return set_error(TVBG_EINVAL, "tvbg_pack_edges: delay out of [0, nh)");
        const uint32_t uc = static_cast<uint32_t>(c);
        out[e].pk = (uc << lognh) | ((uc - static_cast<uint32_t>(d)) & mask);
        out[e].w = weights[e];
    }
    return TVBG_OK;
}

int tvbg_pack_edges_blocked(int32_t N, int32_t nnz, const int32_t* row, const int32_t* col,
                            const float* weights, const int32_t* delays, int32_t lognh,
                            tvbg_edge* out) {
    if (N <= 0 || N > 65536 || nnz < 0 || !row || (nnz > 0 && (!col || !weights || !delays || !out)))
        return set_error(TVBG_EINVAL, "tvbg_pack_edges_blocked: bad arguments");
    if (lognh < 3 || lognh > 16) return set_error(TVBG_EINVAL, "tvbg_pack_edges_blocked: lognh out of [3, 16]");
    const uint64_t nh = 1ull << lognh;
    if (static_cast<uint64_t>(N) * (nh + 8) > (1ull << 32))
        return set_error(TVBG_EINVAL, "tvbg_pack_edges_blocked: ring indices overflow 32 bits");
    if (row[0] != 0 || row[N] != nnz)
        return set_error(TVBG_EINVAL, "tvbg_pack_edges_blocked: row[0] != 0 or row[N] != nnz");
    for (int32_t i = 0; i < N; ++i)
        if (row[i + 1] < row[i]) return set_error(TVBG_EINVAL, "tvbg_pack_edges_blocked: row not monotone");
    const uint32_t mask = static_cast<uint32_t>(nh - 1);
    for (int32_t e = 0; e < nnz; ++e) {
        const int32_t c = col[e];
        const int32_t d = delays[e];
        if (c < 0 || c >= N) return set_error(TVBG_EINVAL, "tvbg_pack_edges_blocked: column out of range");
        if (d < 0 || static_cast<uint64_t>(d) >= nh)
            return set_error(TVBG_EINVAL, "tvbg_pack_edges_blocked: delay out of [0, nh)");
        const uint32_t uc = static_cast<uint32_t>(c);
        out[e].pk = (uc << 16) | ((uc - static_cast<uint32_t>(d)) & mask);
        out[e].w = weights[e];
    }
    return TVBG_OK;
}

int tvbg_delays(int32_t nnz, const float* lengths, float speed, float dt, int32_t rounding,
                int32_t* out) {
    if (nnz < 0 || (nnz > 0 && (!lengths || !out)) || !(speed > 0.0f) || !(dt > 0.0f) || rounding < 0 ||
        rounding > 2)
        return set_error(TVBG_EINVAL, "tvbg_delays: bad arguments");
    // volatile keeps each float32 rounding explicit (no contraction / excess precision)
    const volatile float vs = speed, vdt = dt;
    const volatile float rec = (1.0f / vs) / vdt;
    for (int32_t e = 0; e < nnz; ++e) {
        const float len = lengths[e];
        if (!(len >= 0.0f)) return set_error(TVBG_EINVAL, "tvbg_delays: negative or NaN length");
        float q;
        if (rounding == 2) {
            volatile float m = len * rec;
            q = std::trunc(static_cast<float>(m));
        } else {
            volatile float a = len / vs;
            volatile float b = a / vdt;
            q = rounding == 1 ? std::ceil(static_cast<float>(b)) : std::trunc(static_cast<float>(b));
        }
        if (q > 2147483647.0f) return set_error(TVBG_EINVAL, "tvbg_delays: delay overflows int32");
        out[e] = static_cast<int32_t>(q);
    }
    return TVBG_OK;
}

int tvbg_sweep(const tvbg_instance* d_inst, int32_t n_inst, const tvbg_launch* cfg, void* stream) {
    int rc = check_launch(cfg, d_inst, n_inst);
    if (rc) return rc;
    if (n_inst == 0) return TVBG_OK;
    return launch_step(cfg->model, cfg->cfun, d_inst, n_inst, cfg, false, stream);
}

int tvbg_batch_run(const tvbg_instance* d_inst, int32_t n_inst, const tvbg_launch* cfg, void* stream) {
    int rc = check_launch(cfg, d_inst, n_inst);
    if (rc) return rc;
    if (n_inst == 0) return TVBG_OK;
    return launch_step(cfg->model, cfg->cfun, d_inst, n_inst, cfg, true, stream);
}

int tvbg_philox_normal(uint64_t seed, uint32_t stream_id, float* d_out, int64_t n, void* stream) {
    if (!d_out || n < 0) return set_error(TVBG_EINVAL, "tvbg_philox_normal: bad arguments");
    if (n == 0) return TVBG_OK;
    const long long nb = (n + 3) / 4;
    int grid = static_cast<int>((nb + 255) / 256);
    if (grid > 152 * 32) grid = 152 * 32;
    philox_normal_kernel<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<uint32_t>(seed), stream_id, static_cast<uint32_t>(seed >> 32), d_out, n);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_cuda_error(e, "philox_normal launch");
    return TVBG_OK;
}

int tvbg_philox_u32(uint32_t k0, uint32_t k1, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t* d_out,
                    int64_t n_blocks, void* stream) {
    if (!d_out || n_blocks < 0 || n_blocks > 0xffffffffLL)
        return set_error(TVBG_EINVAL, "tvbg_philox_u32: bad arguments");
    if ((reinterpret_cast<uintptr_t>(d_out) & 15u) != 0)
        return set_error(TVBG_EINVAL, "tvbg_philox_u32: d_out must be 16-byte aligned");
    if (n_blocks == 0) return TVBG_OK;
    int grid = static_cast<int>((n_blocks + 255) / 256);
    if (grid > 152 * 32) grid = 152 * 32;
    philox_u32_kernel<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(k0, k1, c1, c2, c3, d_out,
                                                                           n_blocks);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_cuda_error(e, "philox_u32 launch");
    return TVBG_OK;
}

}  // extern "C"
