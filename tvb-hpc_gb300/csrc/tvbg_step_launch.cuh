// Launch plumbing of the per-step kernels (one instance per CTA, or
// persistent CTAs pulling instances from a counter), shared by the engine
// library and the libraries generated from LEMS models.  Errors are reported
// through the caller's error sink, so each library keeps its own last-error
// record.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "../../include/tvbg.h"

namespace tvbg {

struct ErrSink {
    int (*error)(int code, const char* msg);
    int (*cuda)(cudaError_t e, const char* where);
};

// Argument checks of tvbg_sweep / tvbg_batch_run (and their generated twins).
inline int check_step_launch(const tvbg_launch* cfg, const void* d_inst, int32_t n_inst,
                             const ErrSink& es) {
    if (!cfg || !d_inst || n_inst < 0) return es.error(TVBG_EINVAL, "null launch config or instances");
    if (cfg->threads < 32 || cfg->threads > 1024 || (cfg->threads & 31))
        return es.error(TVBG_EINVAL, "threads must be a multiple of 32 in [32, 1024]");
    if (cfg->tpn != 1 && cfg->tpn != 2 && cfg->tpn != 4 && cfg->tpn != 8)
        return es.error(TVBG_EINVAL, "tpn must be 1, 2, 4 or 8");
    if (cfg->smem_ring < 0 || (cfg->smem_ring & 15))
        return es.error(TVBG_EINVAL, "smem_ring must be a non-negative multiple of 16");
    if (cfg->block_k != 0 && cfg->block_k != 1 && cfg->block_k != 4 && cfg->block_k != 8)
        return es.error(TVBG_EINVAL, "block_k must be 0, 1, 4 or 8");
    if (cfg->nmax < 0 || cfg->nmax > cfg->threads)
        return es.error(TVBG_EINVAL, "nmax must be in [0, threads]");
    return TVBG_OK;
}

// Dynamic shared memory of a per-step launch: ring capacity + per-warp sums + mbarrier.
inline size_t step_smem_bytes(int threads, int smem_ring) {
    return static_cast<size_t>(smem_ring) + 4u * static_cast<size_t>(threads) + 16u;
}

// Set the kernel's shared-memory limit and size the grid: n_inst CTAs, or
// (persistent) cfg->ctas or one CTA per SM with the work counter zeroed on
// `st`.  *grid = 0 means there is nothing to launch.
inline int prepare_step_launch(const void* kfn, size_t smem, int32_t n_inst, const tvbg_launch* cfg,
                               bool persistent, cudaStream_t st, const ErrSink& es, int* grid) {
    *grid = 0;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return es.cuda(e, "cudaGetDevice");
    int optin = 0;
    e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e != cudaSuccess) return es.cuda(e, "cudaDeviceGetAttribute");
    // the kernel's static shared memory (instance descriptor, counter) needs ~300 bytes
    if (smem + 512 > static_cast<size_t>(optin))
        return es.error(TVBG_EINVAL, "ring capacity exceeds the shared memory of one CTA");
    e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return es.cuda(e, "cudaFuncSetAttribute(smem)");
    int g = n_inst;
    if (persistent) {
        if (!cfg->d_counter) return es.error(TVBG_EINVAL, "tvbg_batch_run needs d_counter");
        int sms = 0;
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return es.cuda(e, "cudaDeviceGetAttribute(SMs)");
        g = cfg->ctas > 0 ? cfg->ctas : sms;
        if (g > n_inst) g = n_inst;
        e = cudaMemsetAsync(cfg->d_counter, 0, sizeof(int32_t), st);
        if (e != cudaSuccess) return es.cuda(e, "cudaMemsetAsync(counter)");
    }
    *grid = g;
    return TVBG_OK;
}

}  // namespace tvbg
