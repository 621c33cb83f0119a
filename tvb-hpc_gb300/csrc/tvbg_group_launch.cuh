// Launch plumbing of the lane-interleaved group kernel (one group per CTA or
// per cluster of CTAs), shared by the engine library and the libraries
// generated from LEMS models.
#pragma once

#include <cuda_runtime.h>

#include <cstring>

#include "tvbg_lanes.cuh"
#include "tvbg_step_launch.cuh"

namespace tvbg {

using GroupKernelFn = void (*)(const tvbg_group*, int32_t, const int32_t*, int32_t*);

// Checks of a group launch configuration; *cluster = CTAs per group.
// k_mask: the block lengths built (bit K set for K in {1, 2, 4, 8});
// pipelined: whether the library builds the pipelined kernels (tpn 2).
inline int check_group_cfg(const tvbg_launch* cfg, const ErrSink& es, int* cluster,
                           unsigned k_mask = (1u << 4) | (1u << 8), bool pipelined = false) {
    if (!cfg) return es.error(TVBG_EINVAL, "null launch config");
    if (cfg->threads < 32 || cfg->threads > 1024 || (cfg->threads & 31))
        return es.error(TVBG_EINVAL, "threads must be a multiple of 32 in [32, 1024]");
    if (cfg->block_k < 1 || cfg->block_k > 8 || !((k_mask >> cfg->block_k) & 1u))
        return es.error(TVBG_EINVAL, "tvbg_group_run: block_k not built (4 or 8; 1, 2, 4 or 8 "
                                     "for LEMS libraries)");
    const int c = cfg->cluster <= 0 ? 1 : cfg->cluster;
    if (c < 1 || c > 16) return es.error(TVBG_EINVAL, "cluster must be in [1, 16]");
    if (cfg->tpn == TVBG_GROUP_PIPELINED) {
        if (!pipelined) return es.error(TVBG_EUNSUPPORTED, "tvbg_group_run: pipelined kernel not built");
        if (cfg->threads & 63)
            return es.error(TVBG_EINVAL, "tvbg_group_run: pipelined CTAs need a multiple of 64 threads");
    } else if (cfg->tpn > 1) {
        return es.error(TVBG_EINVAL, "tvbg_group_run: tpn must be 0, 1 or 2 (pipelined)");
    }
    *cluster = c;
    return TVBG_OK;
}

// Ring channels of a coupling id (the group kernel's shared-memory sums scale with it).
inline int group_channels(int cfun) {
    return (cfun == TVBG_CFUN_KURAMOTO || cfun == TVBG_CFUN_LEMS_SC || cfun == TVBG_CFUN_LEMS_2) ? 2
                                                                                                : 1;
}

// Launch n_groups groups of kfn: grid = n_groups * cluster CTAs, clusters of
// `cluster` CTAs, dynamic shared memory `smem` (opted in beyond 48 KB).
inline int launch_group_kernel(GroupKernelFn kfn, const tvbg_group* d_groups, int32_t n_groups,
                               const tvbg_launch* cfg, int cluster, size_t smem, void* stream,
                               const ErrSink& es) {
    if (n_groups < 0 || (n_groups > 0 && !d_groups))
        return es.error(TVBG_EINVAL, "tvbg_group_run: bad group array");
    if (n_groups == 0) return TVBG_OK;
    cudaError_t e = cudaSuccess;
    if (smem + sizeof(tvbg_group) > 48u * 1024u) {  // beyond the default: opt in
        e = cudaFuncSetAttribute(reinterpret_cast<const void*>(kfn),
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        if (e != cudaSuccess) return es.cuda(e, "tvbg_group_run: smem attribute");
    }
    if (cluster > 8) {  // 9..16 CTAs: a non-portable cluster size, opted in per kernel
        e = cudaFuncSetAttribute(reinterpret_cast<const void*>(kfn),
                                 cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        if (e != cudaSuccess) return es.cuda(e, "tvbg_group_run: non-portable cluster attribute");
    }
    cudaLaunchConfig_t lc;
    std::memset(&lc, 0, sizeof(lc));
    lc.gridDim = dim3(static_cast<unsigned>(n_groups) * static_cast<unsigned>(cluster), 1, 1);
    lc.blockDim = dim3(static_cast<unsigned>(cfg->threads), 1, 1);
    lc.dynamicSmemBytes = smem;
    lc.stream = static_cast<cudaStream_t>(stream);
    cudaLaunchAttribute attr[2];
    unsigned na = 0;
    if (cluster > 1) {
        attr[na].id = cudaLaunchAttributeClusterDimension;
        attr[na].val.clusterDim.x = static_cast<unsigned>(cluster);
        attr[na].val.clusterDim.y = 1;
        attr[na].val.clusterDim.z = 1;
        ++na;
    }
    if (cfg->priority != 0) {  // CTA dispatch order against concurrent launches
        int lo = 0, hi = 0;    // lo = least, hi = greatest priority (numerically lowest)
        e = cudaDeviceGetStreamPriorityRange(&lo, &hi);
        if (e != cudaSuccess) return es.cuda(e, "tvbg_group_run: priority range");
        int pr = cfg->priority;
        pr = pr < hi ? hi : (pr > lo ? lo : pr);
        attr[na].id = cudaLaunchAttributePriority;
        attr[na].val.priority = pr;
        ++na;
    }
    lc.attrs = attr;
    lc.numAttrs = na;
    e = cudaLaunchKernelEx(&lc, kfn, d_groups, n_groups, cfg->d_order, cfg->d_status);
    if (e != cudaSuccess) return es.cuda(e, "group kernel launch");
    return TVBG_OK;
}

}  // namespace tvbg
