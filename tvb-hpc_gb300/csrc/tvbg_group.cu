// C ABI of the lane-interleaved group kernels (tvbg_group_run and helpers).
#include <cstring>

#include "tvbg_abi_internal.h"
#include "tvbg_group_launch.cuh"

using namespace tvbg;

namespace {

GroupKernel lookup_group(int model, int cfun, int k, bool pipe) {
    switch (model) {
        case TVBG_MODEL_KURAMOTO: return group_kernel_kuramoto(cfun, k, pipe);
        case TVBG_MODEL_G2DO: return group_kernel_g2do(cfun, k, pipe);
        case TVBG_MODEL_MPR: return group_kernel_mpr(cfun, k, pipe);
        case TVBG_MODEL_LINEAR: return group_kernel_linear(cfun, k, pipe);
        case TVBG_MODEL_G2DOSC: return group_kernel_g2dosc(cfun, k, pipe);
        case TVBG_MODEL_RWW: return group_kernel_rww(cfun, k, pipe);
        case TVBG_MODEL_JANSENRIT: return group_kernel_jansenrit(cfun, k, pipe);
        default: return nullptr;
    }
}

const ErrSink kSink{set_error, set_cuda_error};

// Validate a group launch; its dynamic shared memory holds the K coupling
// sums of every thread.
int check_group_launch(const tvbg_launch* cfg, GroupKernel* kfn, int* cluster, size_t* smem) {
    int rc = check_group_cfg(cfg, kSink, cluster, (1u << 4) | (1u << 8), true);
    if (rc) return rc;
    const bool pipe = cfg->tpn == TVBG_GROUP_PIPELINED;
    *kfn = lookup_group(cfg->model, cfg->cfun, cfg->block_k, pipe);
    if (!*kfn)
        return set_error(TVBG_EUNSUPPORTED, "group kernel not built for this model/coupling/block_k");
    *smem = pipe ? group_pipelined_smem_bytes(cfg->block_k, cfg->threads, group_channels(cfg->cfun))
                 : group_smem_bytes(cfg->block_k, cfg->threads, group_channels(cfg->cfun));
    return TVBG_OK;
}

}  // namespace

GroupKernel tvbg::lookup_group_kernel(int model, int cfun, int k, bool pipe) {
    return lookup_group(model, cfun, k, pipe);
}

extern "C" {

size_t tvbg_group_size(void) { return sizeof(tvbg_group); }

int tvbg_pack_edges_group(int32_t N, int32_t nnz, const int32_t* row, const int32_t* col,
                          const float* weights, const int32_t* delays, int32_t lognh,
                          tvbg_edge* out) {
    if (N < 0 || nnz < 0 || !row || (nnz > 0 && (!col || !weights || !delays || !out)))
        return set_error(TVBG_EINVAL, "tvbg_pack_edges_group: bad arguments");
    if (lognh < 3 || lognh > 16 || N > 65536)
        return set_error(TVBG_EINVAL, "tvbg_pack_edges_group: needs lognh in [3, 16], N <= 65536");
    if (row[0] != 0 || row[N] != nnz)
        return set_error(TVBG_EINVAL, "tvbg_pack_edges_group: row must run from 0 to nnz");
    const uint32_t nh = 1u << lognh;
    const uint32_t mask = nh - 1u;
    for (int32_t i = 0; i < N; ++i) {
        if (row[i + 1] < row[i]) return set_error(TVBG_EINVAL, "tvbg_pack_edges_group: row not monotone");
        for (int32_t e = row[i]; e < row[i + 1]; ++e) {
            const int32_t c = col[e], d = delays[e];
            if (c < 0 || c >= N) return set_error(TVBG_EINVAL, "tvbg_pack_edges_group: col out of range");
            if (d < 0 || static_cast<uint32_t>(d) >= nh)
                return set_error(TVBG_EINVAL, "tvbg_pack_edges_group: delay outside [0, nh)");
            out[e].pk = (static_cast<uint32_t>(c) << 16) | ((nh - static_cast<uint32_t>(d)) & mask);
            out[e].w = weights[e];
        }
    }
    return TVBG_OK;
}

int tvbg_group_run(const tvbg_group* d_groups, int32_t n_groups, const tvbg_launch* cfg,
                   void* stream) {
    GroupKernel kfn = nullptr;
    int cluster = 1;
    size_t smem = 0;
    int rc = check_group_launch(cfg, &kfn, &cluster, &smem);
    if (rc) return rc;
    return launch_group_kernel(kfn, d_groups, n_groups, cfg, cluster, smem, stream, kSink);
}

int tvbg_group_occupancy(const tvbg_launch* cfg, int32_t* ctas_per_sm, int32_t* sms) {
    if (!ctas_per_sm || !sms) return set_error(TVBG_EINVAL, "tvbg_group_occupancy: null");
    GroupKernel kfn = nullptr;
    int cluster = 1;
    size_t smem = 0;
    int rc = check_group_launch(cfg, &kfn, &cluster, &smem);
    if (rc) return rc;
    int n = 0;
    cudaError_t e = cudaSuccess;
    if (smem + sizeof(tvbg_group) > 48u * 1024u) {  // beyond the default: opt in
        e = cudaFuncSetAttribute(reinterpret_cast<const void*>(kfn),
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        if (e != cudaSuccess) return set_cuda_error(e, "tvbg_group_occupancy: smem attribute");
    }
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, reinterpret_cast<const void*>(kfn),
                                                      cfg->threads, smem);
    if (e != cudaSuccess) return set_cuda_error(e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    int dev = 0, nsm = 0;
    e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return set_cuda_error(e, "tvbg_group_occupancy: SM count");
    *ctas_per_sm = n;
    *sms = nsm;
    return TVBG_OK;
}

int tvbg_group_max_clusters(const tvbg_launch* cfg, int32_t* max_clusters) {
    if (!max_clusters) return set_error(TVBG_EINVAL, "tvbg_group_max_clusters: null");
    GroupKernel kfn = nullptr;
    int cluster = 1;
    size_t smem = 0;
    int rc = check_group_launch(cfg, &kfn, &cluster, &smem);
    if (rc) return rc;
    cudaError_t e = cudaSuccess;
    if (smem + sizeof(tvbg_group) > 48u * 1024u) {
        e = cudaFuncSetAttribute(reinterpret_cast<const void*>(kfn),
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        if (e != cudaSuccess) return set_cuda_error(e, "tvbg_group_max_clusters: smem attribute");
    }
    if (cluster > 8) {
        e = cudaFuncSetAttribute(reinterpret_cast<const void*>(kfn),
                                 cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        if (e != cudaSuccess) return set_cuda_error(e, "tvbg_group_max_clusters: cluster attribute");
    }
    cudaLaunchConfig_t lc;
    std::memset(&lc, 0, sizeof(lc));
    lc.gridDim = dim3(static_cast<unsigned>(cluster), 1, 1);
    lc.blockDim = dim3(static_cast<unsigned>(cfg->threads), 1, 1);
    lc.dynamicSmemBytes = smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = static_cast<unsigned>(cluster);
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    lc.attrs = attr;
    lc.numAttrs = 1;
    int n = 0;
    e = cudaOccupancyMaxActiveClusters(&n, reinterpret_cast<const void*>(kfn), &lc);
    if (e != cudaSuccess) {
        cudaGetLastError();  // an unschedulable shape is reported here, before any launch
        n = 0;
    }
    *max_clusters = n;
    return TVBG_OK;
}

}  // extern "C"
