// C ABI of the node-parallel kernel for one very large network (tvbg_net_run).
#include "tvbg_abi_internal.h"
#include "tvbg_net.cuh"

using namespace tvbg;

namespace {

using NetKernel = void (*)(const tvbg_net, long long, int, int32_t*);
using SeedKernel = void (*)(const tvbg_net, long long);

// lanes == 1: one thread per node; lanes == K: K lanes per node.
template <class M, int CF>
NetKernel pick_k(int k, bool lanes) {
    switch (k) {
        case 4: return lanes ? net_kernel_lanes<M, CF, 4> : net_kernel<M, CF, 4>;
        case 8: return lanes ? net_kernel_lanes<M, CF, 8> : net_kernel<M, CF, 8>;
        default: return nullptr;
    }
}

template <class M>
NetKernel pick_cf(int cfun, int k, bool lanes) {
    switch (cfun) {
        case TVBG_CFUN_LINEAR: return pick_k<M, TVBG_CFUN_LINEAR>(k, lanes);
        case TVBG_CFUN_DIFF: return pick_k<M, TVBG_CFUN_DIFF>(k, lanes);
        case TVBG_CFUN_SIGMOIDAL: return pick_k<M, TVBG_CFUN_SIGMOIDAL>(k, lanes);
        default: return nullptr;
    }
}

int lookup(int model, int cfun, int k, bool lanes, NetKernel* kfn, SeedKernel* sfn) {
    switch (model) {
        case TVBG_MODEL_G2DO: *kfn = pick_cf<G2DO>(cfun, k, lanes); *sfn = net_seed_kernel<G2DO>; break;
        case TVBG_MODEL_G2DOSC:
            *kfn = pick_cf<G2DOsc>(cfun, k, lanes);
            *sfn = net_seed_kernel<G2DOsc>;
            break;
        case TVBG_MODEL_MPR: *kfn = pick_cf<MPR>(cfun, k, lanes); *sfn = net_seed_kernel<MPR>; break;
        case TVBG_MODEL_LINEAR:
            *kfn = pick_cf<Linear>(cfun, k, lanes);
            *sfn = net_seed_kernel<Linear>;
            break;
        default: *kfn = nullptr;
    }
    return *kfn ? TVBG_OK : set_error(TVBG_EUNSUPPORTED, "tvbg_net_run: model/coupling/block_k not built");
}

}  // namespace

extern "C" size_t tvbg_net_size(void) { return sizeof(tvbg_net); }

extern "C" int tvbg_net_run(const tvbg_net* net, int64_t t0, int32_t nsteps, const tvbg_launch* cfg,
                            void* stream) {
    if (!net || !cfg || nsteps < 0 || t0 < 0)
        return set_error(TVBG_EINVAL, "tvbg_net_run: bad arguments");
    if (net->N <= 0 || net->lognh < 3 || net->lognh > 16 || !net->row || !net->ring ||
        !net->state || !net->nparam || (net->flags & (TVBG_F_TRACKA | TVBG_F_MIDSYNC)))
        return set_error(TVBG_EINVAL, "tvbg_net_run: bad network descriptor");
    if (cfg->block_k != 4 && cfg->block_k != 8)
        return set_error(TVBG_EINVAL, "tvbg_net_run: block_k must be 4 or 8");
    if (cfg->threads < 32 || cfg->threads > 1024 || (cfg->threads & 31))
        return set_error(TVBG_EINVAL, "threads must be a multiple of 32 in [32, 1024]");
    if (net->model != cfg->model || net->cfun != cfg->cfun)
        return set_error(TVBG_EINVAL, "tvbg_net_run: descriptor and launch disagree on model/coupling");
    const int lanes = cfg->tpn > 1 ? cfg->tpn : 1;
    if (lanes != 1 && lanes != cfg->block_k)
        return set_error(TVBG_EINVAL, "tvbg_net_run: tpn must be 0, 1 or block_k");
    NetKernel kfn = nullptr;
    SeedKernel sfn = nullptr;
    int rc = lookup(net->model, net->cfun, cfg->block_k, lanes > 1, &kfn, &sfn);
    if (rc) return rc;
    const long long seed_blocks = (net->N + cfg->threads - 1) / cfg->threads;
    const long long blocks = (net->N * lanes + cfg->threads - 1) / cfg->threads;
    if (blocks > 0x7fffffffLL) return set_error(TVBG_EINVAL, "tvbg_net_run: N too large");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    sfn<<<static_cast<unsigned>(seed_blocks), cfg->threads, 0, st>>>(*net, t0);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_cuda_error(e, "tvbg_net_run: seed launch");
    for (long long tb = t0; tb < t0 + nsteps; tb += cfg->block_k) {
        const int cnt = static_cast<int>((t0 + nsteps - tb) < cfg->block_k ? (t0 + nsteps - tb)
                                                                            : cfg->block_k);
        kfn<<<static_cast<unsigned>(blocks), cfg->threads, 0, st>>>(*net, tb, cnt, cfg->d_status);
        e = cudaGetLastError();
        if (e != cudaSuccess) return set_cuda_error(e, "tvbg_net_run: step launch");
    }
    return TVBG_OK;
}
