// Lane-interleaved group kernels for the G2DO model: separable couplings
// (LINEAR, DIFF, SIGMOIDAL) x block length 4, 8 x edge slices 1, 2, 4.
#include "tvbg_abi_internal.h"
#include "tvbg_lanes.cuh"

namespace tvbg {

// slices: edge slices per node (1, 2 or 4); the sigmoidal coupling (an
// expf per value) is built with one slice only
template <int CF, int K>
static GroupKernel pick_s(int slices) {
    if constexpr (CF == TVBG_CFUN_SIGMOIDAL) {
        return slices == 1 ? group_kernel<G2DO, CF, K, 1> : nullptr;
    } else {
        switch (slices) {
            case 1: return group_kernel<G2DO, CF, K, 1>;
            case 2: return group_kernel<G2DO, CF, K, 2>;
            case 4: return group_kernel<G2DO, CF, K, 4>;
            default: return nullptr;
        }
    }
}

template <int CF>
static GroupKernel pick_k(int k, int slices) {
    switch (k) {
        case 4: return pick_s<CF, 4>(slices);
        case 8: return pick_s<CF, 8>(slices);
        default: return nullptr;
    }
}

GroupKernel group_kernel_g2do(int cfun, int k, int slices) {
    switch (cfun) {
        case TVBG_CFUN_LINEAR: return pick_k<TVBG_CFUN_LINEAR>(k, slices);
        case TVBG_CFUN_DIFF: return pick_k<TVBG_CFUN_DIFF>(k, slices);
        case TVBG_CFUN_SIGMOIDAL: return pick_k<TVBG_CFUN_SIGMOIDAL>(k, slices);
        default: return nullptr;
    }
}

}  // namespace tvbg
