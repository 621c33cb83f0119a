// Lane-interleaved group kernels for the Linear model: separable couplings
// (LINEAR, DIFF, SIGMOIDAL) x block length 4, 8.
#include "tvbg_abi_internal.h"
#include "tvbg_lanes.cuh"

namespace tvbg {

template <int CF>
static GroupKernel pick_k(int k) {
    switch (k) {
        case 4: return group_kernel<Linear, CF, 4>;
        case 8: return group_kernel<Linear, CF, 8>;
        default: return nullptr;
    }
}

GroupKernel group_kernel_linear(int cfun, int k) {
    switch (cfun) {
        case TVBG_CFUN_LINEAR: return pick_k<TVBG_CFUN_LINEAR>(k);
        case TVBG_CFUN_DIFF: return pick_k<TVBG_CFUN_DIFF>(k);
        case TVBG_CFUN_SIGMOIDAL: return pick_k<TVBG_CFUN_SIGMOIDAL>(k);
        default: return nullptr;
    }
}

}  // namespace tvbg
