// Lane-interleaved group kernels for the Linear model: separable couplings
// (LINEAR, DIFF, SIGMOIDAL) x block length 4, 8 x gather depth 16, 32.
#include "tvbg_abi_internal.h"
#include "tvbg_lanes.cuh"

namespace tvbg {

// depth: sector loads in flight per thread / 8 (2 -> 16, 4 -> 32); the
// sigmoidal coupling (an expf per value) is built with depth 2 only
template <int CF>
static GroupKernel pick_k(int k, int depth) {
    if (CF == TVBG_CFUN_SIGMOIDAL || depth == 2) {
        switch (k) {
            case 4: return group_kernel<Linear, CF, 4, 16>;
            case 8: return group_kernel<Linear, CF, 8, 16>;
            default: return nullptr;
        }
    }
    if constexpr (CF != TVBG_CFUN_SIGMOIDAL) {
        if (depth == 4) {
            switch (k) {
                case 4: return group_kernel<Linear, CF, 4, 32>;
                case 8: return group_kernel<Linear, CF, 8, 32>;
                default: return nullptr;
            }
        }
    }
    return nullptr;
}

GroupKernel group_kernel_linear(int cfun, int k, int depth) {
    switch (cfun) {
        case TVBG_CFUN_LINEAR: return pick_k<TVBG_CFUN_LINEAR>(k, depth);
        case TVBG_CFUN_DIFF: return pick_k<TVBG_CFUN_DIFF>(k, depth);
        case TVBG_CFUN_SIGMOIDAL: return pick_k<TVBG_CFUN_SIGMOIDAL>(k, 2);
        default: return nullptr;
    }
}

}  // namespace tvbg
