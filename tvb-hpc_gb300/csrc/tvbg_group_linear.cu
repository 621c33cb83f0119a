// Lane-interleaved group kernels for the Linear model: separable couplings
// (LINEAR, DIFF, SIGMOIDAL) x block length 4, 8, plain and
// pipelined (group_kernel_pipelined).
#include "tvbg_abi_internal.h"
#include "tvbg_lanes.cuh"

namespace tvbg {

template <int CF>
static GroupKernel pick_k(int k, bool pipe) {
    switch (k) {
        case 4: return pipe ? group_kernel_pipelined<Linear, CF, 4> : group_kernel<Linear, CF, 4>;
        case 8: return pipe ? group_kernel_pipelined<Linear, CF, 8> : group_kernel<Linear, CF, 8>;
        default: return nullptr;
    }
}

GroupKernel group_kernel_linear(int cfun, int k, bool pipe) {
    switch (cfun) {
        case TVBG_CFUN_LINEAR: return pick_k<TVBG_CFUN_LINEAR>(k, pipe);
        case TVBG_CFUN_DIFF: return pick_k<TVBG_CFUN_DIFF>(k, pipe);
        case TVBG_CFUN_SIGMOIDAL: return pick_k<TVBG_CFUN_SIGMOIDAL>(k, pipe);
        default: return nullptr;
    }
}

}  // namespace tvbg
