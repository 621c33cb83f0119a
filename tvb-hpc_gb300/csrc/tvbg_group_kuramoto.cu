// Lane-interleaved group kernels for the Kuramoto model: the Kuramoto
// coupling (sin/cos ring channels) and the separable couplings (LINEAR, DIFF,
// SIGMOIDAL) x block length 4, 8.
#include "tvbg_abi_internal.h"
#include "tvbg_lanes.cuh"

namespace tvbg {

template <int CF>
static GroupKernel pick_k(int k) {
    switch (k) {
        case 4: return group_kernel<Kuramoto, CF, 4>;
        case 8: return group_kernel<Kuramoto, CF, 8>;
        default: return nullptr;
    }
}

GroupKernel group_kernel_kuramoto(int cfun, int k) {
    switch (cfun) {
        case TVBG_CFUN_LINEAR: return pick_k<TVBG_CFUN_LINEAR>(k);
        case TVBG_CFUN_DIFF: return pick_k<TVBG_CFUN_DIFF>(k);
        case TVBG_CFUN_SIGMOIDAL: return pick_k<TVBG_CFUN_SIGMOIDAL>(k);
        case TVBG_CFUN_KURAMOTO: return pick_k<TVBG_CFUN_KURAMOTO>(k);
        default: return nullptr;
    }
}

}  // namespace tvbg
