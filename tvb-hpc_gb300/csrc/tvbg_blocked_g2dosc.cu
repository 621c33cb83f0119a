// Time-blocked step-kernel instances for the G2DOsc model: separable couplings
// (LINEAR, DIFF, SIGMOIDAL) x gather width 2, 4, 8 x block length 4, 8.
#include "tvbg_abi_internal.h"
#include "tvbg_step_blocked.cuh"

namespace tvbg {

template <int CF, int K>
static BlockedKernel pick_tpn_b(int tpn) {
    switch (tpn) {
        case 2: return blocked_kernel<G2DOsc, CF, 2, K>;
        case 4: return blocked_kernel<G2DOsc, CF, 4, K>;
        case 8: return blocked_kernel<G2DOsc, CF, 8, K>;
        default: return nullptr;
    }
}

template <int CF>
static BlockedKernel pick_k(int tpn, int k) {
    switch (k) {
        case 4: return pick_tpn_b<CF, 4>(tpn);
        case 8: return pick_tpn_b<CF, 8>(tpn);
        default: return nullptr;
    }
}

BlockedKernel blocked_kernel_g2dosc(int cfun, int tpn, int k) {
    switch (cfun) {
        case TVBG_CFUN_LINEAR: return pick_k<TVBG_CFUN_LINEAR>(tpn, k);
        case TVBG_CFUN_DIFF: return pick_k<TVBG_CFUN_DIFF>(tpn, k);
        case TVBG_CFUN_SIGMOIDAL: return pick_k<TVBG_CFUN_SIGMOIDAL>(tpn, k);
        default: return nullptr;
    }
}

}  // namespace tvbg
