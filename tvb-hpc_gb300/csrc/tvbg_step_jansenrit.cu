// Step-kernel instances for the JansenRit model: every coupling function and
// gather width (lanes per node) 1, 2, 4, 8.
#include "tvbg_abi_internal.h"
#include "tvbg_step.cuh"

namespace tvbg {

template <int CF>
static StepKernel pick_tpn(int tpn) {
    switch (tpn) {
        case 1: return step_kernel<JansenRit, CF, 1>;
        case 2: return step_kernel<JansenRit, CF, 2>;
        case 4: return step_kernel<JansenRit, CF, 4>;
        case 8: return step_kernel<JansenRit, CF, 8>;
        default: return nullptr;
    }
}

StepKernel step_kernel_jansenrit(int cfun, int tpn) {
    switch (cfun) {
        case TVBG_CFUN_LINEAR: return pick_tpn<TVBG_CFUN_LINEAR>(tpn);
        case TVBG_CFUN_DIFF: return pick_tpn<TVBG_CFUN_DIFF>(tpn);
        case TVBG_CFUN_KURAMOTO: return pick_tpn<TVBG_CFUN_KURAMOTO>(tpn);
        case TVBG_CFUN_SIGMOIDAL: return pick_tpn<TVBG_CFUN_SIGMOIDAL>(tpn);
        default: return nullptr;
    }
}

}  // namespace tvbg
