// Internal helpers shared by the translation units behind the C ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/tvbg.h"

namespace tvbg {

// Record `msg` as the calling thread's last error and return `code`.
int set_error(int code, const char* msg);
// Record a CUDA failure (message + cudaGetErrorString) and return TVBG_ECUDA.
int set_cuda_error(cudaError_t e, const char* where);

// Step kernel signature shared by every (model, coupling, lanes) instance.
using StepKernel = void (*)(const tvbg_instance*, int32_t, const int32_t*, int32_t*, int32_t*,
                            uint32_t);

// Per-model lookup: kernel for (cfun, tpn) or nullptr if not built.
StepKernel step_kernel_kuramoto(int cfun, int tpn);
StepKernel step_kernel_g2do(int cfun, int tpn);
StepKernel step_kernel_mpr(int cfun, int tpn);
StepKernel step_kernel_linear(int cfun, int tpn);

}  // namespace tvbg
