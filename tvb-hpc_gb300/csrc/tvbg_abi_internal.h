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

// Time-blocked kernel signature (adds the largest N of the call).
using BlockedKernel = void (*)(const tvbg_instance*, int32_t, const int32_t*, int32_t*, int32_t*,
                               uint32_t, int32_t);

// Per-model lookup: kernel for (cfun, tpn) or nullptr if not built.
StepKernel step_kernel_kuramoto(int cfun, int tpn);
StepKernel step_kernel_g2do(int cfun, int tpn);
StepKernel step_kernel_mpr(int cfun, int tpn);
StepKernel step_kernel_linear(int cfun, int tpn);
StepKernel step_kernel_g2dosc(int cfun, int tpn);
StepKernel step_kernel_rww(int cfun, int tpn);
StepKernel step_kernel_jansenrit(int cfun, int tpn);
// Per-model lookup of the time-blocked kernel for (cfun, tpn, K); nullptr if not built.
BlockedKernel blocked_kernel_g2do(int cfun, int tpn, int k);
BlockedKernel blocked_kernel_mpr(int cfun, int tpn, int k);
BlockedKernel blocked_kernel_linear(int cfun, int tpn, int k);
BlockedKernel blocked_kernel_g2dosc(int cfun, int tpn, int k);
// Lane-interleaved group kernel signature and per-model lookup for (cfun, K).
using GroupKernel = void (*)(const tvbg_group*, int32_t, const int32_t*, int32_t*);
GroupKernel group_kernel_kuramoto(int cfun, int k, bool pipe);
GroupKernel group_kernel_g2do(int cfun, int k, bool pipe);
GroupKernel group_kernel_mpr(int cfun, int k, bool pipe);
GroupKernel group_kernel_linear(int cfun, int k, bool pipe);
GroupKernel group_kernel_g2dosc(int cfun, int k, bool pipe);
GroupKernel group_kernel_rww(int cfun, int k, bool pipe);
GroupKernel group_kernel_jansenrit(int cfun, int k, bool pipe);
// Group kernel of the engine library for (model, cfun, K), nullptr if not built.
GroupKernel lookup_group_kernel(int model, int cfun, int k, bool pipe = false);
// Shared memory of the blocked kernel beyond the ring (floats): K * nmax * (2 + NS) + 4 * nmax.
uint32_t blocked_aux_bytes(int model, int k, int nmax);

}  // namespace tvbg
