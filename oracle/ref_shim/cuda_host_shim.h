/*
 * Force-included when the reference's CUDA sources are compiled for the host
 * (oracle/Makefile, target `ref`).  TEST INFRASTRUCTURE ONLY.
 *
 * The kernels of dsl/dsl_cuda/CUDAmodels/ are written one thread per
 * instance; with these definitions a kernel body becomes a plain C function
 * that ref_driver.c calls once per instance (threadIdx.x = instance,
 * blockDim.x = instance count, one node loop per call since threadIdx.y = 0
 * and blockDim.y = 1).  __syncthreads() has nothing to order in that form.
 */
#ifndef TVBG_CUDA_HOST_SHIM_H
#define TVBG_CUDA_HOST_SHIM_H
#include <math.h>
#define __global__
#define __device__
typedef struct { unsigned int x, y, z; } tvbg_shim_dim3;
extern tvbg_shim_dim3 threadIdx, blockIdx, blockDim, gridDim;
#define __syncthreads() ((void)0)
static inline float rsqrtf(float v) { return 1.0f / sqrtf(v); }
#endif
