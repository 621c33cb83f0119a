/* Host stand-in for the curand device API used by the reference kernels:
 * the generator is replaced by zeros, so a reference kernel compiled with it
 * runs its deterministic (noise-off) dynamics.  TEST INFRASTRUCTURE ONLY. */
#ifndef TVBG_SHIM_CURAND_KERNEL_H
#define TVBG_SHIM_CURAND_KERNEL_H
typedef struct { int unused; } curandState;
typedef struct { float x, y; } float2;
static inline void curand_init(unsigned long long seed, unsigned long long sub,
                               unsigned long long off, curandState *st) {
    (void)seed; (void)sub; (void)off; st->unused = 0;
}
static inline float2 curand_normal2(curandState *st) {
    float2 r = {0.0f, 0.0f};
    (void)st;
    return r;
}
#endif
