/* Empty host stand-in (the reference kernels include it but use only curand_kernel.h). */
