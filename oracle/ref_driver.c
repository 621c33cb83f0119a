/*
 * ref_driver.c -- calls the reference's own CUDA kernels, compiled for the
 * host by oracle/Makefile (target `ref`), once per instance.
 * TEST INFRASTRUCTURE ONLY: used to pin the oracle restatement against the
 * reference's arithmetic (ring addressing, truncated delays, fmod wrap,
 * balloon update, covariance), never by the product.
 */
#include <stddef.h>

typedef struct { unsigned int x, y, z; } tvbg_shim_dim3;
tvbg_shim_dim3 threadIdx, blockIdx, blockDim, gridDim;

/* dsl/dsl_cuda/CUDAmodels/kuramoto.c:29-39 */
void Kuramoto(unsigned int i_step, unsigned int n_node, unsigned int nh, unsigned int n_step,
              unsigned int n_params, float dt, float speed, float *weights, float *lengths,
              float *params_pwi, float *state_pwi, float *tavg_pwi);
/* dsl/dsl_cuda/CUDAmodels/refs/balloon.c:24-30 */
void bold_update(int n_node, float dt, float *bold_state, float *neural_state, float *out);
/* dsl/dsl_cuda/CUDAmodels/refs/covar.c:78-84, 140-145 */
void update_cov(unsigned int i_sample, unsigned int n_node, float *cov, float *means,
                const float *data);
void cov_to_corr(unsigned int n_sample, unsigned int n_node, float *cov, float *corr);

static void one_block(unsigned int n_work) {
    blockIdx.x = blockIdx.y = blockIdx.z = 0;
    gridDim.x = gridDim.y = gridDim.z = 1;
    blockDim.x = n_work;
    blockDim.y = blockDim.z = 1;
    threadIdx.y = threadIdx.z = 0;
}

/* Layout as cuda_run.py:74-80: params[n_params][n_work] (speed, coupling),
 * state[nh][n_node][n_work], tavg[n_node][n_work]. */
void ref_kuramoto(unsigned int i_step, unsigned int n_node, unsigned int nh, unsigned int n_step,
                  float dt, float *weights, float *lengths, float *params, float *state,
                  float *tavg, unsigned int n_work) {
    unsigned int w;
    one_block(n_work);
    for (w = 0; w < n_work; ++w) {
        threadIdx.x = w;
        Kuramoto(i_step, n_node, nh, n_step, 2, dt, 0.0f, weights, lengths, params, state, tavg);
    }
}

/* bold[4][n_node][n_threads], neural[n_node][n_threads], out[n_node][n_threads] */
void ref_bold_update(int n_node, float dt, float *bold, float *neural, float *out,
                     unsigned int n_threads) {
    unsigned int w;
    one_block(n_threads);
    for (w = 0; w < n_threads; ++w) {
        threadIdx.x = w;
        bold_update(n_node, dt, bold, neural, out);
    }
}

/* single instance (covar.c TEST_COVAR mode: it = 0, nt = 1) */
void ref_update_cov(unsigned int i_sample, unsigned int n_node, float *cov, float *means,
                    const float *data) {
    one_block(1);
    threadIdx.x = 0;
    update_cov(i_sample, n_node, cov, means, data);
}

void ref_cov_to_corr(unsigned int n_sample, unsigned int n_node, float *cov, float *corr) {
    one_block(1);
    threadIdx.x = 0;
    cov_to_corr(n_sample, n_node, cov, corr);
}
