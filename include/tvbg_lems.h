/*
 * C ABI of the libraries generated from LEMS XML models (tvb_hpc.lems).
 *
 * One shared library per model.  Each replaces what the reference emits
 * for that model: dsl/dsl_cuda/LEMS2CUDA.py:37-86 (render_model,
 * cuda_templating) renders the XML through dsl/dsl_cuda/tmpl8_CUDA.py into
 * __global__ void <Model>(i_step, n_node, nh, n_step, n_params, dt, speed,
 * weights, lengths, params, state, tavg) (tmpl8_CUDA.py:42-60), launched by
 * dsl/dsl_cuda/example/cuda_run.py:67-142.  Here the model becomes the
 * device functors of the engine's per-step kernel, driven by the same
 * tvbg_instance / tvbg_launch descriptors as tvbg_sweep (include/tvbg.h),
 * with model = TVBG_MODEL_LEMS and cfun = TVBG_CFUN_LEMS.
 *
 * Per work item, the slots are the swept parameters (the model's
 * <Parameter> elements, in file order) followed by its derived parameters
 * (<DerivedParameter>, in file order): at most TVBG_LEMS_MAX_K floats.  The
 * per-step kernel reads them from tvbg_instance.consts (the coupling) and
 * from the per-node parameter array nparam ([N][NP], replicated over
 * nodes, NP = max(1, slots); the model).
 * Noise ("noise" component "on") takes sigma[v] = nsig / sqrt(dt); models
 * with 5..8 state variables take sigma[0] for every variable.
 *
 * Every entry point returns TVBG_OK (0) or a negative TVBG_E* code with a
 * message in tvbg_lems_last_error() (thread-local, per library).
 */
#ifndef TVBG_LEMS_H
#define TVBG_LEMS_H

#include "tvbg.h"

#ifdef __cplusplus
extern "C" {
#endif

#define TVBG_LEMS_MAX_K 16

/* info[] fields of tvbg_lems_info */
enum {
    TVBG_LEMS_INFO_NS = 0,           /* state variables (1..8)                   */
    TVBG_LEMS_INFO_NPARAMS = 1,      /* swept parameters per work item           */
    TVBG_LEMS_INFO_NDERIVED = 2,     /* derived parameters                       */
    TVBG_LEMS_INFO_NEXPO = 3,        /* exposures (observables)                  */
    TVBG_LEMS_INFO_CVAR = 4,         /* coupled state variable (ring observable) */
    TVBG_LEMS_INFO_NOISE = 5,        /* 1 when the noise component is "on"       */
    TVBG_LEMS_INFO_REC_SPEED_DT = 6, /* consts index of rec_speed_dt, -1 = none  */
    TVBG_LEMS_INFO_NSIG = 7,         /* consts index of nsig, -1 = none          */
    TVBG_LEMS_INFO_ABI = 8,          /* 1                                        */
    TVBG_LEMS_INFO_GROUP = 9,        /* group kernel coupling: 1 = separable     */
                                     /* (TVBG_CFUN_LEMS), 2 = sine difference    */
                                     /* (TVBG_CFUN_LEMS_SC), 0 = per-step only   */
    TVBG_LEMS_INFO_LEN = 10
};

int tvbg_lems_info(int32_t *info);

/* Host evaluation of the per-work-item slots: out[b][0..15] = swept
 * parameters params[b][0..n_params) then the derived parameters, evaluated
 * with the reference's C types (dt float, n_node unsigned int; the template
 * declares them in tmpl8_CUDA.py:47-50,95-100).  Unused slots are zero. */
int tvbg_lems_derived(const float *params, int32_t n_work, int32_t n_params, float dt,
                      int32_t n_node, float *out);

/* One CTA per work item (tvbg_sweep) or persistent CTAs (tvbg_batch_run);
 * block_k must be 0 or 1 (the per-step kernel). */
int tvbg_lems_sweep(const tvbg_instance *d_inst, int32_t n_inst, const tvbg_launch *cfg,
                    void *stream);
int tvbg_lems_batch_run(const tvbg_instance *d_inst, int32_t n_inst, const tvbg_launch *cfg,
                        void *stream);

/* Lane-interleaved groups of eight work items sharing a delay table
 * (tvbg_group_run's records, model = TVBG_MODEL_LEMS and cfun as
 * TVBG_LEMS_INFO_GROUP says).  The per-work-item slots travel in
 * tvbg_group.nparam ([N][NP][8], replicated over nodes); sigma[0..3] =
 * nsig / sqrt(dt) shared by the group.  TVBG_EUNSUPPORTED when the coupling
 * needs the per-step kernel. */
int tvbg_lems_group_run(const tvbg_group *d_groups, int32_t n_groups, const tvbg_launch *cfg,
                        void *stream);

/* The value a separable coupling's ring slot holds for observable o, per
 * work item (slots [n][16] as from tvbg_lems_derived): fills the history
 * before t0 (o = 0) on the host. */
int tvbg_lems_ring_value(const float *slots, int32_t n, float o, float *out);

/* Exposures of n node states: d_state [n][ns] -> d_out [n][nexpo]
 * (tmpl8_CUDA.py:244-249 writes them after the last step of a launch). */
int tvbg_lems_expose(const float *d_state, int64_t n, float *d_out, void *stream);

const char *tvbg_lems_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* TVBG_LEMS_H */
