/*
 * tvbg.h -- C ABI of the GB300 brain-network step engine.
 *
 * The engine runs the per-instance network time step of tvb-hpc: each node
 * gathers delayed neighbour observables from a circular history ring, applies
 * the coupling function and the neural-mass drift, takes an Euler or
 * Euler-Maruyama step with counter-based Philox noise, and optionally feeds a
 * Balloon-Windkessel BOLD monitor.  A Pearson functional-connectivity (FC)
 * kernel and a Philox normal generator complete the path.
 *
 * Conventions shared by every entry point:
 *   - return 0 on success, a negative TVBG_E* code on failure; the message of
 *     the last failure on the calling thread is returned by tvbg_last_error();
 *   - pointers named d_* are device pointers owned by the caller; no entry
 *     point allocates device memory (scratch words such as queue counters and
 *     status words are caller-provided);
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default);
 *     every call is asynchronous with respect to the host unless stated.
 *
 * Reference interfaces replaced (paths inside the tvb-hpc project):
 *   tvbg_sweep         <- the fused loopy kernel of
 *                         tvb_hpc/transforms.py:23-49 (network_time_step,
 *                         called as knl(nstep, nnode, ntime, state, ...),
 *                         tvb_hpc/examples/hackathon.py:48-54) and the CUDA
 *                         DSL step kernel
 *                         dsl/dsl_cuda/CUDAmodels/kuramoto.c:29-146 launched
 *                         by dsl/dsl_cuda/example/cuda_run.py:124-142
 *   tvbg_batch_run     <- the OpenMP subject batch of examples/hcp100.py:65-118
 *                         (lp.to_batched over i_subj), as one persistent launch
 *   tvbg_fc            <- tvb_hpc/metric.py:18-139 (Covar, CovToCorr) and
 *                         dsl/dsl_cuda/CUDAmodels/refs/covar.c:9-109
 *   tvbg_philox_normal <- tvb_hpc/rng.py:30-96 (RNG.fill, tvb_rng)
 *   tvbg_pack_edges    <- tvb_hpc/network.py:66-78 (Connectivity.from_dense)
 *                         plus the delay rule of hackathon.py:44 / kuramoto.c:105
 */
#ifndef TVBG_H
#define TVBG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TVBG_ABI_VERSION 1

/* ---- status codes ------------------------------------------------------ */
#define TVBG_OK 0
#define TVBG_EINVAL (-1)       /* bad argument (size, pointer, combination) */
#define TVBG_ECUDA (-2)        /* a CUDA runtime call failed */
#define TVBG_ETIMEOUT (-3)     /* a bounded device wait gave up */
#define TVBG_EUNSUPPORTED (-4) /* model / coupling pair not built */
#define TVBG_EDEVICE (-5)      /* device-side check failed (status word) */

/* ---- neural-mass models (tvb_hpc/model.py) ------------------------------ */
#define TVBG_MODEL_KURAMOTO 0 /* model.py:169-182  state theta, param omega  */
#define TVBG_MODEL_G2DO 1     /* model.py:262-276  state W V, param a        */
#define TVBG_MODEL_MPR 2      /* Montbrio-Pazo-Roxin 2015, state r V, param eta */
#define TVBG_MODEL_LINEAR 3   /* model.py:250-259  state x, param lam        */
#define TVBG_MODEL_G2DOSC 4   /* generic 2-D oscillator in the form of the CUDA
                                 DSL (dsl/dsl_cuda/CUDAmodels/oscillator.c:149-150):
                                 state V W, cubic in V, coupling into V */
#define TVBG_MODEL_RWW 5      /* model.py:209-223 reduced Wong-Wang, state S,
                                 params w io */
#define TVBG_MODEL_JANSENRIT 6 /* model.py:226-247 Jansen-Rit, state y0..y5,
                                 params v0 r, observable y0 - y1; no noise
                                 (more than 4 state variables) */
#define TVBG_MODEL_LEMS 64    /* a model generated from LEMS XML
                                 (dsl/dsl_cuda/LEMS2CUDA.py); only the
                                 libraries of include/tvbg_lems.h run it */

/* ---- coupling functions (tvb_hpc/coupling.py) --------------------------- */
#define TVBG_CFUN_LINEAR 0    /* pre = x_j,                  post = a*sum + b */
#define TVBG_CFUN_DIFF 1      /* pre = x_j - x_i,            post = a*sum + b */
#define TVBG_CFUN_KURAMOTO 2  /* pre = sin(x_j - x_i),       post = a*mean    */
#define TVBG_CFUN_SIGMOIDAL 3 /* pre = cmax/(1+exp(r(mid-x_j))), post = a*sum */
#define TVBG_CFUN_LEMS 64     /* the coupling of a LEMS model: pre(x_j, x_i)
                                 from its XML, sum passed to the model raw
                                 (group kernel: pre(x_j) applied when the
                                 ring slot is written) */
#define TVBG_CFUN_LEMS_SC 65  /* a LEMS coupling post * sin(x_j - x_i) on the
                                 group kernel: sin and cos ring channels */
#define TVBG_CFUN_LEMS_2 66   /* two separable LEMS couplings (two coupled
                                 inputs) on the group kernel: one ring
                                 channel each */

/* ---- per-instance flags ------------------------------------------------- */
#define TVBG_F_NOISE 1u      /* Euler-Maruyama with Philox normals          */
#define TVBG_F_BOLD 2u       /* integrate the Balloon-Windkessel monitor    */
#define TVBG_F_TRACE 4u      /* write observables every trace_every steps   */
#define TVBG_F_WRAP_FMOD 8u  /* Kuramoto wrap by fmod (CUDA DSL) not shift  */
#define TVBG_F_SMEM_RING 16u /* ring staged in shared memory (planner sets)  */
#define TVBG_F_NO_WRAP 32u   /* disable the model's limit/wrap rule          */
/* Track-A step order (tvb_hpc/transforms.py:30-42, fused loopy kernel): the
 * gather of step t reads ring slot t before the model writes obs(x_t) into
 * it, so post and zero-delay reads see the slot's old content. */
#define TVBG_F_TRACKA 64u
#define TVBG_F_MIDSYNC 128u  /* block barrier between gather and update      */
/* the trace carries one more column per node: the raw coupling sum S of the
 * step (written during the step; used by the adjoint's recomputation) */
#define TVBG_F_TRACE_CSUM 256u
/* time-blocked kernel, warp-specialised: owner warps update block i while
 * the other warps gather block i+1 and integrate the balloon of block i-1
 * (needs block_k <= (d_min + 1) / 2 and more warps than ceil(N/32)) */
#define TVBG_F_PIPELINE 512u

/*
 * Packed connectivity edge, one per CSR non-zero, rows = target node i:
 *   pk = (col << lognh) | ((col - delay) & (nh - 1)),  w = weight bits.
 * The ring of an instance is node-major and skewed:
 *   value of node j at time slot s lives at  j*nh + ((s + j) & (nh-1)),
 * so the delayed read of edge e at slot tm is
 *   ((tm + pk) & (nh-1)) | (pk & ~(nh-1)).
 * nh = 1 << lognh must exceed max(delay) + sync_every.
 */
typedef struct tvbg_edge {
    uint32_t pk;
    float w;
} tvbg_edge;

/*
 * One simulation instance (one parameter point of a sweep).  An array of
 * these lives in device memory; tvbg_instance_size() must equal
 * sizeof(tvbg_instance) on both sides of the FFI.
 */
typedef struct tvbg_instance {
    const tvbg_edge *edges;  /* [nnz] packed edges for this instance's delays */
    const int32_t *row;      /* [N+1] CSR row offsets (in-edges of node i)   */
    float *ring;             /* [N << lognh] history ring backing store      */
    float *state;            /* [N][nsvar] state at t0, updated in place      */
    const float *nparam;     /* [N][npar] per-node model parameter            */
    float *bold;             /* [4][N] balloon s, f-1, v-1, q-1 (rest = 0)    */
    float *bold_out;         /* [bold_len][N] BOLD samples                    */
    float *trace;            /* trace rows, see trace_* (TVBG_F_TRACE)        */
    int64_t t0;              /* absolute step index of the first step         */
    int64_t trace_stride;    /* floats between consecutive trace rows          */
    int32_t nsteps;          /* steps to take in this launch                  */
    int32_t N;               /* nodes (<= 1024)                               */
    int32_t nnz;             /* edges                                         */
    int32_t lognh;           /* ring length nh = 1 << lognh                   */
    int32_t model;           /* TVBG_MODEL_* (must equal the launch's)        */
    int32_t cfun;            /* TVBG_CFUN_* (must equal the launch's)         */
    uint32_t flags;          /* TVBG_F_*                                      */
    int32_t sync_every;      /* steps between block barriers (1..d_min+1)     */
    int32_t trace_every;     /* sample trace when t % trace_every == 0        */
    int32_t trace_len;       /* trace row = (t / trace_every) % trace_len     */
    int32_t trace_nobs;      /* observables per node written to the trace     */
    int32_t bold_period;     /* BOLD sample when (t + 1) % bold_period == 0   */
    int32_t bold_len;        /* rows available in bold_out                    */
    int32_t bold_obs;        /* observable index feeding the BOLD monitor     */
    uint32_t seed_lo;        /* Philox key word 0                             */
    uint32_t seed_hi;        /* Philox counter word 2                         */
    uint32_t inst_id;        /* Philox key word 1 (request-local instance id) */
    int32_t reserved0;
    float dt;                /* integration step (ms)                         */
    float sqrt_dt;           /* sqrtf(dt)                                     */
    float dt_bold;           /* balloon step (s) = dt / 1000                  */
    float cf_a;              /* coupling a (global coupling G)                */
    float cf_b;              /* coupling b                                    */
    float cf_p[3];           /* sigmoidal: cmax, midpoint, r                  */
    float sigma[4];          /* noise amplitude per state variable            */
    float consts[16];        /* model constants, order fixed per model        */
} tvbg_instance;

/* Launch-wide configuration. */
typedef struct tvbg_launch {
    int32_t model;         /* TVBG_MODEL_* shared by every instance of the call */
    int32_t cfun;          /* TVBG_CFUN_* shared by every instance of the call  */
    int32_t threads;       /* CTA size, multiple of 32, >= max N rounded up     */
    int32_t tpn;           /* lanes per node in the gather: 1, 2, 4 or 8        */
    int32_t smem_ring;     /* shared-memory bytes reserved for the ring (0 ok)  */
    int32_t ctas;          /* persistent CTAs (tvbg_batch_run); 0 = 1 per SM    */
    int32_t block_k;       /* 0 or 1: per-step kernel; 4 or 8: time-blocked     */
                           /* kernel (K steps per block, padded ring layout)    */
    int32_t nmax;          /* largest N of the call (blocked kernel); 0 = threads */
    int32_t cluster;       /* tvbg_group_run: CTAs per group (1..16; 0 = 1; 9..16 */
                           /* are non-portable cluster sizes)                   */
    int32_t priority;      /* tvbg_group_run: launch priority (0 = the stream's; */
                           /* lower numbers are higher priority, as CUDA streams) */
    int32_t *d_status;     /* optional device int: first device error code      */
    int32_t *d_counter;    /* tvbg_batch_run work counter (zeroed by the call)  */
    const int32_t *d_order;/* tvbg_batch_run instance order (cost-descending)   */
} tvbg_launch;

/* ---- entry points ------------------------------------------------------ */

/* ABI version (TVBG_ABI_VERSION) and struct sizes, for FFI checks. */
int tvbg_abi_version(void);
size_t tvbg_instance_size(void);
size_t tvbg_launch_size(void);

/* Message for the last failing call on this thread ("" if none). */
const char *tvbg_last_error(void);

/* Largest dynamic shared memory a CTA may use on the current device. */
int tvbg_max_smem(int32_t *bytes);

/*
 * Resident CTAs per SM of the step kernel a launch with `cfg` would use
 * (cudaOccupancyMaxActiveBlocksPerMultiprocessor), and the SM count; used by
 * the batch planner to size persistent grids.
 */
int tvbg_occupancy(const tvbg_launch *cfg, int32_t *ctas_per_sm, int32_t *sms);

/*
 * Host helper: pack CSR connectivity and integer delays into tvbg_edge.
 * row[N+1], col[nnz] (int32), weights[nnz] (float), delays[nnz] (int32 >= 0).
 * Fails if a delay >= nh or N << lognh overflows 32 bits.
 * Replaces the CSR build of tvb_hpc/network.py:66-78 for the kernel layout.
 */
int tvbg_pack_edges(int32_t N, int32_t nnz, const int32_t *row,
                    const int32_t *col, const float *weights,
                    const int32_t *delays, int32_t lognh, tvbg_edge *out);

/*
 * Host helper for the time-blocked kernel (tvbg_launch.block_k = 4 or 8),
 * whose ring rows carry 8 ghost slots: node j, slot s lives at
 * j*(nh+8) + ((s + j) & (nh-1)), and positions < 8 are mirrored at +nh.
 * pk = (col << 16) | ((col - delay) & (nh - 1)); needs N, nh <= 65536.
 */
int tvbg_pack_edges_blocked(int32_t N, int32_t nnz, const int32_t *row,
                            const int32_t *col, const float *weights,
                            const int32_t *delays, int32_t lognh,
                            tvbg_edge *out);

/*
 * Host helper: integer delays d = op(f32(f32(len / speed) / dt)),
 * op = ceil (rounding = 1) or trunc (rounding = 0): the float32 arithmetic of
 * tvb_hpc/examples/hackathon.py:44 under numpy 1.15 casting.  rounding = 2
 * uses the CUDA DSL rule trunc(len * f32(f32(1/speed)/dt)) of
 * dsl/dsl_cuda/CUDAmodels/kuramoto.c:65,105.
 */
int tvbg_delays(int32_t nnz, const float *lengths, float speed, float dt,
                int32_t rounding, int32_t *out);

/*
 * Run every instance of d_inst[0..n_inst) for its nsteps, one CTA per
 * instance, all instances sharing the (model, cfun) pair of cfg.  This is the plain
 * one-sweep-per-launch path (the fused network step of
 * tvb_hpc/transforms.py:23-49 batched over instances).
 */
int tvbg_sweep(const tvbg_instance *d_inst, int32_t n_inst,
               const tvbg_launch *cfg, void *stream);

/*
 * With cfg->block_k = 4 or 8, tvbg_sweep and tvbg_batch_run use the
 * time-blocked kernel: CUDA step order, couplings whose pre-summation term
 * depends on the source only (LINEAR, DIFF, SIGMOIDAL), every delay >=
 * block_k - 1, rings in the padded layout of tvbg_pack_edges_blocked.  It
 * computes the same step (same Philox stream) as the per-step kernel.
 */

/*
 * Persistent batched run: cfg->ctas CTAs pull instances (in d_order order)
 * from the device counter cfg->d_counter until all n_inst are done.
 * Instances may differ in N, nnz, ring length and nsteps; they share the
 * (model, cfun) pair of cfg.  The counter is reset on `stream` before the
 * launch, so the call may be captured into a CUDA graph.
 */
int tvbg_batch_run(const tvbg_instance *d_inst, int32_t n_inst,
                   const tvbg_launch *cfg, void *stream);

/*
 * Reverse-time adjoint of the delayed Euler scheme for one segment of steps
 * [t0, t0 + len), Montbrio-Pazo-Roxin with linear coupling, CUDA step order,
 * deterministic.  With mu(t+1) = lambda(t+1) (r component masked where the
 * rate was clamped):
 *   lambda(t)     = mu + dt J(x(t))^T mu + dL/dr(t) e_r
 *   lambda_r,j(t) += dt G / tau * sum_{edges i <- j, delay d} w mu_V,i(t + d + 1)
 *   deta_j += dt / tau * mu_V,j(t+1);   dG_j += dt / tau * mu_V,j(t+1) S_j(t)
 * (FP64 accumulators).  mu_V is kept in an adjoint ring (skewed node-major
 * layout of tvbg.h, zero before the last segment) gathered over the
 * transposed CSR, pk = (i << lognh) | ((i + d + 1) & (nh - 1)).
 * No counterpart kernel exists in the reference (tvb_hpc builds symbolic
 * partials only, model.py:61-65, scheme.py:42-48).
 */
typedef struct tvbg_adjoint {
    const tvbg_edge *edges_t; /* [nnz] transposed edges (out-edges of node j) */
    const int32_t *row_t;     /* [N+1] out-edge offsets                       */
    const float *seg;         /* [len][N][3]: r, V, S at the start of each step, */
                              /* element stride seg_lanes                      */
    const float *dr;          /* [len][N]: direct dL/dr(t), row t - t0        */
    float *lam;               /* [N][2]: lambda(t0 + len) in, lambda(t0) out  */
    float *ring;              /* [N << lognh] adjoint ring of mu_V            */
    double *deta;             /* [N] accumulated dL/deta                      */
    double *dG;               /* [N] accumulated per-node part of dL/dG       */
    int64_t t0;
    int32_t len, N, lognh;
    int32_t seg_lanes;        /* 0 or 1: seg per instance; 8: seg points at one */
                              /* lane of a lane-interleaved group trace        */
                              /* [len][N][3][8] (TVBG_F_TRACE_CSUM)            */
    float dt, G;
    float consts[4];          /* MPR: Delta, J, tau, I                        */
} tvbg_adjoint;

int tvbg_adjoint_mpr(const tvbg_adjoint *d_adj, int32_t n_inst, int32_t threads,
                     void *stream);
/* The same with the adjoint ring staged in smem_ring bytes of shared memory
 * per CTA (loaded at the start, stored at the end of the call); an instance
 * whose ring (N << lognh floats) does not fit uses its global ring. */
int tvbg_adjoint_mpr_ex(const tvbg_adjoint *d_adj, int32_t n_inst, int32_t threads,
                        int32_t smem_ring, void *stream);

/*
 * The same recursion for lane-interleaved groups of up to 8 instances that
 * share the connectome and delays (one group per CTA or cluster of CTAs,
 * thread = node slot x lane, lane l = instance 8 g + l), time-blocked:
 * with every delay >= block_k, the block_k reverse steps of a block read
 * only adjoint-ring slots written by earlier blocks, so the CTAs meet at
 * one barrier per block.  Each thread sums its node's out-edges for the
 * block's steps with 32-byte loads that carry 8 instances (lane l loads
 * step l of the block), in out-edge order, as tvbg_adjoint_mpr does: the
 * results are the same as tvbg_adjoint_mpr's on the same segment.
 * Adjoint ring: [N][R][8] floats, R = nh + block_k, nh = 1 << lognh >=
 * d_max + block_k; slot s of node i at (i R + (s & (nh-1))) 8 + lane,
 * slots < block_k mirrored at + nh; zero before the last segment.
 * Out-edges packed as in tvbg_group: pk = (i << 16) | d.
 */
typedef struct tvbg_adjoint_group {
    const tvbg_edge *edges_t; /* [nnz] out-edges of node j, pk = (i << 16) | d */
    const int32_t *row_t;     /* [N+1] out-edge offsets                       */
    const int32_t *nodes;     /* [N] node of each slot position, or NULL      */
    const float *seg;         /* [len][N][3][8]: r, V, S of the group's lanes  */
                              /* (a group trace with TVBG_F_TRACE_CSUM)       */
    const float *dr;          /* lane l: dr + l dr_stride, [len][N] rows t - t0 */
    float *lam;               /* lane l: lam + 2 N l, [N][2]                  */
    float *ring;              /* [N][R][8] adjoint ring of mu_V (16-byte aligned) */
    double *deta;             /* lane l: deta + N l, [N]                      */
    double *dG;               /* lane l: dG + N l, [N]                        */
    int64_t t0;
    int64_t dr_stride;        /* floats between the dr rows of two lanes       */
    int32_t len, N, lognh;
    int32_t lanes;            /* live lanes (1..8); others compute, write nothing */
    int32_t dmin;             /* smallest delay (>= block_k, checked)         */
    int32_t flush_every;      /* > 0: deta and dG partial sums added after each */
                              /* step t with t % flush_every == 0 (the grouping */
                              /* of one launch per segment of that length); 0: */
                              /* once, at the end of the launch                */
    float dt;
    float G[8];               /* coupling of each lane                        */
    float consts[4];          /* MPR: Delta, J, tau, I                        */
} tvbg_adjoint_group;

size_t tvbg_adjoint_group_size(void);
/* n_groups records; threads = 8 x node slots per CTA (a multiple of 32, <= 512),
 * cluster CTAs per group (1..16, N <= cluster x threads / 8), block_k 4 or
 * 8.  pipelined = 1: two thread teams per CTA (threads = 2 x 8 x node slots,
 * a multiple of 64; N <= cluster x threads / 16), the out-edge sums of block
 * b + 1 gathered while block b's steps run; needs every delay >= 2 block_k;
 * the same results.  A record that does not match the launch sets *d_status
 * (optional) to TVBG_EINVAL and its group does nothing. */
int tvbg_adjoint_mpr_groups(const tvbg_adjoint_group *d_adj, int32_t n_groups,
                            int32_t threads, int32_t cluster, int32_t block_k,
                            int32_t pipelined, int32_t *d_status, void *stream);

/*
 * Pearson FC per instance over T samples of N nodes, FP64 reduction.
 * d_x: float [n_inst][T][N] (inst_stride floats between instances).
 * d_fc: float [n_inst][N][N].  If d_target ([N][N]) and d_err ([n_inst])
 * are given, d_err[b] = sum_{i<j} (fc_ij - target_ij)^2 in FP64.
 * Replaces tvb_hpc/metric.py:18-139 and refs/covar.c:9-109.
 */
int tvbg_fc(const float *d_x, int32_t n_inst, int32_t T, int32_t N,
            int64_t inst_stride, float *d_fc, const float *d_target,
            double *d_err, void *stream);

/*
 * tvbg_fc with caller scratch: N > 126 needs d_scratch of
 * tvbg_fc_scratch_bytes(n_inst, N) bytes (FP64 means and Gram); smaller N
 * needs none (d_scratch may be NULL).
 */
int tvbg_fc_scratch_bytes(int32_t n_inst, int32_t N, int64_t *bytes);
int tvbg_fc_ex(const float *d_x, int32_t n_inst, int32_t T, int32_t N,
               int64_t inst_stride, float *d_fc, const float *d_target,
               double *d_err, double *d_scratch, void *stream);

/*
 * Allocation-free variant of tvbg_fc_ex, for callers that cannot call
 * cudaMalloc: code whose device memory is owned by a host framework's pool
 * or budget (a serving runtime, a plugin inside another runtime) and loops
 * that may not take cudaMalloc's implicit device synchronisation.  It has no
 * counterpart in the reference.
 *
 * The FP64 scratch of the N > 126 path lives in a file-scope device array of
 * TVBG_FC_NOALLOC_MAX_DOUBLES doubles (8 MiB), which every GPU that loads the
 * library holds until the process exits; a call needs n_inst * N * (N + 1)
 * doubles and is rejected with TVBG_EINVAL beyond that.  The first call on a
 * device looks up the array's device address (cudaGetSymbolAddress) with
 * that device current; make that first call before any stream capture.  All
 * calls share the one array: every scratch entry a call reads it has written
 * first, but calls that overlap on the GPU (different streams, no ordering)
 * race on it and must be serialised by the caller.  The looked-up address is
 * kept per device for the life of the process; cudaDeviceReset unloads the
 * library's device code and invalidates it, so do not call this entry point
 * on a device after a cudaDeviceReset in the same process.
 */
#define TVBG_FC_NOALLOC_MAX_DOUBLES 1048576
int tvbg_fc_noalloc(const float *d_x, int32_t n_inst, int32_t T, int32_t N,
                    int64_t inst_stride, float *d_fc, const float *d_target,
                    double *d_err, void *stream);

/*
 * ---- one very large network ----------------------------------------------
 * A single instance with up to millions of nodes (the case of
 * tvb_hpc/examples/sim515k.py: one network of 515 056 nodes), node-parallel:
 * one thread per node, node-major ring [N][nh + 8] (slot s of node j at
 * j*(nh+8) + (s & (nh-1)), positions < 8 mirrored at +nh), one launch per
 * block of block_k (4 or 8) steps.  Needs every delay >= block_k - 1 and
 * nh >= max(delay) + 1 + block_k; couplings LINEAR, DIFF, SIGMOIDAL; models
 * G2DO, G2DOSC, MPR, LINEAR.  Same step (CUDA order) and Philox stream as
 * instance 0 of tvbg_sweep.  The descriptor is host memory (it is passed to
 * the kernels by value).
 */
typedef struct tvbg_net {
    const int32_t *row;     /* [N+1] CSR offsets (in-edges of node i)          */
    const int32_t *col;     /* [nnz] source node of each edge                  */
    const float *w;         /* [nnz] weight                                    */
    const uint16_t *off;    /* [nnz] (nh - delay) & (nh - 1)                   */
    const float *wsum;      /* [N] sum of in-edge weights (DIFF), else NULL    */
    float *ring;            /* [N][nh + 8]                                     */
    float *state;           /* [N][nsvar], updated in place                    */
    const float *nparam;    /* [N][npar]                                       */
    int64_t N;
    int32_t lognh;          /* 3..16                                           */
    int32_t model;
    int32_t cfun;
    uint32_t flags;         /* NOISE, NO_WRAP                                  */
    uint32_t seed_lo;
    uint32_t seed_hi;
    float dt;
    float sqrt_dt;
    float cf_a;
    float cf_b;
    float cf_p[3];
    float reserved0;
    float sigma[4];
    float consts[16];
} tvbg_net;

size_t tvbg_net_size(void);

/* Advance the network from step t0 by nsteps: one seed launch (slot t0
 * holds obs0 of the state) and ceil(nsteps / cfg->block_k) step launches of
 * cfg->threads threads per CTA on `stream`.  cfg->tpn selects the thread
 * mapping: 0 or 1 = one thread per node, block_k = block_k lanes per node
 * (lane k gathers step k); both give bit-identical results.
 * Graph-capturable. */
int tvbg_net_run(const tvbg_net *net, int64_t t0, int32_t nsteps,
                 const tvbg_launch *cfg, void *stream);

/*
 * Streaming covariance for long runs: fold one sample per instance into an
 * FP64 running state (Welford update).  d_x: sample of instance b at
 * d_x + b * x_stride (N floats); n: samples already folded (0 starts a new
 * state -- the state arrays need no clearing); d_mean: double [n_inst][N];
 * d_m2: double [n_inst][N][N], the co-moment
 * sum_s (x_si - mean_i)(x_sj - mean_j) over the samples folded so far.
 * N <= 3000.  Replaces tvb_hpc/metric.py:87-108 (OnlineCov) and
 * dsl/dsl_cuda/CUDAmodels/refs/covar.c:9-68 (update_cov).
 */
int tvbg_cov_update(const float *d_x, int64_t x_stride, int32_t n_inst,
                    int32_t N, int64_t n, double *d_mean, double *d_m2,
                    void *stream);

/* Pearson correlation of a streaming state: corr_ij = m2_ij / sqrt(m2_ii
 * m2_jj), float [n_inst][N][N].  Replaces refs/covar.c:73-109 (cov_to_corr). */
int tvbg_cov_corr(const double *d_m2, int32_t n_inst, int32_t N, float *d_corr,
                  void *stream);

/*
 * Fill d_out[0..n) with standard normals from Philox4x32-10 (Salmon et al.
 * 2011) + Box-Muller: key = (seed_lo, stream_id), counter = (i/4, 0,
 * seed_hi, 0) for output i.  Replaces tvb_hpc/rng.py:30-96 (RNG.fill).
 */
int tvbg_philox_normal(uint64_t seed, uint32_t stream_id, float *d_out,
                       int64_t n, void *stream);

/* Raw Philox4x32-10 words: d_out[4*i + k] = philox(ctr=(i, c1, c2, c3), key)[k]. */
int tvbg_philox_u32(uint32_t k0, uint32_t k1, uint32_t c1, uint32_t c2,
                    uint32_t c3, uint32_t *d_out, int64_t n_blocks,
                    void *stream);

/*
 * ---- lane-interleaved groups --------------------------------------------
 * TVBG_GROUP_LANES instances that share a connectome, a delay table, the
 * model constants, the coupling b and t0 run as one group: one instance per
 * lane of an 8-lane slice, every per-node array interleaved over the 8
 * instances, so one delayed read of an edge is one 32-byte sector for the
 * group and the edge record is read once for 8 instances.  Same step (CUDA
 * order) and Philox streams as tvbg_sweep; couplings LINEAR, DIFF and
 * SIGMOIDAL, and KURAMOTO with the Kuramoto model; block_k (4 or 8) steps
 * per barrier, which needs every delay
 * >= block_k - 1 and nh >= max(delay) + 1 + block_k.
 * Layouts (L = 8, R = nh + 8, l = lane):
 *   ring     [N][R][L]  slot s of node j at (j*R + (s & (nh-1)))*L + l;
 *                       positions < 8 are mirrored at +nh; with the
 *                       KURAMOTO coupling (Kuramoto model) [N][R][2][L]:
 *                       sin and cos of the observable, zero history (0, 1)
 *   state    [N][nsvar][L]      nparam  [N][npar][L]
 *   bold     [4][N][L]          bold_out [bold_len][N][L]
 *   trace    [trace_len][N][trace_nobs][L]; with TVBG_F_TRACE_CSUM (the
 *            pipelined kernel, one-channel couplings) [trace_len][N]
 *            [trace_nobs + 1][L], the last column the raw coupling sum
 * A lane with nsteps = 0 is padding (its state and ring are not updated).
 * This layout has no counterpart in tvb-hpc; it serves the sweeps of
 * tvb_hpc/examples/hackathon.py:58-89 (a coupling x speed grid, one delay
 * table per speed) and dsl/dsl_cuda/example/cuda_run.py:110-142 (one
 * thread per parameter point).
 */
#define TVBG_GROUP_LANES 8

typedef struct tvbg_lane {
    float cf_a;          /* coupling a (global coupling G) of this instance */
    int32_t nsteps;      /* steps this instance takes, <= the group's nsteps */
    uint32_t inst_id;    /* Philox key word 1 */
    int32_t reserved0;
} tvbg_lane;

typedef struct tvbg_group {
    const tvbg_edge *edges;  /* [nnz] pk = (col << 16) | ((nh - d) & (nh-1)) */
    const int32_t *row;      /* [N+1] CSR row offsets (in-edges of node i)    */
    const float *wsum;       /* [N] sum of in-edge weights (DIFF), else NULL   */
    const int32_t *nodes;    /* [N] node visiting order, NULL = 0..N-1         */
    float *ring;             /* [N][nh + 8][8]                                */
    float *state;            /* [N][nsvar][8]                                 */
    const float *nparam;     /* [N][npar][8]                                  */
    float *bold;             /* [4][N][8] balloon deviations, or NULL         */
    float *bold_out;         /* [bold_len][N][8]                              */
    float *trace;            /* [trace_len][N][trace_nobs][8], or NULL        */
    int64_t t0;              /* absolute step index of the first step         */
    int32_t nsteps;          /* steps of the longest lane                     */
    int32_t N;               /* nodes (< 65536)                               */
    int32_t nnz;
    int32_t lognh;           /* 3..16                                         */
    int32_t model;
    int32_t cfun;
    uint32_t flags;          /* NOISE, BOLD, TRACE, NO_WRAP, WRAP_FMOD         */
    int32_t trace_every;
    int32_t trace_len;
    int32_t trace_nobs;
    int32_t bold_period;
    int32_t bold_len;
    int32_t bold_obs;
    uint32_t seed_lo;
    uint32_t seed_hi;
    int32_t dmin;            /* smallest delay of the group's table; read by  */
                             /* the pipelined kernel (TVBG_GROUP_PIPELINED),   */
                             /* which needs dmin >= 2 block_k - 1             */
    float dt;
    float sqrt_dt;
    float dt_bold;
    float cf_b;
    float cf_p[3];
    float reserved1;
    float sigma[4];
    float consts[16];
    tvbg_lane lanes[TVBG_GROUP_LANES];
} tvbg_group;

size_t tvbg_group_size(void);

/*
 * Host helper for tvbg_group_run: pk = (col << 16) | ((nh - delay) & (nh-1)).
 * Needs N <= 65536, lognh <= 16 and every delay < nh.
 */
int tvbg_pack_edges_group(int32_t N, int32_t nnz, const int32_t *row,
                          const int32_t *col, const float *weights,
                          const int32_t *delays, int32_t lognh,
                          tvbg_edge *out);

/*
 * Run the groups d_groups[0..n_groups): cfg->cluster CTAs of cfg->threads
 * threads per group (a thread-block cluster when > 1; up to 16, sizes above
 * 8 opt in to non-portable clusters), group of cluster c = d_order[c] (or
 * c).  cfg->block_k = 4 or 8; cfg->priority, when non-zero, is the launch's
 * scheduling priority (lower = earlier CTA dispatch, clamped to the
 * device's range); smem_ring, ctas, nmax and d_counter are not used.
 * cfg->tpn = threads per (node, instance): 0 or 1, or TVBG_GROUP_PIPELINED
 * (2): the pipelined kernel, whose CTA is two teams of threads / 2 (a
 * multiple of 64 threads) on the same (node, instance) pairs -- one sums the
 * coupling of block b + 1 while the other runs the K steps of block b.  It
 * needs every group's dmin >= 2 block_k - 1, one node per 8-lane slot
 * (cluster * threads / 16 >= N) and 16-byte aligned rings, else the device
 * status reports TVBG_EINVAL; its gather is transposed (lane l of a node
 * slot loads ring position t + l for the 8 instances, one 32-byte run, and
 * the sums cross lanes through shared memory); results are identical to
 * the plain kernel's.
 * Graph-capturable.
 */
#define TVBG_GROUP_PIPELINED 2
int tvbg_group_run(const tvbg_group *d_groups, int32_t n_groups,
                   const tvbg_launch *cfg, void *stream);

/* Resident CTAs per SM of the group kernel of `cfg`, and the SM count. */
int tvbg_group_occupancy(const tvbg_launch *cfg, int32_t *ctas_per_sm,
                         int32_t *sms);

/*
 * Clusters of cfg->cluster CTAs of the group kernel of `cfg` that can be
 * resident at once (cudaOccupancyMaxActiveClusters); 0 when the shape
 * cannot be launched on the current device.  Used by the batch tuner to
 * skip shapes; no counterpart in the reference (its launch shape is a
 * command-line choice, dsl/dsl_cuda/example/cuda_setup.py:53-86).
 */
int tvbg_group_max_clusters(const tvbg_launch *cfg, int32_t *max_clusters);

/*
 * dL/dZ = Z A of the FC-fit loss for n_inst instances: d_z [n_inst][T][N]
 * (normalised, centred series), d_a [n_inst][N][N], d_out [n_inst][T][N],
 * FP32 (a sum over the N nodes per sample; the FC and the loss, sums over
 * time, are FP64 in the caller).  Used by the FC-fit adjoint
 * (tvb_hpc.adjoint.FCFit); no counterpart in the reference.
 */
int tvbg_fcfit_zgrad(const float *d_z, const float *d_a, float *d_out, int32_t n_inst,
                    int32_t T, int32_t N, void *stream);

/*
 * The FC-fit loss path of the adjoint in one call (tvb_hpc.adjoint.FCFit),
 * for n_inst series X_b [T][N], instance b in block g = b / lanes at lane
 * l = b % lanes (lanes = 1: per-instance arrays; 8: lane-interleaved
 * groups): row s < T - 1 at d_x + g * x_inst_stride + l + (s * N + i) *
 * lanes, row T - 1 at d_last + g * last_inst_stride + l + i *
 * last_node_stride (or from d_x too when d_last is NULL).  Computes the
 * Pearson FC to FP64 accuracy (two-pass: FP64 means, then the centred Gram,
 * upper triangle only, in FP32 error-free arithmetic for N <= 192 -- every
 * product exact, sums carried in two FP32 words, error below 4e-12 of
 * ||c_i|| ||c_j|| -- and in FP64 above; norms from its diagonal; into
 * d_fc [n_inst][N][N] when not NULL), d_loss[b] = mean_{i<j}
 * (FC_ij - target_ij)^2 (FP64) and, when d_dx is not NULL, dL/dX (FP32) at
 * d_dx + b * dx_inst_stride + s * N + i.  target [N][N] FP64; d_scratch of
 * tvbg_fcfit_scratch_bytes().  Restates the Pearson FC of refs/covar.c:70-109
 * (metric.py:111-139) as a two-pass sum; the loss and its gradient have no
 * counterpart in the reference.
 */
int tvbg_fcfit_scratch_bytes(int32_t n_inst, int32_t N, int64_t *bytes);
int tvbg_fcfit_loss(const float *d_x, int64_t x_inst_stride, const float *d_last,
                    int64_t last_inst_stride, int64_t last_node_stride, int32_t lanes,
                    int32_t n_inst, int32_t T, int32_t N, const double *d_target,
                    double *d_loss, float *d_dx, int64_t dx_inst_stride, double *d_fc,
                    void *d_scratch, void *stream);

/*
 * Region mapping (tvb_hpc/network.py:179-202).  to_avg: d_roi[i][j] = sum
 * of d_node[k][j] over the nodes k with d_rmap[k] == i (RMapToAvg zeroes roi
 * and accumulates: a sum), one CTA per region, a fixed reduction tree;
 * from_avg: d_node[k][j] = d_roi[d_rmap[k]][j] (RMapFromAvg).  rmap entries
 * outside [0, nroi) map to no region (their node rows are left unchanged).
 */
int tvbg_rmap_to_avg(int32_t nroi, int32_t nvar, int32_t nnode, const int32_t *d_rmap,
                     const float *d_node, float *d_roi, void *stream);
int tvbg_rmap_from_avg(int32_t nroi, int32_t nvar, int32_t nnode, const int32_t *d_rmap,
                       const float *d_roi, float *d_node, void *stream);

/*
 * ---- serving pool ---------------------------------------------------------
 * Continuous batching of sweep requests in native code: requests are copied
 * in (tvbg_serve_admit), admitted to the device when their footprint fits
 * the pool's HBM budget, advanced chunk by chunk from tvbg_serve_tick (each
 * request's lane-interleaved groups on its own stream, at its own pace),
 * retired when done (final state copied
 * out, device memory freed), and polled or cancelled by id.  The pool is
 * the one object that allocates device memory behind its calls: it is
 * created and destroyed explicitly.  The reference has no serving layer;
 * its DSL launcher runs one sweep per call
 * (dsl/dsl_cuda/example/cuda_run.py:124-142).  A request's result is the
 * group kernel's for the same inputs, alone or in any mix (chunk
 * boundaries are exact; every request keeps its Philox key: seed, and the
 * request-local instance index).
 */
typedef struct tvbg_serve tvbg_serve;

typedef struct tvbg_serve_request {
    int32_t model;            /* TVBG_MODEL_* with a group kernel            */
    int32_t cfun;             /* TVBG_CFUN_* (separable, or Kuramoto pair)   */
    int32_t N;                /* nodes                                       */
    int32_t nnz;              /* edges                                       */
    const int32_t *row;       /* host [N+1] CSR offsets (in-edges)           */
    const int32_t *col;       /* host [nnz]                                  */
    const float *weights;     /* host [nnz]                                  */
    const float *lengths;     /* host [nnz] tract lengths (mm)               */
    int32_t n_inst;           /* instances (parameter points)                */
    int32_t npar;             /* per-node parameters of the model            */
    const float *couplings;   /* host [n_inst] coupling a                    */
    const float *speeds;      /* host [n_inst] conduction speed (mm/ms)      */
    const float *state0;      /* host [n_inst][N][nsvar]                     */
    const float *nparam;      /* host [n_inst][N][npar]                      */
    int64_t nsteps;           /* steps every instance takes                  */
    float dt;                 /* ms                                          */
    int32_t rounding;         /* delay rule: 0 trunc, 1 ceil, 2 DSL          */
    uint64_t seed;            /* Philox key word 0 (lo) / counter word 2 (hi) */
    uint32_t flags;           /* TVBG_F_NOISE or 0                           */
    float cf_b;               /* coupling offset b                           */
    float cf_p[3];            /* sigmoidal coupling parameters               */
    float sigma[4];           /* noise amplitude per state variable          */
    float consts[16];         /* model constants (the model's order)         */
} tvbg_serve_request;

#define TVBG_SERVE_QUEUED 0
#define TVBG_SERVE_ACTIVE 1
#define TVBG_SERVE_DONE 2
#define TVBG_SERVE_CANCELLED 3

/* A pool with `hbm_budget` bytes for admitted requests, advancing each
 * active request by up to `chunk` steps per chunk, every request on a
 * stream of its own (`stream` is reserved: pass NULL).  Creating a pool and
 * admitting requests (host planning only) touch no device. */
int tvbg_serve_create(int64_t hbm_budget, int32_t chunk, void *stream, tvbg_serve **out);
int tvbg_serve_destroy(tvbg_serve *pool);
/* Copy a request in and queue it; *id identifies it.  Rejects requests whose
 * delays are shorter than the group kernel's blocks (d_min < 3) or whose
 * footprint exceeds the whole budget. */
int tvbg_serve_admit(tvbg_serve *pool, const tvbg_serve_request *req, int64_t *id);
/* Admit queued requests that fit and start a chunk for every active request
 * with none running; then, once some chunk is done (waiting at most 20 ms
 * when none is yet), take every finished chunk (status word, progress,
 * retirement of the finished requests: final state copied out, device
 * memory given back) and start the next chunk of its request at once.
 * Requests advance at their own pace, none waits for the others' chunks;
 * device memory is stream-ordered (cudaMallocAsync / cudaFreeAsync), so
 * admission and retirement do not wait for the device either.  *n_active
 * and *n_queued (either may be NULL) count what is left. */
int tvbg_serve_tick(tvbg_serve *pool, int32_t *n_active, int32_t *n_queued);
/* Ids of the requests retired since the last call, oldest first: up to cap
 * of them into ids, *n = how many. */
int tvbg_serve_finished(tvbg_serve *pool, int64_t *ids, int32_t cap, int32_t *n);
/* *status = TVBG_SERVE_*; once done, the final state is copied to
 * state_out (host [n_inst][N][nsvar]) when it is not NULL. */
int tvbg_serve_poll(tvbg_serve *pool, int64_t id, int32_t *status, float *state_out);
/* Drop a queued or active request (its device memory is freed at once). */
int tvbg_serve_cancel(tvbg_serve *pool, int64_t id);
/* Device bytes held by admitted requests and the footprint of request id. */
int tvbg_serve_usage(tvbg_serve *pool, int64_t id, int64_t *used, int64_t *footprint);
/* Admission stops while the active requests' chunks hold max_ctas CTAs or
 * more (an empty pool still admits its next request); 0 = no limit (the
 * default), -1 = three times the device's SM count.  On the mixed serving
 * workload at 50 requests/s no limit served the most node-steps/s: many
 * requests have few instances, so a CTA count underestimates how empty the
 * GPU is. */
int tvbg_serve_set_concurrency(tvbg_serve *pool, int64_t max_ctas);
/* Steps request id has taken so far (every instance takes the same). */
int tvbg_serve_progress(tvbg_serve *pool, int64_t id, int64_t *steps_done);
/* Steps handed to the device for request id: those taken plus the chunk
 * running now. */
int tvbg_serve_issued(tvbg_serve *pool, int64_t id, int64_t *steps);
/* Admission budget of the following ticks, at most the creation budget: a
 * caller that holds device memory of its own under the same budget (the
 * Python serving path beside the pool) passes what it leaves free, so the
 * two together stay within the budget.  Requests already admitted keep
 * their memory; a request larger than the creation budget is still refused
 * by tvbg_serve_admit.  No counterpart in the reference (no serving layer). */
int tvbg_serve_set_budget(tvbg_serve *pool, int64_t budget);

#ifdef __cplusplus
}
#endif

#endif /* TVBG_H */
