/*
 * tvbg_oracle.c -- CPU restatement of the tvb-hpc network time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA engine:
 * only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline /
 * --impl reference legs load it.  The product path never calls it.
 *
 * It restates, in plain C with no fused multiply-adds (-ffp-contract=off):
 *   - the network coupling gather       tvb_hpc/network.py:115-143
 *   - the coupling functions            tvb_hpc/coupling.py:68-121
 *   - the neural-mass drifts            tvb_hpc/model.py:157-276 (+ MPR 2015)
 *   - the Kuramoto wrap                 tvb_hpc/model.py:142-155, and the
 *     fmod wrap of dsl/dsl_cuda/CUDAmodels/kuramoto.c:19-27
 *   - Euler / Euler-Maruyama            tvb_hpc/scheme.py:29-107
 *   - the fused step and time batching  tvb_hpc/transforms.py:23-49
 *   - the ring addressing               dsl/dsl_cuda/CUDAmodels/kuramoto.c:92,108,128
 *   - the Balloon-Windkessel monitor    tvb_hpc/bold.py:24-74, refs/balloon.c:24-67
 *   - Pearson FC                        tvb_hpc/metric.py:18-139, refs/covar.c:9-109
 *   - Philox4x32-10 + Box-Muller        tvb_hpc/rng.py:30-60 (algorithm of
 *     Salmon et al. 2011; the key/counter layout is this engine's)
 * once with float arithmetic in the reference's operation order (the FP32
 * mirror) and once in double (the FP64 oracle).  The ring here is the
 * reference's plain slot-major layout ring[slot][node], slot = t mod nh.
 *
 * Parity pins: the golden fixtures under tests/golden/ (CSR gather of
 * tvb_hpc/tests.py:211-244, coupling stats, region maps), the hackathon
 * FC-SC known-answer test (tvb_hpc/examples/hackathon.py:58-89), and the
 * reference's own CUDA sources compiled for the host by oracle/Makefile
 * (kuramoto.c with noise stubbed out, balloon.c, covar.c).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_MODEL_KURAMOTO 0
#define ORC_MODEL_G2DO 1
#define ORC_MODEL_MPR 2
#define ORC_MODEL_LINEAR 3

#define ORC_CFUN_LINEAR 0
#define ORC_CFUN_DIFF 1
#define ORC_CFUN_KURAMOTO 2
#define ORC_CFUN_SIGMOIDAL 3

/* flag values shared with include/tvbg.h (TVBG_F_*), plus oracle-only bits */
#define ORC_F_NOISE 1u
#define ORC_F_BOLD 2u
#define ORC_F_TRACE 4u
#define ORC_F_WRAP_FMOD 8u
#define ORC_F_NO_WRAP 32u
#define ORC_F_BOLD_DEV 256u /* balloon on deviations from rest (the engine's form) */
/* Track-A order (tvb_hpc/transforms.py:30-42): the network gather of step t
 * runs before the model writes obsrv[t], so slot t is read as it was (post
 * and zero delays see the old row) and is then overwritten with obs(x_t). */
#define ORC_F_TRACKA 64u

/* Launch-wide configuration (host memory). */
typedef struct orc_cfg {
    int32_t model, cfun, N, nnz;
    const int32_t *row, *col;
    const float *weights;
    int32_t nh;          /* ring length (any value > max delay + 1) */
    int32_t nsteps;
    int64_t t0;
    float dt;
    uint32_t flags;
    float sigma[4];
    float consts[16];
    float cf_b;
    float cf_p[3];
    uint32_t seed_lo, seed_hi;
    int32_t trace_every, trace_len, trace_nobs;
    int32_t bold_period, bold_len, bold_obs;
    float dt_bold;
} orc_cfg;

static int nstate(int model) { return (model == ORC_MODEL_G2DO || model == ORC_MODEL_MPR) ? 2 : 1; }

/* ---- Philox4x32-10 (Salmon et al. 2011) -------------------------------- */
static void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
    int r;
    for (r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c[1] ^ k0;
        uint32_t n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0;
        c[1] = lo1;
        c[2] = n2;
        c[3] = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

void orc_philox_u32(uint32_t k0, uint32_t k1, uint32_t c1, uint32_t c2, uint32_t c3,
                    uint32_t *out, int64_t n_blocks) {
    int64_t b;
    for (b = 0; b < n_blocks; ++b) {
        uint32_t c[4] = {(uint32_t)b, c1, c2, c3};
        philox4x32_10(c, k0, k1);
        memcpy(out + 4 * b, c, sizeof(c));
    }
}

/* Box-Muller in double: u1 = ((a>>8)+0.5) 2^-24, u2 = (b>>8) 2^-24. */
static void box_muller(uint32_t a, uint32_t b, double *z0, double *z1) {
    const double u1 = ((double)(a >> 8) + 0.5) * 5.9604644775390625e-8;
    const double u2 = (double)(b >> 8) * 5.9604644775390625e-8;
    const double r = sqrt(-2.0 * log(u1));
    const double pi = 3.14159265358979323846;
    *z0 = r * cos(2.0 * pi * u2);
    *z1 = r * sin(2.0 * pi * u2);
}

static void philox_normals4(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t k0, uint32_t k1,
                            double z[4]) {
    uint32_t c[4] = {c0, c1, c2, 0u};
    philox4x32_10(c, k0, k1);
    box_muller(c[0], c[1], &z[0], &z[1]);
    box_muller(c[2], c[3], &z[2], &z[3]);
}

/* RNG.fill equivalent: key = (seed_lo, stream), counter = (i/4, i>>34, seed_hi, 0). */
void orc_philox_normal(uint64_t seed, uint32_t stream_id, float *out, int64_t n) {
    int64_t b, nb = (n + 3) / 4;
    for (b = 0; b < nb; ++b) {
        double z[4];
        int q;
        philox_normals4((uint32_t)b, (uint32_t)(b >> 32), (uint32_t)(seed >> 32), (uint32_t)seed,
                        stream_id, z);
        for (q = 0; q < 4; ++q)
            if (4 * b + q < n) out[4 * b + q] = (float)z[q];
    }
}

/* ---- the step, written once for REAL = float and REAL = double ---------- */
#define REAL float
#define SUFFIX f32
#define RSIN sinf
#define RCOS cosf
#define REXP expf
#define RPOW powf
#define RFMOD fmodf
#define RLOG1P log1pf
#define REXPM1 expm1f
#include "tvbg_oracle_step.inc"
#undef REAL
#undef SUFFIX
#undef RSIN
#undef RCOS
#undef REXP
#undef RPOW
#undef RFMOD
#undef RLOG1P
#undef REXPM1

#define REAL double
#define SUFFIX f64
#define RSIN sin
#define RCOS cos
#define REXP exp
#define RPOW pow
#define RFMOD fmod
#define RLOG1P log1p
#define REXPM1 expm1
#include "tvbg_oracle_step.inc"

/* ---- Pearson FC, FP64 two-pass (x: [T][N]) ------------------------------ */
void orc_fc(const float *x, int32_t T, int32_t N, double *fc) {
    double *m = (double *)calloc((size_t)N, sizeof(double));
    double *g = (double *)calloc((size_t)N * N, sizeof(double));
    int32_t t, i, j;
    for (t = 0; t < T; ++t)
        for (i = 0; i < N; ++i) m[i] += (double)x[(int64_t)t * N + i];
    for (i = 0; i < N; ++i) m[i] /= (double)T;
    for (t = 0; t < T; ++t)
        for (i = 0; i < N; ++i) {
            const double xi = (double)x[(int64_t)t * N + i] - m[i];
            for (j = 0; j < N; ++j) g[(int64_t)i * N + j] += xi * ((double)x[(int64_t)t * N + j] - m[j]);
        }
    for (i = 0; i < N; ++i)
        for (j = 0; j < N; ++j)
            fc[(int64_t)i * N + j] = g[(int64_t)i * N + j] / sqrt(g[(int64_t)i * N + i] * g[(int64_t)j * N + j]);
    free(m);
    free(g);
}

/* One-pass co-moment with double-buffered means, as refs/covar.c:9-68, in
 * float, followed by the normalisation of covar.c:71-109.  x: [T][N]. */
void orc_fc_onepass_f32(const float *x, int32_t T, int32_t N, float *corr) {
    float *cov = (float *)calloc((size_t)N * N, sizeof(float));
    float *means = (float *)calloc((size_t)2 * N, sizeof(float));
    int32_t s, i, j;
    for (s = 0; s < T; ++s) {
        const float *data = x + (int64_t)s * N;
        if (s == 0) {
            for (i = 0; i < N; ++i) means[i] = data[i];
            continue;
        }
        {
            const float recip_n = 1.0f / (float)s;
            float *next_mean = means, *prev_mean = means;
            if (s % 2 == 0)
                prev_mean += N;
            else
                next_mean += N;
            for (i = 0; i < N; ++i) next_mean[i] = prev_mean[i] + (data[i] - prev_mean[i]) * recip_n;
            for (i = 0; i < N; ++i) {
                const float dmi = data[i] - prev_mean[i];
                for (j = 0; j < N; ++j) cov[j * N + i] += (data[j] - next_mean[j]) * dmi;
            }
        }
    }
    {
        const float rn = 1.0f / (float)T;
        for (i = 0; i < N * N; ++i) cov[i] *= rn;
        for (i = 0; i < N; ++i)
            for (j = 0; j < N; ++j) corr[i * N + j] = cov[i * N + j] * (1.0f / sqrtf(cov[i * N + i] * cov[j * N + j]));
    }
    free(cov);
    free(means);
}

int orc_abi_version(void) { return 1; }
