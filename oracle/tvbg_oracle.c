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
#define ORC_MODEL_G2DOSC 4 /* oscillator.c:149-150 */
#define ORC_MODEL_RWW 5       /* tvb_hpc/model.py:209-223 */
#define ORC_MODEL_JANSENRIT 6 /* tvb_hpc/model.py:226-247 */

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
    int32_t npar; /* parameters per node (nparam is [N][npar] per instance); 0 = 1 */
} orc_cfg;

static int nstate(int model) {
    if (model == ORC_MODEL_JANSENRIT) return 6;
    return (model == ORC_MODEL_G2DO || model == ORC_MODEL_MPR || model == ORC_MODEL_G2DOSC) ? 2 : 1;
}

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

/* ---- FC-fit adjoint of the delayed Euler scheme, FP64 (reference gradient) ----
 *
 * TEST INFRASTRUCTURE ONLY.  Deterministic MPR with linear coupling
 * c_i(t) = G sum_e w_e r_{j_e}(t - d_e) (CUDA step order, zero history,
 * r clamped at 0), T steps from x(0).  The observed series is X[s] = r(s+1),
 * s = 0..T-1; FC = Pearson(X) (FP64); loss = mean_{i<j} (FC_ij - F*_ij)^2.
 * Gradients w.r.t. G and eta_i by the adjoint recursion
 *   mu(t+1)    = lambda(t+1) * [r_pre(t+1) >= 0 for the r component]
 *   lambda(t)  = mu + dt J(x(t))^T mu + dL/dx(t)|direct
 *   lambda_r,j(t) += dt G/tau sum_{e: j -> i} w_e mu_V,i(t + d_e + 1)
 *   dL/deta_i += dt/tau mu_V,i(t+1);  dL/dG += dt/tau mu_V,i(t+1) S_i(t)
 * consts K = [Delta, J, tau, I].
 */
static double mpr_fwd(int N, const int32_t *row, const int32_t *col, const float *w,
                      const int32_t *delays, double G, const double *eta, const double *x0,
                      int T, double dt, const float *Kf, double *X /* (T+1)*N*2 */,
                      double *S /* T*N */) {
    const double Delta = Kf[0], J = Kf[1], tau = Kf[2], I = Kf[3];
    const double pi = 3.14159265358979323846;
    int t, i, e;
    memcpy(X, x0, sizeof(double) * 2 * N);
    for (t = 0; t < T; ++t) {
        const double *x = X + (int64_t)t * N * 2;
        double *xn = X + (int64_t)(t + 1) * N * 2;
        for (i = 0; i < N; ++i) {
            double acc = 0.0;
            for (e = row[i]; e < row[i + 1]; ++e) {
                const int ts = t - delays[e];
                if (ts >= 0) acc += (double)w[e] * X[((int64_t)ts * N + col[e]) * 2];
            }
            S[(int64_t)t * N + i] = acc;
        }
        for (i = 0; i < N; ++i) {
            const double r = x[2 * i], V = x[2 * i + 1];
            const double c = G * S[(int64_t)t * N + i];
            const double ptr = pi * tau * r;
            const double fr = (Delta / (pi * tau) + 2.0 * r * V) / tau;
            const double fV = (V * V + eta[i] + J * tau * r + I + c - ptr * ptr) / tau;
            double rn = r + dt * fr;
            xn[2 * i] = rn < 0.0 ? 0.0 : rn;
            xn[2 * i + 1] = V + dt * fV;
        }
    }
    return 0.0;
}

/* FC of X[s] = r(s+1), loss and dL/dX (FP64); returns the loss. */
static double fc_loss_grad(int N, int T, const double *X, const double *target, double *dX) {
    double *mu = (double *)calloc((size_t)N, sizeof(double));
    double *nrm = (double *)calloc((size_t)N, sizeof(double));
    double *Z = (double *)calloc((size_t)T * N, sizeof(double));
    double *A = (double *)calloc((size_t)N * N, sizeof(double));
    double *gZ = (double *)calloc((size_t)T * N, sizeof(double));
    const double P = (double)N * (N - 1) / 2.0;
    double loss = 0.0;
    int s, i, j;
    for (s = 0; s < T; ++s)
        for (i = 0; i < N; ++i) mu[i] += X[((int64_t)(s + 1) * N + i) * 2];
    for (i = 0; i < N; ++i) mu[i] /= T;
    for (s = 0; s < T; ++s)
        for (i = 0; i < N; ++i) {
            const double v = X[((int64_t)(s + 1) * N + i) * 2] - mu[i];
            Z[(int64_t)s * N + i] = v;
            nrm[i] += v * v;
        }
    for (i = 0; i < N; ++i) nrm[i] = sqrt(nrm[i]);
    for (s = 0; s < T; ++s)
        for (i = 0; i < N; ++i) Z[(int64_t)s * N + i] /= nrm[i];
    for (i = 0; i < N; ++i)
        for (j = i + 1; j < N; ++j) {
            double fc = 0.0;
            for (s = 0; s < T; ++s) fc += Z[(int64_t)s * N + i] * Z[(int64_t)s * N + j];
            const double dd = fc - (double)target[(int64_t)i * N + j];
            loss += dd * dd / P;
            A[(int64_t)i * N + j] = A[(int64_t)j * N + i] = 2.0 * dd / P;
        }
    for (s = 0; s < T; ++s)
        for (i = 0; i < N; ++i) {
            double g = 0.0;
            for (j = 0; j < N; ++j) g += A[(int64_t)i * N + j] * Z[(int64_t)s * N + j];
            gZ[(int64_t)s * N + i] = g;
        }
    for (i = 0; i < N; ++i) {
        double zg = 0.0, m = 0.0;
        for (s = 0; s < T; ++s) zg += Z[(int64_t)s * N + i] * gZ[(int64_t)s * N + i];
        for (s = 0; s < T; ++s) {
            const double v = (gZ[(int64_t)s * N + i] - Z[(int64_t)s * N + i] * zg) / nrm[i];
            dX[(int64_t)s * N + i] = v;
            m += v;
        }
        m /= T;
        for (s = 0; s < T; ++s) dX[(int64_t)s * N + i] -= m;
    }
    free(mu); free(nrm); free(Z); free(A); free(gZ);
    return loss;
}

static int mpr_adjoint_one(int N, const int32_t *row, const int32_t *col, const float *w,
                           const int32_t *delays, int nnz, double G, const double *eta,
                           const double *x0, int T, double dt, const float *Kf,
                           const double *target, double *loss, double *dG, double *deta) {
    const double J = Kf[1], tau = Kf[2];
    const double pi = 3.14159265358979323846;
    double *X = (double *)malloc(sizeof(double) * (size_t)(T + 1) * N * 2);
    double *S = (double *)malloc(sizeof(double) * (size_t)T * N);
    double *dX = (double *)calloc((size_t)T * N, sizeof(double));
    double *lam = (double *)calloc((size_t)2 * N, sizeof(double));
    double *muV = (double *)calloc((size_t)(T + 2) * N, sizeof(double)); /* mu_V(t), t = 0..T+1 */
    int t, i, e;
    if (!X || !S || !dX || !lam || !muV) return -1;
    mpr_fwd(N, row, col, w, delays, G, eta, x0, T, dt, Kf, X, S);
    *loss = fc_loss_grad(N, T, X, target, dX);
    *dG = 0.0;
    for (i = 0; i < N; ++i) deta[i] = 0.0;
    /* lambda(T) = direct gradient on r(T) = X[T-1] */
    for (i = 0; i < N; ++i) {
        lam[2 * i] = dX[(int64_t)(T - 1) * N + i];
        lam[2 * i + 1] = 0.0;
    }
    for (t = T - 1; t >= 0; --t) {
        const double *x = X + (int64_t)t * N * 2;
        double *mu = (double *)malloc(sizeof(double) * 2 * N);
        double *coup = (double *)calloc((size_t)N, sizeof(double));
        for (i = 0; i < N; ++i) {
            const double r = x[2 * i], V = x[2 * i + 1];
            const double fr = (Kf[0] / (pi * tau) + 2.0 * r * V) / tau;
            const double rpre = r + dt * fr;
            mu[2 * i] = rpre >= 0.0 ? lam[2 * i] : 0.0;
            mu[2 * i + 1] = lam[2 * i + 1];
            muV[(int64_t)(t + 1) * N + i] = mu[2 * i + 1];
        }
        /* coupling: r_j(t) feeds c_i(t + d) for every edge i <- j */
        for (i = 0; i < N; ++i)
            for (e = row[i]; e < row[i + 1]; ++e) {
                const int tt = t + delays[e];
                if (tt < T) coup[col[e]] += (double)w[e] * muV[(int64_t)(tt + 1) * N + i];
            }
        for (i = 0; i < N; ++i) {
            const double r = x[2 * i], V = x[2 * i + 1];
            const double mr = mu[2 * i], mv = mu[2 * i + 1];
            const double dfr_dr = 2.0 * V / tau, dfr_dV = 2.0 * r / tau;
            const double dfV_dr = (J * tau - 2.0 * pi * pi * tau * tau * r) / tau;
            const double dfV_dV = 2.0 * V / tau;
            double lr = mr + dt * (mr * dfr_dr + mv * dfV_dr) + dt * G / tau * coup[i];
            double lv = mv + dt * (mr * dfr_dV + mv * dfV_dV);
            if (t >= 1) lr += dX[(int64_t)(t - 1) * N + i];
            deta[i] += dt / tau * mv;
            *dG += dt / tau * mv * S[(int64_t)t * N + i];
            lam[2 * i] = lr;
            lam[2 * i + 1] = lv;
        }
        free(mu);
        free(coup);
    }
    (void)nnz;
    free(X); free(S); free(dX); free(lam); free(muV);
    return 0;
}

/* n_inst instances: G [I], eta [I][N], x0 [I][N][2], delays [I][nnz]. */
int orc_mpr_adjoint_f64(int32_t N, const int32_t *row, const int32_t *col, const float *w,
                        int32_t nnz, int32_t n_inst, const int32_t *delays, const double *G,
                        const double *eta, const double *x0, int32_t T, double dt,
                        const float *consts, const double *target, double *loss, double *dG,
                        double *deta, int32_t nthreads) {
    int b, bad = 0;
    if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads) reduction(| : bad)
    for (b = 0; b < n_inst; ++b)
        if (mpr_adjoint_one(N, row, col, w, delays + (int64_t)b * nnz, nnz, G[b], eta + (int64_t)b * N,
                            x0 + (int64_t)b * N * 2, T, dt, consts, target, loss + b, dG + b,
                            deta + (int64_t)b * N))
            bad = 1;
    return bad ? -1 : 0;
}

/* Forward + loss only (FP64), for finite differences. */
int orc_mpr_loss_f64(int32_t N, const int32_t *row, const int32_t *col, const float *w,
                     int32_t nnz, const int32_t *delays, double G, const double *eta,
                     const double *x0, int32_t T, double dt, const float *consts,
                     const double *target, double *loss) {
    double *X = (double *)malloc(sizeof(double) * (size_t)(T + 1) * N * 2);
    double *S = (double *)malloc(sizeof(double) * (size_t)T * N);
    double *dX = (double *)calloc((size_t)T * N, sizeof(double));
    (void)nnz;
    if (!X || !S || !dX) return -1;
    mpr_fwd(N, row, col, w, delays, G, eta, x0, T, dt, consts, X, S);
    *loss = fc_loss_grad(N, T, X, target, dX);
    free(X); free(S); free(dX);
    return 0;
}
