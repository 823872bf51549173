/*
 * lmm_oracle.c -- TEST INFRASTRUCTURE ONLY. This is the checker, never the
 * product: only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg load it. The product path (the CUDA library) never links or calls it.
 *
 * FP64 CPU restatement of the LIBOR Market Model swaption-portfolio Monte
 * Carlo with pathwise adjoint Greeks of intel/Financial-Services-Workload-Samples,
 * LiborMarketModel/liborSwaptionGreeks.cpp:
 *   blk_forward  restates path_calc_b1  (:34-82)   Euler log-step of the NN
 *                forward rates over NMAT steps, storing the trajectory L2.
 *   blk_payoff   restates portfolio_b   (:120-211) annuity/discount build,
 *                payer-swaption payoffs x100, discounting and payoff adjoint.
 *   blk_reverse  restates path_calc_b2  (:86-117)  reverse sweep of the rate
 *                adjoint back to t=0 (gives dV/dL0[i]).
 * Additions that the reference does not have:
 *   - the vega adjoint dV/dlambda[k], derived by differentiating :68-72 with
 *     respect to lambda[k] (lambda enters through con1 = delta*lambda in the
 *     drift sum v and through the exponent);
 *   - a switch between the reference's aliased payoff adjoint (:178 overwrites
 *     L[n] with its adjoint and :181 reads it back as a rate) and the fixed
 *     form in which the rate and its adjoint are separate values;
 *   - ragged path counts (the reference needs numPaths % SIMDVLEN == 0, :282);
 *   - runtime NN/NMAT/portfolio instead of params.h compile-time constants;
 *   - seeded normals: Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel
 *     random numbers: as easy as 1, 2, 3", SC'11) + Box-Muller, restated
 *     here so that the tests can regenerate, on the CPU, exactly the counters
 *     the CUDA library consumes. The reference draws MKL MRG32k3a/ICDF normals
 *     (LiborMarketModel/mklRng.cpp:25,31,91); MKL is closed and absent, so
 *     both sides of every parity check are fed the same normals instead.
 *
 * Paths are processed in blocks of BLK=16 lanes laid out [index][lane], the
 * same vectorisation axis as the reference (SIMDVLEN=16 in FP64,
 * params.h:16), so that timing this port on the host is a fair stand-in for
 * the reference's own CPU path.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define BLK 16

typedef struct {
    int32_t nn;          /* number of forward rates            (params.h:27) */
    int32_t nmat;        /* time steps / normals per path       (params.h:28) */
    int32_t nopt;        /* swaptions in the portfolio          (params.h:30) */
    int32_t reserved;
    double delta;        /* accrual fraction DELTA              (params.h:33) */
    const double *L0;    /* [nn] initial curve   (liborSwaptionGreeks.cpp:271) */
    const double *lambda;/* [nn] vol by time to maturity, read as lambda[i-n-1] (:65,:102) */
    const int32_t *maturities; /* [nopt] swap length in periods (params.h:38) */
    const double *swaprates;   /* [nopt] strikes                (params.h:39) */
    const double *weights;     /* [nopt] notional weight of each swaption (the
                                  reference's portfolio: all 1); NULL = all 1 */
} lmmo_params;

/* ------------------------------------------------------------------ */
/* Philox4x32-10 and Box-Muller normals                                */
/* ------------------------------------------------------------------ */

static inline uint32_t mulhilo(uint32_t a, uint32_t b, uint32_t *hi)
{
    uint64_t p = (uint64_t)a * (uint64_t)b;
    *hi = (uint32_t)(p >> 32);
    return (uint32_t)p;
}

/* Philox4x32 with 10 rounds; multipliers and Weyl key increments as
 * published by Salmon et al. (SC'11, section 4.2). */
void lmmo_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        if (r > 0) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        uint32_t hi0, hi1;
        uint32_t lo0 = mulhilo(0xD2511F53u, c0, &hi0);
        uint32_t lo1 = mulhilo(0xCD9E8D57u, c2, &hi1);
        uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* Counter layout shared with the CUDA library: normals 4q..4q+3 of global
 * path p come from ctr = {q, 0, lo32(p), hi32(p)}, key = {lo32(seed), hi32(seed)}. */
static void philox_quad(uint64_t seed, uint64_t path, uint32_t q, uint32_t x[4])
{
    uint32_t ctr[4] = { q, 0u, (uint32_t)path, (uint32_t)(path >> 32) };
    uint32_t key[2] = { (uint32_t)seed, (uint32_t)(seed >> 32) };
    lmmo_philox4x32_10(ctr, key, x);
}

/* FP64 variant: 32-bit uniforms u1 = (x+1)/2^32 in (0,1], u2 = x/2^32 in [0,1),
 * z0 = r cos(2 pi u2), z1 = r sin(2 pi u2), r = sqrt(-2 ln u1). Output is
 * path-major z[p*nmat + n] as in the reference (liborSwaptionGreeks.cpp:56). */
void lmmo_normals_f64(uint64_t seed, int64_t path0, int64_t paths, int32_t nmat,
                      double mean, double sd, double *z)
{
    const double two32inv = 1.0 / 4294967296.0;
    const double twopi = 6.283185307179586476925286766559;
    const int32_t nq = (nmat + 3) / 4;
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < paths; ++p) {
        double *zp = z + p * (int64_t)nmat;
        for (int32_t q = 0; q < nq; ++q) {
            uint32_t x[4];
            philox_quad(seed, (uint64_t)(path0 + p), (uint32_t)q, x);
            double g[4];
            for (int h = 0; h < 2; ++h) {
                double u1 = ((double)x[2 * h] + 1.0) * two32inv;
                double u2 = (double)x[2 * h + 1] * two32inv;
                double r = sqrt(-2.0 * log(u1));
                double th = twopi * u2;
                g[2 * h] = r * cos(th);
                g[2 * h + 1] = r * sin(th);
            }
            for (int e = 0; e < 4; ++e) {
                int32_t n = 4 * q + e;
                if (n < nmat) zp[n] = mean + sd * g[e];
            }
        }
    }
}

/* FP32 variant (the spec of the CUDA in-kernel generator): 24-bit uniforms
 * u1 = ((x>>8)+1)/2^24 in (0,1], u2 = (x>>8)/2^24 in [0,1); same transform,
 * evaluated here in FP64 and rounded once to float. */
void lmmo_normals_f32(uint64_t seed, int64_t path0, int64_t paths, int32_t nmat, float *z)
{
    const double two24inv = 1.0 / 16777216.0;
    const double twopi = 6.283185307179586476925286766559;
    const int32_t nq = (nmat + 3) / 4;
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < paths; ++p) {
        float *zp = z + p * (int64_t)nmat;
        for (int32_t q = 0; q < nq; ++q) {
            uint32_t x[4];
            philox_quad(seed, (uint64_t)(path0 + p), (uint32_t)q, x);
            double g[4];
            for (int h = 0; h < 2; ++h) {
                double u1 = ((double)(x[2 * h] >> 8) + 1.0) * two24inv;
                double u2 = (double)(x[2 * h + 1] >> 8) * two24inv;
                double r = sqrt(-2.0 * log(u1));
                double th = twopi * u2;
                g[2 * h] = r * cos(th);
                g[2 * h + 1] = r * sin(th);
            }
            for (int e = 0; e < 4; ++e) {
                int32_t n = 4 * q + e;
                if (n < nmat) zp[n] = (float)g[e];
            }
        }
    }
}

/* ------------------------------------------------------------------ */
/* Per-block kernels                                                    */
/* ------------------------------------------------------------------ */

typedef struct {
    double *L;     /* [nn][BLK]            rates, later the rate adjoint  */
    double *L2;    /* [(nmat+1)*nn][BLK]   stored trajectory              */
    double *B, *S, *Bb, *Sb;               /* [nn-nmat][BLK] payoff work */
    double *vf;    /* [nn][BLK] drift prefix sums of one step (vega)      */
    double *vega;  /* [nn][BLK]                                           */
    double *zb;    /* [BLK][nmat] normals of the block                    */
} blk_work;

static int work_alloc(blk_work *w, const lmmo_params *p)
{
    const size_t nn = (size_t)p->nn, nmat = (size_t)p->nmat, M = nn - nmat;
    memset(w, 0, sizeof(*w));
    w->L = (double *)calloc(nn * BLK, sizeof(double));
    w->L2 = (double *)calloc((nmat + 1) * nn * BLK, sizeof(double));
    w->B = (double *)calloc(M * BLK, sizeof(double));
    w->S = (double *)calloc(M * BLK, sizeof(double));
    w->Bb = (double *)calloc(M * BLK, sizeof(double));
    w->Sb = (double *)calloc(M * BLK, sizeof(double));
    w->vf = (double *)calloc(nn * BLK, sizeof(double));
    w->vega = (double *)calloc(nn * BLK, sizeof(double));
    w->zb = (double *)calloc(nmat * BLK, sizeof(double));
    return (w->L && w->L2 && w->B && w->S && w->Bb && w->Sb && w->vf && w->vega && w->zb) ? 0 : -1;
}

static void work_free(blk_work *w)
{
    free(w->L); free(w->L2); free(w->B); free(w->S); free(w->Bb); free(w->Sb);
    free(w->vf); free(w->vega); free(w->zb);
}

/* path_calc_b1 (liborSwaptionGreeks.cpp:34-82). z is [BLK][nmat]. */
static void blk_forward(const lmmo_params *p, const double *z, double *L, double *L2)
{
    const int nn = p->nn, nmat = p->nmat;
    const double d = p->delta, sqd = sqrt(p->delta);
    for (int i = 0; i < nn; ++i)
        for (int j = 0; j < BLK; ++j) L2[i * BLK + j] = L[i * BLK + j];
    for (int n = 0; n < nmat; ++n) {
        double sqez[BLK], v[BLK];
        for (int j = 0; j < BLK; ++j) { sqez[j] = sqd * z[j * nmat + n]; v[j] = 0.0; }
        for (int i = n + 1; i < nn; ++i) {
            const double lam = p->lambda[i - n - 1];
            const double con1 = d * lam;
            double *Li = L + i * BLK;
            double *Ls = L2 + ((size_t)(n + 1) * nn + i) * BLK;
#pragma omp simd
            for (int j = 0; j < BLK; ++j) {
                v[j] += con1 * Li[j] / (1.0 + d * Li[j]);
                double vrat = exp(con1 * v[j] + lam * (sqez[j] - 0.5 * con1));
                Li[j] = Li[j] * vrat;
                Ls[j] = Li[j];
            }
        }
    }
}

/* portfolio_b (liborSwaptionGreeks.cpp:120-211). On entry L holds the
 * terminal rates, on exit their adjoint dV/dL (discounted). v receives the
 * discounted portfolio value per lane. aliased != 0 reproduces :178/:181
 * exactly (the rate is overwritten by its adjoint and then read back). */
static void blk_payoff(const lmmo_params *p, blk_work *w, double *L, double *v, int aliased)
{
    const int nn = p->nn, nmat = p->nmat, M = nn - nmat;
    const double d = p->delta;
    double b[BLK], s[BLK];
    for (int j = 0; j < BLK; ++j) { b[j] = 1.0; s[j] = 0.0; v[j] = 0.0; }
    for (int m = 0; m < M; ++m) {
        const double *Ln = L + (m + nmat) * BLK;
#pragma omp simd
        for (int j = 0; j < BLK; ++j) {
            b[j] = b[j] / (1.0 + d * Ln[j]);
            s[j] = s[j] + d * b[j];
            w->B[m * BLK + j] = b[j];
            w->S[m * BLK + j] = s[j];
        }
    }
    memset(w->Bb, 0, sizeof(double) * (size_t)M * BLK);
    memset(w->Sb, 0, sizeof(double) * (size_t)M * BLK);
    for (int o = 0; o < p->nopt; ++o) {
        const int m = p->maturities[o] - 1;
        const double K = p->swaprates[o];
        const double wo = p->weights ? p->weights[o] : 1.0;
#pragma omp simd
        for (int j = 0; j < BLK; ++j) {
            double swapval = w->B[m * BLK + j] + K * w->S[m * BLK + j] - 1.0;
            if (swapval < 0.0) {
                v[j] += (-100.0 * swapval) * wo;
                w->Sb[m * BLK + j] += (-100.0 * K) * wo;
                w->Bb[m * BLK + j] += -100.0 * wo;
            }
        }
    }
    for (int m = M - 1; m >= 0; --m) {
        double *Ln = L + (m + nmat) * BLK;
#pragma omp simd
        for (int j = 0; j < BLK; ++j) {
            w->Bb[m * BLK + j] += d * w->Sb[m * BLK + j];
            if (aliased) {
                Ln[j] = -w->Bb[m * BLK + j] * w->B[m * BLK + j] * d / (1.0 + d * Ln[j]);
                if (m > 0) {
                    w->Sb[(m - 1) * BLK + j] += w->Sb[m * BLK + j];
                    w->Bb[(m - 1) * BLK + j] += w->Bb[m * BLK + j] / (1.0 + d * Ln[j]);
                }
            } else {
                const double rate = Ln[j];
                const double adj = -w->Bb[m * BLK + j] * w->B[m * BLK + j] * d / (1.0 + d * rate);
                if (m > 0) {
                    w->Sb[(m - 1) * BLK + j] += w->Sb[m * BLK + j];
                    w->Bb[(m - 1) * BLK + j] += w->Bb[m * BLK + j] / (1.0 + d * rate);
                }
                Ln[j] = adj;
            }
        }
    }
    for (int j = 0; j < BLK; ++j) b[j] = 1.0;
    for (int n = 0; n < nmat; ++n)
        for (int j = 0; j < BLK; ++j) b[j] = b[j] / (1.0 + d * L[n * BLK + j]);
    for (int j = 0; j < BLK; ++j) v[j] = b[j] * v[j];
    for (int n = 0; n < nmat; ++n)
        for (int j = 0; j < BLK; ++j) L[n * BLK + j] = -v[j] * d / (1.0 + d * L[n * BLK + j]);
    for (int n = nmat; n < nn; ++n)
        for (int j = 0; j < BLK; ++j) L[n * BLK + j] = b[j] * L[n * BLK + j];
}

/* path_calc_b2 (liborSwaptionGreeks.cpp:86-117) plus the vega adjoint.
 * With w = con1*v_i + lam*(sqez - con1/2), con1 = delta*lam_k and
 * v_i = sum_{j<=i} con1_j L_j/(1+delta L_j), cell (n,i) adds to vega[k=i-n-1]
 *   Pb_i * (delta*v_i + sqez - delta*lam_k) + delta^2 * L_i/(1+delta L_i) * v1_i
 * where Pb_i = L_{n+1,i} * Lb_i is the adjoint of log L_{n+1,i} and
 * v1_i = sum_{j>=i} lam_j Pb_j is the reference's running sum v1 (:108). */
static void blk_reverse(const lmmo_params *p, blk_work *w, double *Lb, const double *L2,
                        const double *z, int want_vega)
{
    const int nn = p->nn, nmat = p->nmat;
    const double d = p->delta, sqd = sqrt(p->delta);
    for (int n = nmat - 1; n >= 0; --n) {
        double v1[BLK], sqez[BLK];
        if (want_vega) {
            double acc[BLK];
            for (int j = 0; j < BLK; ++j) { acc[j] = 0.0; sqez[j] = sqd * z[j * nmat + n]; }
            for (int i = n + 1; i < nn; ++i) {
                const double con1 = d * p->lambda[i - n - 1];
                const double *Ln = L2 + ((size_t)n * nn + i) * BLK;
                for (int j = 0; j < BLK; ++j) {
                    acc[j] += con1 * Ln[j] / (1.0 + d * Ln[j]);
                    w->vf[i * BLK + j] = acc[j];
                }
            }
        }
        for (int j = 0; j < BLK; ++j) v1[j] = 0.0;
        for (int i = nn - 1; i > n; --i) {
            const double lam = p->lambda[i - n - 1];
            const double *Ln = L2 + ((size_t)n * nn + i) * BLK;
            const double *Lp = L2 + ((size_t)(n + 1) * nn + i) * BLK;
            double *Lbi = Lb + i * BLK;
            double *vg = w->vega + (i - n - 1) * BLK;
#pragma omp simd
            for (int j = 0; j < BLK; ++j) {
                v1[j] += lam * Lp[j] * Lbi[j];
                const double faci = d / (1.0 + d * Ln[j]);
                if (want_vega) {
                    const double Pb = Lp[j] * Lbi[j];
                    const double t = Ln[j] / (1.0 + d * Ln[j]);
                    vg[j] += Pb * (d * w->vf[i * BLK + j] + sqez[j] - d * lam) + d * d * t * v1[j];
                }
                Lbi[j] = Lbi[j] * Lp[j] / Ln[j] + v1[j] * lam * faci * faci;
            }
        }
    }
}

/* One block of up to BLK paths. z points at the first path (path-major);
 * lanes >= nb reuse lane 0's normals and are ignored by the caller.
 * res is [BLK][1+2nn]: value, deltas, vegas per lane. */
static void blk_eval(const lmmo_params *p, blk_work *w, const double *z, int nb,
                     int want_adj, int want_vega, int aliased, double *res)
{
    const int nn = p->nn, nmat = p->nmat, nout = 1 + 2 * nn;
    for (int j = 0; j < BLK; ++j) {
        const double *src = z + (size_t)(j < nb ? j : 0) * nmat;
        memcpy(w->zb + (size_t)j * nmat, src, sizeof(double) * (size_t)nmat);
    }
    for (int i = 0; i < nn; ++i)
        for (int j = 0; j < BLK; ++j) w->L[i * BLK + j] = p->L0[i];
    memset(w->vega, 0, sizeof(double) * (size_t)nn * BLK);
    double v[BLK];
    blk_forward(p, w->zb, w->L, w->L2);
    blk_payoff(p, w, w->L, v, aliased);
    if (want_adj) blk_reverse(p, w, w->L, w->L2, w->zb, want_vega);
    for (int j = 0; j < BLK; ++j) {
        double *r = res + (size_t)j * nout;
        r[0] = v[j];
        for (int i = 0; i < nn; ++i) {
            r[1 + i] = want_adj ? w->L[i * BLK + j] : 0.0;
            r[1 + nn + i] = want_vega ? w->vega[i * BLK + j] : 0.0;
        }
    }
}

static int check_params(const lmmo_params *p)
{
    if (!p || p->nn < 2 || p->nmat < 1 || p->nmat >= p->nn || p->nopt < 0) return -1;
    if (!p->L0 || !p->lambda || (p->nopt > 0 && (!p->maturities || !p->swaprates))) return -1;
    for (int o = 0; o < p->nopt; ++o)
        if (p->maturities[o] < 1 || p->maturities[o] > p->nn - p->nmat) return -1;
    return 0;
}

/* ------------------------------------------------------------------ */
/* Public entry points (ctypes)                                          */
/* ------------------------------------------------------------------ */

/* Per-path results, res is [paths][1+2nn]. */
int lmmo_paths(const lmmo_params *p, const double *z, int64_t paths, int32_t want_vega,
               int32_t aliased, double *res)
{
    if (check_params(p) || paths < 0 || (paths > 0 && (!z || !res))) return -1;
    const int nout = 1 + 2 * p->nn;
    const int64_t nblk = (paths + BLK - 1) / BLK;
    int err = 0;
#pragma omp parallel
    {
        blk_work w;
        double *tmp = (double *)malloc(sizeof(double) * (size_t)BLK * nout);
        int ok = (work_alloc(&w, p) == 0 && tmp);
        if (!ok) {
#pragma omp atomic write
            err = 1;
        }
#pragma omp for schedule(static)
        for (int64_t b = 0; b < nblk; ++b) {
            if (!ok) continue;
            const int64_t p0 = b * BLK;
            const int nb = (int)((paths - p0) < BLK ? (paths - p0) : BLK);
            blk_eval(p, &w, z + p0 * p->nmat, nb, 1, want_vega, aliased, tmp);
            memcpy(res + p0 * nout, tmp, sizeof(double) * (size_t)nb * nout);
        }
        work_free(&w);
        free(tmp);
    }
    return err ? -2 : 0;
}

/* Monte Carlo means and standard errors of value, the nn deltas and the nn
 * vegas. Sums run per chunk of 64 blocks in FP64 and chunks are added in
 * order, so the result does not depend on the thread count. */
static int greeks_impl(const lmmo_params *p, const double *z, int64_t paths, int want_adj,
                       int want_vega, int aliased, int nthreads, double *mean, double *se)
{
    if (check_params(p) || paths < 1 || !z || !mean) return -1;
    const int nout = 1 + 2 * p->nn;
    const int64_t nblk = (paths + BLK - 1) / BLK;
    const int64_t CH = 64;
    const int64_t nch = (nblk + CH - 1) / CH;
    double *part = (double *)calloc((size_t)nch * 2 * nout, sizeof(double));
    if (!part) return -2;
    int err = 0;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#else
    nthreads = 1;
#endif
#pragma omp parallel num_threads(nthreads)
    {
        blk_work w;
        double *tmp = (double *)malloc(sizeof(double) * (size_t)BLK * nout);
        int ok = (work_alloc(&w, p) == 0 && tmp);
        if (!ok) {
#pragma omp atomic write
            err = 1;
        }
#pragma omp for schedule(dynamic, 1)
        for (int64_t c = 0; c < nch; ++c) {
            if (!ok) continue;
            double *ps = part + (size_t)c * 2 * nout;
            for (int64_t b = c * CH; b < (c + 1) * CH && b < nblk; ++b) {
                const int64_t p0 = b * BLK;
                const int nb = (int)((paths - p0) < BLK ? (paths - p0) : BLK);
                blk_eval(p, &w, z + p0 * p->nmat, nb, want_adj, want_vega, aliased, tmp);
                for (int j = 0; j < nb; ++j)
                    for (int o = 0; o < nout; ++o) {
                        const double x = tmp[(size_t)j * nout + o];
                        ps[o] += x;
                        ps[nout + o] += x * x;
                    }
            }
        }
        work_free(&w);
        free(tmp);
    }
    if (err) { free(part); return -2; }
    for (int o = 0; o < nout; ++o) {
        double s = 0.0, s2 = 0.0;
        for (int64_t c = 0; c < nch; ++c) {
            s += part[(size_t)c * 2 * nout + o];
            s2 += part[(size_t)c * 2 * nout + nout + o];
        }
        const double m = s / (double)paths;
        mean[o] = m;
        if (se) {
            double var = paths > 1 ? (s2 - s * m) / (double)(paths - 1) : 0.0;
            se[o] = var > 0.0 ? sqrt(var / (double)paths) : 0.0;
        }
    }
    free(part);
    return 0;
}

int lmmo_greeks(const lmmo_params *p, const double *z, int64_t paths, int32_t aliased,
                int32_t nthreads, double *mean, double *se)
{
    return greeks_impl(p, z, paths, 1, 1, aliased, nthreads, mean, se);
}

/* Discounted portfolio value only (forward + payoff), for finite differences. */
int lmmo_value(const lmmo_params *p, const double *z, int64_t paths, int32_t nthreads,
               double *mean, double *se)
{
    if (check_params(p)) return -1;
    const int nout = 1 + 2 * p->nn;
    double *m = (double *)calloc((size_t)nout, sizeof(double));
    double *s = (double *)calloc((size_t)nout, sizeof(double));
    if (!m || !s) { free(m); free(s); return -2; }
    int rc = greeks_impl(p, z, paths, 0, 0, 0, nthreads, m, s);
    if (rc == 0) { *mean = m[0]; if (se) *se = s[0]; }
    free(m); free(s);
    return rc;
}

/* Central finite differences under common random numbers: out is
 * [1+2nn] = value, dV/dL0[i], dV/dlambda[k], with bump h on each input. */
int lmmo_fd_greeks(const lmmo_params *p, const double *z, int64_t paths, double h,
                   int32_t nthreads, double *out)
{
    if (check_params(p) || !(h > 0.0)) return -1;
    const int nn = p->nn;
    double *L0 = (double *)malloc(sizeof(double) * nn);
    double *lam = (double *)malloc(sizeof(double) * nn);
    if (!L0 || !lam) { free(L0); free(lam); return -2; }
    memcpy(L0, p->L0, sizeof(double) * nn);
    memcpy(lam, p->lambda, sizeof(double) * nn);
    lmmo_params q = *p;
    q.L0 = L0; q.lambda = lam;
    int rc = lmmo_value(&q, z, paths, nthreads, &out[0], NULL);
    for (int i = 0; i < nn && rc == 0; ++i) {
        double up, dn;
        L0[i] = p->L0[i] + h; rc |= lmmo_value(&q, z, paths, nthreads, &up, NULL);
        L0[i] = p->L0[i] - h; rc |= lmmo_value(&q, z, paths, nthreads, &dn, NULL);
        L0[i] = p->L0[i];
        out[1 + i] = (up - dn) / (2.0 * h);
        lam[i] = p->lambda[i] + h; rc |= lmmo_value(&q, z, paths, nthreads, &up, NULL);
        lam[i] = p->lambda[i] - h; rc |= lmmo_value(&q, z, paths, nthreads, &dn, NULL);
        lam[i] = p->lambda[i];
        out[1 + nn + i] = (up - dn) / (2.0 * h);
    }
    free(L0); free(lam);
    return rc;
}

/* The reference's own unit of work, for the CPU baseline: per path the
 * forward, the payoff and the full delta adjoint (no vegas, which the
 * reference never computes), summing the value and dV/dL0[nn-1] in FP64 as
 * liborSwaptionGreeks.cpp:276-344 does, with the aliasing fixed. Returns the
 * means (the reference additionally multiplies them by NLOOPS, :278,:355). */
int lmmo_reference_work(const lmmo_params *p, const double *z, int64_t paths, int32_t nthreads,
                        double *value, double *delta_last)
{
    if (check_params(p) || paths < 1 || !z) return -1;
    const int nn = p->nn, nout = 1 + 2 * nn;
    const int64_t nblk = (paths + BLK - 1) / BLK;
    double sv = 0.0, sl = 0.0;
    int err = 0;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#else
    nthreads = 1;
#endif
#pragma omp parallel num_threads(nthreads) reduction(+ : sv, sl)
    {
        blk_work w;
        double *tmp = (double *)malloc(sizeof(double) * (size_t)BLK * nout);
        int ok = (work_alloc(&w, p) == 0 && tmp);
        if (!ok) {
#pragma omp atomic write
            err = 1;
        }
#pragma omp for schedule(static)
        for (int64_t b = 0; b < nblk; ++b) {
            if (!ok) continue;
            const int64_t p0 = b * BLK;
            const int nb = (int)((paths - p0) < BLK ? (paths - p0) : BLK);
            blk_eval(p, &w, z + p0 * p->nmat, nb, 1, 0, 0, tmp);
            for (int j = 0; j < nb; ++j) {
                sv += tmp[(size_t)j * nout];
                sl += tmp[(size_t)j * nout + nn];
            }
        }
        work_free(&w);
        free(tmp);
    }
    if (err) return -2;
    *value = sv / (double)paths;
    *delta_last = sl / (double)paths;
    return 0;
}

int lmmo_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
