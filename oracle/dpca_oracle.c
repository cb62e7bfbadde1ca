/*
 * dpca_oracle.c -- CPU restatement of DistPCA's hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: tests/, the smoke()
 * entry point and bench.py's CPU-baseline leg load it (liboracle.so) to
 * produce expected results.  The product (distpca_gb300/, libdpca.so) never
 * links, loads or calls it.
 *
 * Each function restates one piece of the reference (paths relative to the
 * DistPCA checkout):
 *   oracle_decode_row     src/utilities.cpp:351-414  decode_plink_sse2, LUT {0,3,1,2}
 *   oracle_standardize    src/utilities.cpp:272-306  standardize
 *   oracle_lut_row        src/methods.cpp:819-843    norm_precomp cache (sd > 1e-9)
 *   oracle_rand_val       src/gennorm.c:44-72        Park-Miller LCG, Schrage's method
 *   oracle_norm2          src/gennorm.c:21-42        Box-Muller, cos branch, PI=3.14159265
 *   oracle_omega          src/distpca.cpp:384-394    start block, reseed with int jj*M+kk
 *   oracle_pass           src/methods.cpp:786-936    Z = sum_b X_b^T (X_b Omega), blocked
 *   oracle_solve          src/methods.cpp:702-1118   out-of-core subspace iteration, and
 *                         src/methods.cpp:24-325     in-core variant (bsize >= n_snp)
 * Dense products, Householder QR and the symmetric eigensolve go through the
 * same CBLAS/LAPACKE calls the reference makes (OpenBLAS from the scipy wheel).
 *
 * Parity is pinned against the reference itself: oracle/build_ref.sh compiles
 * the unmodified reference sources into oracle/_ref/, and
 * tests/golden/make_golden.py records their outputs as fixtures.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "shim/dpca_blas_shim.h"

#define ORACLE_MISSING 3
#define ORACLE_PI 3.14159265 /* truncated, as gennorm.h:23 */

typedef struct {
    int n_ind;  /* individuals (reference: M) */
    int n_snp;  /* SNPs (reference: N) */
    int nsv;
    int nrhs;
    int power;
    int crit;   /* 0 trace, 1 per-sigma, 2 MEV */
    int miter;
    int bsize;  /* SNP rows per block; >= n_snp selects the in-core variant */
    double tol;
    int threads; /* BLAS threads; <= 0 leaves the library default */
} oracle_cfg;

static double oracle_now(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* ---------------------------------------------------------------- decode */

/* 2-bit codes, sample i at bits 2*(i%4) of byte i/4; LUT {0,3,1,2}. */
void oracle_decode_row(const uint8_t *in, int n_ind, uint8_t *out) {
    static const uint8_t lut[4] = {0, 3, 1, 2};
    for (int i = 0; i < n_ind; ++i) out[i] = lut[(in[i >> 2] >> (2 * (i & 3))) & 3];
}

/* Mean over non-missing, binomial sd, scaled standardized row; NaN -> 0. */
void oracle_standardize(const uint8_t *dec, int n_ind, double inv_sqrt_nsnp, double *avg_out, double *sd_out,
                        double *row_out) {
    double sum = 0;
    unsigned int ctr = 0;
    for (int i = 0; i < n_ind; ++i)
        if (dec[i] != ORACLE_MISSING) {
            sum += (double)dec[i];
            ctr++;
        }
    double freq = sum / ctr;
    double p = freq / 2.0;
    double sd = sqrt(2.0 * p * (1 - p));
    *avg_out = freq;
    *sd_out = sd;
    if (row_out)
        for (int i = 0; i < n_ind; ++i) {
            double x = (double)dec[i];
            double v = (x == ORACLE_MISSING) ? 0.0 : (x - freq) / sd * inv_sqrt_nsnp;
            row_out[i] = isnan(v) ? 0.0 : v;
        }
}

/* Per-SNP cache indexed by b = {3,1,2,0}[code] (decode_plink_precomp_sse2,
 * utilities.cpp:419): lut[3] = (0-avg)/sd (code 00), lut[2] = (1-avg)/sd
 * (code 10), lut[0] = (2-avg)/sd (code 11), lut[1] = 0 (code 01, missing);
 * all zero unless sd > 1e-9.  Later passes multiply by 1/sqrt(n_snp)
 * (methods.cpp:842). */
void oracle_lut_row(double avg, double sd, double lut[4]) {
    lut[0] = lut[1] = lut[2] = lut[3] = 0.0;
    if (sd > 1e-9) {
        lut[3] = (0 - avg) / sd;
        lut[2] = (1 - avg) / sd;
        lut[0] = (2 - avg) / sd;
        lut[1] = 0;
    }
}

/* Statistics of every SNP row of a packed matrix (rows of ceil(n_ind/4) bytes). */
void oracle_decode_stats(const uint8_t *packed, int n_ind, int n_snp, double *avg, double *sd, uint8_t *codes) {
    size_t np = ((size_t)n_ind + 3) / 4;
    uint8_t *dec = (uint8_t *)malloc((size_t)n_ind);
    for (int s = 0; s < n_snp; ++s) {
        oracle_decode_row(packed + (size_t)s * np, n_ind, dec);
        oracle_standardize(dec, n_ind, 1.0, &avg[s], &sd[s], NULL);
        if (codes) memcpy(codes + (size_t)s * n_ind, dec, (size_t)n_ind);
    }
    free(dec);
}

/* ---------------------------------------------------------------- RNG */

static long oracle_lcg_state = 0; /* static state starts at 0 */

double oracle_rand_val(int seed) {
    const long a = 16807, m = 2147483647, q = 127773, r = 2836;
    if (seed > 0) {
        oracle_lcg_state = seed;
        return 0.0;
    }
    long hi = oracle_lcg_state / q, lo = oracle_lcg_state % q;
    long nx = a * lo - r * hi;
    oracle_lcg_state = nx > 0 ? nx : nx + m;
    return (double)oracle_lcg_state / m;
}

double oracle_norm2(double mean, double sd) {
    double u = 0.0;
    while (u == 0.0) u = oracle_rand_val(0);
    double rr = sqrt(-2.0 * log(u));
    double th = 0.0;
    while (th == 0.0) th = 2.0 * ORACLE_PI * oracle_rand_val(0);
    return rr * cos(th) * sd + mean;
}

/* Row-major n_ind x k start block; seed jj*n_ind+kk wraps as a 32-bit int. */
void oracle_omega(int n_ind, int k, double *out) {
    oracle_lcg_state = 0;
    for (int j = 0; j < n_ind; ++j)
        for (int c = 0; c < k; ++c) {
            int seed = (int)((uint32_t)j * (uint32_t)n_ind + (uint32_t)c);
            oracle_rand_val(seed);
            out[(size_t)j * k + c] = oracle_norm2(0.0, 1.0);
        }
}

/* ---------------------------------------------------------------- passes */

typedef struct {
    const uint8_t *packed;
    int n_ind, n_snp, k, bsize;
    double inv_sqrt_nsnp;
    double *lut;        /* 4 per SNP */
    uint8_t *seen;      /* per SNP */
    double *blk;        /* bsize x n_ind */
    double *yb;         /* bsize x k */
    uint8_t *dec;
    double t_load, t_mm_a, t_mm_at;
} oracle_ctx;

/* Fill rows [s0, s0+rows) of the standardized matrix, first sight via
 * standardize(), later via the cached LUT (methods.cpp:819-843). */
static void oracle_fill_block(oracle_ctx *c, int s0, int rows, double *dst) {
    size_t np = ((size_t)c->n_ind + 3) / 4;
    static const uint8_t lut_pre[4] = {3, 1, 2, 0}; /* decode_plink_precomp_sse2 */
    for (int r = 0; r < rows; ++r) {
        int s = s0 + r;
        const uint8_t *row = c->packed + (size_t)s * np;
        double *out = dst + (size_t)r * c->n_ind;
        if (!c->seen[s]) {
            double avg, sd;
            oracle_decode_row(row, c->n_ind, c->dec);
            oracle_standardize(c->dec, c->n_ind, c->inv_sqrt_nsnp, &avg, &sd, out);
            oracle_lut_row(avg, sd, c->lut + 4 * (size_t)s);
            c->seen[s] = 1;
        } else {
            const double *l = c->lut + 4 * (size_t)s;
            for (int i = 0; i < c->n_ind; ++i) {
                int b = lut_pre[(row[i >> 2] >> (2 * (i & 3))) & 3];
                out[i] = l[b] * c->inv_sqrt_nsnp;
            }
        }
    }
}

/* Z = sum over SNP blocks of X_b^T (X_b Omega); Omega, Z row-major n_ind x k. */
static void oracle_pass_ctx(oracle_ctx *c, const double *omega, double *z) {
    int n = c->n_ind, k = c->k;
    memset(z, 0, (size_t)n * k * sizeof(double));
    for (int s0 = 0; s0 < c->n_snp; s0 += c->bsize) {
        int rows = c->n_snp - s0 < c->bsize ? c->n_snp - s0 : c->bsize;
        double t0 = oracle_now();
        oracle_fill_block(c, s0, rows, c->blk);
        double t1 = oracle_now();
        cblas_dgemm(CblasRowMajor, CblasNoTrans, CblasNoTrans, rows, k, n, 1.0, c->blk, n, omega, k, 0.0, c->yb, k);
        double t2 = oracle_now();
        cblas_dgemm(CblasRowMajor, CblasTrans, CblasNoTrans, n, k, rows, 1.0, c->blk, n, c->yb, k, 1.0, z, k);
        double t3 = oracle_now();
        c->t_load += t1 - t0;
        c->t_mm_a += t2 - t1;
        c->t_mm_at += t3 - t2;
    }
}

static int oracle_ctx_init(oracle_ctx *c, const uint8_t *packed, int n_ind, int n_snp, int k, int bsize) {
    memset(c, 0, sizeof(*c));
    c->packed = packed;
    c->n_ind = n_ind;
    c->n_snp = n_snp;
    c->k = k;
    c->bsize = bsize < 1 ? 1 : (bsize > n_snp ? n_snp : bsize);
    c->inv_sqrt_nsnp = 1.0 / sqrt((double)n_snp);
    c->lut = (double *)calloc(4 * (size_t)n_snp, sizeof(double));
    c->seen = (uint8_t *)calloc((size_t)n_snp, 1);
    c->blk = (double *)malloc((size_t)c->bsize * n_ind * sizeof(double));
    c->yb = (double *)malloc((size_t)c->bsize * k * sizeof(double));
    c->dec = (uint8_t *)malloc((size_t)n_ind);
    return (c->lut && c->seen && c->blk && c->yb && c->dec) ? 0 : -1;
}

static void oracle_ctx_free(oracle_ctx *c) {
    free(c->lut);
    free(c->seen);
    free(c->blk);
    free(c->yb);
    free(c->dec);
}

/* npasses passes over the same matrix; the first decodes and standardizes
 * (methods.cpp:819-835), later ones use the LUT cache (methods.cpp:837-843).
 * z receives the last pass.  times[4] (nullable): load/decode, X*Omega,
 * X^T*Y and wall seconds of the LAST pass; walls[npasses] (nullable): the
 * wall seconds of every pass. */
int oracle_pass(const uint8_t *packed, int n_ind, int n_snp, int bsize, const double *omega, int k, double *z,
                int npasses, double *times, double *walls) {
    oracle_ctx c;
    if (oracle_ctx_init(&c, packed, n_ind, n_snp, k, bsize)) {
        oracle_ctx_free(&c);
        return -1;
    }
    for (int p = 0; p < (npasses < 1 ? 1 : npasses); ++p) {
        c.t_load = c.t_mm_a = c.t_mm_at = 0;
        double t0 = oracle_now();
        oracle_pass_ctx(&c, omega, z);
        double w = oracle_now() - t0;
        if (times) times[3] = w;
        if (walls) walls[p] = w;
    }
    if (times) {
        times[0] = c.t_load;
        times[1] = c.t_mm_a;
        times[2] = c.t_mm_at;
    }
    oracle_ctx_free(&c);
    return 0;
}

/* Input generation for CPU-side baselines: packed rows [s0, s1) of the seeded
 * Balding-Nichols cohort, the same bytes as distpca_gb300/synth.py::pack_rows
 * (2-bit codes 00/10/11 for g = 0/1/2, 01 missing, pads 00). */
static uint64_t oracle_fmix(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

void oracle_synth_rows(uint64_t key, int n_ind, int s0, int s1, const uint8_t *pop, const uint32_t *miss_thr,
                       const uint32_t *snp_thr, int n_pop, uint8_t *out) {
    size_t np = ((size_t)n_ind + 3) / 4;
    for (int s = s0; s < s1; ++s) {
        uint8_t *row = out + (size_t)(s - s0) * np;
        memset(row, 0, np);
        const uint32_t *t = snp_thr + (size_t)s * n_pop;
        for (int i = 0; i < n_ind; ++i) {
            uint64_t x = (((uint64_t)s) << 32 | (uint64_t)i) ^ key;
            uint64_t hg = oracle_fmix(x + 0x9E3779B97F4A7C15ull);
            uint64_t hm = oracle_fmix(x ^ 0xD6E8FEB86659FD93ull);
            uint32_t th = t[pop[i]];
            unsigned g = ((uint32_t)hg < th) + ((uint32_t)(hg >> 32) < th);
            unsigned code = g == 0 ? 0u : (g == 1 ? 2u : 3u);
            if ((uint32_t)hm < miss_thr[i]) code = 1u;
            row[i >> 2] |= (uint8_t)(code << (2 * (i & 3)));
        }
    }
}

/* Householder QR of the n x k row-major panel in place -> explicit Q. */
static void oracle_qr(double *a, int n, int k, double *tau) {
    LAPACKE_dgeqrf(LAPACK_ROW_MAJOR, n, k, a, k, tau);
    LAPACKE_dorgqr(LAPACK_ROW_MAJOR, n, k, k, a, k, tau);
}

/* Symmetric eigensolve of the upper triangle of b (k x k), eigenvalues
 * ascending in w; then columns reversed into descending order in out. */
static void oracle_eig_desc(double *b, int k, double *w, double *out) {
    for (int i = 0; i < k; ++i)
        for (int j = 0; j < i; ++j) b[i * k + j] = 0.0;
    LAPACKE_dsyev(LAPACK_ROW_MAJOR, 'V', 'U', k, b, k, w);
    for (int i = 0; i < k; ++i)
        for (int j = 0; j < k; ++j) out[i * k + j] = b[i * k + (k - 1 - j)];
}

/*
 * Full solve.  omega (n_ind x nrhs, row-major) is the start block on entry
 * and the final Ritz block on exit, as RHS2 in the reference.
 * sigma[nsv], u[n_ind*nsv] receive the results; its_out the iteration count;
 * crit_vals[miter] (nullable) the per-iteration criterion value (NaN at ii=0);
 * timers[6] (nullable): load, mm_a, mm_at, qr, rr, total seconds.
 */
int oracle_solve(const oracle_cfg *cfg, const uint8_t *packed, double *omega, double *sigma, double *u,
                 int *its_out, double *crit_vals, double *timers) {
    int n = cfg->n_ind, k = cfg->nrhs, nsv = cfg->nsv, miter = cfg->miter;
    int in_core = cfg->bsize >= cfg->n_snp;
    if (cfg->threads > 0) scipy_openblas_set_num_threads(cfg->threads);
    double t_begin = oracle_now(), t_qr = 0, t_rr = 0;

    oracle_ctx c;
    if (oracle_ctx_init(&c, packed, n, cfg->n_snp, k, cfg->bsize)) {
        oracle_ctx_free(&c);
        return -1;
    }
    size_t nk = (size_t)n * k;
    double *z = (double *)malloc(nk * sizeof(double));
    double *q = (double *)malloc(nk * sizeof(double));
    double *old = (double *)malloc(nk * sizeof(double));
    double *tau = (double *)malloc((size_t)k * sizeof(double));
    double *b = (double *)malloc((size_t)k * k * sizeof(double));
    double *wv = (double *)malloc((size_t)k * k * sizeof(double));
    double *w = (double *)malloc((size_t)k * sizeof(double));
    double *sv = (double *)calloc((size_t)nsv, sizeof(double));
    double *sv_old = (double *)calloc((size_t)nsv, sizeof(double));
    double *delta = (double *)calloc((size_t)(miter > 0 ? miter : 1), sizeof(double));
    /* in-core: X materialised once (Read_Bed_Local, utilities.cpp:482-518) */
    double *xfull = NULL, *yfull = NULL;
    if (in_core) {
        xfull = (double *)malloc((size_t)cfg->n_snp * n * sizeof(double));
        yfull = (double *)malloc((size_t)cfg->n_snp * k * sizeof(double));
        double t0 = oracle_now();
        for (int s = 0; s < cfg->n_snp; ++s) {
            double avg, sd;
            oracle_decode_row(packed + (size_t)s * ((n + 3) / 4), n, c.dec);
            oracle_standardize(c.dec, n, c.inv_sqrt_nsnp, &avg, &sd, xfull + (size_t)s * n);
        }
        c.t_load += oracle_now() - t0;
    }
    if (cfg->crit == 2) memcpy(old, omega, nk * sizeof(double));

    /* in-core pass: RHS_local = X Omega, ARHS = X^T RHS_local (methods.cpp:55-75) */
#define PASS(src)                                                                                              \
    do {                                                                                                       \
        if (in_core) {                                                                                         \
            double ta = oracle_now();                                                                          \
            cblas_dgemm(CblasRowMajor, CblasNoTrans, CblasNoTrans, cfg->n_snp, k, n, 1.0, xfull, n, (src), k,  \
                        0.0, yfull, k);                                                                        \
            double tb = oracle_now();                                                                          \
            cblas_dgemm(CblasRowMajor, CblasTrans, CblasNoTrans, n, k, cfg->n_snp, 1.0, xfull, n, yfull, k,    \
                        0.0, z, k);                                                                            \
            c.t_mm_a += tb - ta;                                                                               \
            c.t_mm_at += oracle_now() - tb;                                                                    \
        } else {                                                                                               \
            oracle_pass_ctx(&c, (src), z);                                                                     \
        }                                                                                                      \
    } while (0)

    int ii;
    for (ii = 0; ii < miter; ++ii) {
        PASS(omega);
        for (int kk = 0; kk < cfg->power - 1; ++kk) {
            double t0 = oracle_now();
            oracle_qr(z, n, k, tau);
            t_qr += oracle_now() - t0;
            memcpy(omega, z, nk * sizeof(double));
            PASS(omega);
        }
        double t0 = oracle_now();
        oracle_qr(z, n, k, tau);
        t_qr += oracle_now() - t0;
        memcpy(q, z, nk * sizeof(double));
        t0 = oracle_now();
        if (in_core) {
            /* B = (X Q)^T (X Q) (methods.cpp:129-150) */
            cblas_dgemm(CblasRowMajor, CblasNoTrans, CblasNoTrans, cfg->n_snp, k, n, 1.0, xfull, n, q, k, 0.0,
                        yfull, k);
            double tb = oracle_now();
            c.t_mm_a += tb - t0;
            cblas_dgemm(CblasRowMajor, CblasTrans, CblasNoTrans, k, k, cfg->n_snp, 1.0, yfull, k, yfull, k, 0.0,
                        b, k);
            c.t_mm_at += oracle_now() - tb;
        } else {
            /* last pass on Q, then B = Q^T (A A^T Q) (methods.cpp:958-973) */
            memcpy(omega, q, nk * sizeof(double));
            oracle_pass_ctx(&c, omega, z);
            cblas_dgemm(CblasRowMajor, CblasTrans, CblasNoTrans, k, k, n, 1.0, q, k, z, k, 0.0, b, k);
        }
        double t1 = oracle_now();
        oracle_eig_desc(b, k, w, wv);
        /* Omega = Q W (methods.cpp:1002-1007) */
        cblas_dgemm(CblasRowMajor, CblasNoTrans, CblasNoTrans, n, k, k, 1.0, q, k, wv, k, 0.0, omega, k);
        t_rr += oracle_now() - t1;
        delta[ii] = 0.0;
        for (int j = 0; j < nsv; ++j) {
            sv[j] = sqrt(w[k - 1 - j]);
            delta[ii] += sv[j];
        }
        double cval = NAN;
        int stop = 0;
        if (ii > 0) {
            if (cfg->crit == 0) {
                cval = fabs(delta[ii - 1] - delta[ii]) / delta[ii];
                stop = cval <= cfg->tol;
            } else if (cfg->crit == 1) {
                int conv = 0;
                for (int j = 0; j < nsv; ++j)
                    if (fabs((sv[j] - sv_old[j]) / sv[j]) <= cfg->tol) conv++;
                cval = conv;
                stop = conv == nsv;
            } else if (cfg->crit == 2) {
                double mev = 0.0;
                for (int j = 0; j < nsv; ++j) {
                    double d = 0.0;
                    for (int i = 0; i < n; ++i) d += old[(size_t)i * k + j] * omega[(size_t)i * k + j];
                    mev += d * d;
                }
                mev /= nsv;
                cval = 1.0 - mev;
                stop = cval <= cfg->tol;
            }
        }
        if (crit_vals) crit_vals[ii] = cval;
        if (stop) break;
        memcpy(sv_old, sv, (size_t)nsv * sizeof(double));
        if (cfg->crit == 2) memcpy(old, omega, nk * sizeof(double));
    }
#undef PASS
    *its_out = ii < miter ? ii + 1 : ii;
    memcpy(sigma, sv, (size_t)nsv * sizeof(double));
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < nsv; ++j) u[(size_t)i * nsv + j] = omega[(size_t)i * k + j];
    if (timers) {
        timers[0] = c.t_load;
        timers[1] = c.t_mm_a;
        timers[2] = c.t_mm_at;
        timers[3] = t_qr;
        timers[4] = t_rr;
        timers[5] = oracle_now() - t_begin;
    }
    free(z); free(q); free(old); free(tau); free(b); free(wv); free(w);
    free(sv); free(sv_old); free(delta); free(xfull); free(yfull);
    oracle_ctx_free(&c);
    return 0;
}

void oracle_set_threads(int n) { scipy_openblas_set_num_threads(n); }
