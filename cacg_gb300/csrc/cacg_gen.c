/*
 * cacg_gen.c -- seeded synthetic SPD systems and right-hand sides.
 *
 * Shared verbatim by the GPU library (libcacg.so) and the CPU oracle
 * (liboracle.so), so both consume bit-identical CSR arrays and RHS blocks.
 * Compiled with -ffp-contract=off and without libm transcendentals (log/exp
 * below are written out from their series), so x86-64 and aarch64 hosts
 * generate identical bits.
 *
 * Layout: CSR with int32 row_ptr/col_idx, double values, rows in
 * lexicographic grid order (x fastest), columns ascending within a row,
 * Dirichlet boundaries (neighbours outside the grid are dropped).  RHS blocks
 * are n x m row-major (element (i, c) at i*m + c), the reference's layout
 * (src/GetRHS.c:8, src/BLAS3.c:103-104).
 *
 * RNG: splitmix64 stream; u01 = (next >> 11) * 2^-53 in [0, 1);
 * normal = Marsaglia polar method (pairs, rejection on s >= 1 or s == 0);
 * lognormal(0, sigma) = exp(sigma * normal);
 * Beta(2, 5) = second-smallest of six u01 draws (order statistic).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "cacg.h"

typedef struct {
    uint64_t s;
    int have_spare;
    double spare;
} rng_t;

static uint64_t sm64_next(rng_t *r) {
    uint64_t z = (r->s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

static void rng_init(rng_t *r, uint64_t seed, uint64_t tag) {
    r->s = seed ^ (tag * 0xD1B54A32D192ED03ULL);
    r->have_spare = 0;
    r->spare = 0.0;
    (void)sm64_next(r);
}

static double u01(rng_t *r) { return (double)(sm64_next(r) >> 11) * 0x1.0p-53; }

static const double LN2_HI = 6.93147180369123816490e-01;
static const double LN2_LO = 1.90821492927058770002e-10;

/* natural log of x > 0: x = f 2^e, f in [sqrt(1/2), sqrt(2)),
 * log f = 2 atanh((f-1)/(f+1)) summed to 40 terms (|t| <= 0.1716). */
double cacg_det_log(double x) {
    int e;
    double f = frexp(x, &e);
    if (f < 0.70710678118654752440) {
        f = f * 2.0;
        e -= 1;
    }
    double t = (f - 1.0) / (f + 1.0);
    double t2 = t * t;
    double term = t, sum = 0.0;
    for (int k = 0; k < 40; k++) {
        sum = sum + term / (double)(2 * k + 1);
        term = term * t2;
    }
    return (double)e * LN2_HI + ((double)e * LN2_LO + 2.0 * sum);
}

/* exp(x): x = k ln2 + r, |r| <= ln2/2, Taylor series to 30 terms, scaled by 2^k. */
double cacg_det_exp(double x) {
    if (x > 709.0) return HUGE_VAL;
    if (x < -745.0) return 0.0;
    double k = floor(x * 1.44269504088896338700 + 0.5);
    double r = (x - k * LN2_HI) - k * LN2_LO;
    double term = 1.0, sum = 1.0;
    for (int i = 1; i < 30; i++) {
        term = term * r / (double)i;
        sum = sum + term;
    }
    return ldexp(sum, (int)k);
}

static double normal01(rng_t *r) {
    if (r->have_spare) {
        r->have_spare = 0;
        return r->spare;
    }
    double u, v, s;
    do {
        u = 2.0 * u01(r) - 1.0;
        v = 2.0 * u01(r) - 1.0;
        s = u * u + v * v;
    } while (s >= 1.0 || s == 0.0);
    double f = sqrt(-2.0 * cacg_det_log(s) / s);
    r->spare = v * f;
    r->have_spare = 1;
    return u * f;
}

static double beta25(rng_t *r) {
    /* second-smallest of six uniforms ~ Beta(2, 5) */
    double a = 2.0, b = 2.0; /* a <= b: the two smallest so far */
    for (int i = 0; i < 6; i++) {
        double x = u01(r);
        if (x < a) {
            b = a;
            a = x;
        } else if (x < b) {
            b = x;
        }
    }
    return b;
}

int64_t cacg_gen_rows(int kind, int64_t N) {
    switch (kind) {
    case CACG_GEN_LAPLACE2D_5PT:
    case CACG_GEN_VARCOEF2D_5PT: return N * N;
    case CACG_GEN_LAPLACE3D_7PT:
    case CACG_GEN_STENCIL3D_27PT: return N * N * N;
    default: return -1;
    }
}

int64_t cacg_gen_nnz(int kind, int64_t N) {
    switch (kind) {
    case CACG_GEN_LAPLACE2D_5PT:
    case CACG_GEN_VARCOEF2D_5PT: return 5 * N * N - 4 * N;
    case CACG_GEN_LAPLACE3D_7PT: return 7 * N * N * N - 6 * N * N;
    case CACG_GEN_STENCIL3D_27PT: return (3 * N - 2) * (3 * N - 2) * (3 * N - 2);
    default: return -1;
    }
}

/*
 * Fill row_ptr (n+1), col_idx (nnz), val (nnz).
 *   LAPLACE2D_5PT : diag 4 + shift, neighbours -1
 *   LAPLACE3D_7PT : diag 6 + shift, neighbours -1
 *   STENCIL3D_27PT: diag 26 + shift, the 26 cube neighbours -1
 *   VARCOEF2D_5PT : -div(c grad u) with edge conductivities c ~ lognormal(0, sigma)
 *                   (stream seed/tag 1: the N(N+1) x-edges row by row, then the
 *                   N(N+1) y-edges); diag = sum of the 4 incident edges
 *                   (boundary edges included) + shift.
 * Returns 0, or -1 for bad arguments / index overflow of int32.
 */
int cacg_gen_matrix(int kind, int64_t N, double shift, double sigma, uint64_t seed,
                    int32_t *row_ptr, int32_t *col_idx, double *val) {
    int64_t n = cacg_gen_rows(kind, N);
    int64_t nnz = cacg_gen_nnz(kind, N);
    if (n <= 0 || nnz <= 0 || nnz > INT32_MAX || n > INT32_MAX) return -1;
    int64_t p = 0;
    if (kind == CACG_GEN_LAPLACE2D_5PT) {
        for (int64_t y = 0; y < N; y++)
            for (int64_t x = 0; x < N; x++) {
                int64_t i = x + N * y;
                row_ptr[i] = (int32_t)p;
                if (y > 0) { col_idx[p] = (int32_t)(i - N); val[p++] = -1.0; }
                if (x > 0) { col_idx[p] = (int32_t)(i - 1); val[p++] = -1.0; }
                col_idx[p] = (int32_t)i; val[p++] = 4.0 + shift;
                if (x < N - 1) { col_idx[p] = (int32_t)(i + 1); val[p++] = -1.0; }
                if (y < N - 1) { col_idx[p] = (int32_t)(i + N); val[p++] = -1.0; }
            }
    } else if (kind == CACG_GEN_LAPLACE3D_7PT) {
        int64_t N2 = N * N;
        for (int64_t z = 0; z < N; z++)
            for (int64_t y = 0; y < N; y++)
                for (int64_t x = 0; x < N; x++) {
                    int64_t i = x + N * y + N2 * z;
                    row_ptr[i] = (int32_t)p;
                    if (z > 0) { col_idx[p] = (int32_t)(i - N2); val[p++] = -1.0; }
                    if (y > 0) { col_idx[p] = (int32_t)(i - N); val[p++] = -1.0; }
                    if (x > 0) { col_idx[p] = (int32_t)(i - 1); val[p++] = -1.0; }
                    col_idx[p] = (int32_t)i; val[p++] = 6.0 + shift;
                    if (x < N - 1) { col_idx[p] = (int32_t)(i + 1); val[p++] = -1.0; }
                    if (y < N - 1) { col_idx[p] = (int32_t)(i + N); val[p++] = -1.0; }
                    if (z < N - 1) { col_idx[p] = (int32_t)(i + N2); val[p++] = -1.0; }
                }
    } else if (kind == CACG_GEN_STENCIL3D_27PT) {
        int64_t N2 = N * N;
        for (int64_t z = 0; z < N; z++)
            for (int64_t y = 0; y < N; y++)
                for (int64_t x = 0; x < N; x++) {
                    int64_t i = x + N * y + N2 * z;
                    row_ptr[i] = (int32_t)p;
                    for (int dz = -1; dz <= 1; dz++) {
                        if (z + dz < 0 || z + dz >= N) continue;
                        for (int dy = -1; dy <= 1; dy++) {
                            if (y + dy < 0 || y + dy >= N) continue;
                            for (int dx = -1; dx <= 1; dx++) {
                                if (x + dx < 0 || x + dx >= N) continue;
                                int64_t j = i + dx + N * dy + N2 * dz;
                                col_idx[p] = (int32_t)j;
                                val[p++] = (j == i) ? 26.0 + shift : -1.0;
                            }
                        }
                    }
                }
    } else if (kind == CACG_GEN_VARCOEF2D_5PT) {
        /* cx[y*(N+1) + e]: edge between x = e-1 and x = e in row y;
         * cy[e*N + x]    : edge between y = e-1 and y = e in column x. */
        rng_t r;
        rng_init(&r, seed, 1);
        int64_t ncx = N * (N + 1);
        double *cx = (double *)malloc((size_t)(2 * ncx) * sizeof(double));
        if (!cx) return -1;
        double *cy = cx + ncx;
        for (int64_t e = 0; e < ncx; e++) cx[e] = cacg_det_exp(sigma * normal01(&r));
        for (int64_t e = 0; e < ncx; e++) cy[e] = cacg_det_exp(sigma * normal01(&r));
        for (int64_t y = 0; y < N; y++)
            for (int64_t x = 0; x < N; x++) {
                int64_t i = x + N * y;
                double w = cx[y * (N + 1) + x];
                double e_ = cx[y * (N + 1) + x + 1];
                double s_ = cy[y * N + x];
                double n_ = cy[(y + 1) * N + x];
                row_ptr[i] = (int32_t)p;
                if (y > 0) { col_idx[p] = (int32_t)(i - N); val[p++] = -s_; }
                if (x > 0) { col_idx[p] = (int32_t)(i - 1); val[p++] = -w; }
                col_idx[p] = (int32_t)i; val[p++] = ((w + e_) + (s_ + n_)) + shift;
                if (x < N - 1) { col_idx[p] = (int32_t)(i + 1); val[p++] = -e_; }
                if (y < N - 1) { col_idx[p] = (int32_t)(i + N); val[p++] = -n_; }
            }
        free(cx);
    } else {
        return -1;
    }
    row_ptr[n] = (int32_t)p;
    return p == nnz ? 0 : -1;
}

/*
 * n x m row-major block; element (i, c) is draw number i*m + c of the stream
 * (seed, tag 2).  dist: CACG_RHS_UNIFORM -> U[a, b); CACG_RHS_NORMAL -> N(0,1);
 * CACG_RHS_BETA25 -> Beta(2, 5); CACG_RHS_ONES -> 1.
 */
int cacg_gen_rhs(int dist, int64_t n, int m, uint64_t seed, double a, double b,
                 double *out) {
    if (n <= 0 || m <= 0) return -1;
    rng_t r;
    rng_init(&r, seed, 2);
    int64_t tot = n * (int64_t)m;
    for (int64_t i = 0; i < tot; i++) {
        switch (dist) {
        case CACG_RHS_UNIFORM: out[i] = a + (b - a) * u01(&r); break;
        case CACG_RHS_NORMAL: out[i] = normal01(&r); break;
        case CACG_RHS_BETA25: out[i] = beta25(&r); break;
        case CACG_RHS_ONES: out[i] = 1.0; break;
        default: return -1;
        }
    }
    return 0;
}
