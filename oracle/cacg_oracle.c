/*
 * cacg_oracle.c -- CPU restatement of the sclc/cacg CA Chebyshev-basis CG hot
 * path, written for this project as the ORACLE of the GPU implementation.
 *
 * Test infrastructure only: loaded by tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py, never by the cacg_gb300 product.
 *
 * Every function follows one reference routine statement for statement in
 * the same loop and accumulation order, so that (built with
 * -ffp-contract=off) it reproduces the reference bit for bit on one rank.
 * That equality is pinned by tests/test_oracle_pins.py against
 * oracle/_ref/libcacgref.so and the committed fixtures in tests/golden/.
 *
 * Layout: dense blocks are row-major (element (i, c) at i*ncols + c), the
 * reference's layout (src/GetRHS.c:8, src/BLAS3.c:103-104); CSR indices are
 * int32 (the reference uses long, src/DataTypes.h:28-40; values are equal).
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* src/common.c:53-106 gerschgorin_v1 (one rank; out[0]=min, out[1]=max).
 * Note the reference initialises the running max with DBL_MIN. */
void or_gerschgorin(int64_t n, const int32_t *rp, const int32_t *ci, const double *v,
                    double *out) {
    double local_max = DBL_MIN;
    double local_min = DBL_MAX;
    for (int64_t i = 0; i < n; i++) {
        double acc = 0.0, diag = 0.0;
        for (int64_t e = rp[i]; e < rp[i + 1]; e++) {
            if (i != ci[e])
                acc += (v[e] > 0 ? v[e] : -v[e]);
            else
                diag = v[e];
        }
        if (local_max < (acc + diag)) local_max = acc + diag;
        if (local_min > (diag - acc)) local_min = diag - acc;
    }
    out[0] = local_min;
    out[1] = local_max;
}

/* src/BLAS3.c:78-112 (spmm_csr_v1) == :207-222 (spmm_csr_v2): Y = A X,
 * X is n x w row-major with row stride ldx, Y row stride ldy. */
void or_spmm(int64_t n, const int32_t *rp, const int32_t *ci, const double *v,
             const double *X, int64_t ldx, int64_t w, double *Y, int64_t ldy) {
    for (int64_t i = 0; i < n; i++) {
        double *y = Y + i * ldy;
        for (int64_t c = 0; c < w; c++) y[c] = 0.0;
        for (int64_t e = rp[i]; e < rp[i + 1]; e++) {
            int64_t col = ci[e];
            double a = v[e];
            for (int64_t c = 0; c < w; c++) y[c] += a * X[col * ldx + c];
        }
    }
}

/* src/common.c:182-256 (BCBCG) and :109-179 (CBCG, m == 1): Chebyshev basis.
 *   T0 = R; T1 = alpha*(A R) + beta*R                (src/BLAS3.c:843-844)
 *   Tj = 2alpha*(A Tj-1) + 2beta*Tj-1 + (-1)*Tj-2   (src/BLAS3.c:989-991)
 * then the chunk transpose (src/MatrixOperations.c:70-92): S[i, j*m + c] = Tj[i, c].
 * S is n x (s*m) row-major. */
void or_basis(int64_t n, const int32_t *rp, const int32_t *ci, const double *v,
              const double *R, int64_t m, int64_t s, double alpha, double beta,
              double *S) {
    int64_t chunk = n * m;
    double *T = (double *)calloc((size_t)(chunk * s), sizeof(double));
    double *AT = (double *)calloc((size_t)chunk, sizeof(double));
    double a2 = 2.0 * alpha, b2 = 2.0 * beta;
    for (int64_t j = 0; j < s; j++) {
        double *Tj = T + j * chunk;
        if (j == 0) {
            memcpy(Tj, R, (size_t)chunk * sizeof(double));
        } else if (j == 1) {
            or_spmm(n, rp, ci, v, R, m, m, AT, m);
            for (int64_t q = 0; q < chunk; q++) Tj[q] = alpha * AT[q] + beta * R[q];
        } else {
            const double *T1 = T + (j - 1) * chunk, *T2 = T + (j - 2) * chunk;
            or_spmm(n, rp, ci, v, T1, m, m, AT, m);
            for (int64_t q = 0; q < chunk; q++)
                Tj[q] = a2 * AT[q] + b2 * T1[q] + -1.0 * T2[q];
        }
    }
    for (int64_t i = 0; i < n; i++)
        for (int64_t j = 0; j < s; j++)
            for (int64_t c = 0; c < m; c++)
                S[i * s * m + j * m + c] = T[j * chunk + i * m + c];
    free(T);
    free(AT);
}

/* src/BLAS3.c:730-758 distributedMatLTransposeMatRMul_updated (one rank):
 * C (ka x kb) = L^T R; L n x ka, R n x kb, row-major.  Loop order k, row, col.
 * (src/BLAS3.c:699-726, the square variant, computes the same thing in the
 * same order.) */
void or_gram(int64_t n, const double *L, int64_t ka, const double *R, int64_t kb,
             double *C) {
    memset(C, 0, (size_t)(ka * kb) * sizeof(double));
    for (int64_t k = 0; k < n; k++)
        for (int64_t r = 0; r < ka; r++) {
            double t = L[k * ka + r];
            for (int64_t c = 0; c < kb; c++) C[r * kb + c] += R[k * kb + c] * t;
        }
}

/* src/BLAS3.c:794-825 dense_distributedMatL_localMatR_Mul_v1: Y = L W,
 * L n x ka, W ka x kb.  Loop order row, k, col. */
void or_tallsmall(int64_t n, const double *L, int64_t ka, const double *W, int64_t kb,
                  double *Y) {
    memset(Y, 0, (size_t)(n * kb) * sizeof(double));
    for (int64_t i = 0; i < n; i++)
        for (int64_t k = 0; k < ka; k++) {
            double t = L[i * ka + k];
            for (int64_t c = 0; c < kb; c++) Y[i * kb + c] += W[k * kb + c] * t;
        }
}

/* src/DLSsolvers.c:106-208 LUsolver_v1_KeeplhsMat: Crout LU with unit-diagonal
 * U and no pivoting, then forward (divide by L's diagonal through a
 * reciprocal) and backward substitution.  M is k x k, RHS and Y are k x r. */
void or_lu(int64_t k, const double *M, int64_t r, const double *RHS, double *Y) {
    double *L = (double *)malloc((size_t)(k * k) * sizeof(double));
    double *Z = (double *)calloc((size_t)(k * r), sizeof(double));
    memcpy(L, M, (size_t)(k * k) * sizeof(double));
    for (int64_t d = 0; d < k; d++) {
        double inv = 1.0 / L[d * k + d];
        for (int64_t c = d + 1; c < k; c++) L[d * k + c] *= inv;
        for (int64_t i = d + 1; i < k; i++) {
            double p = L[i * k + d];
            for (int64_t c = d + 1; c < k; c++) L[i * k + c] = L[i * k + c] - p * L[d * k + c];
        }
    }
    for (int64_t i = 0; i < k; i++) {
        for (int64_t j = 0; j < r; j++) Z[i * r + j] = RHS[i * r + j];
        for (int64_t q = 0; q < i; q++) {
            double l = L[i * k + q];
            for (int64_t j = 0; j < r; j++) Z[i * r + j] -= Z[q * r + j] * l;
        }
        double inv = 1.0 / L[i * k + i];
        for (int64_t j = 0; j < r; j++) Z[i * r + j] *= inv;
    }
    for (int64_t j = 0; j < r; j++) Y[(k - 1) * r + j] = Z[(k - 1) * r + j];
    for (int64_t i = k - 2; i >= 0; i--) {
        for (int64_t j = 0; j < r; j++) Y[i * r + j] = Z[i * r + j];
        for (int64_t q = i + 1; q < k; q++) {
            double u = L[i * k + q];
            for (int64_t j = 0; j < r; j++) Y[i * r + j] -= Y[q * r + j] * u;
        }
    }
    free(L);
    free(Z);
}

/*
 * src/bcbcgKernel.c:27-556 bcbcg_v1 (and src/cbcgKernel.c:23-250 cbcg_v1,
 * which is the same sequence for m == 1) on one rank:
 *   bounds (Gerschgorin, or injected as the harness does), s_alpha, s_beta
 *   R = B - A X
 *   loop: S = basis(R); it 0: Q = S; else QtAS = AQ^T S, beta = LU(QtAQ, QtAS),
 *         Q = S - Q beta;  AQ = A Q;  QtAQ = Q^T AQ;  QtR = Q^T R;
 *         alpha = LU(QtAQ, QtR);  X += Q alpha;  R -= AQ alpha;
 *         stop when sqrt(||R(:,0)||^2) < eps.
 * Returns the number of outer iterations executed; hist (may be NULL) gets
 * ||R(:,0)|| per iteration.
 */
int64_t or_solve(int64_t n, const int32_t *rp, const int32_t *ci, const double *v,
                 const double *B, double *X, int64_t m, int64_t s, double eps,
                 int bounds_mode, double lmin, double lmax, int64_t maxit, double *hist,
                 int64_t hist_cap) {
    int64_t k = s * m;
    double bnd[2];
    if (bounds_mode == 0) {
        or_gerschgorin(n, rp, ci, v, bnd);
    } else {
        bnd[0] = lmin;
        bnd[1] = lmax;
    }
    double sa = 2.0 / (bnd[1] - bnd[0]);
    double sb = -(bnd[1] + bnd[0]) / (bnd[1] - bnd[0]);

    double *R = (double *)malloc((size_t)(n * m) * sizeof(double));
    double *AX = (double *)malloc((size_t)(n * m) * sizeof(double));
    double *S = (double *)calloc((size_t)(n * k), sizeof(double));
    double *Q = (double *)calloc((size_t)(n * k), sizeof(double));
    double *AQ = (double *)calloc((size_t)(n * k), sizeof(double));
    double *Qb = (double *)calloc((size_t)(n * k), sizeof(double));
    double *Qa = (double *)calloc((size_t)(n * m), sizeof(double));
    double *AQa = (double *)calloc((size_t)(n * m), sizeof(double));
    double *QtAQ = (double *)calloc((size_t)(k * k), sizeof(double));
    double *QtAS = (double *)calloc((size_t)(k * k), sizeof(double));
    double *QtR = (double *)calloc((size_t)(k * m), sizeof(double));
    double *al = (double *)calloc((size_t)(k * m), sizeof(double));
    double *be = (double *)calloc((size_t)(k * k), sizeof(double));

    or_spmm(n, rp, ci, v, X, m, m, AX, m);
    for (int64_t q = 0; q < n * m; q++) R[q] = 1.0 * B[q] + -1.0 * AX[q];

    int64_t it;
    for (it = 0; it < maxit; it++) {
        or_basis(n, rp, ci, v, R, m, s, sa, sb, S);
        if (it == 0) {
            double *t = Q; Q = S; S = t;
        } else {
            or_gram(n, AQ, k, S, k, QtAS);
            or_lu(k, QtAQ, k, QtAS, be);
            or_tallsmall(n, Q, k, be, k, Qb);
            for (int64_t q = 0; q < n * k; q++) Q[q] = 1.0 * S[q] + -1.0 * Qb[q];
        }
        or_spmm(n, rp, ci, v, Q, k, k, AQ, k);
        or_gram(n, Q, k, AQ, k, QtAQ);
        or_gram(n, Q, k, R, m, QtR);
        or_lu(k, QtAQ, m, QtR, al);
        or_tallsmall(n, Q, k, al, m, Qa);
        or_tallsmall(n, AQ, k, al, m, AQa);
        for (int64_t q = 0; q < n * m; q++) X[q] = 1.0 * X[q] + 1.0 * Qa[q];
        for (int64_t q = 0; q < n * m; q++) R[q] = 1.0 * R[q] + -1.0 * AQa[q];
        double nr = 0.0;
        for (int64_t i = 0; i < n; i++) nr += R[i * m] * R[i * m];
        if (hist && it < hist_cap) hist[it] = sqrt(nr);
        if (sqrt(nr) < eps) {
            it++;
            break;
        }
    }
    free(R); free(AX); free(S); free(Q); free(AQ); free(Qb); free(Qa); free(AQa);
    free(QtAQ); free(QtAS); free(QtR); free(al); free(be);
    return it;
}

/* True residual ||b_c - A x_c||_2 / ||b_c||_2 per column (FP64, no reference
 * counterpart: the reference never forms the true residual). */
void or_true_relres(int64_t n, const int32_t *rp, const int32_t *ci, const double *v,
                    const double *B, const double *X, int64_t m, double *out) {
    double *AX = (double *)malloc((size_t)(n * m) * sizeof(double));
    or_spmm(n, rp, ci, v, X, m, m, AX, m);
    for (int64_t c = 0; c < m; c++) {
        double num = 0.0, den = 0.0;
        for (int64_t i = 0; i < n; i++) {
            double r = B[i * m + c] - AX[i * m + c];
            num += r * r;
            den += B[i * m + c] * B[i * m + c];
        }
        out[c] = den > 0 ? sqrt(num / den) : sqrt(num);
    }
    free(AX);
}
