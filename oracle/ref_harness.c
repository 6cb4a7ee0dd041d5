/*
 * ref_harness.c -- drives the reference CPU solver (sclc/cacg src/*.c, built
 * unmodified apart from the MAXITER constants by oracle/build_ref.py) so that
 * it can serve as the oracle and as the timed CPU baseline.
 *
 * Oracle/test infrastructure: only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py load the library built from this file.
 *
 * What the harness adds around the reference code, all by link-level
 * interposition (no reference statement is changed):
 *   - gerschgorin_v1 (src/common.c:53) is compiled as gerschgorin_v1_ref and
 *     this file supplies gerschgorin_v1: it returns either the reference's own
 *     Gerschgorin bounds or bounds injected by the caller (analytic, given,
 *     Lanczos), which is how the configurations choose their Chebyshev
 *     interval while the reference solvers still compute
 *     s_alpha/s_beta themselves (src/bcbcgKernel.c:113-115).
 *   - norm2square_dist_denseMat_col_n (src/MatrixOperations.c:110), as called
 *     from the two solver loops (src/bcbcgKernel.c:447, src/cbcgKernel.c:214),
 *     is routed through cacg_ref_norm_hook, which records the per-iteration
 *     residual norm history -- the reference returns nothing else.
 *   - MAXITER / CBCG_MAXITER (src/bcbcgKernel.c:3, src/cbcgKernel.c:2) read
 *     the variable cacg_ref_maxiter (shipped values: 100 and 1000).
 *   - Block-row distribution over ranks follows
 *     src/SparseMatrixDistribution.c:64-87 (rows_per = n/np, the last rank takes
 *     the remainder; global column indices; mat.start = first global row).
 */
#include <fcntl.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include "mpi.h"
#include "DataTypes.h"

/* reference entry points (src/bcbcgKernel.h:22, src/cbcgKernel.h:21, ...) */
void bcbcg_v1(csrType_local mat, denseType B, denseType X, long s, double epsilon,
              int myid, int numprocs);
void cbcg_v1(csrType_local mat, denseType B, denseType X, long s, double epsilon,
             int myid, int numprocs);
void gerschgorin_v1_ref(double *output, csrType_local mat);
void norm2square_dist_denseMat_col_n(denseType mat, double *result, long n,
                                     int myid, int numprocs);
void BCBCG_chebyshevPolynomialBasisGen(denseType S_mat, csrType_local mat, denseType R,
                                       long s, double s_alpha, double s_beta,
                                       int myid, int numprocs);
void CBCG_chebyshevPolynomialBasisGen(denseType S_mat, csrType_local mat, denseType R,
                                      long s, double s_alpha, double s_beta,
                                      int myid, int numprocs);
void spmm_csr_v2(csrType_local csr_mat, denseType dense_mat, denseType *res_mat,
                 int myid, int numprocs);
void distributedMatLTransposeMatRMul_updated(denseType *resMat, denseType matL,
                                             denseType matR, int myid, int numprocs);
void distributedMatLTransposeMatRMul(denseType *resMat, denseType matL,
                                     denseType matR, int myid, int numprocs);
void dense_distributedMatL_localMatR_Mul_v1(denseType *res_mat, denseType matDistL,
                                            denseType matLocalR, int myid, int numprocs);
void LUsolver_v1_KeeplhsMat(denseType *resMat, denseType lhsMatdb, denseType rhsMat,
                            int myid, int numprocs);

long cacg_ref_maxiter = 100;

static int g_bounds_mode = 0; /* 0: reference Gerschgorin, 1: injected */
static double g_bounds[2];

void gerschgorin_v1(double *output, csrType_local mat) {
    if (g_bounds_mode == 0) {
        gerschgorin_v1_ref(output, mat);
    } else {
        output[0] = g_bounds[0];
        output[1] = g_bounds[1];
    }
}

#define HIST_CAP 100000
static long g_iters = 0;
static double *g_hist = NULL;

void cacg_ref_norm_hook(denseType mat, double *result, long n, int myid, int numprocs) {
    norm2square_dist_denseMat_col_n(mat, result, n, myid, numprocs);
    if (myid == 0) {
        if (g_hist && g_iters < HIST_CAP) g_hist[g_iters] = sqrt(*result);
        g_iters++;
    }
}

void bcg_v1(csrType_local mat, denseType B, denseType X, double epsilon, int myid,
            int numprocs);

/* src/bcgKernel.c:597 bcg_Scalapack_qr (never called by bcg_v1) refers to
 * BLACS/ScaLAPACK, which this build does not have: these stand-ins satisfy
 * the link and stop the process if that path were ever reached. */
static void no_scalapack(void) {
    fprintf(stderr, "oracle: ScaLAPACK path of src/bcgKernel.c is not built\n");
    abort();
}
void Cblacs_pinfo(long *a, long *b) { (void)a; (void)b; no_scalapack(); }
void Cblacs_get(long a, long b, long *c) { (void)a; (void)b; (void)c; no_scalapack(); }
void Cblacs_gridinfo(long a, long *b, long *c, long *d, long *e) {
    (void)a; (void)b; (void)c; (void)d; (void)e; no_scalapack();
}
void Cblacs_gridmap(void) { no_scalapack(); }
void descinit_(void) { no_scalapack(); }
long numroc_(void) { no_scalapack(); return 0; }

typedef struct {
    int solver; /* 1 = cbcg_v1, 2 = bcbcg_v1, 3 = bcg_v1 */
    long n, m, s;
    const long *row_ptr, *col_idx;
    const double *val, *B;
    double *X;
    double eps;
    double seconds;
} job_t;

static void rank_body(int rank, void *p) {
    job_t *j = (job_t *)p;
    int np;
    MPI_Comm_size(MPI_COMM_WORLD, &np);
    long rows_per = j->n / np;
    long start = (long)rank * rows_per;
    long nloc = (rank == np - 1) ? j->n - rows_per * (np - 1) : rows_per;

    csrType_local A;
    A.num_rows = nloc;
    A.num_cols = j->n;
    A.start = start;
    long base = j->row_ptr[start];
    A.nnz = j->row_ptr[start + nloc] - base;
    A.row_start = (long *)malloc((size_t)(nloc + 1) * sizeof(long));
    for (long i = 0; i <= nloc; i++) A.row_start[i] = j->row_ptr[start + i] - base;
    A.col_idx = (long *)(j->col_idx + base);
    A.csrdata = (double *)(j->val + base);

    denseType B, X;
    B.local_num_row = X.local_num_row = nloc;
    B.local_num_col = X.local_num_col = j->m;
    B.global_num_row = X.global_num_row = j->n;
    B.global_num_col = X.global_num_col = j->m;
    B.start_idx = X.start_idx = start;
    size_t bytes = (size_t)nloc * (size_t)j->m * sizeof(double);
    B.data = (double *)malloc(bytes);
    X.data = (double *)malloc(bytes);
    memcpy(B.data, j->B + start * j->m, bytes);
    memcpy(X.data, j->X + start * j->m, bytes);

    MPI_Barrier(MPI_COMM_WORLD);
    double t0 = MPI_Wtime();
    if (j->solver == 1)
        cbcg_v1(A, B, X, j->s, j->eps, rank, np);
    else if (j->solver == 3)
        bcg_v1(A, B, X, j->eps, rank, np);
    else
        bcbcg_v1(A, B, X, j->s, j->eps, rank, np);
    MPI_Barrier(MPI_COMM_WORLD);
    double t1 = MPI_Wtime();
    if (rank == 0) j->seconds = t1 - t0;

    memcpy(j->X + start * j->m, X.data, bytes);
    free(A.row_start);
    free(B.data);
    free(X.data);
}

/*
 * Run the reference solver.  solver: 1 = cbcg_v1 (m must be 1), 2 = bcbcg_v1,
 * 3 = bcg_v1 (block CG, no s).
 * bounds_mode 0 = the reference's Gerschgorin bounds, 1 = [lmin, lmax].
 * eps is the reference's absolute threshold on ||R(:,0)||.  X is in/out.
 * hist (capacity hist_cap, may be NULL) receives ||R(:,0)|| per outer
 * iteration.  quiet != 0 silences the reference's printf output.
 * Returns the number of outer iterations executed; *seconds = solver wall time.
 */
long cacg_ref_solve(int solver, int nranks, long n, const long *row_ptr,
                    const long *col_idx, const double *val, const double *B,
                    double *X, long m, long s, double eps, int bounds_mode,
                    double lmin, double lmax, long maxit, double *hist,
                    long hist_cap, int quiet, double *seconds) {
    job_t j;
    j.solver = solver; j.n = n; j.m = m; j.s = s;
    j.row_ptr = row_ptr; j.col_idx = col_idx; j.val = val; j.B = B; j.X = X;
    j.eps = eps; j.seconds = 0.0;
    g_bounds_mode = bounds_mode;
    g_bounds[0] = lmin;
    g_bounds[1] = lmax;
    cacg_ref_maxiter = maxit;
    g_iters = 0;
    double *tmp = (double *)calloc(HIST_CAP, sizeof(double));
    g_hist = tmp;

    int saved = -1;
    if (quiet) {
        fflush(stdout);
        saved = dup(1);
        int dn = open("/dev/null", O_WRONLY);
        if (dn >= 0) { dup2(dn, 1); close(dn); }
    }
    cacg_mpi_run(nranks, rank_body, &j);
    if (quiet && saved >= 0) {
        fflush(stdout);
        dup2(saved, 1);
        close(saved);
    }
    long it = g_iters;
    if (hist) {
        long c = it < hist_cap ? it : hist_cap;
        if (c > HIST_CAP) c = HIST_CAP;
        memcpy(hist, tmp, (size_t)c * sizeof(double));
    }
    g_hist = NULL;
    free(tmp);
    if (seconds) *seconds = j.seconds;
    return it;
}

/* ---- single-rank kernel entry points, for per-kernel golden vectors ---- */

static csrType_local make_csr(long n, const long *rp, const long *ci, const double *v) {
    csrType_local A;
    A.num_rows = n; A.num_cols = n; A.nnz = rp[n]; A.start = 0;
    A.row_start = (long *)rp; A.col_idx = (long *)ci; A.csrdata = (double *)v;
    return A;
}

static denseType make_dense(long r, long c, double *data) {
    denseType D;
    D.local_num_row = D.global_num_row = r;
    D.local_num_col = D.global_num_col = c;
    D.start_idx = 0;
    D.data = data;
    return D;
}

/* src/common.c:53 as shipped: out[0] = min, out[1] = max */
void cacg_ref_gerschgorin(long n, const long *rp, const long *ci, const double *v,
                          double *out) {
    gerschgorin_v1_ref(out, make_csr(n, rp, ci, v));
}

/* src/common.c:182 (m > 1 or m == 1) / src/common.c:109 (cbcg == 1, m == 1):
 * S (n x s*m, row-major) from R (n x m). */
void cacg_ref_basis(int cbcg, long n, const long *rp, const long *ci, const double *v,
                    const double *R, long m, long s, double alpha, double beta,
                    double *S) {
    double *Rc = (double *)malloc((size_t)n * m * sizeof(double));
    memcpy(Rc, R, (size_t)n * m * sizeof(double));
    denseType Rd = make_dense(n, m, Rc);
    denseType Sd = make_dense(n, s * m, S);
    if (cbcg)
        CBCG_chebyshevPolynomialBasisGen(Sd, make_csr(n, rp, ci, v), Rd, s, alpha, beta, 0, 1);
    else
        BCBCG_chebyshevPolynomialBasisGen(Sd, make_csr(n, rp, ci, v), Rd, s, alpha, beta, 0, 1);
    free(Rc);
}

/* src/BLAS3.c:157 spmm_csr_v2: Y (n x w) = A X */
void cacg_ref_spmm(long n, const long *rp, const long *ci, const double *v,
                   const double *X, long w, double *Y) {
    double *Xc = (double *)malloc((size_t)n * w * sizeof(double));
    memcpy(Xc, X, (size_t)n * w * sizeof(double));
    denseType Xd = make_dense(n, w, Xc);
    denseType Yd = make_dense(n, w, (double *)calloc((size_t)n * w, sizeof(double)));
    spmm_csr_v2(make_csr(n, rp, ci, v), Xd, &Yd, 0, 1);
    memcpy(Y, Yd.data, (size_t)n * w * sizeof(double));
    free(Yd.data);
    free(Xc);
}

/* src/BLAS3.c:730 (sym == 0) or src/BLAS3.c:699 (sym == 1, ka == kb):
 * C (ka x kb) = L^T R with L n x ka, R n x kb */
void cacg_ref_gram(int square, long n, const double *L, long ka, const double *R,
                   long kb, double *C) {
    denseType Ld = make_dense(n, ka, (double *)L);
    denseType Rd = make_dense(n, kb, (double *)R);
    denseType Cd = make_dense(ka, kb, C);
    if (square)
        distributedMatLTransposeMatRMul(&Cd, Ld, Rd, 0, 1);
    else
        distributedMatLTransposeMatRMul_updated(&Cd, Ld, Rd, 0, 1);
}

/* src/BLAS3.c:794: Y (n x kb) = L (n x ka) * W (ka x kb) */
void cacg_ref_tallsmall(long n, const double *L, long ka, const double *W, long kb,
                        double *Y) {
    denseType Ld = make_dense(n, ka, (double *)L);
    denseType Wd = make_dense(ka, kb, (double *)W);
    denseType Yd = make_dense(n, kb, (double *)calloc((size_t)n * kb, sizeof(double)));
    dense_distributedMatL_localMatR_Mul_v1(&Yd, Ld, Wd, 0, 1);
    memcpy(Y, Yd.data, (size_t)n * kb * sizeof(double));
    free(Yd.data);
}

/* src/DLSsolvers.c:106: Y (k x r) solves M Y = RHS by no-pivot Crout LU */
void cacg_ref_lu(long k, const double *M, long r, const double *RHS, double *Y) {
    denseType Md = make_dense(k, k, (double *)M);
    denseType Rd = make_dense(k, r, (double *)RHS);
    denseType Yd = make_dense(k, r, Y);
    LUsolver_v1_KeeplhsMat(&Yd, Md, Rd, 0, 1);
}

/* ---------------------------------------------------------- input files */
void readMtx_info_and_coo(char *path, char *name, matInfo *info, cooType *mat);
void Converter_Coo2Csr(cooType src, csrType_local *target, matInfo *mat_info);
void parseCSV(char *filename, double **output, long numRows, long numCols);

/* src/readMTX.c:8-135 then src/matrixType.c:4-52, as
 * Sparse_Csr_Matrix_Distribution runs them on rank 0
 * (src/SparseMatrixDistribution.c:43-51).  The arrays are the reference's
 * own allocations (release with cacg_ref_free).  The reference exits on a
 * malformed file: call it with valid files only. */
long cacg_ref_read_mtx(const char *dir, const char *name, long *nrows, long *ncols,
                       long **rp, long **ci, double **v) {
    matInfo info;
    cooType coo;
    csrType_local csr;
    readMtx_info_and_coo((char *)dir, (char *)name, &info, &coo);
    Converter_Coo2Csr(coo, &csr, &info);
    free(coo.rowIdx);
    free(coo.colIdx);
    free(coo.coodata);
    *nrows = csr.num_rows;
    *ncols = csr.num_cols;
    *rp = csr.row_start;
    *ci = csr.col_idx;
    *v = csr.csrdata;
    return csr.nnz;
}

void cacg_ref_free(void *p) { free(p); }

/* src/common.c:16-48: rows x cols values into out */
void cacg_ref_parse_csv(const char *path, long rows, long cols, double *out) {
    double *buf = NULL;
    parseCSV((char *)path, &buf, rows, cols);
    memcpy(out, buf, (size_t)rows * cols * sizeof(double));
    free(buf);
}
