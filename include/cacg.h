/*
 * cacg.h -- C ABI of libcacg.so, the GB300 (sm_103a) implementation of the
 * sclc/cacg communication-avoiding Chebyshev-basis (block) CG hot path.
 *
 * Three layers, all extern "C", plain pointers and sizes:
 *   1. Drop-in replacements for the reference solver entry points
 *      (cbcg_v1, bcbcg_v1), same symbols, same by-value structs, same
 *      semantics, for one rank's work on one GPU.
 *   2. The extended solver API (cacg_solve*, cacg_matrix_*), with explicit
 *      bounds / tolerance / precision / residual-replacement parameters and a
 *      status code instead of exit().
 *   3. Kernel-level entry points (cacg_k_*) on device pointers, one per hot
 *      operation of the reference, used by the parity tests.
 * Plus the serving loop (cacg_server_*) and the seeded input generators.
 *
 * Errors: every int-returning function returns CACG_OK (0) or a negative
 * CACG_ERR_* code; nothing calls exit().  The drop-ins return void like the
 * reference, and leave their status in cacg_last_status().
 */
#ifndef CACG_H
#define CACG_H

#include <stddef.h>
#include <stdint.h>

#include "cacg_ref_types.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
#define CACG_OK 0
#define CACG_NOT_CONVERGED 1 /* result valid, tolerance not reached in maxit */
#define CACG_PENDING 2       /* server: request not finished yet */
#define CACG_ERR_ARG (-1)
#define CACG_ERR_OOM (-2)
#define CACG_ERR_CUDA (-3)
#define CACG_ERR_BREAKDOWN (-4) /* zero/non-finite pivot or NaN/Inf in the iteration */
#define CACG_ERR_TIMEOUT (-5)   /* a bounded device-side wait ran out */
#define CACG_ERR_UNSUPPORTED (-6)
#define CACG_ERR_BUSY (-7)      /* server: admission refused (memory budget) */
#define CACG_ERR_NODEV (-8)     /* no CUDA device */

/* ----------------------------------------------------------------- enums */
#define CACG_BOUNDS_GERSCHGORIN 0 /* reference behaviour, src/common.c:53 */
#define CACG_BOUNDS_GIVEN 1       /* [lambda_min, lambda_max] from params */
#define CACG_BOUNDS_LANCZOS 2     /* lanczos_steps-step Lanczos estimate */

#define CACG_TOL_ABS_COL0 0 /* reference: ||R(:,0)|| < tol (src/bcbcgKernel.c:524) */
#define CACG_TOL_REL_ALL 1  /* max_c ||b_c - A x_c|| / ||b_c|| <= tol (true residual) */

#define CACG_FP64 0  /* plain FP64 everywhere */
#define CACG_MIXED 1 /* FP32 basis/SpMM/updates, FP64 Gram accumulation, LU, X, R,
                        FP64 residual replacement */

#define CACG_GRAM_AUTO 0
#define CACG_GRAM_FMA 1  /* FP64 FMA pipe */
#define CACG_GRAM_DMMA 2 /* FP64 tensor core (mma.sync m8n8k4 f64) */
#define CACG_GRAM_TC 3   /* FP32 inputs on the bf16 tensor cores: three bf16 slices
                            per value, six slice products, FP32 accumulation over
                            256-row groups, FP64 across groups */
#define CACG_GRAM_TC_SLICES 4 /* same products, from bf16 slice planes written by the
                                 producers (cacg_k_gram splits its inputs first) */
#define CACG_GRAM_TC5 5  /* same products on the 5th-generation tensor cores
                            (tcgen05.mma, accumulator in tensor memory, FP32 over
                            64-row groups, float-float sums across groups) */

#define CACG_ALG_CACG 0 /* s-step Chebyshev-basis CG: cbcg_v1 (m = 1) / bcbcg_v1 */
#define CACG_ALG_BCG 1  /* block CG, bcg_v1 (src/bcgKernel.c:22) */

#define CACG_SPMM_AUTO 0
#define CACG_SPMM_CSR 1 /* always the CSR kernels */
#define CACG_SPMM_DIA_UNSTAGED 2 /* the DIA view, read through the caches only (no
                                    shared-memory staging of X); results identical */

#define CACG_RESID_AUTO 0
#define CACG_RESID_FP64 1 /* residual replacements in FP64 as well */

#define CACG_VAL_F64 0
#define CACG_VAL_F32 1
#define CACG_XR_EXACT 16 /* or-ed into cacg_k_xrupdate's vtype: float-float sums */
#define CACG_VAL_TC5 32  /* or-ed into the vtype of cacg_k_qupdate / cacg_k_xrupdate
                            (FP32 only): the products on the 5th-generation tensor
                            cores (three bf16 slices per value, six slice products,
                            FP32 accumulation).  Returns CACG_ERR_UNSUPPORTED outside
                            qupdate: k % 16 == 0, k <= 96; xrupdate: k % 4 == 0,
                            k <= 256, m <= 16 dividing 32; both: 16-byte aligned rows */
#define CACG_VAL_TC5_CPASYNC 64 /* with CACG_VAL_TC5 in cacg_k_qupdate: the cp.async-fed
                                   kernel instead of the TMA-fed one (bit-identical) */
#define CACG_XR_FFSTATE 128 /* or-ed into cacg_k_xrupdate's vtype (FP32, m = 16): X and R
                               are float-float pairs, each n x 16 FP32 high parts followed
                               by n x 16 low parts (the byte size of n x 16 doubles) -- the
                               mixed solve's state; S0 = R32 = the high part of R */

/* generators (cacg_gen_*) */
#define CACG_GEN_LAPLACE2D_5PT 1
#define CACG_GEN_LAPLACE3D_7PT 2
#define CACG_GEN_STENCIL3D_27PT 3
#define CACG_GEN_VARCOEF2D_5PT 4
#define CACG_RHS_UNIFORM 0
#define CACG_RHS_NORMAL 1
#define CACG_RHS_BETA25 2
#define CACG_RHS_ONES 3

/* --------------------------------------------------------------- structs */
typedef struct cacg_csr {
    int64_t n;              /* rows == columns */
    int64_t nnz;
    const int32_t *row_ptr; /* n + 1 */
    const int32_t *col_idx; /* nnz, ascending within a row not required */
    const double *val;      /* nnz */
} cacg_csr;

typedef struct cacg_params {
    int32_t s;            /* basis length (s-step), >= 2 */
    int32_t bounds_mode;  /* CACG_BOUNDS_* */
    double lambda_min;    /* used with CACG_BOUNDS_GIVEN */
    double lambda_max;
    int32_t lanczos_steps; /* used with CACG_BOUNDS_LANCZOS (default 50) */
    int32_t tol_mode;     /* CACG_TOL_* */
    double tol;           /* absolute (ABS_COL0) or relative (REL_ALL) */
    int32_t maxit;        /* outer iterations */
    int32_t precision;    /* CACG_FP64 / CACG_MIXED */
    int32_t rr_period;    /* MIXED: FP64 residual replacement every rr_period
                             outer iterations (0: only when the recurrence
                             residual says converged) */
    int32_t gram_variant; /* CACG_GRAM_* */
    uint64_t lanczos_seed;
    void *stream;         /* cudaStream_t, NULL = the library's own stream */
    int32_t use_graph;    /* on a non-default stream: capture the outer iteration
                             (from the third on) in CUDA graphs and replay them */
    int32_t exact_updates; /* MIXED: X/R update products summed in float-float
                              instead of FP32 FMAs */
    int32_t spmm_format;  /* CACG_SPMM_*: AUTO uses the matrix's DIA view when it
                             has one (results bit-identical to CSR); MIXED with
                             16-column blocks stages the X rows of each band of
                             diagonals in shared memory (TMA) */
    int32_t residual_precision; /* CACG_RESID_*: MIXED with a DIA view computes the
                                   periodic residual replacements in float-float
                                   (about 44 bits, FP32 pipe) unless FP64 is asked
                                   for; convergence checks are always FP64 */
    int32_t algorithm;    /* CACG_ALG_*: the s-step Chebyshev solvers (default) or
                             block CG (bcg_v1; FP64 only, s and bounds unused) */
    int32_t reserved[3];
} cacg_params;

typedef struct cacg_result {
    int32_t status;      /* CACG_OK / CACG_NOT_CONVERGED / CACG_ERR_* */
    int32_t iterations;  /* outer iterations executed */
    int32_t residual_replacements;
    int32_t m;
    double lambda_min;   /* Chebyshev interval actually used */
    double lambda_max;
    double recurrence_norm0; /* ||R(:,0)|| of the recurrence residual at exit */
    double true_relres_max;  /* max_c ||b_c - A x_c|| / ||b_c|| (FP64) */
    double *true_relres;     /* optional caller array of m entries */
    double seconds;          /* solve time on the device (CUDA events) */
    int64_t launches;        /* kernels launched by the solve */
    int32_t reserved[6];
} cacg_result;

/* ------------------------------------------------- 1. drop-in (reference) */
/* Replaces void cbcg_v1(csrType_local, denseType, denseType, long s,
 * double epsilon, int myid, int numprocs), src/cbcgKernel.h:21.
 * One rank only (numprocs must be 1); B/X local n x 1 row-major; X in/out;
 * Gerschgorin bounds; stops when ||R(:,0)|| < epsilon or after 1000 outer
 * iterations (src/cbcgKernel.c:2). */
void cbcg_v1(csrType_local mat, denseType B, denseType X, long s, double epsilon,
             int myid, int numprocs);
/* Replaces void bcbcg_v1(...), src/bcbcgKernel.h:22.  Same contract with
 * m = B.local_num_col right-hand sides and 100 outer iterations
 * (src/bcbcgKernel.c:3). */
void bcbcg_v1(csrType_local mat, denseType B, denseType X, long s, double epsilon,
              int myid, int numprocs);
/* Replaces void bcg_v1(csrType_local mat, denseType B, denseType X,
 * double epsilon, int myid, int numprocs), src/bcgKernel.h:22: block CG (no
 * s-step basis), FP64, X in/out, stops when ||R(:,0)|| < epsilon -- tested
 * on the residual before the iteration's R update, after X has moved, as
 * src/bcgKernel.c:311-424 does -- or after 1000 iterations
 * (src/bcgKernel.c:2). */
void bcg_v1(csrType_local mat, denseType B, denseType X, double epsilon, int myid,
            int numprocs);
/* Status of the calling thread's last drop-in call (they return void). */
int cacg_last_status(void);
/* Iterations / final ||R(:,0)|| of the calling thread's last drop-in call. */
int cacg_last_iterations(void);
/* Override the drop-ins' outer-iteration cap (0 restores 1000 / 100). */
void cacg_set_dropin_maxit(int maxit);

/* --------------------------------------------------- 2. extended solver API */
void cacg_params_default(cacg_params *p);
const char *cacg_status_string(int status);

/* Host pointers in and out: copies A, B to the device, solves, copies X
 * (initial guess in, solution out) back.  m right-hand sides, n x m row-major. */
int cacg_solve(const cacg_csr *A, const double *B, double *X, int32_t m,
               const cacg_params *p, cacg_result *res);

/* A resident matrix (FP64 values, plus FP32 values when mixed is requested). */
typedef struct cacg_matrix cacg_matrix;
int cacg_matrix_create(const cacg_csr *A_host, int32_t want_fp32, cacg_matrix **out);
int cacg_matrix_destroy(cacg_matrix *A);
int64_t cacg_matrix_device_bytes(const cacg_matrix *A);
/* No counterpart in the reference (CSR only there).  Diagonals of the
 * matrix's DIA view, built at creation when every nonzero lies on one of at
 * most 32 diagonals with at most 1.5x padding (stencil matrices); 0 when the
 * matrix is kept as CSR only. */
int32_t cacg_matrix_diagonals(const cacg_matrix *A);
/* Device pointers: B_dev, X_dev are n x m row-major doubles on the device. */
int cacg_solve_device(cacg_matrix *A, const double *B_dev, double *X_dev, int32_t m,
                      const cacg_params *p, cacg_result *res);
/* Device bytes of solver state for (n, m, s, precision): the admission cost. */
int64_t cacg_workspace_bytes(int64_t n, int32_t m, int32_t s, int32_t precision);

/* ------------------------------------------------ 3. kernel entry points */
/* All pointers are device pointers; stream may be NULL (legacy default
 * stream).  Each call is asynchronous on that stream. */

/* src/common.c:53-106 gerschgorin_v1: out[0] = min_i(d_i - sum|a_ij|),
 * out[1] = max_i(d_i + sum|a_ij|) (max initialised to DBL_MIN as in the
 * reference).  out is 2 device doubles. */
int cacg_k_gerschgorin(int64_t n, const int32_t *row_ptr, const int32_t *col_idx,
                       const double *val, double *out, void *stream);

/* Fused CSR SpMM + three-term epilogue (src/BLAS3.c:20-155, 913-976, 978-994):
 *   Y = ca * (A X) + cb * Z1 + cc * Z2        (Z1 / Z2 may be NULL)
 * X, Y, Z1, Z2 are n x w row-major with the given row strides (elements).
 * vtype selects double or float for val / X / Y / Z (CACG_VAL_*). */
int cacg_k_spmm(int32_t vtype, int64_t n, const int32_t *row_ptr,
                const int32_t *col_idx, const void *val, int32_t w, const void *X,
                int64_t ldx, void *Y, int64_t ldy, const void *Z1, int64_t ldz1,
                const void *Z2, int64_t ldz2, double ca, double cb, double cc,
                void *stream);

/* src/common.c:182-256 BCBCG_chebyshevPolynomialBasisGen (and :109-179 for
 * m == 1): S (n x s*m, row stride lds) with S[:, 0:m] = R on entry already
 * or copied from R when R != NULL; column block j = T_j. */
int cacg_k_basis(int32_t vtype, int64_t n, const int32_t *row_ptr,
                 const int32_t *col_idx, const void *val, const void *R, int32_t m,
                 int32_t s, double alpha, double beta, void *S, int64_t lds,
                 void *stream);

/* src/BLAS3.c:699-758 distributedMatLTransposeMatRMul(_updated):
 *   C (ka x (kb1 + kb2)) = L^T [R1 | R2]   accumulated in FP64.
 * L (n x ka), R1 (n x kb1), R2 (n x kb2, may be NULL with kb2 == 0).
 * vtype: inputs double (accumulate FP64) or float (FP64-accurate accumulation
 * of FP32 products).  variant: CACG_GRAM_*.  C is row-major, ldc >= kb1+kb2. */
int cacg_k_gram(int32_t vtype, int32_t variant, int64_t n, const void *L, int64_t ldl,
                int32_t ka, const void *R1, int64_t ldr1, int32_t kb1, const void *R2,
                int64_t ldr2, int32_t kb2, double *C, int32_t ldc, void *stream);

/* No counterpart in the reference.  Same product as cacg_k_gram, for callers
 * that cannot let the library allocate device memory (their device memory is
 * owned by their own allocator, or an allocation could synchronise a
 * latency-critical loop): the split-K scratch is a fixed 16 MiB device array
 * inside libcacg.so, held by every GPU that loads the library until exit.
 * Calls no cudaMalloc/cudaFree.  Shapes whose single-chunk scratch exceeds
 * 16 MiB return CACG_ERR_ARG.  variant: CACG_GRAM_AUTO, CACG_GRAM_FMA or
 * CACG_GRAM_DMMA only (others: CACG_ERR_UNSUPPORTED); FP32 inputs take the
 * FP64-accurate CUDA-core product.  All calls share the array: calls that
 * overlap on the GPU race.  The first call in each device context (again
 * after a cudaDeviceReset) looks up the array's device address; make it
 * before any stream capture. */
int cacg_k_gram_noalloc(int32_t vtype, int32_t variant, int64_t n, const void *L,
                        int64_t ldl, int32_t ka, const void *R1, int64_t ldr1, int32_t kb1,
                        const void *R2, int64_t ldr2, int32_t kb2, double *C, int32_t ldc,
                        void *stream);

/* No counterpart in the reference.  Every wait of the tcgen05 kernels on an
 * mbarrier is bounded; on expiry the kernel drains its own copies and MMAs in
 * flight, frees its tensor memory, sets a status word and returns, and the
 * solver reports CACG_ERR_TIMEOUT.  This sets the poll limit of the tcgen05
 * Gram's pipeline waits (process-wide; polls < 0 restores the default of
 * 2^22) so that a test can make them run out; the drain waits keep the full
 * bound. */
int cacg_set_pipeline_wait_limit(int64_t polls);

/* src/BLAS3.c:794-825 + :579-612 fused: Q = S - Q * beta (in place on Q),
 * Q, S n x k (strides ldq, lds), beta k x k FP64 row-major. */
int cacg_k_qupdate(int32_t vtype, int64_t n, int32_t k, void *Q, int64_t ldq,
                   const void *S, int64_t lds, const double *beta, void *stream);

/* src/BLAS3.c:794-825 + :579-612 + src/MatrixOperations.c:110-142 fused:
 *   X += Q alpha;  R -= AQ alpha;  S0 = R (cast to vtype, may be NULL);
 *   norms[c] = ||R(:,c)||^2 for c < m (may be NULL).
 * Q, AQ n x k (vtype, strides ldq), alpha k x m FP64, X, R n x m FP64. */
int cacg_k_xrupdate(int32_t vtype, int64_t n, int32_t k, int32_t m, const void *Q,
                    const void *AQ, int64_t ldq, const double *alpha, double *X,
                    double *R, void *S0, int64_t lds, double *norms, void *stream);

/* Tall-skinny QR, V (n x k, FP64, row-major, stride ldv) = Q R: Q (n x k,
 * stride ldq) with orthonormal columns, R (k x k row-major) upper triangular
 * with a positive diagonal; k <= 128, n >= k.  The reference's TSQR
 * (src/TSQR.c) is empty and its Householder QR (src/MatrixDecomposition.c:3-93)
 * unfinished, so this has no reference behaviour to match: CholeskyQR2 on the
 * split-K FP64 Gram, orthogonal to working accuracy for cond(V) < ~1e8;
 * CACG_ERR_BREAKDOWN when V is numerically rank-deficient. */
int cacg_k_tsqr(int64_t n, int32_t k, const double *V, int64_t ldv, double *Q, int64_t ldq,
                double *R, void *stream);

/* src/DLSsolvers.c:106-208 LUsolver_v1_KeeplhsMat: Y (k x r) = M^{-1} RHS by
 * Crout LU without pivoting (U unit-diagonal).  status (device int, may be
 * NULL) is set to 1 on a zero or non-finite pivot. */
int cacg_k_lu(int32_t k, const double *M, int32_t r, const double *RHS, double *Y,
              int *status, void *stream);

/* Number of CUDA kernels this library has launched in this process. */
int64_t cacg_launch_count(void);

/* ------------------------------------------------------- phase profiling */
/* The GPU counterpart of the reference's TIME_MEASURE_BCBCG_* phase timers
 * (src/bcbcgKernel.c:19-24, 454-522): when enabled, every solve records CUDA
 * events around each phase's kernels on the solve's stream and accumulates
 * device time, launches, and the phase's algorithmic bytes and flops. */
#define CACG_PHASE_BASIS 0    /* Chebyshev-step SpMM (width m) */
#define CACG_PHASE_AQ 1       /* AQ = A Q SpMM (width k) */
#define CACG_PHASE_GRAM 2     /* Q^T [AQ | R], (AQ)^T S */
#define CACG_PHASE_QUPDATE 3  /* Q = S - Q beta */
#define CACG_PHASE_XRUPDATE 4 /* X += Q alpha, R -= AQ alpha, norms */
#define CACG_PHASE_LU 5       /* factor + solves */
#define CACG_PHASE_RESIDUAL 6 /* R = B - A X (start, replacement, final) */
#define CACG_PHASE_BOUNDS 7   /* Gerschgorin / Lanczos */
#define CACG_NUM_PHASES 8
void cacg_profile_enable(int on);
void cacg_profile_reset(void);
int cacg_profile_get(int phase, double *ms, int64_t *launches, double *bytes, double *flops);
/* Timed calls of a phase (one Gram product, one basis step, ...; a call may
 * launch more than one kernel, e.g. a split-K product and its reduction). */
int64_t cacg_profile_calls(int phase);
const char *cacg_profile_name(int phase);

/* ----------------------------------------------------------- serving loop */
/* Serving engines: BATCHED (default) advances every admitted request one
 * outer iteration per step, each phase one launch over all requests of a
 * precision class, the step replayed from a CUDA graph; requests beyond its
 * kernels' limits (s * m > 64, m > 32, s > 16, Lanczos bounds, block CG) and
 * requests above batch_max_rows rows run on per-request stream workers with
 * the single-request solver.  STREAMS runs every request that way.
 * max_active bounds the requests in flight on both paths together. */
#define CACG_SERVER_BATCHED 0
#define CACG_SERVER_STREAMS 1

typedef struct cacg_server cacg_server;
typedef struct cacg_server_config {
    int64_t mem_budget_bytes; /* device bytes admitted requests may hold */
    int32_t max_active;       /* concurrent requests on the device */
    int32_t engine;           /* CACG_SERVER_BATCHED (0) or CACG_SERVER_STREAMS */
    int32_t no_graphs;        /* batched engine: 1 launches each step directly
                                 instead of replaying its CUDA graph */
    int32_t batch_max_rows;   /* batched engine: requests with more rows take a
                                 stream worker and the single-request solver's
                                 kernels (0: 65536; negative: no limit) */
    int32_t reserved[4];
} cacg_server_config;

int cacg_server_create(const cacg_server_config *cfg, cacg_server **out);
/* Enqueue one request: the server copies A, B (host) at admission; X_out
 * (host, n x m) receives the solution.  Non-blocking; *ticket identifies it. */
int cacg_server_submit(cacg_server *srv, const cacg_csr *A, const double *B,
                       int32_t m, const cacg_params *p, double *X_out,
                       int64_t *ticket);
/* CACG_PENDING while running, else the request's final status; res filled. */
int cacg_server_poll(cacg_server *srv, int64_t ticket, cacg_result *res);
int cacg_server_wait(cacg_server *srv, int64_t ticket, cacg_result *res);
/* Queue depth, active requests and device bytes in use. */
int cacg_server_stats(cacg_server *srv, int64_t *queued, int64_t *active,
                      int64_t *bytes_in_use);
/* Batched engine: steps run, steps replayed from a CUDA graph, and the
 * autotuned blocks per SM of its kernels (FP64 class: SpMM, Gram, Q update,
 * X/R update, then the same four for the FP32 class; 0 = not tuned yet). */
int cacg_server_engine_stats(cacg_server *srv, int64_t *steps, int64_t *graph_replays,
                             int32_t *blocks_per_sm, int32_t nvals);
int cacg_server_destroy(cacg_server *srv);

/* ----------------------------------------------------------- input files
 * The reference's file inputs and its 1-D row-block split, on the host.
 * Where the reference calls exit() or assert(), these return CACG_ERR_ARG
 * (malformed input), CACG_ERR_UNSUPPORTED (valid file of a kind the
 * reference refuses) or CACG_ERR_OOM, and leave the outputs zeroed. */

/* Replaces readMtx_info_and_coo (src/readMTX.c:8-135) followed by
 * Converter_Coo2Csr (src/matrixType.c:4-52): a Matrix Market coordinate file
 * (field real, integer or pattern -- pattern entries read as 1.0; symmetry
 * general, skew-symmetric read as stored, or symmetric with each
 * off-diagonal entry followed by its mirror) into *out: 0-based long
 * indices, a row's entries in file order, start = 0, arrays malloc'ed by the
 * library (cacg_csr_free).  Array and complex files: CACG_ERR_UNSUPPORTED. */
int cacg_read_mtx(const char *path, csrType_local *out);
void cacg_csr_free(csrType_local *mat);

/* Replaces the row split of Sparse_Csr_Matrix_Distribution
 * (src/SparseMatrixDistribution.c:7-205): rank myid of numprocs gets rows
 * [myid * (n / numprocs), ...), n / numprocs of them (the last rank also the
 * remainder), row_start rebased to 0, global column indices, start = its
 * first row.  A copy (cacg_csr_free). */
int cacg_csr_row_block(const csrType_local *A, int myid, int numprocs,
                       csrType_local *local);

/* Replaces parseCSV (src/common.c:16-48): `rows` lines of `cols`
 * comma-separated numbers (atof) into out (rows x cols, row-major).  Lines
 * past `rows` are ignored; a shorter file leaves the remaining rows zero as
 * the reference does (*rows_read, may be NULL, says how many were read); a
 * line with another number of fields is CACG_ERR_ARG (the reference
 * asserts).  No line-length limit (the reference reads 1024-byte lines). */
int cacg_read_csv(const char *path, int64_t rows, int64_t cols, double *out,
                  int64_t *rows_read);

/* Replaces the split of GenVector_ReadCSV (src/GetRHS.c:124-208): rank
 * myid's block of rows of a rows x cols row-major array, as a denseType with
 * the reference's field values (start_idx = myid * cols * (rows / numprocs)).
 * A copy (cacg_dense_free). */
int cacg_dense_row_block(const double *global, int64_t rows, int64_t cols, int myid,
                         int numprocs, denseType *local);
void cacg_dense_free(denseType *d);

/* ------------------------------------------------------------ generators */
int64_t cacg_gen_rows(int kind, int64_t N);
int64_t cacg_gen_nnz(int kind, int64_t N);
int cacg_gen_matrix(int kind, int64_t N, double shift, double sigma, uint64_t seed,
                    int32_t *row_ptr, int32_t *col_idx, double *val);
int cacg_gen_rhs(int dist, int64_t n, int m, uint64_t seed, double a, double b,
                 double *out);
double cacg_det_log(double x);
double cacg_det_exp(double x);

#ifdef __cplusplus
}
#endif

#endif /* CACG_H */
