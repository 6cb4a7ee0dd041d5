// cacg_solver.h -- internal interface between the solver and the server.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "cacg.h"

namespace cacg {

constexpr int kDiaMax = 32;      // diagonals of a DIA view
constexpr int kDiaGroupMax = 4;  // adjacent diagonals sharing one X register window

// Diagonal offsets (sorted) and groups of adjacent offsets of a DIA view;
// passed to kernels by value.
struct DiaDesc {
    int ndiag, ngroups;
    int64_t off[kDiaMax];
    int gstart[kDiaMax + 1];
};

// A CSR matrix resident on the device: int32 indices, FP64 values, and FP32
// values when the mixed mode needs them; plus a DIA view (values per
// diagonal, ndiag x dia_npad, zero where a row lacks the diagonal) when every
// nonzero lies on one of at most kDiaMax diagonals with little padding.
struct DevMatrix {
    int64_t n = 0, nnz = 0;
    double avg_nnz = 0;
    int32_t *rp = nullptr, *ci = nullptr;
    double *val = nullptr;
    float *val32 = nullptr;
    int dia_ndiag = 0;  // 0: CSR only
    int64_t dia_npad = 0;
    DiaDesc dia{};
    double *dia64 = nullptr;
    float *dia32 = nullptr;    // FP32 values (hi) ...
    float *dia32lo = nullptr;  // ... and val - hi, same allocation
    size_t owned_bytes = 0;
    cudaStream_t st = nullptr;  // stream of the stream-ordered allocations
    static int create(const cacg_csr *A, bool want_f32, DevMatrix *M, cudaStream_t st);
    int build_dia(const cacg_csr *A, bool want_f32, cudaStream_t st);
    int ensure_f32(cudaStream_t st);
    void release();
};

int launch_dia_hilo(cudaStream_t st, int64_t count, const double *v64, float *hi, float *lo);
int launch_ff_split(cudaStream_t st, int64_t count, const double *x, float *hi, float *lo);
// x = hi + lo in FP64 (k_dia.cu)
int launch_ff_join(cudaStream_t st, int64_t count, const float *hi, const float *lo, double *x);
// R = B - A X in float-float over the DIA view, with S0 = R32 = (float)R and
// the column norms of R; Xh, Xl: n x m FP32 scratch, filled from X (X ==
// NULL: they already hold X).  Rff != NULL (m = 16): R written as a
// normalised float-float pair (n x 16 high parts, then low parts) instead of
// FP64 R (k_dia.cu)
int launch_dia_residual_ff(cudaStream_t st, const DevMatrix *A, int m, const double *X,
                           const double *B, double *R, float *Xh, float *Xl, float *S0,
                           int64_t lds, float *R32, double *norms, double *ws,
                           int64_t ws_doubles, float *Rff = nullptr);

// Y = ca A X + cb Z1 + cc Z2 over the DIA view (k_dia.cu);
// CACG_ERR_UNSUPPORTED when the matrix has no view of this precision.
template <typename T>
int launch_dia_spmm(cudaStream_t st, const DevMatrix *A, int w, const T *X, int64_t ldx, T *Y,
                    int64_t ldy, const T *Z1, int64_t ldz1, const T *Z2, int64_t ldz2,
                    double ca, double cb, double cc);

// The same product for FP32 blocks of 16k columns with the X rows of each
// band of diagonals staged in shared memory by TMA (k_dia_ring.cu);
// CACG_ERR_UNSUPPORTED when the operands or the diagonals do not fit its
// layout.  *status gets kStatusTimeout if a bounded wait expires.
int launch_dia_ring(cudaStream_t st, const DevMatrix *A, int w, const float *X, int64_t ldx,
                    float *Y, int64_t ldy, const float *Z1, int64_t ldz1, const float *Z2,
                    int64_t ldz2, double ca, double cb, double cc, int *status);

// The same product without recurrence terms (Z1 = Z2 = NULL: the A Q product)
// for FP32 blocks whose width (64 or 96) is also their row stride, with
// compile-time strides (k_dia_wide.cu); bit-identical to launch_dia_spmm.
// CACG_ERR_UNSUPPORTED for other shapes.
int launch_dia_wide(cudaStream_t st, const DevMatrix *A, int w, const float *X, int64_t ldx,
                    float *Y, int64_t ldy, const float *Z1, int64_t ldz1, const float *Z2,
                    int64_t ldz2, double ca, double cb, double cc);

// Per-thread pinned host scratch of at least `bytes` (reused across calls).
double *pinned_scratch(size_t bytes);

// Block CG (bcg_v1, src/bcgKernel.c:22-462), FP64, on the same kernels
// (bcg.cu).  tol_mode, tol, maxit, gram_variant, spmm_format and stream of p
// apply; s, bounds and the mixed-precision fields do not.
int solve_bcg_on_device(const DevMatrix *A, const double *B, double *X, int m,
                        const cacg_params *p, cacg_result *res);

// Device bytes of one solve's state (S, Q, AQ, R, small matrices, reduction
// workspaces), the admission cost of a request.
size_t solve_workspace_bytes(int64_t n, int m, int s, int prec, bool lanczos);

// Solve with device B, X.  ws_external (>= solve_workspace_bytes) may be
// given; otherwise a cached workspace is used.
void keep_pool_memory();
// phase profiler (cacg_profile_*): on/off, and a call timed by another component
bool profile_enabled();
void profile_accumulate(int phase, double ms, int64_t launches);

int solve_on_device(const DevMatrix *A, const double *B, double *X, int m,
                    const cacg_params *p, cacg_result *res, void *ws_external,
                    size_t ws_external_bytes);

}  // namespace cacg
