// cacg_solver.h -- internal interface between the solver and the server.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "cacg.h"

namespace cacg {

// A CSR matrix resident on the device: int32 indices, FP64 values, and FP32
// values when the mixed mode needs them.
struct DevMatrix {
    int64_t n = 0, nnz = 0;
    double avg_nnz = 0;
    int32_t *rp = nullptr, *ci = nullptr;
    double *val = nullptr;
    float *val32 = nullptr;
    size_t owned_bytes = 0;
    cudaStream_t st = nullptr;  // stream of the stream-ordered allocations
    static int create(const cacg_csr *A, bool want_f32, DevMatrix *M, cudaStream_t st);
    int ensure_f32(cudaStream_t st);
    void release();
};

// Device bytes of one solve's state (S, Q, AQ, R, small matrices, reduction
// workspaces), the admission cost of a request.
size_t solve_workspace_bytes(int64_t n, int m, int s, int prec, bool lanczos);

// Solve with device B, X.  ws_external (>= solve_workspace_bytes) may be
// given; otherwise a cached workspace is used.
void keep_pool_memory();

int solve_on_device(const DevMatrix *A, const double *B, double *X, int m,
                    const cacg_params *p, cacg_result *res, void *ws_external,
                    size_t ws_external_bytes);

}  // namespace cacg
