// bcg.cu -- block CG, bcg_v1 (src/bcgKernel.c:22-462): the block conjugate
// gradient method that the s-step Chebyshev solvers are measured against,
// on the same GB300 kernels and in FP64, as the reference runs it:
//
//   R = B - A X;  P = R;  G = R^T R                        (src/bcgKernel.c:113-197)
//   repeat:
//     AP = A P;  alpha = (P^T AP)^{-1} G                   (:267-307)
//     X += P alpha;  R -= AP alpha                         (:311-336, :427-431)
//     stop if ||R(:,0)|| < eps, R taken before this update (:339-424)
//     G' = R^T R;  beta = G^{-1} G';  P = R + P beta;  G = G'  (:433-457)
//
// The reference updates X, tests the residual of the previous iteration,
// and only then updates R; R is internal, so updating X and R in one fused
// pass and testing G(0,0) (= ||R(:,0)||^2 of the pre-update R) gives the same
// iterate at the same iteration.  alpha and beta: the no-pivot Crout LU of
// k_lu.cu (LUsolver_v1, src/DLSsolvers.c:6-91, factors its left-hand side in
// place; a solve on a copy gives the same values).  P = R + P beta runs as
// P' = R - P (-beta) through the tall x small update into a second buffer
// (P is read while it is written), then the buffers swap.
//
// Host synchronisation: the copy of G (and the LU status) for the test of
// iteration i is queued when G is formed in iteration i - 1; the host waits
// for it only after queueing iteration i's SpMM, Gram, solve and update, so
// the device does not idle on the read-back.
#include <algorithm>
#include <cmath>
#include <vector>

#include "cacg_internal.cuh"
#include "cacg_solver.h"

namespace cacg {

namespace {

__global__ void bcg_negate_kernel(int count, const double *__restrict__ in,
                                  double *__restrict__ out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
        out[i] = -in[i];
}

struct BcgState {
    const DevMatrix *A = nullptr;
    cacg_params p{};
    cudaStream_t st = nullptr;
    int m = 0;
    int64_t n = 0;
    double *R = nullptr, *P = nullptr, *P2 = nullptr, *AP = nullptr, *T = nullptr;
    double *G = nullptr, *G2 = nullptr, *PtAP = nullptr, *alpha = nullptr, *beta = nullptr,
           *nbeta = nullptr, *F = nullptr, *norms = nullptr, *bnorm = nullptr;
    double *gram_ws = nullptr, *norm_ws = nullptr;
    size_t gram_ws_bytes = 0;
    int *status = nullptr;
    void *block = nullptr;
    double *h = nullptr;  // pinned: G (m*m), status, norms (m), bnorm (m)

    int spmm(const double *X, double *Y, const double *Z1, double ca, double cb) {
        if (p.spmm_format != CACG_SPMM_CSR && A->dia_ndiag > 0) {
            int rc = launch_dia_spmm<double>(st, A, m, X, m, Y, m, Z1, m, nullptr, 0, ca, cb,
                                             0.0);
            if (rc != CACG_ERR_UNSUPPORTED) return rc;
        }
        return launch_spmm<double>(st, n, A->rp, A->ci, A->val, m, X, m, Y, m, Z1, m, nullptr,
                                   0, ca, cb, 0.0, A->avg_nnz);
    }
    int gram(const double *L, const double *Rm, double *C) {
        return launch_gram<double>(st, p.gram_variant, n, L, m, m, Rm, m, m, nullptr, 0, 0, C,
                                   m, nullptr, 0, gram_ws, gram_ws_bytes);
    }
    // Y = M^{-1} RHS (m x m), M factored into F
    int solve(const double *M, const double *RHS, double *Y) {
        int rc = launch_lu_factor(st, m, M, F, status);
        if (rc) return rc;
        return launch_lu_solve(st, m, F, m, RHS, Y);
    }
    // queue the copy of G and the status word for the host test
    int queue_readback() {
        CACG_CUDA_TRY(cudaMemcpyAsync(h, G, sizeof(double) * m * m, cudaMemcpyDeviceToHost, st));
        CACG_CUDA_TRY(cudaMemcpyAsync(h + m * m, status, sizeof(int), cudaMemcpyDeviceToHost,
                                      st));
        return CACG_OK;
    }
    // true residual of X into T, column norms into h + m*m + 1 (host)
    int true_residual(const double *B, const double *X, double *out_relres) {
        int rc = spmm(X, T, B, -1.0, 1.0);
        if (!rc) rc = launch_colnorm(st, n, m, T, norms, norm_ws);
        if (rc) return rc;
        double *hn = h + m * m + 2;
        CACG_CUDA_TRY(cudaMemcpyAsync(hn, norms, sizeof(double) * m, cudaMemcpyDeviceToHost, st));
        CACG_CUDA_TRY(cudaMemcpyAsync(hn + m, bnorm, sizeof(double) * m, cudaMemcpyDeviceToHost,
                                      st));
        CACG_CUDA_TRY(cudaStreamSynchronize(st));
        for (int c = 0; c < m; ++c) {
            const double den = hn[m + c] > 0 ? std::sqrt(hn[m + c]) : 1.0;
            out_relres[c] = std::sqrt(std::max(hn[c], 0.0)) / den;
        }
        return CACG_OK;
    }
};

}  // namespace

int solve_bcg_on_device(const DevMatrix *A, const double *B, double *X, int m,
                        const cacg_params *pin, cacg_result *res) {
    if (!A || !B || !X || m <= 0 || m > 256 || !pin || !res) return CACG_ERR_ARG;
    if (pin->maxit < 0) return CACG_ERR_ARG;
    if (pin->precision != CACG_FP64) return CACG_ERR_UNSUPPORTED;  // the reference's arithmetic
    keep_pool_memory();
    BcgState S;
    S.A = A;
    S.p = *pin;
    S.st = (cudaStream_t)pin->stream;
    S.m = m;
    S.n = A->n;
    const int64_t n = A->n;
    const size_t nm = (size_t)n * m, mm = (size_t)m * m;
    S.gram_ws_bytes = gram_workspace_bytes(n, m, m);
    const size_t nws = norm_workspace_doubles(n, m);
    const size_t doubles = 5 * nm + 7 * mm + (2 * mm + m) + 2 * (size_t)m + nws + 16;
    const size_t bytes = doubles * sizeof(double) + S.gram_ws_bytes + 256;
    if (cudaMallocAsync(&S.block, bytes, S.st) != cudaSuccess) {
        cudaGetLastError();
        return CACG_ERR_OOM;
    }
    double *q = (double *)S.block;
    auto take = [&](size_t cnt) {
        double *r = q;
        q += (cnt + 1) & ~(size_t)1;  // 16-byte steps
        return r;
    };
    S.R = take(nm);
    S.P = take(nm);
    S.P2 = take(nm);
    S.AP = take(nm);
    S.T = take(nm);
    S.G = take(mm);
    S.G2 = take(mm);
    S.PtAP = take(mm);
    S.alpha = take(mm);
    S.beta = take(mm);
    S.nbeta = take(mm);
    S.F = take(2 * mm + m);
    S.norms = take(m);
    S.bnorm = take(m);
    S.norm_ws = take(nws);
    S.status = (int *)take(2);
    S.gram_ws = q;
    S.h = pinned_scratch(sizeof(double) * (mm + 4 + 2 * (size_t)m));
    int rc = S.h ? CACG_OK : CACG_ERR_OOM;

    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, S.st);
    const int64_t l0 = g_launches.load();
    const bool abs_col0 = pin->tol_mode == CACG_TOL_ABS_COL0;
    std::vector<double> relres(m, 0.0);
    bool converged = false;
    int it = 0;
    if (!rc) rc = cudaMemsetAsync(S.status, 0, sizeof(int), S.st) == cudaSuccess ? CACG_OK
                                                                             : CACG_ERR_CUDA;
    // R = B - A X; P = R; G = R^T R; ||B(:,c)||^2 for the relative test
    if (!rc) rc = S.spmm(X, S.R, B, -1.0, 1.0);
    if (!rc && cudaMemcpyAsync(S.P, S.R, nm * sizeof(double), cudaMemcpyDeviceToDevice, S.st) !=
                   cudaSuccess)
        rc = CACG_ERR_CUDA;
    if (!rc) rc = S.gram(S.R, S.R, S.G);
    if (!rc) rc = launch_colnorm(S.st, n, m, B, S.bnorm, S.norm_ws);
    if (!rc) rc = S.queue_readback();
    std::vector<double> bn(m, 1.0);
    if (!rc) {
        CACG_CUDA_TRY(cudaMemcpyAsync(S.h + mm + 2, S.bnorm, sizeof(double) * m,
                                      cudaMemcpyDeviceToHost, S.st));
        if (cudaStreamSynchronize(S.st) != cudaSuccess) rc = CACG_ERR_CUDA;
        for (int c = 0; !rc && c < m; ++c)
            bn[c] = S.h[mm + 2 + c] > 0 ? std::sqrt(S.h[mm + 2 + c]) : 1.0;
        if (!rc) rc = S.queue_readback();
    }
    for (it = 0; !rc && it < pin->maxit; ++it) {
        // iteration work that does not depend on the test
        rc = S.spmm(S.P, S.AP, nullptr, 1.0, 0.0);
        if (!rc) rc = S.gram(S.P, S.AP, S.PtAP);
        if (!rc) rc = S.solve(S.PtAP, S.G, S.alpha);
        if (!rc)
            rc = launch_xrupdate_fast<double>(S.st, n, m, m, S.P, S.AP, m, S.alpha, X, S.R,
                                              nullptr, 0, nullptr, nullptr, nullptr);
        if (rc) break;
        // the test on the residual before this iteration's update
        if (cudaStreamSynchronize(S.st) != cudaSuccess) {
            rc = CACG_ERR_CUDA;
            break;
        }
        const int stv = *reinterpret_cast<int *>(S.h + mm);
        res->iterations = it + 1;
        res->recurrence_norm0 = std::sqrt(std::max(S.h[0], 0.0));
        if (stv & kStatusBreakdown) {
            rc = CACG_ERR_BREAKDOWN;
            break;
        }
        bool finite = true;
        for (int c = 0; c < m; ++c) finite = finite && std::isfinite(S.h[(size_t)c * m + c]);
        if (!finite) {
            rc = CACG_ERR_BREAKDOWN;
            break;
        }
        if (abs_col0) {
            if (std::sqrt(S.h[0]) < pin->tol) {  // src/bcgKernel.c:422
                converged = true;
                break;
            }
        } else {
            double mx = 0.0;
            for (int c = 0; c < m; ++c) {
                const double v = std::sqrt(std::max(S.h[(size_t)c * m + c], 0.0)) / bn[c];
                if (!(v <= mx)) mx = v;
            }
            if (mx <= pin->tol) {
                // confirmed on the true residual of the updated X
                rc = S.true_residual(B, X, relres.data());
                if (rc) break;
                double tmx = 0.0;
                for (int c = 0; c < m; ++c) tmx = std::max(tmx, relres[c]);
                if (tmx <= pin->tol) {
                    converged = true;
                    break;
                }
            }
        }
        // G' = R^T R; beta = G^{-1} G'; P = R + P beta
        rc = S.gram(S.R, S.R, S.G2);
        if (!rc) rc = S.solve(S.G, S.G2, S.beta);
        if (!rc) {
            bcg_negate_kernel<<<1, 256, 0, S.st>>>((int)mm, S.beta, S.nbeta);
            rc = check_launch();
        }
        if (!rc) rc = launch_qupdate<double>(S.st, n, m, S.P2, m, S.P, m, S.R, m, S.nbeta);
        if (rc) break;
        std::swap(S.P, S.P2);
        std::swap(S.G, S.G2);
        rc = S.queue_readback();
    }
    // reported residual: FP64, every column
    if (rc >= 0) {
        int r2 = S.true_residual(B, X, relres.data());
        if (r2) rc = r2;
    }
    double mx = 0.0;
    for (int c = 0; c < m; ++c) {
        if (res->true_relres) res->true_relres[c] = relres[c];
        if (!(relres[c] <= mx)) mx = relres[c];
    }
    res->true_relres_max = mx;
    res->m = m;
    res->residual_replacements = 0;
    res->lambda_min = res->lambda_max = 0.0;
    cudaEventRecord(e1, S.st);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    res->seconds = ms * 1e-3;
    res->launches = g_launches.load() - l0;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFreeAsync(S.block, S.st);
    cudaStreamSynchronize(S.st);
    cudaGetLastError();
    if (rc < 0) {
        res->status = rc;
        return rc;
    }
    res->status = converged ? CACG_OK : CACG_NOT_CONVERGED;
    return res->status;
}

}  // namespace cacg
