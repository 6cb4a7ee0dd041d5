// k_lu.cu -- the small dense solve of the CA iteration, in FP64.
//
// Reference operation replaced (sclc/cacg): LUsolver_v1_KeeplhsMat,
// src/DLSsolvers.c:106-208 -- Crout LU with unit-diagonal U and NO pivoting
// (reciprocal of the pivot times the pivot row, then the trailing update),
// forward substitution dividing by L's diagonal through a reciprocal, back
// substitution with U's unit diagonal.  The same elimination order is kept
// so the GPU result matches the reference to rounding.
//
// The reference refactors Q^T AQ inside every call (twice per iteration:
// for alpha, and one iteration later for beta); here the factor of each
// Q^T AQ is computed once and reused by both solves.
//
// The factor F is 2*k*k + k doubles: the Crout factors, the reciprocals of
// L's diagonal (the reference multiplies by 1/L_ii, src/DLSsolvers.c:168),
// and the factors again, transposed, for the column-sweep solves.
// A zero or non-finite pivot sets *status = 1 (CACG_ERR_BREAKDOWN at the
// host) instead of trapping; the arithmetic continues as the reference's
// does (inf/NaN propagate) and the host stops the iteration.
#include <cooperative_groups.h>

#include "cacg_internal.cuh"

namespace cacg {

namespace cgrp = cooperative_groups;

constexpr int kLuThreads = 512;
constexpr int kLuSmemK = 144;  // factor in shared memory up to k = 144 (162 KB)

// One CTA.  W is the working matrix: shared memory when it fits, else F.
__global__ void __launch_bounds__(kLuThreads)
    lu_factor_kernel(int k, const double *__restrict__ M, double *__restrict__ F,
                     int *__restrict__ status, int use_smem) {
    extern __shared__ __align__(16) double Ws[];
    double *W = use_smem ? Ws : F;
    const int kk = k * k;
    for (int i = threadIdx.x; i < kk; i += blockDim.x) W[i] = M[i];
    __syncthreads();
    int bad = 0;
    double *Dinv = F + (size_t)kk;  // reciprocals of L's diagonal, read by the solves
    for (int d = 0; d < k; ++d) {
        // warp 0 scales the pivot row; one FP64 division per step
        if (threadIdx.x < 32) {
            double inv = 0.0;
            if (threadIdx.x == 0) {
                const double piv = W[d * k + d];
                if (piv == 0.0 || !isfinite(piv)) bad = 1;
                inv = 1.0 / piv;
                Dinv[d] = inv;
            }
            inv = __shfl_sync(0xffffffffu, inv, 0);
            for (int c = d + 1 + threadIdx.x; c < k; c += 32) W[d * k + c] *= inv;
        }
        __syncthreads();
        // trailing update, rows by warp, columns by lane (no index division)
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        for (int i = d + 1 + warp; i < k; i += kLuThreads / 32) {
            const double lid = W[i * k + d];
            for (int c = d + 1 + lane; c < k; c += 32)
                W[i * k + c] = W[i * k + c] - lid * W[d * k + c];
        }
        __syncthreads();
    }
    if (use_smem)
        for (int i = threadIdx.x; i < kk; i += blockDim.x) F[i] = W[i];
    // transposed copy for the column-sweep solves: FT[i][j] = F[j][i]
    double *FT = F + (size_t)kk + k;
    for (int idx = threadIdx.x; idx < kk; idx += blockDim.x) {
        const int i = idx / k, j = idx % k;
        FT[idx] = W[(size_t)j * k + i];
    }
    if (threadIdx.x == 0 && bad && status) atomicOr(status, kStatusBreakdown);
}

// The same factor spread over a cluster of kLucCtas CTAs (one SM each): CTA r
// owns rows i = r (mod kLucCtas) in its shared memory.  Step d: the owner of
// row d scales it by the pivot's reciprocal; one cluster barrier; every CTA
// copies the scaled row d from the owner's shared memory (distributed shared
// memory) and updates its rows i > d.  Every element sees the same
// operations in the same order as lu_factor_kernel (bit-identical factors);
// the trailing update's FP64 work is split over kLucCtas SMs' FP64 pipes.
constexpr int kLucCtas = 8;
constexpr int kLucThreads = 256;
constexpr int kLucMaxK = 256;

__global__ void __cluster_dims__(kLucCtas, 1, 1) __launch_bounds__(kLucThreads)
    lu_factor_cluster_kernel(int k, const double *__restrict__ M, double *__restrict__ F,
                             int *__restrict__ status) {
    extern __shared__ __align__(16) double luc_sm[];
    cgrp::cluster_group cluster = cgrp::this_cluster();
    const int rank = (int)cluster.block_rank();
    const int nloc = (k - rank + kLucCtas - 1) / kLucCtas;  // rows rank, rank + C, ...
    const int rows_max = (k + kLucCtas - 1) / kLucCtas;
    double *Wl = luc_sm;                        // nloc x k: local rows
    double *prow = luc_sm + (size_t)rows_max * k;  // the current pivot row
    for (int idx = threadIdx.x; idx < nloc * k; idx += blockDim.x) {
        const int li = idx / k, c = idx - li * k;
        Wl[idx] = M[(size_t)(li * kLucCtas + rank) * k + c];
    }
    double *Dinv = F + (size_t)k * k;
    int bad = 0;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    for (int d = 0; d < k; ++d) {
        const int owner = d % kLucCtas;
        if (rank == owner && warp == 0) {
            double *rd = Wl + (size_t)(d / kLucCtas) * k;
            double inv = 0.0;
            if (lane == 0) {
                const double piv = rd[d];
                if (piv == 0.0 || !isfinite(piv)) bad = 1;
                inv = 1.0 / piv;
                Dinv[d] = inv;
            }
            inv = __shfl_sync(0xffffffffu, inv, 0);
            for (int c = d + 1 + lane; c < k; c += 32) rd[c] *= inv;
        }
        cluster.sync();  // row d scaled, visible to the cluster
        const double *src = cluster.map_shared_rank(Wl + (size_t)(d / kLucCtas) * k, owner);
        for (int c = d + 1 + threadIdx.x; c < k; c += blockDim.x) prow[c] = src[c];
        __syncthreads();
        // local rows i > d: rows by warp, columns by lane
        const int li0 = (d + 1 - rank + kLucCtas - 1) / kLucCtas;  // first local row past d
        for (int li = li0 + warp; li < nloc; li += kLucThreads / 32) {
            double *wi = Wl + (size_t)li * k;
            const double lid = wi[d];
            for (int c = d + 1 + lane; c < k; c += 32) wi[c] = wi[c] - lid * prow[c];
        }
        __syncthreads();
    }
    // factors and their transpose (the column-sweep solves read FT)
    double *FT = F + (size_t)k * k + k;
    for (int idx = threadIdx.x; idx < nloc * k; idx += blockDim.x) {
        const int li = idx / k, c = idx - li * k;
        const int i = li * kLucCtas + rank;
        F[(size_t)i * k + c] = Wl[idx];
        FT[(size_t)c * k + i] = Wl[idx];
    }
    if (threadIdx.x == 0 && bad && status) atomicOr(status, kStatusBreakdown);
    cluster.sync();  // no CTA leaves while another may still read its rows
}

// One CTA with one barrier per elimination step (k <= kLuLaMaxK): warp 0
// updates row d + 1 at step d and at once takes its pivot and scales it into
// U's row -- the next step's critical path -- while warps 1..7 update rows
// d + 2 .. k - 1 as one flat range of (row, column) entries, so every FP64
// instruction of the trailing update carries 32 useful lanes.  Every element
// sees the same operations in the same order as lu_factor_kernel
// (bit-identical factors); the two-barrier factor and the cluster factor pay
// a barrier (a cluster barrier) and the serial pivot work at every step.
constexpr int kLuLaThreads = 256;
constexpr int kLuLaMaxK = 128;  // k x k doubles in shared memory (128 KB); taken for k <= 64

__device__ __forceinline__ void lu_pivot_row(double *W, int k, int i, double *Dinv, int lane,
                                             int &bad) {
    double inv = 0.0;
    if (lane == 0) {
        const double piv = W[i * k + i];
        if (piv == 0.0 || !isfinite(piv)) bad = 1;
        inv = 1.0 / piv;
        Dinv[i] = inv;
    }
    inv = __shfl_sync(0xffffffffu, inv, 0);
    for (int c = i + 1 + lane; c < k; c += 32) W[i * k + c] *= inv;
}

__global__ void __launch_bounds__(kLuLaThreads)
    lu_factor_la_kernel(int k, const double *__restrict__ M, double *__restrict__ F,
                        int *__restrict__ status) {
    extern __shared__ __align__(16) double lw[];
    const int kk = k * k;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    for (int i = tid; i < kk; i += blockDim.x) lw[i] = M[i];
    __syncthreads();
    double *Dinv = F + (size_t)kk;
    int bad = 0;
    if (warp == 0) lu_pivot_row(lw, k, 0, Dinv, lane, bad);
    __syncthreads();
    for (int d = 0; d + 1 < k; ++d) {
        const int x = k - d - 1;  // trailing columns d + 1 .. k - 1
        const double *U = lw + (size_t)d * k;
        if (warp == 0) {
            double *wr = lw + (size_t)(d + 1) * k;
            const double lid = wr[d];
            for (int c = d + 1 + lane; c < k; c += 32) wr[c] = wr[c] - lid * U[c];
            __syncwarp();
            lu_pivot_row(lw, k, d + 1, Dinv, lane, bad);
        } else {
            // entry e = q x + r of rows d + 2 .. k - 1: row d + 2 + q, column
            // d + 1 + r; q = floor(e / x) as the high word of e * ceil(2^32 / x)
            // (exact for e < 2^32 / x)
            const uint32_t mg = x > 1 ? 0xFFFFFFFFu / (uint32_t)x + 1u : 0u;
            for (int e = tid - 32; e < (x - 1) * x; e += kLuLaThreads - 32) {
                const int q = x > 1 ? (int)__umulhi((uint32_t)e, mg) : e;
                double *wr = lw + (size_t)(d + 2 + q) * k;
                const int c = d + 1 + (e - q * x);
                wr[c] = wr[c] - wr[d] * U[c];
            }
        }
        __syncthreads();
    }
    double *FT = F + (size_t)kk + k;
    for (int idx = tid; idx < kk; idx += blockDim.x) {
        const int i = idx / k, j = idx - i * k;
        F[idx] = lw[idx];
        FT[idx] = lw[(size_t)j * k + i];
    }
    if (bad && status) atomicOr(status, kStatusBreakdown);
}

// Y (k x r) from the factor F (k*k factors + k reciprocal diagonal) and RHS
// (k x r).  Each CTA solves kLuRC columns with kLuTPC threads per column
// splitting the inner products; many CTAs spread the FP64 work over SMs.
constexpr int kLuRC = 8;    // right-hand-side columns per CTA
constexpr int kLuTPC = 16;  // threads per column

__global__ void __launch_bounds__(kLuRC * kLuTPC)
    lu_solve_kernel(int k, const double *__restrict__ F, int r, const double *__restrict__ RHS,
                    double *__restrict__ Y, int use_smem) {
    extern __shared__ __align__(16) double sm[];
    double *Fs = use_smem ? sm : nullptr;
    double *Z = sm + (use_smem ? (size_t)k * k + k : 0);  // k x kLuRC
    const double *Fm = use_smem ? Fs : F;
    if (use_smem)
        for (int i = threadIdx.x; i < k * k + k; i += blockDim.x) Fs[i] = F[i];
    const int c0 = blockIdx.x * kLuRC;
    const int cl = threadIdx.x / kLuTPC, sub = threadIdx.x % kLuTPC;
    const int col = c0 + cl;
    const bool active = col < r;
    for (int i = threadIdx.x; i < k * kLuRC; i += blockDim.x) {
        int row = i / kLuRC, cc = i % kLuRC;
        Z[i] = (c0 + cc < r) ? RHS[(size_t)row * r + c0 + cc] : 0.0;
    }
    __syncthreads();
    // forward: Z[i] = (Z[i] - sum_{q<i} L[i][q] Z[q]) * (1 / L[i][i])
    for (int i = 0; i < k; ++i) {
        double s = 0.0;
        for (int q = sub; q < i; q += kLuTPC) s = fma(Fm[i * k + q], Z[q * kLuRC + cl], s);
#pragma unroll
        for (int o = kLuTPC / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, kLuTPC);
        if (sub == 0 && active) Z[i * kLuRC + cl] = (Z[i * kLuRC + cl] - s) * Fm[k * k + i];
        __syncthreads();
    }
    // backward: Y[i] = Z[i] - sum_{q>i} U[i][q] Y[q]   (U unit diagonal)
    for (int i = k - 2; i >= 0; --i) {
        double s = 0.0;
        for (int q = i + 1 + sub; q < k; q += kLuTPC) s = fma(Fm[i * k + q], Z[q * kLuRC + cl], s);
#pragma unroll
        for (int o = kLuTPC / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, kLuTPC);
        if (sub == 0 && active) Z[i * kLuRC + cl] = Z[i * kLuRC + cl] - s;
        __syncthreads();
    }
    for (int i = threadIdx.x; i < k * kLuRC; i += blockDim.x) {
        int row = i / kLuRC, cc = i % kLuRC;
        if (c0 + cc < r) Y[(size_t)row * r + c0 + cc] = Z[i];
    }
}

// Column-sweep ("axpy") triangular solves, one warp per right-hand side:
// lane l owns rows l, l+32, ...; at forward step i the owner's value times
// the stored reciprocal pivot is y_i, broadcast with one shuffle, and every
// lane subtracts L[j][i] y_i from its rows j > i; the backward sweep does the
// same with the unit upper factor.  The factor is staged transposed in shared
// memory (FT[i][j] = F[j][i]), so step i reads row i of FT, conflict-free.
// Same arithmetic as the substitution above, summed column by column
// (agrees with the reference to rounding).  T = ceil(k / 32) rows per lane.
constexpr int kLuWarpsPerCta = 2;

template <int T>
__global__ void __launch_bounds__(32 * kLuWarpsPerCta)
    lu_solve_sweep_kernel(int k, const double *__restrict__ F, int r,
                          const double *__restrict__ RHS, double *__restrict__ Y) {
    extern __shared__ __align__(16) double FT[];  // k * k transposed, then k reciprocal pivots
    double *Dinv = FT + (size_t)k * k;
    {
        // the factor kernel wrote FT after F and the pivots: contiguous copy,
        // 16-byte loads issued 8 at a time (k (k + 1) is even: aligned)
        const double2 *src = reinterpret_cast<const double2 *>(F + (size_t)k * k + k);
        double2 *dst = reinterpret_cast<double2 *>(FT);
        const int n2 = k * k / 2;
        int q = threadIdx.x;
        for (; q + 7 * (int)blockDim.x < n2; q += 8 * blockDim.x) {
            double2 v[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) v[u] = src[q + u * blockDim.x];
#pragma unroll
            for (int u = 0; u < 8; ++u) dst[q + u * blockDim.x] = v[u];
        }
        for (; q < n2; q += blockDim.x) dst[q] = src[q];
        if ((k * k) & 1 && threadIdx.x == 0) FT[k * k - 1] = F[(size_t)k * k + k + k * k - 1];
    }
    for (int i = threadIdx.x; i < k; i += blockDim.x) Dinv[i] = F[(size_t)k * k + i];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int c = blockIdx.x * kLuWarpsPerCta + (threadIdx.x >> 5);
    if (c >= r) return;  // no block-wide barrier follows
    double z[T];
#pragma unroll
    for (int t = 0; t < T; ++t) {
        const int j = lane + 32 * t;
        z[t] = j < k ? RHS[(size_t)j * r + c] : 0.0;
    }
    // forward: y_i = z_i / L_ii; z_j -= L_ji y_i (j > i)
#pragma unroll
    for (int t = 0; t < T; ++t) {
        for (int ii = 0; ii < 32; ++ii) {
            const int i = 32 * t + ii;
            if (i >= k) break;
            const double yi = __shfl_sync(0xffffffffu, z[t], ii) * Dinv[i];
            if (lane == ii) z[t] = yi;
            const double *col = FT + (size_t)i * k;
#pragma unroll
            for (int tt = t; tt < T; ++tt) {
                const int j = lane + 32 * tt;
                if (j > i && j < k) z[tt] = fma(-col[j], yi, z[tt]);
            }
        }
    }
    // backward (U unit diagonal): x_i = z_i; z_j -= U_ji x_i (j < i)
#pragma unroll
    for (int t = T - 1; t >= 0; --t) {
        for (int ii = 31; ii >= 0; --ii) {
            const int i = 32 * t + ii;
            if (i >= k) continue;
            const double xi = __shfl_sync(0xffffffffu, z[t], ii);
            const double *col = FT + (size_t)i * k;
#pragma unroll
            for (int tt = 0; tt <= t; ++tt) {
                const int j = lane + 32 * tt;
                if (j < i) z[tt] = fma(-col[j], xi, z[tt]);
            }
        }
    }
#pragma unroll
    for (int t = 0; t < T; ++t) {
        const int j = lane + 32 * t;
        if (j < k) Y[(size_t)j * r + c] = z[t];
    }
}

template <int T>
static int launch_sweep(cudaStream_t st, int k, const double *F, int r, const double *RHS,
                        double *Y, size_t smem) {
    set_smem_attr(lu_solve_sweep_kernel<T>, (int)max_smem_optin());
    const int blocks = (r + kLuWarpsPerCta - 1) / kLuWarpsPerCta;
    lu_solve_sweep_kernel<T><<<blocks, 32 * kLuWarpsPerCta, smem, st>>>(k, F, r, RHS, Y);
    return check_launch();
}

int launch_lu_factor(cudaStream_t st, int k, const double *M, double *F, int *status) {
    if (k <= 0) return CACG_ERR_ARG;
    // k <= 64 (the serving stream's shapes): one CTA; larger k: the cluster
    // (at k = 96 it measured 8 % less LU time per outer iteration)
    if (k <= 64) {
        const size_t smem = (size_t)k * k * sizeof(double);
        set_smem_attr(lu_factor_la_kernel, kLuLaMaxK * kLuLaMaxK * (int)sizeof(double));
        lu_factor_la_kernel<<<1, kLuLaThreads, smem, st>>>(k, M, F, status);
        return check_launch();
    }
    if (k >= kLucCtas && k <= kLucMaxK) {
        const size_t csmem = ((size_t)((k + kLucCtas - 1) / kLucCtas) * k + k) * sizeof(double);
        set_smem_attr(lu_factor_cluster_kernel, (int)(((size_t)(kLucMaxK / kLucCtas) * kLucMaxK + kLucMaxK) * sizeof(double)));
        lu_factor_cluster_kernel<<<kLucCtas, kLucThreads, csmem, st>>>(k, M, F, status);
        if (cudaPeekAtLastError() == cudaSuccess) return check_launch();  // counted
        cudaGetLastError();  // cluster launch refused: the one-CTA factor below
    }
    int use_smem = k <= kLuSmemK;
    size_t smem = use_smem ? (size_t)k * k * sizeof(double) : 0;
    set_smem_attr(lu_factor_kernel, (int)max_smem_optin());
    lu_factor_kernel<<<1, kLuThreads, smem, st>>>(k, M, F, status, use_smem);
    return check_launch();
}

int launch_lu_solve(cudaStream_t st, int k, const double *F, int r, const double *RHS,
                    double *Y) {
    if (k <= 0 || r <= 0) return CACG_ERR_ARG;
    {
        const size_t sweep_smem = ((size_t)k * k + k) * sizeof(double);
        if (k <= 160 && sweep_smem <= max_smem_optin()) {
            switch ((k + 31) / 32) {
                case 1: return launch_sweep<1>(st, k, F, r, RHS, Y, sweep_smem);
                case 2: return launch_sweep<2>(st, k, F, r, RHS, Y, sweep_smem);
                case 3: return launch_sweep<3>(st, k, F, r, RHS, Y, sweep_smem);
                case 4: return launch_sweep<4>(st, k, F, r, RHS, Y, sweep_smem);
                case 5: return launch_sweep<5>(st, k, F, r, RHS, Y, sweep_smem);
            }
        }
    }
    size_t zbytes = (size_t)k * kLuRC * sizeof(double);
    size_t fbytes = ((size_t)k * k + k) * sizeof(double);
    int use_smem = (fbytes + zbytes) <= max_smem_optin() - 1024;
    size_t smem = zbytes + (use_smem ? fbytes : 0);
    if (smem > max_smem_optin()) return CACG_ERR_UNSUPPORTED;
    set_smem_attr(lu_solve_kernel, (int)max_smem_optin());
    int blocks = (r + kLuRC - 1) / kLuRC;
    lu_solve_kernel<<<blocks, kLuRC * kLuTPC, smem, st>>>(k, F, r, RHS, Y, use_smem);
    return check_launch();
}

}  // namespace cacg

using namespace cacg;

extern "C" int cacg_k_lu(int32_t k, const double *M, int32_t r, const double *RHS, double *Y,
                         int *status, void *stream) {
    cudaStream_t st = (cudaStream_t)stream;
    double *F = nullptr;
    if (cudaMallocAsync((void **)&F, ((size_t)2 * k * k + k) * sizeof(double), st) != cudaSuccess)
        return CACG_ERR_OOM;
    int rc = launch_lu_factor(st, k, M, F, status);
    if (rc == CACG_OK) rc = launch_lu_solve(st, k, F, r, RHS, Y);
    cudaFreeAsync(F, st);
    return rc;
}
