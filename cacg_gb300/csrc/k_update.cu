// k_update.cu -- tall x small products with fused epilogues, norms,
// Gerschgorin bounds, casts.
//
// Reference operations replaced (sclc/cacg):
//   dense_distributedMatL_localMatR_Mul_v1  src/BLAS3.c:794-825  Q beta, Q alpha, AQ alpha
//   dense_mat_mat_add_TP                    src/BLAS3.c:579-612  Q = S - Qbeta,
//                                                                 X += Qalpha, R -= AQalpha
//   norm2square_dist_denseMat_col_n         src/MatrixOperations.c:110-142 (+ Allreduce)
//   gerschgorin_v1                          src/common.c:53-106 (+ Allreduce MIN/MAX)
// The reference materialises Qbeta / Qalpha / AQalpha (n x k and n x m) and
// then runs a separate axpby pass; here the product and the axpby are one
// kernel, and the X/R update also writes the next basis block T_0 = R and the
// per-column residual norms, so R is touched once per outer iteration.
//
// Reductions (norms, bounds, dots) are two-pass with a fixed grid and fixed
// order, hence deterministic.
#include <algorithm>
#include <cfloat>

#include "cacg_internal.cuh"

namespace cacg {

constexpr int kRowThreads = 256;
constexpr int kRedBlocks = 304;  // fixed partial count for two-pass reductions

template <typename T>
static bool direct_ok(int k, int64_t ld, const void *a, const void *b);
template <typename T>
int launch_xrupdate_direct(cudaStream_t st, int64_t n, int k, int m, const T *Q, const T *AQ,
                           int64_t ldq, const double *alpha, double *X, double *R, T *S0,
                           int64_t lds, float *R32, double *norms, double *ws, Slices s0sl,
                           Slices r32sl);

// --------------------------------------------------------------- qupdate
// Qout[i][c] = S[i][c] - sum_j Qin[i][j] * W[j][c]; W = beta (k x k FP64)
// staged in shared memory as T in column blocks of BC; the Qin tile is staged
// transposed (Qt[j][r]) so a thread's 8 rows are two 16-byte vectors.
constexpr int kQuTR = 64;  // rows per tile
constexpr int kQuM = 8;    // micro tile rows
constexpr int kQuN = 4;    // micro tile cols

template <typename T>
__global__ void __launch_bounds__(512)
    qupdate_kernel(int64_t n, int k, int BC, T *Qout, int64_t ldo, const T *__restrict__ Qin,
                   int64_t ldq, const T *S, int64_t lds, const double *__restrict__ beta) {
    // Qout may alias S (each element is read, then written, by one thread)
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int TRP = kQuTR + 16 / sizeof(T);  // padded row length of Qt
    T *Ws = reinterpret_cast<T *>(smem_raw);      // k x BC
    T *Qt = Ws + (size_t)k * BC;                  // k x TRP
    const int c0 = blockIdx.y * BC;
    const int bc = min(BC, k - c0);
    for (int idx = threadIdx.x; idx < k * BC; idx += blockDim.x) {
        int j = idx / BC, c = idx % BC;
        Ws[idx] = c < bc ? T(beta[(size_t)j * k + c0 + c]) : T(0);
    }
    const int nc = BC / kQuN;
    const int tr = threadIdx.x / nc, tc = threadIdx.x % nc;
    const bool active = tr < kQuTR / kQuM;
    for (int64_t r0 = (int64_t)blockIdx.x * kQuTR; r0 < n; r0 += (int64_t)gridDim.x * kQuTR) {
        __syncthreads();
        for (int idx = threadIdx.x; idx < kQuTR * k; idx += blockDim.x) {
            int r = idx / k, j = idx % k;
            int64_t row = r0 + r;
            Qt[j * TRP + r] = row < n ? Qin[row * ldq + j] : T(0);
        }
        __syncthreads();
        if (active) {
            T acc[kQuM][kQuN];
#pragma unroll
            for (int i = 0; i < kQuM; ++i)
#pragma unroll
                for (int q = 0; q < kQuN; ++q) acc[i][q] = T(0);
#pragma unroll 2
            for (int j = 0; j < k; ++j) {
                T qv[kQuM], wv[kQuN];
#pragma unroll
                for (int i = 0; i < kQuM; ++i) qv[i] = Qt[j * TRP + tr * kQuM + i];
#pragma unroll
                for (int q = 0; q < kQuN; ++q) wv[q] = Ws[j * BC + tc * kQuN + q];
#pragma unroll
                for (int i = 0; i < kQuM; ++i)
#pragma unroll
                    for (int q = 0; q < kQuN; ++q) acc[i][q] = fma(qv[i], wv[q], acc[i][q]);
            }
#pragma unroll
            for (int i = 0; i < kQuM; ++i) {
                int64_t row = r0 + tr * kQuM + i;
                if (row >= n) continue;
#pragma unroll
                for (int q = 0; q < kQuN; ++q) {
                    int c = tc * kQuN + q;
                    if (c < bc) Qout[row * ldo + c0 + c] = S[row * lds + c0 + c] - acc[i][q];
                }
            }
        }
    }
}

template <typename T>
int launch_qupdate_direct(cudaStream_t st, int64_t n, int k, T *Qout, int64_t ldo,
                          const T *Qin, int64_t ldq, const T *S, int64_t lds,
                          const double *beta, Slices qsl);

template <typename T>
int launch_qupdate(cudaStream_t st, int64_t n, int k, T *Qout, int64_t ldo, const T *Qin,
                   int64_t ldq, const T *S, int64_t lds, const double *beta) {
    if (n <= 0) return CACG_OK;
    if (k <= 0 || (const void *)Qout == (const void *)Qin) return CACG_ERR_ARG;
    if (k % 4 == 0 && k / 4 <= 256 && ldq % 4 == 0 && (size_t)k * k * sizeof(T) <= 160 * 1024 &&
        aligned16(Qin))
        return launch_qupdate_direct<T>(st, n, k, Qout, ldo, Qin, ldq, S, lds, beta, Slices());
    constexpr int TRP = kQuTR + 16 / sizeof(T);
    size_t budget = max_smem_optin() - 1024;
    auto need = [&](int bc) { return ((size_t)k * bc + (size_t)k * TRP) * sizeof(T); };
    int BC = (k + kQuN - 1) / kQuN * kQuN;
    while (BC > kQuN && need(BC) > budget) BC = (BC / 2 + kQuN - 1) / kQuN * kQuN;
    while (BC > kQuN && (kQuTR / kQuM) * (BC / kQuN) > 512) BC -= kQuN;
    if (need(BC) > budget) return CACG_ERR_UNSUPPORTED;
    int threads = (kQuTR / kQuM) * (BC / kQuN);
    threads = (threads + 31) / 32 * 32;
    size_t smem = need(BC);
    set_smem_attr(qupdate_kernel<T>, (int)max_smem_optin());
    int64_t tiles = (n + kQuTR - 1) / kQuTR;
    int64_t cap = (int64_t)sm_count() * 4;
    dim3 grid((unsigned)(tiles < cap ? tiles : cap), (k + BC - 1) / BC);
    qupdate_kernel<T><<<grid, threads, smem, st>>>(n, k, BC, Qout, ldo, Qin, ldq, S, lds, beta);
    return check_launch();
}

template int launch_qupdate<double>(cudaStream_t, int64_t, int, double *, int64_t,
                                    const double *, int64_t, const double *, int64_t,
                                    const double *);
template int launch_qupdate<float>(cudaStream_t, int64_t, int, float *, int64_t, const float *,
                                   int64_t, const float *, int64_t, const double *);

// -------------------------------------------------------------- xrupdate
// One thread per (row, column c < m); a block covers XR_ROWS rows.  alpha is
// staged in shared memory (FP64, or float-float hi/lo for FP32 inputs).
struct FF2 {
    float s, c;
};

template <typename T>
__global__ void __launch_bounds__(kRowThreads)
    xrupdate_kernel(int64_t n, int k, int m, int mp, const T *__restrict__ Q,
                    const T *__restrict__ AQ, int64_t ldq, const double *__restrict__ alpha,
                    double *__restrict__ X, double *__restrict__ R, T *__restrict__ S0,
                    int64_t lds, float *__restrict__ R32, double *__restrict__ part) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int rows = blockDim.x / mp;
    double *al = reinterpret_cast<double *>(smem_raw);  // k x m (FP64 path)
    float *alh = reinterpret_cast<float *>(al + (size_t)k * m);  // k x m hi
    float *all = alh + (size_t)k * m;                            // k x m lo
    T *Qs = reinterpret_cast<T *>(all + (size_t)k * m + 4);      // rows x k
    T *AQs = Qs + (size_t)rows * k;
    double *red = reinterpret_cast<double *>(AQs + (size_t)rows * k + 4);  // rows x mp
    // alignment fix-up for red
    red = reinterpret_cast<double *>((reinterpret_cast<uintptr_t>(red) + 15) & ~uintptr_t(15));

    for (int idx = threadIdx.x; idx < k * m; idx += blockDim.x) {
        double a = alpha[idx];
        al[idx] = a;
        float h = (float)a;
        alh[idx] = h;
        all[idx] = (float)(a - (double)h);
    }
    const int r = threadIdx.x / mp, c = threadIdx.x % mp;
    const bool active = r < rows && c < m;
    double sq = 0.0;
    for (int64_t r0 = (int64_t)blockIdx.x * rows; r0 < n; r0 += (int64_t)gridDim.x * rows) {
        __syncthreads();
        for (int idx = threadIdx.x; idx < rows * k; idx += blockDim.x) {
            int rr = idx / k, j = idx % k;
            int64_t row = r0 + rr;
            Qs[idx] = row < n ? Q[row * ldq + j] : T(0);
            AQs[idx] = row < n ? AQ[row * ldq + j] : T(0);
        }
        __syncthreads();
        const int64_t row = r0 + r;
        if (active && row < n) {
            double dx, dr;
            if constexpr (sizeof(T) == 8) {
                double ax = 0.0, ar = 0.0;
                for (int j = 0; j < k; ++j) {
                    double a = al[j * m + c];
                    ax = fma((double)Qs[r * k + j], a, ax);
                    ar = fma((double)AQs[r * k + j], a, ar);
                }
                dx = ax;
                dr = ar;
            } else {
                // float-float: q * (ah + al) with the q*ah product split exactly
                float sx = 0.f, cx = 0.f, sr = 0.f, cr = 0.f;
                for (int j = 0; j < k; ++j) {
                    float ah = alh[j * m + c], alo = all[j * m + c];
                    float q = (float)Qs[r * k + j], aq = (float)AQs[r * k + j];
                    float p = q * ah, e = fmaf(q, ah, -p);
                    float t = sx + p, bp = t - sx;
                    cx += ((sx - (t - bp)) + (p - bp)) + e + q * alo;
                    sx = t;
                    p = aq * ah;
                    e = fmaf(aq, ah, -p);
                    t = sr + p;
                    bp = t - sr;
                    cr += ((sr - (t - bp)) + (p - bp)) + e + aq * alo;
                    sr = t;
                }
                dx = (double)sx + (double)cx;
                dr = (double)sr + (double)cr;
            }
            double x = X[row * m + c] + dx;
            double rv = R[row * m + c] - dr;
            X[row * m + c] = x;
            R[row * m + c] = rv;
            if (S0) S0[row * lds + c] = (T)rv;
            if (R32) R32[row * m + c] = (float)rv;
            sq = fma(rv, rv, sq);
        }
    }
    // block reduction of sq over rows, per column, fixed order
    __syncthreads();
    if (part) {
        if (r < rows) red[r * mp + c] = (active ? sq : 0.0);
        __syncthreads();
        if (threadIdx.x < m) {
            double s = 0.0;
            for (int rr = 0; rr < rows; ++rr) s += red[rr * mp + threadIdx.x];
            part[(size_t)blockIdx.x * m + threadIdx.x] = s;
        }
    }
}

// out[c] = sum over g < G of part[g*m + c]; non-finite -> status bit
// out[c] = sum over g of part[g * m + c]: one block per column, each thread
// sums a strided subset in g order, then a fixed shared-memory tree.
constexpr int kColsumThreads = 256;

__global__ void __launch_bounds__(kColsumThreads)
    colsum_kernel(const double *__restrict__ part, int G, int m, double *__restrict__ out) {
    __shared__ double red[kColsumThreads];
    const int c = blockIdx.x;
    double s = 0.0;
    for (int g = threadIdx.x; g < G; g += kColsumThreads) s += part[(size_t)g * m + c];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = kColsumThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[c] = red[0];
}

int launch_colsum(cudaStream_t st, const double *part, int G, int m, double *norms) {
    if (m <= 0) return CACG_OK;
    colsum_kernel<<<m, kColsumThreads, 0, st>>>(part, G, m, norms);
    return check_launch();
}

size_t norm_workspace_doubles(int64_t n, int m) {
    (void)n;
    return (size_t)2048 * (size_t)(m > 0 ? m : 1);  // >= kRedBlocks and kXrMaxBlocks
}

static int pow2ceil(int x) {
    int p = 1;
    while (p < x) p <<= 1;
    return p;
}

template <typename T>
int launch_xrupdate(cudaStream_t st, int64_t n, int k, int m, const T *Q, const T *AQ,
                    int64_t ldq, const double *alpha, double *X, double *R, T *S0, int64_t lds,
                    float *R32, double *norms, double *ws) {
    if (m <= 0 || k <= 0 || m > kRowThreads) return CACG_ERR_ARG;
    if (norms && !ws) return CACG_ERR_ARG;
    int mp = pow2ceil(m);
    int rows = kRowThreads / mp;
    size_t smem = (size_t)k * m * (8 + 4 + 4) + 16 + (size_t)2 * rows * k * sizeof(T) + 32 +
                  (size_t)rows * mp * 8;
    if (smem > max_smem_optin()) return CACG_ERR_UNSUPPORTED;
    set_smem_attr(xrupdate_kernel<T>, (int)max_smem_optin());
    int G = kRedBlocks;
    int64_t tiles = (n + rows - 1) / rows;
    if (tiles < G) G = (int)(tiles > 0 ? tiles : 1);
    xrupdate_kernel<T><<<G, kRowThreads, smem, st>>>(n, k, m, mp, Q, AQ, ldq, alpha, X, R, S0,
                                                     lds, R32, norms ? ws : nullptr);
    int rc = check_launch();
    if (rc != CACG_OK || !norms) return rc;
    return launch_colsum(st, ws, G, m, norms);
}

template int launch_xrupdate<double>(cudaStream_t, int64_t, int, int, const double *,
                                     const double *, int64_t, const double *, double *,
                                     double *, double *, int64_t, float *, double *, double *);
template int launch_xrupdate<float>(cudaStream_t, int64_t, int, int, const float *,
                                    const float *, int64_t, const double *, double *, double *,
                                    float *, int64_t, float *, double *, double *);

// ------------------------------------------------- xrupdate (fast path)
// X += Q alpha; R -= AQ alpha with products accumulated in T (FP32 FMAs in the
// mixed mode, FP64 in the FP64 mode); the X/R additions are FP64.  A thread
// owns one row and 4 consecutive columns; Q and AQ tiles are staged in shared
// memory with a padded row length, alpha as T.
constexpr int kXrG = 4;  // columns per thread

template <typename T>
__global__ void __launch_bounds__(kRowThreads)
    xrupdate_fast_kernel(int64_t n, int k, int m, const T *__restrict__ Q,
                         const T *__restrict__ AQ, int64_t ldq, const double *__restrict__ alpha,
                         double *__restrict__ X, double *__restrict__ R, T *__restrict__ S0,
                         int64_t lds, float *__restrict__ R32, double *__restrict__ part) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int G = (m + kXrG - 1) / kXrG;  // column groups per row
    const int mp = G * kXrG;
    const int TR = blockDim.x / G;        // rows per tile
    const int kp = k + 16 / (int)sizeof(T);
    T *As = reinterpret_cast<T *>(smem_raw);  // k x mp
    T *Qs = As + (size_t)k * mp;              // TR x kp
    T *AQs = Qs + (size_t)TR * kp;            // TR x kp
    double *red = reinterpret_cast<double *>(AQs + (size_t)TR * kp);  // TR x mp
    for (int idx = threadIdx.x; idx < k * mp; idx += blockDim.x) {
        int j = idx / mp, c = idx % mp;
        As[idx] = c < m ? T(alpha[(size_t)j * m + c]) : T(0);
    }
    const int r = threadIdx.x / G, g = threadIdx.x % G;
    const bool active = r < TR;
    double sq[kXrG] = {0.0, 0.0, 0.0, 0.0};
    for (int64_t r0 = (int64_t)blockIdx.x * TR; r0 < n; r0 += (int64_t)gridDim.x * TR) {
        __syncthreads();
        for (int idx = threadIdx.x; idx < TR * k; idx += blockDim.x) {
            int rr = idx / k, j = idx % k;
            int64_t row = r0 + rr;
            Qs[rr * kp + j] = row < n ? Q[row * ldq + j] : T(0);
            AQs[rr * kp + j] = row < n ? AQ[row * ldq + j] : T(0);
        }
        __syncthreads();
        const int64_t row = r0 + r;
        if (active && row < n) {
            T ax[kXrG], ar[kXrG];
#pragma unroll
            for (int q = 0; q < kXrG; ++q) ax[q] = ar[q] = T(0);
#pragma unroll 4
            for (int j = 0; j < k; ++j) {
                const T qv = Qs[r * kp + j], aqv = AQs[r * kp + j];
                const T *aj = As + (size_t)j * mp + g * kXrG;
#pragma unroll
                for (int q = 0; q < kXrG; ++q) {
                    ax[q] = fma(qv, aj[q], ax[q]);
                    ar[q] = fma(aqv, aj[q], ar[q]);
                }
            }
#pragma unroll
            for (int q = 0; q < kXrG; ++q) {
                const int c = g * kXrG + q;
                if (c < m) {
                    double x = X[row * m + c] + (double)ax[q];
                    double rv = R[row * m + c] - (double)ar[q];
                    X[row * m + c] = x;
                    R[row * m + c] = rv;
                    if (S0) S0[row * lds + c] = (T)rv;
                    if (R32) R32[row * m + c] = (float)rv;
                    sq[q] = fma(rv, rv, sq[q]);
                }
            }
        }
    }
    __syncthreads();
    if (part) {
        if (active)
#pragma unroll
            for (int q = 0; q < kXrG; ++q) red[r * mp + g * kXrG + q] = sq[q];
        __syncthreads();
        for (int c = threadIdx.x; c < m; c += blockDim.x) {
            double s = 0.0;
            for (int rr = 0; rr < TR; ++rr) s += red[rr * mp + c];
            part[(size_t)blockIdx.x * m + c] = s;
        }
    }
}

template <typename T>
int launch_xrupdate_fast(cudaStream_t st, int64_t n, int k, int m, const T *Q, const T *AQ,
                         int64_t ldq, const double *alpha, double *X, double *R, T *S0,
                         int64_t lds, float *R32, double *norms, double *ws) {
    if (m <= 0 || k <= 0) return CACG_ERR_ARG;
    if (norms && !ws) return CACG_ERR_ARG;
    if constexpr (std::is_same<T, float>::value) {
        if (m == 16) {
            int rc = launch_xrupdate_m16(st, n, k, Q, AQ, ldq, alpha, X, R, S0, lds, R32, norms,
                                         ws);
            if (rc != CACG_ERR_UNSUPPORTED) return rc;
        }
    }
    if (direct_ok<T>(k, ldq, Q, AQ))
        return launch_xrupdate_direct<T>(st, n, k, m, Q, AQ, ldq, alpha, X, R, S0, lds, R32, norms,
                                         ws, Slices(), Slices());
    const int G = (m + kXrG - 1) / kXrG;
    if (G > kRowThreads) return CACG_ERR_ARG;
    const int mp = G * kXrG;
    const int TR = kRowThreads / G;
    const int kp = k + 16 / (int)sizeof(T);
    size_t smem = ((size_t)k * mp + 2 * (size_t)TR * kp) * sizeof(T) + (size_t)TR * mp * 8 + 16;
    if (smem > max_smem_optin()) return CACG_ERR_UNSUPPORTED;
    set_smem_attr(xrupdate_fast_kernel<T>, (int)max_smem_optin());
    int G2 = kRedBlocks;
    int64_t tiles = (n + TR - 1) / TR;
    if (tiles < G2) G2 = (int)(tiles > 0 ? tiles : 1);
    xrupdate_fast_kernel<T><<<G2, kRowThreads, smem, st>>>(n, k, m, Q, AQ, ldq, alpha, X, R, S0,
                                                           lds, R32, norms ? ws : nullptr);
    int rc = check_launch();
    if (rc != CACG_OK || !norms) return rc;
    return launch_colsum(st, ws, G2, m, norms);
}

template int launch_xrupdate_fast<double>(cudaStream_t, int64_t, int, int, const double *,
                                          const double *, int64_t, const double *, double *,
                                          double *, double *, int64_t, float *, double *,
                                          double *);
template int launch_xrupdate_fast<float>(cudaStream_t, int64_t, int, int, const float *,
                                         const float *, int64_t, const double *, double *,
                                         double *, float *, int64_t, float *, double *, double *);

// ----------------------------------------------- direct-load update kernels
// Tall operand rows are read straight from global memory as 16-byte vectors
// (threads sharing a row hit the same L1 lines), the small coefficient matrix
// lives in shared memory as T, and there is no per-tile staging or barrier.
// Used when k and the row strides are multiples of the vector width.

// Qout[i][c..c+3] = S[i][c..c+3] - sum_j Qin[i][j] beta[j][c..c+3]; a thread
// owns kDqRows rows x 4 columns.
constexpr int kDqRows = 4;

template <typename T>
__global__ void __launch_bounds__(256)
    qupdate_direct_kernel(int64_t n, int k, T *Qout, int64_t ldo, const T *__restrict__ Qin,
                          int64_t ldq, const T *S, int64_t lds, const double *__restrict__ beta,
                          Slices qsl) {
    // Qout may alias S (each element is read, then written, by one thread)
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *Ws = reinterpret_cast<T *>(smem_raw);  // k x k
    for (int idx = threadIdx.x; idx < k * k; idx += blockDim.x) Ws[idx] = T(beta[idx]);
    __syncthreads();
    const int G = k / 4;                       // column groups
    const int groups_per_block = blockDim.x / G;
    const int lg = threadIdx.x / G, cg = threadIdx.x % G;
    if (lg >= groups_per_block) return;
    const int64_t ngroups = (n + kDqRows - 1) / kDqRows;
    for (int64_t rg = (int64_t)blockIdx.x * groups_per_block + lg; rg < ngroups;
         rg += (int64_t)gridDim.x * groups_per_block) {
        const int64_t r0 = rg * kDqRows;
        T acc[kDqRows][4];
#pragma unroll
        for (int i = 0; i < kDqRows; ++i)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[i][q] = T(0);
        for (int j = 0; j < k; j += 4) {
            T qv[kDqRows][4];
#pragma unroll
            for (int i = 0; i < kDqRows; ++i) {
                const int64_t row = r0 + i < n ? r0 + i : n - 1;
                if constexpr (sizeof(T) == 4) {
                    float4 v = __ldg(reinterpret_cast<const float4 *>(Qin + row * ldq + j));
                    qv[i][0] = v.x; qv[i][1] = v.y; qv[i][2] = v.z; qv[i][3] = v.w;
                } else {
                    double2 v0 = __ldg(reinterpret_cast<const double2 *>(Qin + row * ldq + j));
                    double2 v1 = __ldg(reinterpret_cast<const double2 *>(Qin + row * ldq + j + 2));
                    qv[i][0] = v0.x; qv[i][1] = v0.y; qv[i][2] = v1.x; qv[i][3] = v1.y;
                }
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const T *w = Ws + (size_t)(j + u) * k + cg * 4;
                T w0, w1, w2, w3;
                if constexpr (sizeof(T) == 4) {
                    float4 wv = *reinterpret_cast<const float4 *>(w);
                    w0 = wv.x; w1 = wv.y; w2 = wv.z; w3 = wv.w;
                } else {
                    double2 wa = *reinterpret_cast<const double2 *>(w);
                    double2 wb = *reinterpret_cast<const double2 *>(w + 2);
                    w0 = wa.x; w1 = wa.y; w2 = wb.x; w3 = wb.y;
                }
#pragma unroll
                for (int i = 0; i < kDqRows; ++i) {
                    acc[i][0] = fma(qv[i][u], w0, acc[i][0]);
                    acc[i][1] = fma(qv[i][u], w1, acc[i][1]);
                    acc[i][2] = fma(qv[i][u], w2, acc[i][2]);
                    acc[i][3] = fma(qv[i][u], w3, acc[i][3]);
                }
            }
        }
#pragma unroll
        for (int i = 0; i < kDqRows; ++i) {
            const int64_t row = r0 + i;
            if (row >= n) break;
            const T *sp = S + row * lds + cg * 4;
            T *op = Qout + row * ldo + cg * 4;
            T o[4] = {sp[0] - acc[i][0], sp[1] - acc[i][1], sp[2] - acc[i][2], sp[3] - acc[i][3]};
            op[0] = o[0];
            op[1] = o[1];
            op[2] = o[2];
            op[3] = o[3];
            if constexpr (sizeof(T) == 4) {
                if (qsl.p) store_slices4(qsl, row * ldo + cg * 4, o);
            }
        }
    }
}

// X += Q alpha; R -= AQ alpha (products in T, additions in FP64); a thread
// owns one row x 4 columns; norms partials per block.
template <typename T>
__global__ void __launch_bounds__(256)
    xrupdate_direct_kernel(int64_t n, int k, int m, const T *__restrict__ Q,
                           const T *__restrict__ AQ, int64_t ldq,
                           const double *__restrict__ alpha, double *__restrict__ X,
                           double *__restrict__ R, T *__restrict__ S0, int64_t lds,
                           float *__restrict__ R32, double *__restrict__ part, Slices s0sl,
                           Slices r32sl) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int G = (m + 3) / 4, mp = G * 4;
    T *As = reinterpret_cast<T *>(smem_raw);  // k x mp
    double *red = reinterpret_cast<double *>(As + (size_t)k * mp +
                                             ((size_t)k * mp * sizeof(T) % 16 ? 2 : 0));
    for (int idx = threadIdx.x; idx < k * mp; idx += blockDim.x) {
        int j = idx / mp, c = idx % mp;
        As[idx] = c < m ? T(alpha[(size_t)j * m + c]) : T(0);
    }
    __syncthreads();
    const int rows_per_block = blockDim.x / G;
    const int lr = threadIdx.x / G, g = threadIdx.x % G;
    const bool active = lr < rows_per_block;
    double sq[4] = {0.0, 0.0, 0.0, 0.0};
    for (int64_t row = (int64_t)blockIdx.x * rows_per_block + lr; active && row < n;
         row += (int64_t)gridDim.x * rows_per_block) {
        T ax[4] = {T(0), T(0), T(0), T(0)}, ar[4] = {T(0), T(0), T(0), T(0)};
        const T *qr = Q + row * ldq, *aqr = AQ + row * ldq;
        for (int j = 0; j < k; j += 4) {
            T q4[4], a4[4];
            if constexpr (sizeof(T) == 4) {
                float4 v = __ldg(reinterpret_cast<const float4 *>(qr + j));
                float4 w = __ldg(reinterpret_cast<const float4 *>(aqr + j));
                q4[0] = v.x; q4[1] = v.y; q4[2] = v.z; q4[3] = v.w;
                a4[0] = w.x; a4[1] = w.y; a4[2] = w.z; a4[3] = w.w;
            } else {
                double2 v0 = __ldg(reinterpret_cast<const double2 *>(qr + j));
                double2 v1 = __ldg(reinterpret_cast<const double2 *>(qr + j + 2));
                double2 w0 = __ldg(reinterpret_cast<const double2 *>(aqr + j));
                double2 w1 = __ldg(reinterpret_cast<const double2 *>(aqr + j + 2));
                q4[0] = v0.x; q4[1] = v0.y; q4[2] = v1.x; q4[3] = v1.y;
                a4[0] = w0.x; a4[1] = w0.y; a4[2] = w1.x; a4[3] = w1.y;
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const T *al = As + (size_t)(j + u) * mp + g * 4;
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    ax[q] = fma(q4[u], al[q], ax[q]);
                    ar[q] = fma(a4[u], al[q], ar[q]);
                }
            }
        }
        float rf[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int c = g * 4 + q;
            if (c < m) {
                double x = X[row * m + c] + (double)ax[q];
                double rv = R[row * m + c] - (double)ar[q];
                X[row * m + c] = x;
                R[row * m + c] = rv;
                if (S0) S0[row * lds + c] = (T)rv;
                if (R32) R32[row * m + c] = (float)rv;
                rf[q] = (float)rv;
                sq[q] = fma(rv, rv, sq[q]);
            }
        }
        // slice planes (used only with m % 4 == 0, so the group is full)
        if (s0sl.p) store_slices4(s0sl, row * lds + g * 4, rf);
        if (r32sl.p) store_slices4(r32sl, row * m + g * 4, rf);
    }
    if (!part) return;
    __syncthreads();
    if (active)
#pragma unroll
        for (int q = 0; q < 4; ++q) red[lr * mp + g * 4 + q] = sq[q];
    __syncthreads();
    for (int c = threadIdx.x; c < m; c += blockDim.x) {
        double t = 0.0;
        for (int rr = 0; rr < rows_per_block; ++rr) t += red[rr * mp + c];
        part[(size_t)blockIdx.x * m + c] = t;
    }
}

template <typename T>
static bool direct_ok(int k, int64_t ld, const void *a, const void *b) {
    return k % 4 == 0 && ld % 4 == 0 && aligned16(a) && (!b || aligned16(b));
}

template <typename T>
int launch_qupdate_direct(cudaStream_t st, int64_t n, int k, T *Qout, int64_t ldo,
                          const T *Qin, int64_t ldq, const T *S, int64_t lds,
                          const double *beta, Slices qsl) {
    const int G = k / 4;
    int threads = std::max(G, (256 / G) * G);
    if (threads > 256) threads = G;  // G <= 256 here
    const int groups_per_block = threads / G;
    size_t smem = (size_t)k * k * sizeof(T);
    set_smem_attr(qupdate_direct_kernel<T>, (int)max_smem_optin());
    int64_t ngroups = (n + kDqRows - 1) / kDqRows;
    int64_t blocks = (ngroups + groups_per_block - 1) / groups_per_block;
    int64_t cap = (int64_t)sm_count() * 8;
    if (blocks > cap) blocks = cap;
    qupdate_direct_kernel<T><<<(unsigned)blocks, threads, smem, st>>>(n, k, Qout, ldo, Qin, ldq, S,
                                                                      lds, beta, qsl);
    return check_launch();
}

constexpr int kXrMaxBlocks = 2048;  // norm partials per xrupdate launch (upper bound)

template <typename T>
int launch_xrupdate_direct(cudaStream_t st, int64_t n, int k, int m, const T *Q, const T *AQ,
                           int64_t ldq, const double *alpha, double *X, double *R, T *S0,
                           int64_t lds, float *R32, double *norms, double *ws, Slices s0sl,
                           Slices r32sl) {
    const int G = (m + 3) / 4, mp = G * 4;
    if (G > 256) return CACG_ERR_ARG;
    const int threads = (256 / G) * G;
    const int rows_per_block = threads / G;
    size_t smem = (size_t)k * mp * sizeof(T) + 16 + (size_t)rows_per_block * mp * 8;
    if (smem > max_smem_optin()) return CACG_ERR_UNSUPPORTED;
    set_smem_attr(xrupdate_direct_kernel<T>, (int)max_smem_optin());
    int64_t blocks = (n + rows_per_block - 1) / rows_per_block;
    int64_t cap = std::min<int64_t>((int64_t)sm_count() * 8, kXrMaxBlocks);
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    xrupdate_direct_kernel<T><<<(unsigned)blocks, threads, smem, st>>>(
        n, k, m, Q, AQ, ldq, alpha, X, R, S0, lds, R32, norms ? ws : nullptr, s0sl, r32sl);
    int rc = check_launch();
    if (rc != CACG_OK || !norms) return rc;
    return launch_colsum(st, ws, (int)blocks, m, norms);
}

// dst = src for an n x w FP32 block, rows of lds and ldd values
__global__ void copy_rows_f32_kernel(int64_t n, int w, const float *__restrict__ src, int64_t lds,
                                     float *__restrict__ dst, int64_t ldd) {
    const int64_t total = n * w;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = e / w;
        const int c = (int)(e - r * w);
        dst[r * ldd + c] = src[r * lds + c];
    }
}

int launch_copy_rows_f32(cudaStream_t st, int64_t n, int w, const float *src, int64_t lds,
                         float *dst, int64_t ldd) {
    if (n <= 0 || w <= 0) return CACG_OK;
    const int64_t blocks =
        std::min<int64_t>((n * w + 255) / 256, (int64_t)sm_count() * 16);
    copy_rows_f32_kernel<<<(unsigned)blocks, 256, 0, st>>>(n, w, src, lds, dst, ldd);
    return check_launch();
}

// ------------------------------------------------------ residual epilogue
// After R = B - A X (launch_spmm): S0 = cast(R), R32 = (float)R, norm partials.
template <typename T>
__global__ void __launch_bounds__(kRowThreads)
    rowpost_kernel(int64_t n, int m, int mp, const double *__restrict__ R, T *__restrict__ S0,
                   int64_t lds, float *__restrict__ R32, double *__restrict__ part,
                   Slices s0sl = Slices(), Slices r32sl = Slices()) {
    __shared__ double red[kRowThreads];
    const int rows = blockDim.x / mp;
    const int r = threadIdx.x / mp, c = threadIdx.x % mp;
    const bool active = r < rows && c < m;
    double sq = 0.0;
    for (int64_t r0 = (int64_t)blockIdx.x * rows; r0 < n; r0 += (int64_t)gridDim.x * rows) {
        int64_t row = r0 + r;
        if (active && row < n) {
            double v = R[row * m + c];
            if (S0) S0[row * lds + c] = (T)v;
            if (R32) R32[row * m + c] = (float)v;
            if (s0sl.p) store_slices1(s0sl, row * lds + c, (float)v);
            if (r32sl.p) store_slices1(r32sl, row * m + c, (float)v);
            sq = fma(v, v, sq);
        }
    }
    red[threadIdx.x] = active ? sq : 0.0;
    __syncthreads();
    if (part && threadIdx.x < m) {
        double s = 0.0;
        for (int rr = 0; rr < rows; ++rr) s += red[rr * mp + threadIdx.x];
        part[(size_t)blockIdx.x * m + threadIdx.x] = s;
    }
}

int launch_residual(cudaStream_t st, int64_t n, const int32_t *rp, const int32_t *ci,
                    const double *val, int m, const double *X, const double *B, double *R,
                    void *S0, int s0_is_f32, int64_t lds, double *norms, double *ws,
                    double avg_nnz) {
    int rc = launch_spmm<double>(st, n, rp, ci, val, m, X, m, R, m, B, m, nullptr, 0, -1.0,
                                 1.0, 0.0, avg_nnz);
    if (rc != CACG_OK) return rc;
    return launch_residual_post(st, n, m, R, S0, s0_is_f32, lds, norms, ws);
}

// R = B - A X already formed: S0 = cast(R), norm partials, column norms.
int launch_residual_post(cudaStream_t st, int64_t n, int m, double *R, void *S0, int s0_is_f32,
                         int64_t lds, double *norms, double *ws) {
    int rc;
    if (m > kRowThreads) return CACG_ERR_ARG;
    int mp = pow2ceil(m);
    int rows = kRowThreads / mp;
    int G = kRedBlocks;
    int64_t tiles = (n + rows - 1) / rows;
    if (tiles < G) G = (int)(tiles > 0 ? tiles : 1);
    if (s0_is_f32)
        rowpost_kernel<float><<<G, kRowThreads, 0, st>>>(n, m, mp, R, (float *)S0, lds, nullptr,
                                                         norms ? ws : nullptr);
    else
        rowpost_kernel<double><<<G, kRowThreads, 0, st>>>(n, m, mp, R, (double *)S0, lds,
                                                          nullptr, norms ? ws : nullptr);
    rc = check_launch();
    if (rc != CACG_OK || !norms) return rc;
    return launch_colsum(st, ws, G, m, norms);
}

int launch_colnorm(cudaStream_t st, int64_t n, int m, const double *R, double *norms,
                   double *ws) {
    if (m > kRowThreads || m <= 0) return CACG_ERR_ARG;
    int mp = pow2ceil(m);
    int rows = kRowThreads / mp;
    int G = kRedBlocks;
    int64_t tiles = (n + rows - 1) / rows;
    if (tiles < G) G = (int)(tiles > 0 ? tiles : 1);
    rowpost_kernel<double><<<G, kRowThreads, 0, st>>>(n, m, mp, R, nullptr, 0, nullptr, ws);
    int rc = check_launch();
    if (rc != CACG_OK) return rc;
    return launch_colsum(st, ws, G, m, norms);
}

int launch_residual_sl(cudaStream_t st, int64_t n, const int32_t *rp, const int32_t *ci,
                       const double *val, int m, const double *X, const double *B, double *R,
                       float *S0, int64_t lds, float *R32, double *norms, double *ws,
                       double avg_nnz, Slices S0sl, Slices R32sl) {
    int rc = launch_spmm<double>(st, n, rp, ci, val, m, X, m, R, m, B, m, nullptr, 0, -1.0,
                                 1.0, 0.0, avg_nnz);
    if (rc != CACG_OK) return rc;
    if (m > kRowThreads) return CACG_ERR_ARG;
    int mp = pow2ceil(m);
    int rows = kRowThreads / mp;
    int G = kRedBlocks;
    int64_t tiles = (n + rows - 1) / rows;
    if (tiles < G) G = (int)(tiles > 0 ? tiles : 1);
    rowpost_kernel<float><<<G, kRowThreads, 0, st>>>(n, m, mp, R, S0, lds, R32,
                                                     norms ? ws : nullptr, S0sl, R32sl);
    rc = check_launch();
    if (rc != CACG_OK || !norms) return rc;
    return launch_colsum(st, ws, G, m, norms);
}

int launch_qupdate_sl(cudaStream_t st, int64_t n, int k, float *Qout, int64_t ldo,
                      const float *Qin, int64_t ldq, const float *S, int64_t lds,
                      const double *beta, Slices Qsl) {
    if (n <= 0) return CACG_OK;
    if (!(k % 4 == 0 && k / 4 <= 256 && ldq % 4 == 0 && ldo % 4 == 0 &&
          (size_t)k * k * sizeof(float) <= 160 * 1024 && aligned16(Qin)) ||
        (const void *)Qout == (const void *)Qin)
        return CACG_ERR_ARG;
    return launch_qupdate_direct<float>(st, n, k, Qout, ldo, Qin, ldq, S, lds, beta, Qsl);
}

int launch_xrupdate_sl(cudaStream_t st, int64_t n, int k, int m, const float *Q,
                       const float *AQ, int64_t ldq, const double *alpha, double *X, double *R,
                       float *S0, int64_t lds, float *R32, double *norms, double *ws,
                       Slices S0sl, Slices R32sl) {
    if (m % 4 != 0 || !direct_ok<float>(k, ldq, Q, AQ) || (norms && !ws)) return CACG_ERR_ARG;
    return launch_xrupdate_direct<float>(st, n, k, m, Q, AQ, ldq, alpha, X, R, S0, lds, R32,
                                         norms, ws, S0sl, R32sl);
}

// ------------------------------------------------------------ Gerschgorin
__global__ void __launch_bounds__(kRowThreads)
    gersch_kernel(int64_t n, const int32_t *__restrict__ rp, const int32_t *__restrict__ ci,
                  const double *__restrict__ v, double *__restrict__ part) {
    __shared__ double smin[kRowThreads], smax[kRowThreads];
    double lmin = DBL_MAX, lmax = DBL_MIN;  // reference initial values
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        double acc = 0.0, diag = 0.0;
        for (int p = rp[i]; p < rp[i + 1]; ++p) {
            double a = v[p];
            if ((int64_t)ci[p] != i)
                acc += fabs(a);
            else
                diag = a;
        }
        lmax = fmax(lmax, acc + diag);
        lmin = fmin(lmin, diag - acc);
    }
    smin[threadIdx.x] = lmin;
    smax[threadIdx.x] = lmax;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            smin[threadIdx.x] = fmin(smin[threadIdx.x], smin[threadIdx.x + o]);
            smax[threadIdx.x] = fmax(smax[threadIdx.x], smax[threadIdx.x + o]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = smin[0];
        part[2 * blockIdx.x + 1] = smax[0];
    }
}

__global__ void gersch_final_kernel(const double *__restrict__ part, int G,
                                    double *__restrict__ out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double lmin = DBL_MAX, lmax = DBL_MIN;
    for (int g = 0; g < G; ++g) {
        lmin = fmin(lmin, part[2 * g]);
        lmax = fmax(lmax, part[2 * g + 1]);
    }
    out[0] = lmin;
    out[1] = lmax;
}

int launch_gerschgorin(cudaStream_t st, int64_t n, const int32_t *rp, const int32_t *ci,
                       const double *val, double *out, double *ws) {
    int G = kRedBlocks;
    int64_t need = (n + kRowThreads - 1) / kRowThreads;
    if (need < G) G = (int)(need > 0 ? need : 1);
    gersch_kernel<<<G, kRowThreads, 0, st>>>(n, rp, ci, val, ws);
    int rc = check_launch();
    if (rc != CACG_OK) return rc;
    gersch_final_kernel<<<1, 32, 0, st>>>(ws, G, out);
    return check_launch();
}

// ------------------------------------------------------------------ casts
__global__ void cast_kernel(int64_t count, const double *__restrict__ in, float *__restrict__ out) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
         i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (float)in[i];
}

int launch_cast_f64_f32(cudaStream_t st, int64_t count, const double *in, float *out) {
    if (count <= 0) return CACG_OK;
    int64_t blocks = (count + 255) / 256;
    int64_t cap = (int64_t)sm_count() * 8;
    cast_kernel<<<(unsigned)(blocks < cap ? blocks : cap), 256, 0, st>>>(count, in, out);
    return check_launch();
}

template <typename T>
__global__ void cast_strided_kernel(int64_t n, int w, const double *__restrict__ in, int64_t ldi,
                                    T *__restrict__ out, int64_t ldo) {
    int64_t tot = n * w;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < tot;
         q += (int64_t)gridDim.x * blockDim.x) {
        int64_t i = q / w;
        int c = (int)(q % w);
        out[i * ldo + c] = (T)in[i * ldi + c];
    }
}

int launch_cast_strided(cudaStream_t st, int64_t n, int w, const double *in, int64_t ldi,
                        void *out, int out_is_f32, int64_t ldo) {
    if (n <= 0) return CACG_OK;
    int64_t blocks = (n * w + 255) / 256;
    int64_t cap = (int64_t)sm_count() * 8;
    unsigned g = (unsigned)(blocks < cap ? blocks : cap);
    if (out_is_f32)
        cast_strided_kernel<float><<<g, 256, 0, st>>>(n, w, in, ldi, (float *)out, ldo);
    else
        cast_strided_kernel<double><<<g, 256, 0, st>>>(n, w, in, ldi, (double *)out, ldo);
    return check_launch();
}

// ----------------------------------------------------------- dot / axpby
__global__ void __launch_bounds__(kRowThreads)
    dot_kernel(int64_t n, const double *__restrict__ a, const double *__restrict__ b,
               double *__restrict__ part) {
    __shared__ double red[kRowThreads];
    double s = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        s = fma(a[i], b[i], s);
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

int launch_dot(cudaStream_t st, int64_t n, const double *a, const double *b, double *out,
               double *ws) {
    int G = kRedBlocks;
    int64_t need = (n + kRowThreads - 1) / kRowThreads;
    if (need < G) G = (int)(need > 0 ? need : 1);
    dot_kernel<<<G, kRowThreads, 0, st>>>(n, a, b, ws);
    int rc = check_launch();
    if (rc != CACG_OK) return rc;
    colsum_kernel<<<1, kColsumThreads, 0, st>>>(ws, G, 1, out);
    return check_launch();
}

__global__ void axpby_kernel(int64_t n, double a, const double *__restrict__ x, double b,
                             double *__restrict__ y) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        y[i] = a * x[i] + b * y[i];
}

int launch_axpby(cudaStream_t st, int64_t n, double a, const double *x, double b, double *y) {
    if (n <= 0) return CACG_OK;
    int64_t blocks = (n + 255) / 256;
    int64_t cap = (int64_t)sm_count() * 8;
    axpby_kernel<<<(unsigned)(blocks < cap ? blocks : cap), 256, 0, st>>>(n, a, x, b, y);
    return check_launch();
}

}  // namespace cacg

using namespace cacg;

extern "C" int cacg_k_gerschgorin(int64_t n, const int32_t *row_ptr, const int32_t *col_idx,
                                  const double *val, double *out, void *stream) {
    cudaStream_t st = (cudaStream_t)stream;
    double *ws = nullptr;
    if (cudaMallocAsync((void **)&ws, 2 * kRedBlocks * sizeof(double), st) != cudaSuccess)
        return CACG_ERR_OOM;
    int rc = launch_gerschgorin(st, n, row_ptr, col_idx, val, out, ws);
    cudaFreeAsync(ws, st);
    return rc;
}

// Runs a launcher that reports bounded-wait expiry in a device status word;
// maps the word to CACG_ERR_TIMEOUT (synchronises the stream).
template <typename F>
static int run_with_status(cudaStream_t st, F &&launch) {
    int *dstat = nullptr;
    if (cudaMallocAsync((void **)&dstat, sizeof(int), st) != cudaSuccess) return CACG_ERR_OOM;
    cudaMemsetAsync(dstat, 0, sizeof(int), st);
    int rc = launch(dstat);
    int hstat = 0;
    if (rc == CACG_OK) {
        cudaMemcpyAsync(&hstat, dstat, sizeof(int), cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess)
            rc = CACG_ERR_CUDA;
        else if (hstat & kStatusTimeout)
            rc = CACG_ERR_TIMEOUT;
    }
    cudaFreeAsync(dstat, st);
    return rc;
}

extern "C" int cacg_k_qupdate(int32_t vtype, int64_t n, int32_t k, void *Q, int64_t ldq,
                              const void *S, int64_t lds, const double *beta, void *stream) {
    // in place on Q: the product reads all of Q's row, so stage a copy first
    cudaStream_t st = (cudaStream_t)stream;
    size_t es = vtype == CACG_VAL_F64 ? 8 : 4;
    void *Qin = nullptr;
    size_t bytes = (size_t)n * ldq * es;
    if (cudaMallocAsync(&Qin, bytes > 0 ? bytes : 16, st) != cudaSuccess) return CACG_ERR_OOM;
    cudaMemcpyAsync(Qin, Q, bytes, cudaMemcpyDeviceToDevice, st);
    int rc;
    if (vtype == CACG_VAL_F64) {
        rc = launch_qupdate<double>(st, n, k, (double *)Q, ldq, (const double *)Qin, ldq,
                                    (const double *)S, lds, beta);
    } else if (vtype == CACG_VAL_F32) {
        rc = launch_qupdate<float>(st, n, k, (float *)Q, ldq, (const float *)Qin, ldq,
                                   (const float *)S, lds, beta);
    } else if (vtype == (CACG_VAL_F32 | CACG_VAL_TC5) ||
               vtype == (CACG_VAL_F32 | CACG_VAL_TC5 | CACG_VAL_TC5_CPASYNC)) {
        const bool tma = (vtype & CACG_VAL_TC5_CPASYNC) == 0;
        rc = run_with_status(st, [&](int *dstat) {
            return launch_qupdate_tc5(st, n, k, (float *)Q, ldq, (const float *)Qin, ldq,
                                      (const float *)S, lds, beta, dstat, tma);
        });
    } else {
        rc = CACG_ERR_ARG;
    }
    cudaFreeAsync(Qin, st);
    return rc;
}

extern "C" int cacg_k_xrupdate(int32_t vtype, int64_t n, int32_t k, int32_t m, const void *Q,
                               const void *AQ, int64_t ldq, const double *alpha, double *X,
                               double *R, void *S0, int64_t lds, double *norms, void *stream) {
    cudaStream_t st = (cudaStream_t)stream;
    double *ws = nullptr;
    if (cudaMallocAsync((void **)&ws, norm_workspace_doubles(n, m) * sizeof(double), st) !=
        cudaSuccess)
        return CACG_ERR_OOM;
    int rc;
    // vtype | CACG_XR_EXACT selects the float-float product sums
    const bool exact = (vtype & CACG_XR_EXACT) != 0;
    const bool ffstate = (vtype & CACG_XR_FFSTATE) != 0;
    vtype &= ~(CACG_XR_EXACT | CACG_XR_FFSTATE);
    if (ffstate) {  // float-float X and R (TMA-fed kernel only)
        int rc2 = CACG_ERR_ARG;
        if (vtype == CACG_VAL_F32 && !exact && m == 16)
            rc2 = run_with_status(st, [&](int *dstat) {
                return launch_xrupdate_m16_ff(st, n, k, (const float *)Q, (const float *)AQ, ldq,
                                              alpha, (float *)X, (float *)R, (float *)S0, lds,
                                              nullptr, norms, ws, dstat);
            });
        cudaFreeAsync(ws, st);
        return rc2;
    }
    if (vtype == CACG_VAL_F64)
        rc = exact ? launch_xrupdate<double>(st, n, k, m, (const double *)Q, (const double *)AQ,
                                             ldq, alpha, X, R, (double *)S0, lds, nullptr,
                                             norms, ws)
                   : launch_xrupdate_fast<double>(st, n, k, m, (const double *)Q,
                                                  (const double *)AQ, ldq, alpha, X, R,
                                                  (double *)S0, lds, nullptr, norms, ws);
    else if (vtype == CACG_VAL_F32 && exact)
        rc = launch_xrupdate<float>(st, n, k, m, (const float *)Q, (const float *)AQ, ldq, alpha,
                                    X, R, (float *)S0, lds, nullptr, norms, ws);
    else if (vtype == CACG_VAL_F32) {
        rc = CACG_ERR_UNSUPPORTED;
        if (m == 16)  // TMA-fed kernel where the operands allow it
            rc = run_with_status(st, [&](int *dstat) {
                return launch_xrupdate_m16_tma(st, n, k, (const float *)Q, (const float *)AQ, ldq,
                                               alpha, X, R, (float *)S0, lds, nullptr, norms, ws,
                                               dstat);
            });
        if (rc == CACG_ERR_UNSUPPORTED)
            rc = launch_xrupdate_fast<float>(st, n, k, m, (const float *)Q, (const float *)AQ,
                                             ldq, alpha, X, R, (float *)S0, lds, nullptr, norms,
                                             ws);
    }
    else if (vtype == (CACG_VAL_F32 | CACG_VAL_TC5) && !exact)
        rc = run_with_status(st, [&](int *dstat) {
            return launch_xrupdate_tc5(st, n, k, m, (const float *)Q, (const float *)AQ, ldq, alpha,
                                       X, R, (float *)S0, lds, nullptr, norms, ws, dstat);
        });
    else
        rc = CACG_ERR_ARG;
    cudaFreeAsync(ws, st);
    return rc;
}
