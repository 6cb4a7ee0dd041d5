// k_tsqr.cu -- tall-skinny QR of an n x k block (FP64): V = Q R with Q's
// columns orthonormal and R upper triangular with a positive diagonal.
//
// The reference names a TSQR (src/TSQR.c, src/TSQR.h) but its file is empty
// and its Householder QR (src/MatrixDecomposition.c:3-93) is unfinished and
// never called, so there is no reference behaviour to match; this is the
// GB300 form of the operation the s-step basis would use to orthonormalise a
// block.  It is CholeskyQR2 (Fukaya, Nakatsukasa, Yanagisawa, Yamamoto 2014):
//   G = V^T V,  R1 = chol(G) (upper),  Q1 = V R1^{-1},
//   G2 = Q1^T Q1, R2 = chol(G2),       Q  = Q1 R2^{-1},   R = R2 R1,
// which is orthogonal to working accuracy while the 2-norm condition number
// of V stays below about u^{-1/2} (1e8); the Gram products are the split-K
// FP64 Gram of k_gram.cu (symmetric: upper triangle computed), the small
// Cholesky factors and triangular inverses run in one CTA, the tall x small
// products stream V once.  A Cholesky pivot that is not positive and finite
// (V numerically rank-deficient) returns CACG_ERR_BREAKDOWN.
#include "cacg_internal.cuh"

namespace cacg {

constexpr int kQrMaxK = 128;
constexpr int kQrThreads = 256;

// One CTA: R = chol(G) (upper, G = R^T R) in shared memory, Rinv = R^{-1};
// both k x k row-major with zeros below the diagonal.  *bad set on a pivot
// that is not positive and finite.
__global__ void __launch_bounds__(kQrThreads)
    chol_inv_kernel(int k, const double *__restrict__ G, double *__restrict__ R,
                    double *__restrict__ Rinv, int *__restrict__ bad) {
    extern __shared__ __align__(16) double qr_sm[];
    double *A = qr_sm;  // k x k
    const int tid = threadIdx.x, kk = k * k;
    for (int i = tid; i < kk; i += blockDim.x) A[i] = G[i];
    __syncthreads();
    for (int j = 0; j < k; ++j) {
        // row j of R: A[j][j] = sqrt(pivot), A[j][l] /= it (l > j)
        const double piv = A[j * k + j];
        const bool ok = piv > 0.0 && isfinite(piv);
        const double d = ok ? sqrt(piv) : 0.0;
        __syncthreads();
        if (tid == 0) {
            A[j * k + j] = d;
            if (!ok) *bad = 1;
        }
        for (int l = j + 1 + tid; l < k; l += blockDim.x) A[j * k + l] = ok ? A[j * k + l] / d : 0.0;
        __syncthreads();
        // trailing upper part: A[i][l] -= R[j][i] R[j][l], j < i <= l
        const int w = k - j - 1;
        for (int e = tid; e < w * w; e += blockDim.x) {
            const int i = j + 1 + e / w, l = j + 1 + e % w;
            if (l >= i) A[i * k + l] = fma(-A[j * k + i], A[j * k + l], A[i * k + l]);
        }
        __syncthreads();
    }
    for (int e = tid; e < kk; e += blockDim.x) {
        const int i = e / k, l = e % k;
        R[e] = l >= i ? A[e] : 0.0;
    }
    // R^{-1}, one column per thread: x_c = 1 / R_cc, x_i = -(sum_{l=i+1..c} R_il x_l) / R_ii
    for (int c = tid; c < k; c += blockDim.x) {
        for (int i = 0; i < k; ++i)
            if (i > c) Rinv[i * k + c] = 0.0;
        Rinv[c * k + c] = 1.0 / A[c * k + c];
        for (int i = c - 1; i >= 0; --i) {
            double s = 0.0;
            for (int l = i + 1; l <= c; ++l) s = fma(A[i * k + l], Rinv[l * k + c], s);
            Rinv[i * k + c] = -s / A[i * k + i];
        }
    }
}

// Y = X W with W k x k upper triangular (row-major, in shared memory):
// Y[r][c] = sum_{j <= c} X[r][j] W[j][c], one thread per output.
__global__ void __launch_bounds__(kQrThreads)
    tallsmall_triu_kernel(int64_t n, int k, const double *__restrict__ X, int64_t ldx,
                          const double *__restrict__ W, double *__restrict__ Y, int64_t ldy) {
    extern __shared__ __align__(16) double ts_sm[];
    for (int i = threadIdx.x; i < k * k; i += blockDim.x) ts_sm[i] = W[i];
    __syncthreads();
    const int64_t total = n * (int64_t)k;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = e / k;
        const int c = (int)(e - r * k);
        const double *x = X + r * ldx;
        double s = 0.0;
        for (int j = 0; j <= c; ++j) s = fma(x[j], ts_sm[j * k + c], s);
        Y[r * ldy + c] = s;
    }
}

// R = A B for upper triangular k x k A, B (one CTA)
__global__ void triu_mul_kernel(int k, const double *__restrict__ A, const double *__restrict__ B,
                                double *__restrict__ R) {
    for (int e = threadIdx.x; e < k * k; e += blockDim.x) {
        const int i = e / k, c = e % k;
        double s = 0.0;
        for (int j = i; j <= c; ++j) s = fma(A[i * k + j], B[j * k + c], s);
        R[e] = c >= i ? s : 0.0;
    }
}

// the opt-in (set once per device) covers the largest k
constexpr int kQrSmemMax = kQrMaxK * kQrMaxK * (int)sizeof(double);

static int chol_inv(cudaStream_t st, int k, const double *G, double *R, double *Rinv, int *bad) {
    const int smem = (int)((size_t)k * k * sizeof(double));
    set_smem_attr(chol_inv_kernel, kQrSmemMax);
    chol_inv_kernel<<<1, kQrThreads, smem, st>>>(k, G, R, Rinv, bad);
    return check_launch();
}

static int tallsmall_triu(cudaStream_t st, int64_t n, int k, const double *X, int64_t ldx,
                          const double *W, double *Y, int64_t ldy) {
    if (n <= 0) return CACG_OK;
    const int smem = (int)((size_t)k * k * sizeof(double));
    set_smem_attr(tallsmall_triu_kernel, kQrSmemMax);
    const int64_t blocks = std::min<int64_t>((n * k + kQrThreads - 1) / kQrThreads,
                                             (int64_t)sm_count() * 4);
    tallsmall_triu_kernel<<<(unsigned)blocks, kQrThreads, smem, st>>>(n, k, X, ldx, W, Y, ldy);
    return check_launch();
}

}  // namespace cacg

using namespace cacg;

extern "C" int cacg_k_tsqr(int64_t n, int32_t k, const double *V, int64_t ldv, double *Q,
                           int64_t ldq, double *R, void *stream) {
    cudaStream_t st = (cudaStream_t)stream;
    if (n < k || k <= 0 || k > kQrMaxK || !V || !Q || !R || ldv < k || ldq < k)
        return CACG_ERR_ARG;
    const size_t gws = (gram_workspace_bytes(n, k, k) + 255) / 256 * 256;
    const size_t q1b = ((size_t)n * k * sizeof(double) + 255) / 256 * 256;
    const size_t small = (size_t)5 * k * k * sizeof(double);
    char *buf = nullptr;
    if (cudaMallocAsync((void **)&buf, gws + q1b + small + 256, st) != cudaSuccess) {
        cudaGetLastError();
        return CACG_ERR_OOM;
    }
    double *ws = (double *)buf;
    double *Q1 = (double *)(buf + gws);  // n x k, the first pass's factor
    double *G = (double *)(buf + gws + q1b), *R1 = G + (size_t)k * k, *R1i = R1 + (size_t)k * k,
           *R2 = R1i + (size_t)k * k, *R2i = R2 + (size_t)k * k;
    int *bad = (int *)(R2i + (size_t)k * k);
    int rc = cudaMemsetAsync(bad, 0, sizeof(int), st) == cudaSuccess ? CACG_OK : CACG_ERR_CUDA;
    // pass 1: G = V^T V, R1, Q1 = V R1^{-1}
    if (rc == CACG_OK)
        rc = launch_gram<double>(st, CACG_GRAM_FMA, n, V, ldv, k, V, ldv, k, nullptr, 0, 0, G, k,
                                 nullptr, 0, ws, gws, true);
    if (rc == CACG_OK) rc = chol_inv(st, k, G, R1, R1i, bad);
    if (rc == CACG_OK) rc = tallsmall_triu(st, n, k, V, ldv, R1i, Q1, k);
    // pass 2: G2 = Q1^T Q1, R2, Q = Q1 R2^{-1}
    if (rc == CACG_OK)
        rc = launch_gram<double>(st, CACG_GRAM_FMA, n, Q1, k, k, Q1, k, k, nullptr, 0, 0, G, k,
                                 nullptr, 0, ws, gws, true);
    if (rc == CACG_OK) rc = chol_inv(st, k, G, R2, R2i, bad);
    if (rc == CACG_OK) rc = tallsmall_triu(st, n, k, Q1, k, R2i, Q, ldq);
    if (rc == CACG_OK) {
        triu_mul_kernel<<<1, kQrThreads, 0, st>>>(k, R2, R1, R);
        rc = check_launch();
    }
    int hb = 0;
    if (rc == CACG_OK) {
        if (cudaMemcpyAsync(&hb, bad, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            rc = CACG_ERR_CUDA;
    }
    cudaFreeAsync(buf, st);
    if (rc != CACG_OK) cudaGetLastError();  // a refused launch leaves no error behind
    if (rc == CACG_OK && hb) rc = CACG_ERR_BREAKDOWN;
    return rc;
}
