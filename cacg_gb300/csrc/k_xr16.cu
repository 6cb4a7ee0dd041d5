// k_xr16.cu -- X/R update of the mixed mode for blocks of 16 right-hand sides
// (src/bcbcgKernel.c, the X += Q alpha and R -= AQ alpha updates):
//
//   X[i][c] += sum_j Q[i][j] alpha[j][c],   R[i][c] -= sum_j AQ[i][j] alpha[j][c],
//   S0[i][c] = R32[i][c] = (float)R[i][c],  partials of ||R(:, c)||^2,
//
// Q, AQ FP32 (n x k, row stride ldq), X, R FP64 (n x 16), alpha FP64 (k x 16).
//
// Four threads share a row and split its k columns into interleaved 16-byte
// chunks (thread g takes chunks g, g + 4, ...), so a warp's loads of Q and AQ
// cover 64 contiguous bytes of each of its eight rows and no row is read
// twice.  Each thread accumulates all 16 columns over its chunks; a
// reduce-scatter over the four lanes (two shuffle rounds) leaves thread g
// with columns 4g .. 4g + 3.  alpha sits in shared memory as FP32 with its
// rows permuted (row 16i + 4g + u at 16i + 4u + g) and an 80-byte pitch, so
// the four 16-byte loads a warp issues per coefficient row fall on distinct
// banks.
//
// FP64 work per element is the two additions into X and R: the float <->
// double conversions are exact bit operations (GB300 runs FP64 at 1/64 of
// the FP32 rate), and the squares for the norms are float-float sums of the
// split R values per thread (about 2^-44 relative) and FP64 across the block.
#include <algorithm>

#include "cacg_internal.cuh"
#include "ff_util.cuh"

namespace cacg {

namespace {

constexpr int kXr16Threads = 256;  // 64 rows x 4 threads
constexpr int kXr16Rows = kXr16Threads / 4;
constexpr int kXr16Pitch = 20;     // floats per staged alpha row (80 bytes)
constexpr int kXr16MaxBlocks = 2048;  // norm partials per launch (the workspace holds 2048 x m)

__device__ __forceinline__ void xr_fma4(float s, const float4 &a, float *acc) {
    acc[0] = fmaf(s, a.x, acc[0]);
    acc[1] = fmaf(s, a.y, acc[1]);
    acc[2] = fmaf(s, a.z, acc[2]);
    acc[3] = fmaf(s, a.w, acc[3]);
}

// 16 partial sums per lane -> lane g of each aligned group of four holds the
// totals of columns 4g .. 4g + 3 in out[0..3]
__device__ __forceinline__ void xr_reduce_scatter(const float (&v)[16], int g, float (&out)[4]) {
    float h[8];
    const bool hi = (g >> 1) != 0;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const float keep = hi ? v[8 + q] : v[q];
        const float give = hi ? v[q] : v[8 + q];
        h[q] = keep + __shfl_xor_sync(0xffffffffu, give, 2);
    }
    const bool odd = (g & 1) != 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const float keep = odd ? h[4 + q] : h[q];
        const float give = odd ? h[q] : h[4 + q];
        out[q] = keep + __shfl_xor_sync(0xffffffffu, give, 1);
    }
}

__global__ void __launch_bounds__(kXr16Threads)
    xrupdate16_kernel(int64_t n, int k, const float *__restrict__ Q, const float *__restrict__ AQ,
                      int64_t ldq, const double *__restrict__ alpha, double *__restrict__ X,
                      double *__restrict__ R, float *__restrict__ S0, int64_t lds,
                      float *__restrict__ R32, double *__restrict__ part) {
    extern __shared__ __align__(16) float xr_al[];  // k rows x kXr16Pitch
    __shared__ double red[kXr16Rows][16];
    for (int idx = threadIdx.x; idx < k * 16; idx += blockDim.x) {
        const int j = idx >> 4, c = idx & 15;
        const int i = j >> 4, gg = (j >> 2) & 3, u = j & 3;
        xr_al[(16 * i + 4 * u + gg) * kXr16Pitch + c] = (float)alpha[(size_t)j * 16 + c];
    }
    __syncthreads();
    const int lr = threadIdx.x >> 2, g = threadIdx.x & 3;
    const int kc = k >> 4;  // chunk rounds (16 columns each)
    float sq_hi[4] = {0.f, 0.f, 0.f, 0.f}, sq_lo[4] = {0.f, 0.f, 0.f, 0.f};
    for (int64_t r0 = (int64_t)blockIdx.x * kXr16Rows; r0 < n;
         r0 += (int64_t)gridDim.x * kXr16Rows) {
        const int64_t row = r0 + lr;
        const bool valid = row < n;
        float ax[16], ar[16];
#pragma unroll
        for (int q = 0; q < 16; ++q) ax[q] = ar[q] = 0.f;
        const float *qr = Q + (valid ? row : 0) * ldq + 4 * g;
        const float *aqr = AQ + (valid ? row : 0) * ldq + 4 * g;
#pragma unroll 2
        for (int i = 0; i < kc; ++i) {
            float4 qv = make_float4(0.f, 0.f, 0.f, 0.f), av = qv;
            if (valid) {
                qv = __ldg(reinterpret_cast<const float4 *>(qr + 16 * i));
                av = __ldg(reinterpret_cast<const float4 *>(aqr + 16 * i));
            }
            const float qs[4] = {qv.x, qv.y, qv.z, qv.w}, as[4] = {av.x, av.y, av.z, av.w};
            const float *al = xr_al + (16 * i + g) * kXr16Pitch;
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const float *a = al + 4 * u * kXr16Pitch;
#pragma unroll
                for (int q4 = 0; q4 < 4; ++q4) {
                    const float4 w = *reinterpret_cast<const float4 *>(a + 4 * q4);
                    xr_fma4(qs[u], w, ax + 4 * q4);
                    xr_fma4(as[u], w, ar + 4 * q4);
                }
            }
        }
        float xs[4], rs[4];
        xr_reduce_scatter(ax, g, xs);
        xr_reduce_scatter(ar, g, rs);
        if (valid) {
            double *xp = X + row * 16 + 4 * g;
            double *rp = R + row * 16 + 4 * g;
            const double2 x01 = *reinterpret_cast<const double2 *>(xp);
            const double2 x23 = *reinterpret_cast<const double2 *>(xp + 2);
            const double2 r01 = *reinterpret_cast<const double2 *>(rp);
            const double2 r23 = *reinterpret_cast<const double2 *>(rp + 2);
            const double xo[4] = {x01.x, x01.y, x23.x, x23.y};
            const double ro[4] = {r01.x, r01.y, r23.x, r23.y};
            double xn[4], rn[4];
            float rf[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                xn[q] = xo[q] + ff_widen(xs[q]);
                rn[q] = ro[q] - ff_widen(rs[q]);
                rf[q] = ff_narrow(rn[q]);
                float rh, rl;
                ff_split_bits(rn[q], rh, rl);
                ff_add_square(rh, rl, sq_hi[q], sq_lo[q]);
            }
            *reinterpret_cast<double2 *>(xp) = make_double2(xn[0], xn[1]);
            *reinterpret_cast<double2 *>(xp + 2) = make_double2(xn[2], xn[3]);
            *reinterpret_cast<double2 *>(rp) = make_double2(rn[0], rn[1]);
            *reinterpret_cast<double2 *>(rp + 2) = make_double2(rn[2], rn[3]);
            const float4 r4 = make_float4(rf[0], rf[1], rf[2], rf[3]);
            if (S0) *reinterpret_cast<float4 *>(S0 + row * lds + 4 * g) = r4;
            if (R32) *reinterpret_cast<float4 *>(R32 + row * 16 + 4 * g) = r4;
        }
    }
    if (!part) return;
#pragma unroll
    for (int q = 0; q < 4; ++q) red[lr][4 * g + q] = ff_widen(sq_hi[q]) + ff_widen(sq_lo[q]);
    __syncthreads();
    if (threadIdx.x < 16) {
        double t = 0.0;
        for (int r = 0; r < kXr16Rows; ++r) t += red[r][threadIdx.x];
        part[(size_t)blockIdx.x * 16 + threadIdx.x] = t;
    }
}

bool a16(const void *p) { return ((uintptr_t)p & 15) == 0; }

}  // namespace

int launch_xrupdate_m16(cudaStream_t st, int64_t n, int k, const float *Q, const float *AQ,
                        int64_t ldq, const double *alpha, double *X, double *R, float *S0,
                        int64_t lds, float *R32, double *norms, double *ws) {
    if (k <= 0 || k % 16 != 0 || ldq % 4 || !a16(Q) || !a16(AQ) || !a16(X) || !a16(R))
        return CACG_ERR_UNSUPPORTED;
    if (S0 && (lds % 4 || !a16(S0))) return CACG_ERR_UNSUPPORTED;
    if (R32 && !a16(R32)) return CACG_ERR_UNSUPPORTED;
    if (norms && !ws) return CACG_ERR_ARG;
    const size_t smem = (size_t)k * kXr16Pitch * sizeof(float);
    if (smem + sizeof(double) * kXr16Rows * 16 > 48 * 1024) return CACG_ERR_UNSUPPORTED;
    int64_t blocks = (n + kXr16Rows - 1) / kXr16Rows;
    blocks = std::min<int64_t>(blocks, std::min<int64_t>((int64_t)sm_count() * 8, kXr16MaxBlocks));
    if (blocks < 1) blocks = 1;
    xrupdate16_kernel<<<(unsigned)blocks, kXr16Threads, smem, st>>>(
        n, k, Q, AQ, ldq, alpha, X, R, S0, lds, R32, norms ? ws : nullptr);
    int rc = check_launch();
    if (rc != CACG_OK || !norms) return rc;
    return launch_colsum(st, ws, (int)blocks, 16, norms);
}

}  // namespace cacg
