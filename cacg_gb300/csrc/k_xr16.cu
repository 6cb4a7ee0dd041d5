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
#include "tc5_util.cuh"
#include "tma_util.cuh"

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

// ---------------------------------------------------------------------------
// The same update with Q and AQ fed by TMA (16-byte aligned operands and row
// strides).  Persistent CTAs walk 128-row tiles: a loader thread streams each
// tile's Q and AQ as 32-column boxes (128-byte swizzle) into a ring of two
// or more stages; eight compute warps take 16 rows each, a thread two rows x
// output columns 4c .. 4c + 3 over all k (no cross-lane reduction).  Per
// chunk of four coefficients a thread reads one 16-byte piece of each of its
// Q and AQ rows (swizzled positions: the eight rows a warp reads at once hit
// distinct banks) and four alpha rows (FP32, broadcast); the FMAs go out as
// packed pairs (fma.rn.f32x2), summing over k in increasing order.
// X and R rows are read with coalesced loads issued before the stage wait:
// FP64 rows (the epilogue of xrupdate16_kernel), or float-float pairs (FF:
// the additions in float-float, no FP64 instruction).  Every compute thread
// releases the stage after its epilogue, behind a proxy fence.
constexpr int kXtWarps = 8;                       // compute warps
constexpr int kXtSlots = 8 * kXtWarps;            // row slots (a thread's first row)
constexpr int kXtThreads = 32 * (kXtWarps + 1);   // + the loader warp
constexpr int kXtMaxStages = 4;
// two rows a thread (rows rl and rl + 64 of a 128-row tile): twice the
// independent FMA chains and half the alpha loads per FMA of one row a
// thread (0.61 ms against 0.79 ms per outer iteration at 128^3, k = 96)
constexpr int kXtRpt = 2;

__host__ __device__ constexpr size_t xt_smem(int nbx, int rpt, int stages) {
    return (size_t)stages * 2 * nbx * (kXtSlots * rpt * 128) + (size_t)32 * nbx * 16 * 4 +
           (size_t)kXtSlots * 16 * 8 + 16 * kXtMaxStages + 16;
}

// (hi, lo) + b as a float-float pair, renormalised (two TwoSums: exact
// error of hi + b, then of the sum with the low parts; no ordering assumed,
// since R cancels heavily near convergence)
__device__ __forceinline__ void ff_add_float(float &hi, float &lo, float b) {
    const float s = hi + b;
    const float bp = s - hi;
    const float e = (hi - (s - bp)) + (b - bp);
    const float l = e + lo;
    const float t = s + l;
    const float tp = t - s;
    lo = (s - (t - tp)) + (l - tp);
    hi = t;
}

// FF = false: X, R FP64 (n x 16).  FF = true: X and R as float-float pairs,
// each n x 16 high parts followed by n x 16 low parts (the mixed solve's
// state between FP64 checks): the updates are float-float additions on the
// FP32 pipe, no FP64 instruction.
template <int NBX, bool FF>  // 32-column boxes per operand: k <= 32 NBX
__global__ void __launch_bounds__(kXtThreads, 1)
    xrupdate16_tma_kernel(const __grid_constant__ CUtensorMap tmQ,
                          const __grid_constant__ CUtensorMap tmAQ, int64_t n, int k, int stages,
                          const double *__restrict__ alpha, void *__restrict__ Xv,
                          void *__restrict__ Rv, float *__restrict__ S0, int64_t lds,
                          float *__restrict__ R32, double *__restrict__ part,
                          int *__restrict__ status) {
    double *X = static_cast<double *>(Xv), *R = static_cast<double *>(Rv);
    float *Xh = static_cast<float *>(Xv), *Rh = static_cast<float *>(Rv);
    float *Xl = Xh + n * 16, *Rl = Rh + n * 16;
    constexpr int KP = 32 * NBX;
    constexpr int RPT = kXtRpt;
    constexpr int kXtRows = kXtSlots * RPT;            // rows per tile
    constexpr unsigned kXtBox = kXtRows * 32 * 4;       // one box: tile rows x 32 columns
    constexpr unsigned stage_bytes = 2 * NBX * kXtBox;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    // [ring: stages x (Q boxes, AQ boxes)][alpha KP x 16 FP32][norm partials
    // 64 x 16 FP64][full, empty mbarriers][abort]
    unsigned char *ring = smem_raw;
    float *al = reinterpret_cast<float *>(ring + (size_t)stages * stage_bytes);
    double *red = reinterpret_cast<double *>(al + KP * 16);
    uint64_t *full = reinterpret_cast<uint64_t *>(red + kXtSlots * 16);
    uint64_t *empty = full + kXtMaxStages;
    volatile int *abort_flag = reinterpret_cast<volatile int *>(empty + kXtMaxStages);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    for (int i = tid; i < KP * 16; i += kXtThreads) {
        const int j = i >> 4;
        al[i] = j < k ? (float)alpha[i] : 0.f;  // alpha is k x 16, row-major
    }
    if (tid == 0) {
        for (int q = 0; q < stages; ++q) {
            t5_mbar_init(&full[q], 1);
            t5_mbar_init(&empty[q], kXtWarps * 32);  // every compute thread releases
        }
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    const int64_t ntiles = (n + kXtRows - 1) / kXtRows;
    const int64_t my_tiles =
        ntiles > blockIdx.x ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    auto fail = [&]() {
        *abort_flag = 1;
        atomicOr(status, kStatusTimeout);
    };

    if (warp == kXtWarps) {
        // ---------------------------------------------------------- loader
        if (lane == 0) {
            int64_t issued = 0;
            int q = 0;
            unsigned qph = 0;  // phase of stage q's current fill (stepped, no division)
            for (int64_t t = 0; t < my_tiles; ++t) {
                if (t > 0 && q == 0) qph ^= 1u;
                if (t >= stages && !t5_mbar_wait_or_abort(&empty[q], qph ^ 1u, abort_flag)) {
                    fail();
                    break;
                }
                unsigned char *dst = ring + (size_t)q * stage_bytes;
                const int y = (int)((blockIdx.x + t * gridDim.x) * kXtRows);
                tma_expect_tx(&full[q], stage_bytes);
#pragma unroll
                for (int b = 0; b < NBX; ++b) {
                    tma_load_2d(dst + b * kXtBox, &tmQ, 32 * b, y, &full[q]);
                    tma_load_2d(dst + (NBX + b) * kXtBox, &tmAQ, 32 * b, y, &full[q]);
                }
                issued = t + 1;
                if (++q == stages) q = 0;
            }
            if (*abort_flag)  // the loads in flight land before the CTA exits (bounded)
                for (int64_t t = issued > stages ? issued - stages : 0; t < issued; ++t)
                    t5_mbar_wait(&full[t % stages], (unsigned)((t / stages) & 1));
        }
    } else {
        // ---------------------------------------------------------- compute
        // thread rows rl + kXtSlots i (same swizzle phase), columns 4c .. 4c + 3
        const int rl = 8 * warp + (lane >> 2), c4 = lane & 3;
        const int sw = rl & 7;
        float sq_hi[4] = {0.f, 0.f, 0.f, 0.f}, sq_lo[4] = {0.f, 0.f, 0.f, 0.f};
        bool ok = true;
        int q = 0;
        unsigned qph = 0;
        for (int64_t t = 0; t < my_tiles; ++t) {
            const int64_t row0 = (blockIdx.x + t * gridDim.x) * (int64_t)kXtRows + rl;
            double2 xo[RPT][2], ro[RPT][2];   // FP64 state
            float4 xhv[RPT], xlv[RPT], rhv[RPT], rlv[RPT];  // float-float state
#pragma unroll
            for (int i = 0; i < RPT; ++i) {
                const int64_t row = row0 + kXtSlots * i;
                if constexpr (FF) {
                    xhv[i] = xlv[i] = rhv[i] = rlv[i] = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (row < n) {
                        const int64_t e = row * 16 + 4 * c4;
                        xhv[i] = *reinterpret_cast<const float4 *>(Xh + e);
                        xlv[i] = *reinterpret_cast<const float4 *>(Xl + e);
                        rhv[i] = *reinterpret_cast<const float4 *>(Rh + e);
                        rlv[i] = *reinterpret_cast<const float4 *>(Rl + e);
                    }
                } else {
                    xo[i][0] = xo[i][1] = ro[i][0] = ro[i][1] = make_double2(0.0, 0.0);
                    if (row < n) {
                        const double *xp = X + row * 16 + 4 * c4, *rp = R + row * 16 + 4 * c4;
                        xo[i][0] = *reinterpret_cast<const double2 *>(xp);
                        xo[i][1] = *reinterpret_cast<const double2 *>(xp + 2);
                        ro[i][0] = *reinterpret_cast<const double2 *>(rp);
                        ro[i][1] = *reinterpret_cast<const double2 *>(rp + 2);
                    }
                }
            }
            const bool w = t5_mbar_wait_or_abort(&full[q], qph, abort_flag);
            if (!__all_sync(0xffffffffu, w)) {
                ok = false;
                break;
            }
            const unsigned char *stq = ring + (size_t)q * stage_bytes + rl * 128;
            float ax[RPT][4], ar[RPT][4];
#pragma unroll
            for (int i = 0; i < RPT; ++i)
#pragma unroll
                for (int c = 0; c < 4; ++c) ax[i][c] = ar[i][c] = 0.f;
#pragma unroll
            for (int b = 0; b < NBX; ++b) {
                const unsigned char *qrow = stq + b * kXtBox;
                const unsigned char *arow = stq + (NBX + b) * kXtBox;
#pragma unroll
                for (int ch = 0; ch < 8; ++ch) {
                    float4 qv[RPT], av[RPT];
#pragma unroll
                    for (int i = 0; i < RPT; ++i) {
                        const int off = kXtSlots * 128 * i + ((ch ^ sw) << 4);
                        qv[i] = *reinterpret_cast<const float4 *>(qrow + off);
                        av[i] = *reinterpret_cast<const float4 *>(arow + off);
                    }
                    const float *ap = al + (32 * b + 4 * ch) * 16 + 4 * c4;
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const float4 wv = *reinterpret_cast<const float4 *>(ap + 16 * u);
#pragma unroll
                        for (int i = 0; i < RPT; ++i) {
                            const float qs = u == 0 ? qv[i].x : u == 1 ? qv[i].y : u == 2 ? qv[i].z : qv[i].w;
                            const float as = u == 0 ? av[i].x : u == 1 ? av[i].y : u == 2 ? av[i].z : av[i].w;
                            fma2_bcast(ax[i][0], ax[i][1], qs, wv.x, wv.y);
                            fma2_bcast(ax[i][2], ax[i][3], qs, wv.z, wv.w);
                            fma2_bcast(ar[i][0], ar[i][1], as, wv.x, wv.y);
                            fma2_bcast(ar[i][2], ar[i][3], as, wv.z, wv.w);
                        }
                    }
                }
            }
            const int qdone = q;
            if (++q == stages) {
                q = 0;
                qph ^= 1u;
            }
#pragma unroll
            for (int i = 0; i < RPT; ++i) {
                const int64_t row = row0 + kXtSlots * i;
                if (row >= n) break;
                if constexpr (FF) {
                    float xh[4] = {xhv[i].x, xhv[i].y, xhv[i].z, xhv[i].w};
                    float xl[4] = {xlv[i].x, xlv[i].y, xlv[i].z, xlv[i].w};
                    float rh[4] = {rhv[i].x, rhv[i].y, rhv[i].z, rhv[i].w};
                    float rl[4] = {rlv[i].x, rlv[i].y, rlv[i].z, rlv[i].w};
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        ff_add_float(xh[c], xl[c], ax[i][c]);
                        ff_add_float(rh[c], rl[c], -ar[i][c]);
                        ff_add_square(rh[c], rl[c], sq_hi[c], sq_lo[c]);
                    }
                    const int64_t e = row * 16 + 4 * c4;
                    *reinterpret_cast<float4 *>(Xh + e) = make_float4(xh[0], xh[1], xh[2], xh[3]);
                    *reinterpret_cast<float4 *>(Xl + e) = make_float4(xl[0], xl[1], xl[2], xl[3]);
                    const float4 r4 = make_float4(rh[0], rh[1], rh[2], rh[3]);
                    *reinterpret_cast<float4 *>(Rh + e) = r4;
                    *reinterpret_cast<float4 *>(Rl + e) = make_float4(rl[0], rl[1], rl[2], rl[3]);
                    if (S0) *reinterpret_cast<float4 *>(S0 + row * lds + 4 * c4) = r4;
                    if (R32) *reinterpret_cast<float4 *>(R32 + e) = r4;
                    continue;
                }
                const double xv[4] = {xo[i][0].x, xo[i][0].y, xo[i][1].x, xo[i][1].y};
                const double rv[4] = {ro[i][0].x, ro[i][0].y, ro[i][1].x, ro[i][1].y};
                double xn[4], rn[4];
                float rf[4];
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    xn[c] = xv[c] + ff_widen(ax[i][c]);
                    rn[c] = rv[c] - ff_widen(ar[i][c]);
                    rf[c] = ff_narrow(rn[c]);
                    float rh, rlo;
                    ff_split_bits(rn[c], rh, rlo);
                    ff_add_square(rh, rlo, sq_hi[c], sq_lo[c]);
                }
                double *xp = X + row * 16 + 4 * c4, *rp = R + row * 16 + 4 * c4;
                *reinterpret_cast<double2 *>(xp) = make_double2(xn[0], xn[1]);
                *reinterpret_cast<double2 *>(xp + 2) = make_double2(xn[2], xn[3]);
                *reinterpret_cast<double2 *>(rp) = make_double2(rn[0], rn[1]);
                *reinterpret_cast<double2 *>(rp + 2) = make_double2(rn[2], rn[3]);
                const float4 r4 = make_float4(rf[0], rf[1], rf[2], rf[3]);
                if (S0) *reinterpret_cast<float4 *>(S0 + row * lds + 4 * c4) = r4;
                if (R32) *reinterpret_cast<float4 *>(R32 + row * 16 + 4 * c4) = r4;
            }
            // every thread releases its own reads of the stage, after the
            // epilogue and behind a proxy fence: released right after the FMA
            // loop by lane 0 (after __syncwarp), the next TMA fill overwrote
            // rows whose shared-memory loads had not completed (seen as
            // run-to-run differences in a few rows of a tile)
            t5_fence_proxy_async();
            t5_mbar_arrive(&empty[qdone]);
        }
        if (!ok && lane == 0) fail();
#pragma unroll
        for (int c = 0; c < 4; ++c) red[rl * 16 + 4 * c4 + c] = ff_widen(sq_hi[c]) + ff_widen(sq_lo[c]);
    }
    __syncthreads();
    if (part && tid < 16) {
        double s = 0.0;
        for (int r = 0; r < kXtSlots; ++r) s += red[r * 16 + tid];
        part[(size_t)blockIdx.x * 16 + tid] = s;
    }
}

template <int NBX, bool FF>
int launch_xt(cudaStream_t st, int64_t n, int k, const float *Q, const float *AQ, int64_t ldq,
              const double *alpha, void *X, void *R, float *S0, int64_t lds, float *R32,
              double *norms, double *ws, int *status) {
    constexpr int kXtRows = kXtSlots * kXtRpt;
    const size_t budget = (size_t)max_smem_optin();
    int stages = kXtMaxStages;
    while (stages > 2 && xt_smem(NBX, kXtRpt, stages) > budget) --stages;
    const size_t smem = xt_smem(NBX, kXtRpt, stages);
    if (smem > budget || n > (int64_t)INT32_MAX - kXtRows) return CACG_ERR_UNSUPPORTED;
    CUtensorMap mq, ma;
    if (!tma_encode_2d(&mq, Q, (uint64_t)k, (uint64_t)n, (uint64_t)ldq * 4, 32, kXtRows,
                       CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B) ||
        !tma_encode_2d(&ma, AQ, (uint64_t)k, (uint64_t)n, (uint64_t)ldq * 4, 32, kXtRows,
                       CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B))
        return CACG_ERR_UNSUPPORTED;
    set_smem_attr(xrupdate16_tma_kernel<NBX, FF>, (int)max_smem_optin());
    const int64_t ntiles = (n + kXtRows - 1) / kXtRows;
    const int grid =
        (int)std::min<int64_t>(ntiles, std::min<int64_t>(sm_count(), kXr16MaxBlocks));
    xrupdate16_tma_kernel<NBX, FF><<<grid, kXtThreads, smem, st>>>(
        mq, ma, n, k, stages, alpha, X, R, S0, lds, R32, norms ? ws : nullptr, status);
    int rc = check_launch();
    if (rc != CACG_OK || !norms) return rc;
    return launch_colsum(st, ws, grid, 16, norms);
}

bool a16(const void *p) { return ((uintptr_t)p & 15) == 0; }

}  // namespace

static int launch_xt_any(cudaStream_t st, int64_t n, int k, const float *Q, const float *AQ,
                        int64_t ldq, const double *alpha, void *X, void *R, float *S0,
                        int64_t lds, float *R32, double *norms, double *ws, int *status, bool ff) {
    if (k <= 0 || k % 4 != 0 || k > 128 || ldq % 4 || !a16(Q) || !a16(AQ) || !a16(X) ||
        !a16(R) || !status)
        return CACG_ERR_UNSUPPORTED;
    if (S0 && (lds % 4 || lds < 16 || !a16(S0))) return CACG_ERR_UNSUPPORTED;
    if (R32 && !a16(R32)) return CACG_ERR_UNSUPPORTED;
    if (norms && !ws) return CACG_ERR_ARG;
    if (n <= 0) return CACG_ERR_UNSUPPORTED;
#define XT_CASE(B)                                                                               \
    case B:                                                                                      \
        return ff ? launch_xt<B, true>(st, n, k, Q, AQ, ldq, alpha, X, R, S0, lds, R32, norms,  \
                                       ws, status)                                              \
                  : launch_xt<B, false>(st, n, k, Q, AQ, ldq, alpha, X, R, S0, lds, R32, norms, \
                                        ws, status);
    switch ((k + 31) / 32) {
        XT_CASE(1)
        XT_CASE(2)
        XT_CASE(3)
        XT_CASE(4)
    }
#undef XT_CASE
    return CACG_ERR_UNSUPPORTED;
}

int launch_xrupdate_m16_tma(cudaStream_t st, int64_t n, int k, const float *Q, const float *AQ,
                            int64_t ldq, const double *alpha, double *X, double *R, float *S0,
                            int64_t lds, float *R32, double *norms, double *ws, int *status) {
    return launch_xt_any(st, n, k, Q, AQ, ldq, alpha, X, R, S0, lds, R32, norms, ws, status,
                         false);
}

int launch_xrupdate_m16_ff(cudaStream_t st, int64_t n, int k, const float *Q, const float *AQ,
                           int64_t ldq, const double *alpha, float *Xff, float *Rff, float *S0,
                           int64_t lds, float *R32, double *norms, double *ws, int *status) {
    return launch_xt_any(st, n, k, Q, AQ, ldq, alpha, Xff, Rff, S0, lds, R32, norms, ws, status,
                         true);
}

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
