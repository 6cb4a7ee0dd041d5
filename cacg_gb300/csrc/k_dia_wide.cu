// k_dia_wide.cu -- SpMM over the DIA view for wide FP32 blocks whose row
// stride equals the block width (the A Q product of the mixed mode: Q and
// AQ are n x k, k = s m), with the width a compile-time constant.
//
// Reference operation replaced (sclc/cacg): spmm_csr_info_data_sep_BCBCG
// (src/BLAS3.c:913-976) computing AQ = A Q in bcbcg_v1 (src/bcbcgKernel.c).
//
// Same arithmetic as dia_spmm_kernel (k_dia.cu): a thread owns R = 8
// consecutive rows x one 16-byte column chunk, walks the groups of adjacent
// diagonals with a register window of R + G - 1 X rows, and for every row
// runs the FMAs over the diagonals in increasing offset order, so the result
// is bit-identical to the CSR kernel (the FMAs go out as packed FP32 pairs,
// fma.rn.f32x2: two independent round-to-nearest FMAs, one per column).
// What differs is the address work:
// with the row stride known at compile time every window row is an
// immediate offset from one pointer per group, the values of a block sit in
// shared memory at compile-time strides, and the group table (offset x
// width, first diagonal, size) is read once per group from shared memory.
// The generic kernel spends more integer and constant-load instructions on
// 64-bit addresses than FMAs at width 96.
#include <algorithm>

#include "cacg_internal.cuh"
#include "cacg_solver.h"

namespace cacg {

namespace {

constexpr int kWideR = 8;          // rows per thread
constexpr int kWideThreads = 192;  // 8 runs x 24 chunks at width 96, 12 x 16 at 64
constexpr int kWideGMax = kDiaGroupMax;
// three CTAs (18 warps) per SM: the X windows are L2 reads, and more warps in
// flight beat the few registers spilled at 96 a thread (0.54 ms against 0.67
// ms with two CTAs for A Q at 128^3, width 96)
constexpr int kWideCtas = 3;

__device__ __forceinline__ void wide_cp16(void *smem, const void *g, int bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(
                     (unsigned)__cvta_generic_to_shared(smem)),
                 "l"(g), "r"(bytes));
}

// Y = ca A X, both n x COLS row-major (row stride COLS)
template <int COLS>
__global__ void __launch_bounds__(kWideThreads, kWideCtas)
    dia_wide_kernel(int64_t n, int64_t npad, const __grid_constant__ DiaDesc desc,
                    const float *__restrict__ vals, const float *__restrict__ X,
                    float *__restrict__ Y, float ca) {
    constexpr int CPR = COLS / 4;                 // 16-byte chunks per row
    constexpr int RUNS = kWideThreads / CPR;      // row runs per block
    constexpr int BR = RUNS * kWideR;             // rows per block
    constexpr int W = kWideR + kWideGMax - 1;     // window rows
    extern __shared__ __align__(16) float wide_vs[];  // [2][ndiag][BR]
    __shared__ int64_t g_off[kDiaMax];             // group offset x COLS
    __shared__ int g_d0[kDiaMax], g_size[kDiaMax];
    const int nd = desc.ndiag, ng = desc.ngroups;
    for (int g = threadIdx.x; g < ng; g += blockDim.x) {
        g_off[g] = desc.off[desc.gstart[g]] * COLS;
        g_d0[g] = desc.gstart[g];
        g_size[g] = desc.gstart[g + 1] - desc.gstart[g];
    }
    const int lr = threadIdx.x / CPR, c = threadIdx.x % CPR;
    const int64_t nblk = (n + BR - 1) / BR;
    const int64_t omin = desc.off[0], omax = desc.off[nd - 1];

    auto stage = [&](int64_t blk, int buf) {
        if (blk < nblk) {
            float *dst = wide_vs + (size_t)buf * nd * BR;
            constexpr int per = BR / 4;  // 16-byte chunks per diagonal
            for (int idx = threadIdx.x; idx < nd * per; idx += kWideThreads) {
                const int d = idx / per, q = idx - d * per;
                const int64_t e0 = blk * BR + 4 * q;
                const int64_t left = npad - e0;
                const int by = left >= 4 ? 16 : (left > 0 ? (int)left * 4 : 0);
                wide_cp16(dst + d * BR + 4 * q, by ? (const void *)(vals + (size_t)d * npad + e0)
                                                   : vals, by);
            }
        }
        asm volatile("cp.async.commit_group;\n" ::);
    };

    int buf = 0;
    stage(blockIdx.x, 0);
    for (int64_t blk = blockIdx.x; blk < nblk; blk += gridDim.x, buf ^= 1) {
        stage(blk + gridDim.x, buf ^ 1);
        asm volatile("cp.async.wait_group 1;\n" ::: "memory");
        __syncthreads();
        const int64_t r0 = blk * BR + (int64_t)lr * kWideR;
        // every window of the block inside the matrix: no clamping
        const bool inside = blk * BR + omin >= 0 && blk * BR + BR - 1 + omax < n;
        const float *xb = X + r0 * COLS + 4 * c;
        const float *vb = wide_vs + (size_t)buf * nd * BR + lr * kWideR;
        float acc[kWideR][4];
#pragma unroll
        for (int i = 0; i < kWideR; ++i)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[i][q] = 0.f;
        for (int g = 0; g < ng; ++g) {
            const int G = g_size[g];
            const float *vg = vb + g_d0[g] * BR;
            float4 win[W];
            if (inside) {
                const float *xp = xb + g_off[g];
#pragma unroll
                for (int t = 0; t < W; ++t)
                    if (t < kWideR + G - 1)
                        win[t] = __ldg(reinterpret_cast<const float4 *>(xp + t * COLS));
            } else {
                const int64_t x0 = r0 + g_off[g] / COLS;
#pragma unroll
                for (int t = 0; t < W; ++t) {
                    if (t < kWideR + G - 1) {
                        int64_t xr = x0 + t;
                        xr = xr < 0 ? 0 : (xr >= n ? n - 1 : xr);  // value is 0 there
                        win[t] = __ldg(reinterpret_cast<const float4 *>(X + xr * COLS + 4 * c));
                    }
                }
            }
#pragma unroll
            for (int j = 0; j < kWideGMax; ++j) {
                if (j < G) {
                    const float4 v0 = *reinterpret_cast<const float4 *>(vg + j * BR);
                    const float4 v1 = *reinterpret_cast<const float4 *>(vg + j * BR + 4);
                    const float vv[kWideR] = {v0.x, v0.y, v0.z, v0.w, v1.x, v1.y, v1.z, v1.w};
#pragma unroll
                    for (int i = 0; i < kWideR; ++i) {
                        const float4 x = win[i + j];
                        fma2_bcast(acc[i][0], acc[i][1], vv[i], x.x, x.y);
                        fma2_bcast(acc[i][2], acc[i][3], vv[i], x.z, x.w);
                    }
                }
            }
        }
#pragma unroll
        for (int i = 0; i < kWideR; ++i) {
            const int64_t row = r0 + i;
            if (row >= n) break;
            float y[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) y[q] = ca * acc[i][q];
            const int64_t e = row * COLS + 4 * c;
            *reinterpret_cast<float4 *>(Y + e) = make_float4(y[0], y[1], y[2], y[3]);
        }
        __syncthreads();  // buffer `buf` is refilled two blocks on
    }
    asm volatile("cp.async.wait_all;\n" ::: "memory");
}

template <int COLS>
int launch_wide(cudaStream_t st, const DevMatrix *A, const float *X, float *Y, float ca) {
    constexpr int BR = (kWideThreads / (COLS / 4)) * kWideR;
    const size_t smem = 2 * (size_t)A->dia_ndiag * BR * sizeof(float);
    if (smem > 96 * 1024) return CACG_ERR_UNSUPPORTED;
    set_smem_attr(dia_wide_kernel<COLS>, 96 * 1024);
    const int64_t nblk = (A->n + BR - 1) / BR;
    const int64_t blocks = std::min<int64_t>(nblk, (int64_t)sm_count() * kWideCtas);
    dia_wide_kernel<COLS><<<(unsigned)blocks, kWideThreads, smem, st>>>(
        A->n, A->dia_npad, A->dia, A->dia32, X, Y, ca);
    return check_launch();
}

bool a16w(const void *p) { return ((uintptr_t)p & 15) == 0; }

}  // namespace

int launch_dia_wide(cudaStream_t st, const DevMatrix *A, int w, const float *X, int64_t ldx,
                    float *Y, int64_t ldy, const float *Z1, int64_t ldz1, const float *Z2,
                    int64_t ldz2, double ca, double cb, double cc) {
    if (!A || A->dia_ndiag <= 0 || !A->dia32 || A->dia.ngroups > kDiaMax)
        return CACG_ERR_UNSUPPORTED;
    // the A Q product only: no recurrence terms (the basis steps take the rings)
    if (Z1 || Z2 || cb != 0.0 || cc != 0.0) return CACG_ERR_UNSUPPORTED;
    (void)ldz1;
    (void)ldz2;
    if (ldx != w || ldy != w || !a16w(X) || !a16w(Y)) return CACG_ERR_UNSUPPORTED;
    if (A->n <= 0) return CACG_OK;
    switch (w) {
        case 96:
            return launch_wide<96>(st, A, X, Y, (float)ca);
        case 64:
            return launch_wide<64>(st, A, X, Y, (float)ca);
        default:
            return CACG_ERR_UNSUPPORTED;
    }
}

}  // namespace cacg
