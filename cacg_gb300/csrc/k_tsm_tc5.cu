// k_tsm_tc5.cu -- tall-skinny x small products on the 5th-generation tensor
// cores (tcgen05, sm_103a): the mixed-precision Q update
//     Q_out = S - Q_in * beta      (Q_in, S: n x k FP32; beta: k x k FP64)
//
// Reference operations replaced (sclc/cacg): dense_distributedMatL_localMatR_Mul_v1
// (src/BLAS3.c:794-825) forming Q*beta and dense_mat_mat_add_TP
// (src/BLAS3.c:579-612) forming S - Q*beta, fused into one pass.
//
// Work split: persistent CTAs (one per SM) walk 128-row tiles of Q; a tile
// is K = k columns deep, processed in steps of 32 columns.
//   * warps 0-7 (producers) stream each step's 128 x 32 FP32 block of Q_in
//     through a 4-stage cp.async ring (rows padded to 36 floats so the
//     conversion reads are conflict-free) and split it into three bf16
//     slices in the K-major core-matrix layout (8 rows x 16 bytes, LBO =
//     128 B, SBO = 512 B); thread 0 issues the step's 12 MMAs (six slice
//     products, two K = 16 halves) against beta's slices, which stay resident
//     in shared memory for the whole launch (N = k rows, SBO = k/8 * 128 B);
//   * the tile's FP32 accumulator (128 lanes x k columns) lives in one of two
//     TMEM buffers; after the tile's last MMAs the issuer commits to that
//     buffer's "full" mbarrier;
//   * warps 8-11 (epilogue, one per TMEM lane quadrant) load their S row
//     before the wait, then read the accumulator with tcgen05.ld, write
//     S - acc to Q_out and release the buffer ("empty" mbarrier), so the
//     epilogue of tile t overlaps the MMAs of tile t+1.
// Products: six bf16 slice products of order <= 2^-16 (FP32-level products),
// FP32 accumulation over K = k, as the CUDA-core kernel's FP32 FMA chain.
// Every mbarrier wait is bounded; on expiry kStatusTimeout is recorded, the
// producers leave together at their next named barrier, the epilogue warps
// stop at the abort flag, the issuer waits (bounded) for its committed MMAs
// and TMEM is freed.
#include <cuda_bf16.h>

#include <algorithm>

#include "cacg_internal.cuh"
#include "tc5_util.cuh"
#include "tma_util.cuh"

namespace cacg {

constexpr int kTsM = 128;                     // rows per tile (UMMA M)
constexpr int kTsKT = 32;                     // K columns per step
constexpr int kTsStages = 4;                  // FP32 ring depth
constexpr int kTsProd = 256;                  // producer threads (warps 0-7)
constexpr int kTsEpi = 128;                   // epilogue threads (warps 8-11)
constexpr int kTsThreads = kTsProd + kTsEpi;  // 12 warps
constexpr int kTsRingLd = kTsKT + 4;          // padded ring row (floats)
constexpr int kTsMaxNN = 6;                   // k <= 96: S row of the epilogue in registers
constexpr unsigned kTsABytes = kTsM * kTsKT * 2;  // one A slice of a step

template <int NN>
__global__ void __launch_bounds__(kTsThreads, 1)
    tsm_q_tc5_kernel(int64_t n, float *Qout, int64_t ldo, const float *__restrict__ Qin,
                     int64_t ldq, const float *S, int64_t lds, const double *__restrict__ beta,
                     int tmem_half, int *__restrict__ status) {
    constexpr int K = 16 * NN;               // = k = N
    constexpr int Kp = (K + 31) / 32 * 32;   // K padded to whole steps
    constexpr int KS = Kp / kTsKT;           // steps per tile
    constexpr unsigned w_bytes = K * Kp * 2;  // one slice of beta^T (N x Kp)
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    // [beta slices 3 x w_bytes][A slices 2 x 3 x kTsABytes][ring][mbar x6][tmem slot][abort]
    unsigned char *wsl = smem_raw;
    unsigned char *asl = smem_raw + 3 * w_bytes;
    float *ring = reinterpret_cast<float *>(asl + 2 * 3 * kTsABytes);
    uint64_t *mbar = reinterpret_cast<uint64_t *>(ring + kTsStages * kTsM * kTsRingLd);
    uint64_t *mma_done = mbar, *acc_full = mbar + 2, *acc_empty = mbar + 4;
    unsigned *tmem_slot = reinterpret_cast<unsigned *>(mbar + 6);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t ntiles = (n + kTsM - 1) / kTsM;
    const int64_t my_tiles =
        ntiles > blockIdx.x ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    const int64_t nsteps = my_tiles * KS;

    // ---- setup: beta^T slices (B operand: row c = output column, K-major),
    // zero-padded to Kp; barriers; TMEM (two accumulator buffers)
    for (int pidx = tid; pidx < K * Kp / 2; pidx += kTsThreads) {
        const int c = pidx / (Kp / 2), j = 2 * (pidx % (Kp / 2));
        const float w0 = j < K ? (float)beta[(size_t)j * K + c] : 0.f;
        const float w1 = j + 1 < K ? (float)beta[(size_t)(j + 1) * K + c] : 0.f;
        unsigned hw, mw, lw;
        t5_split2(w0, w1, hw, mw, lw);
        const unsigned off = (((c >> 3) * (Kp / 8) + (j >> 3)) * 64 + (c & 7) * 8 + (j & 7)) * 2;
        *reinterpret_cast<unsigned *>(wsl + off) = hw;
        *reinterpret_cast<unsigned *>(wsl + w_bytes + off) = mw;
        *reinterpret_cast<unsigned *>(wsl + 2 * w_bytes + off) = lw;
    }
    if (tid == 0) {
        for (int i = 0; i < 2; ++i) {
            t5_mbar_init(&mma_done[i], 1);
            t5_mbar_init(&acc_full[i], 1);
            t5_mbar_init(&acc_empty[i], kTsEpi / 32);
        }
        *abort_flag = 0;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                         t5_smem_u32(tmem_slot)),
                     "r"(2 * tmem_half));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    t5_fence_proxy_async();
    t5_fence_before();
    __syncthreads();
    t5_fence_after();
    const unsigned tmem = *tmem_slot;

    if (warp < kTsProd / 32) {
        // ================================ producers
        auto tile_row0 = [&](int64_t tj) { return (blockIdx.x + tj * gridDim.x) * (int64_t)kTsM; };
        auto issue_loads = [&](int64_t j) {
            if (j < nsteps) {
                float *dst = ring + (int)(j % kTsStages) * kTsM * kTsRingLd;
                const int64_t r0 = tile_row0(j / KS);
                const int c0 = (int)(j % KS) * kTsKT;
#pragma unroll
                for (int v = 0; v < kTsM * kTsKT / 4 / kTsProd; ++v) {
                    const int id = tid + v * kTsProd;
                    const int r = id >> 3, c4 = id & 7;
                    const int64_t row = r0 + r;
                    const int col = c0 + 4 * c4;
                    const bool ok = row < n && col < K;
                    t5_cp16(dst + r * kTsRingLd + 4 * c4, ok ? (const void *)(Qin + row * ldq + col) : Qin,
                            ok ? 16 : 0);
                }
            }
            t5_cp_commit();
        };
        auto convert = [&](int stage, int buf) {
            const float *src = ring + stage * kTsM * kTsRingLd;
            unsigned char *dst = asl + buf * 3 * kTsABytes;
#pragma unroll
            for (int u = 0; u < kTsM * kTsKT / 8 / kTsProd; ++u) {
                const int id = tid + u * kTsProd;
                const int q = id & 7, o = (id >> 3) & 3, g = id >> 5;
                const int row = 8 * g + q;
                const float4 x0 = *reinterpret_cast<const float4 *>(src + row * kTsRingLd + 8 * o);
                const float4 x1 =
                    *reinterpret_cast<const float4 *>(src + row * kTsRingLd + 8 * o + 4);
                unsigned hw[4], mw[4], lw[4];
                t5_split2(x0.x, x0.y, hw[0], mw[0], lw[0]);
                t5_split2(x0.z, x0.w, hw[1], mw[1], lw[1]);
                t5_split2(x1.x, x1.y, hw[2], mw[2], lw[2]);
                t5_split2(x1.z, x1.w, hw[3], mw[3], lw[3]);
                const unsigned off = ((row >> 3) * (kTsKT / 8) + o) * 128 + (row & 7) * 16;
                *reinterpret_cast<uint4 *>(dst + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
                *reinterpret_cast<uint4 *>(dst + kTsABytes + off) =
                    make_uint4(mw[0], mw[1], mw[2], mw[3]);
                *reinterpret_cast<uint4 *>(dst + 2 * kTsABytes + off) =
                    make_uint4(lw[0], lw[1], lw[2], lw[3]);
            }
        };
        constexpr unsigned idesc = t5_idesc(kTsM, K);
        // thread 0: the 12 MMAs of step j; false if the accumulator buffer
        // did not come free in time
        auto issue_mma = [&](int64_t j) -> bool {
            const int buf = (int)(j & 1);
            const int64_t tj = j / KS;
            const int kc = (int)(j % KS);
            const int tb = (int)(tj & 1);
            if (kc == 0 && tj >= 2) {
                if (!t5_mbar_wait(&acc_empty[tb], (unsigned)(((tj - 2) >> 1) & 1))) return false;
                t5_fence_after();
            }
            const unsigned d = tmem + (unsigned)(tb * tmem_half);
            const unsigned abase = t5_smem_u32(asl + buf * 3 * kTsABytes);
            const unsigned wbase = t5_smem_u32(wsl);
            unsigned accumulate = kc != 0;
            const int pa[6] = {2, 1, 0, 1, 0, 0}, pb[6] = {0, 1, 2, 0, 1, 0};
#pragma unroll
            for (int pr = 0; pr < 6; ++pr) {
#pragma unroll
                for (int kk = 0; kk < kTsKT / 16; ++kk) {
                    if (kc * kTsKT + kk * 16 >= K) continue;  // K-padding half
                    const uint64_t ad = t5_desc(abase + pa[pr] * kTsABytes + kk * 256, 512);
                    const uint64_t bd = t5_desc(wbase + pb[pr] * w_bytes + (kc * 4 + kk * 2) * 128,
                                                (Kp / 8) * 128);
                    t5_mma(d, ad, bd, idesc, accumulate);
                    accumulate = 1;
                }
            }
            t5_commit(&mma_done[buf]);
            if (kc == KS - 1) t5_commit(&acc_full[tb]);
            return true;
        };

        int timed_out = 0, aborted = 0;
        int64_t last_committed = -1;
        for (int j = 0; j < kTsStages - 1; ++j) issue_loads(j);
        for (int64_t i = 0; i <= nsteps; ++i) {
            if (i < nsteps) asm volatile("cp.async.wait_group %0;\n" ::"n"(kTsStages - 2));
            t5_fence_proxy_async();
            t5_fence_before();
            aborted = t5_bar_or(1, kTsProd, timed_out);
            t5_fence_after();
            if (aborted) break;
            if (i >= 1 && tid == 0) {
                if (issue_mma(i - 1)) {
                    last_committed = i - 1;
                } else {
                    atomicOr(status, kStatusTimeout);
                    timed_out = 1;
                }
            }
            if (i == nsteps) break;
            issue_loads(i + kTsStages - 1);
            if (i >= 2 && !__all_sync(0xffffffffu, t5_mbar_wait(&mma_done[i & 1],
                                                                (unsigned)(((i - 2) >> 1) & 1)))) {
                if (lane == 0) atomicOr(status, kStatusTimeout);
                timed_out = 1;
            }
            convert((int)(i % kTsStages), (int)(i & 1));
        }
        asm volatile("cp.async.wait_all;\n" ::: "memory");
        if (aborted) {
            if (tid == 0) {
                *abort_flag = 1;
                if (last_committed >= 0)
                    t5_mbar_wait(&mma_done[last_committed & 1],
                                 (unsigned)((last_committed >> 1) & 1));
            }
        }
    } else {
        // ================================ epilogue: rows 32 * quad + lane of each tile
        const int quad = warp & 3;
        for (int64_t tj = 0; tj < my_tiles; ++tj) {
            const int64_t row = (blockIdx.x + tj * gridDim.x) * (int64_t)kTsM + 32 * quad + lane;
            const bool rv = row < n;
            float4 sv[NN * 4];
#pragma unroll
            for (int q = 0; q < NN * 4; ++q)
                sv[q] = rv ? *reinterpret_cast<const float4 *>(S + row * lds + 4 * q)
                           : make_float4(0.f, 0.f, 0.f, 0.f);
            const int tb = (int)(tj & 1);
            const bool ok = __all_sync(0xffffffffu, t5_mbar_wait_or_abort(
                                                        &acc_full[tb], (unsigned)((tj >> 1) & 1),
                                                        abort_flag));
            if (!ok) {
                if (lane == 0) {
                    if (!*abort_flag) atomicOr(status, kStatusTimeout);
                    *abort_flag = 1;
                }
                break;
            }
            t5_fence_after();
            const unsigned tbase = tmem + ((unsigned)(32 * quad) << 16) + (unsigned)(tb * tmem_half);
#pragma unroll
            for (int c8 = 0; c8 < 2 * NN; ++c8) {
                float v[8];
                t5_ld8(tbase + 8 * c8, v);
                const float4 a = sv[2 * c8], b = sv[2 * c8 + 1];
                if (rv) {
                    float4 *o = reinterpret_cast<float4 *>(Qout + row * ldo + 8 * c8);
                    o[0] = make_float4(a.x - v[0], a.y - v[1], a.z - v[2], a.w - v[3]);
                    o[1] = make_float4(b.x - v[4], b.y - v[5], b.z - v[6], b.w - v[7]);
                }
            }
            t5_fence_before();
            __syncwarp();
            if (lane == 0) t5_mbar_arrive(&acc_empty[tb]);
        }
    }
    t5_fence_before();
    __syncthreads();
    if (warp == 0) {
        t5_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem),
                     "r"(2 * tmem_half));
    }
}

// ---------------------------------------------------------------------------
// The same Q update fed by TMA, warp-specialised (operands with 16-byte
// aligned bases and row strides).  Per tile of 128 rows:
//   * a loader thread streams the tile's K steps of Q_in (128 rows x 32
//     columns FP32 boxes, 128-byte swizzle) into a 4-stage ring; a second
//     loader brings the tile's S (k/32 boxes of 128 x 32) into one staging
//     buffer as soon as the previous tile's stores have read it;
//   * 8 converter warps split each ring stage into the three bf16 slices
//     (K-major core matrices, as tsm_q_tc5_kernel) and release the stage;
//     the MMA thread issues the step's 12 MMAs into one of two TMEM
//     accumulators;
//   * 4 epilogue warps (one per TMEM lane quadrant) subtract the
//     accumulator from the staged S in place (a thread's row, 16-byte chunks
//     at swizzled positions: conflict-free) and write their 32 rows with TMA
//     stores, so every global access is whole 128-byte row pieces.
// Hand-offs are mbarriers with bounded waits (kStatusTimeout and the abort
// flag on expiry); no CTA-wide barrier after the setup.  The MMAs and their
// order are those of tsm_q_tc5_kernel, so the results are bit-identical.
constexpr int kQwConvWarps = 8;
constexpr int kQwConv = 32 * kQwConvWarps;       // converter threads (warps 0-7)
constexpr int kQwEpiWarp0 = kQwConvWarps;        // warps 8-11: epilogue
constexpr int kQwLoadWarp = kQwEpiWarp0 + 4;     // warp 12: Q_in loader
constexpr int kQwMmaWarp = kQwLoadWarp + 1;      // warp 13: MMA issuer
constexpr int kQwSWarp = kQwMmaWarp + 1;         // warp 14: S loader
constexpr int kQwThreads = 32 * (kQwSWarp + 1);  // 480
constexpr int kQwStages = 4;
constexpr unsigned kQwBox = kTsM * kTsKT * 4;    // one 128 x 32 FP32 box (16 KB)
constexpr int kQwBars = 2 * kQwStages + 10;  // full, empty; sfull, sfree, afull, afree; stfull, stfree

struct QwLayout {
    unsigned asl, ring, stg, bars, total;
};
__host__ __device__ constexpr unsigned qw_align1k(unsigned x) { return (x + 1023u) & ~1023u; }
// [beta slices 3 x k x Kp bf16][A slices 2 x 3 x 8 KB][ring 4 x 16 KB][S staging
// Kp/32 x 16 KB][mbarriers][tmem slot][abort]; the ring and the staging 1 KB
// aligned (128-byte swizzle)
__host__ __device__ constexpr QwLayout qw_layout(int K) {
    const unsigned Kp = (unsigned)(K + 31) / 32 * 32;
    const unsigned asl = qw_align1k(3u * (unsigned)K * Kp * 2u);
    const unsigned ring = qw_align1k(asl + 2u * 3u * kTsABytes);
    const unsigned stg = ring + (unsigned)kQwStages * kQwBox;
    const unsigned bars = stg + Kp / 32u * kQwBox;
    return QwLayout{asl, ring, stg, bars, bars + 8u * (unsigned)kQwBars + 16u};
}

template <int NN>
__global__ void __launch_bounds__(kQwThreads, 1)
    tsm_q_tc5w_kernel(const __grid_constant__ CUtensorMap tmQ,
                      const __grid_constant__ CUtensorMap tmS,
                      const __grid_constant__ CUtensorMap tmO, int64_t n,
                      const double *__restrict__ beta, int tmem_half, int *__restrict__ status) {
    constexpr int K = 16 * NN;
    constexpr int Kp = (K + 31) / 32 * 32;
    constexpr int KS = Kp / kTsKT;  // steps per tile = S boxes per tile
    constexpr unsigned w_bytes = K * Kp * 2;
    constexpr QwLayout L = qw_layout(K);
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *wsl = smem_raw;
    unsigned char *asl = smem_raw + L.asl;
    unsigned char *ring = smem_raw + L.ring;
    unsigned char *stg = smem_raw + L.stg;
    uint64_t *full = reinterpret_cast<uint64_t *>(smem_raw + L.bars);
    uint64_t *empty = full + kQwStages;
    uint64_t *sfull = empty + kQwStages;  // A slice buffers converted
    uint64_t *sfree = sfull + 2;          // A slice buffers read by the MMAs
    uint64_t *afull = sfree + 2;          // accumulators complete
    uint64_t *afree = afull + 2;          // accumulators read
    uint64_t *stfull = afree + 2;         // S staging loaded
    uint64_t *stfree = stfull + 1;        // S staging stored
    unsigned *tmem_slot = reinterpret_cast<unsigned *>(stfree + 1);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t ntiles = (n + kTsM - 1) / kTsM;
    const int64_t my_tiles =
        ntiles > blockIdx.x ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    const int64_t nsteps = my_tiles * KS;

    // beta^T slices (B operand: row c = output column, K-major), zero-padded to Kp
    for (int pidx = tid; pidx < K * Kp / 2; pidx += kQwThreads) {
        const int c = pidx / (Kp / 2), j = 2 * (pidx % (Kp / 2));
        const float w0 = j < K ? (float)beta[(size_t)j * K + c] : 0.f;
        const float w1 = j + 1 < K ? (float)beta[(size_t)(j + 1) * K + c] : 0.f;
        unsigned hw, mw, lw;
        t5_split2(w0, w1, hw, mw, lw);
        const unsigned off = (((c >> 3) * (Kp / 8) + (j >> 3)) * 64 + (c & 7) * 8 + (j & 7)) * 2;
        *reinterpret_cast<unsigned *>(wsl + off) = hw;
        *reinterpret_cast<unsigned *>(wsl + w_bytes + off) = mw;
        *reinterpret_cast<unsigned *>(wsl + 2 * w_bytes + off) = lw;
    }
    if (tid == 0) {
        for (int q = 0; q < kQwStages; ++q) {
            t5_mbar_init(&full[q], 1);
            t5_mbar_init(&empty[q], kQwConvWarps);
        }
        for (int b = 0; b < 2; ++b) {
            t5_mbar_init(&sfull[b], kQwConvWarps);
            t5_mbar_init(&sfree[b], 1);
            t5_mbar_init(&afull[b], 1);
            t5_mbar_init(&afree[b], 4);
        }
        t5_mbar_init(stfull, 1);
        t5_mbar_init(stfree, 4);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                         t5_smem_u32(tmem_slot)),
                     "r"(2 * tmem_half));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    t5_fence_proxy_async();
    t5_fence_before();
    __syncthreads();
    t5_fence_after();
    const unsigned tmem = *tmem_slot;
    auto fail = [&]() {
        *abort_flag = 1;
        atomicOr(status, kStatusTimeout);
    };
    auto tile_row0 = [&](int64_t tj) { return (int)((blockIdx.x + tj * gridDim.x) * kTsM); };

    if (warp < kQwConvWarps) {
        // ------------------------------------------------------ converters
        // unit u: row 8g + q8 of the tile, K columns 8o .. 8o + 7 of the step
        int urow[2], uo[2];
        unsigned udst[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const int id = tid + u * kQwConv;
            const int q8 = id & 7, o = (id >> 3) & 3, g = id >> 5;
            urow[u] = 8 * g + q8;
            uo[u] = o;
            udst[u] = (unsigned)(((urow[u] >> 3) * (kTsKT / 8) + o) * 128 + (urow[u] & 7) * 16);
        }
        bool ok = true;
        for (int64_t j = 0; j < nsteps; ++j) {
            const int q = (int)(j % kQwStages), b = (int)(j & 1);
            bool w = t5_mbar_wait_or_abort(&full[q], (unsigned)((j / kQwStages) & 1), abort_flag);
            if (w && j >= 2)
                w = t5_mbar_wait_or_abort(&sfree[b], (unsigned)(((j >> 1) - 1) & 1), abort_flag);
            if (!__all_sync(0xffffffffu, w)) {
                ok = false;
                break;
            }
            const unsigned char *src = ring + (size_t)q * kQwBox;
            unsigned char *dst = asl + b * 3 * kTsABytes;
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int sw = urow[u] & 7;
                const unsigned char *rp = src + urow[u] * 128;
                const float4 x0 = *reinterpret_cast<const float4 *>(rp + (((2 * uo[u]) ^ sw) << 4));
                const float4 x1 =
                    *reinterpret_cast<const float4 *>(rp + (((2 * uo[u] + 1) ^ sw) << 4));
                unsigned hw[4], mw[4], lw[4];
                t5_split2(x0.x, x0.y, hw[0], mw[0], lw[0]);
                t5_split2(x0.z, x0.w, hw[1], mw[1], lw[1]);
                t5_split2(x1.x, x1.y, hw[2], mw[2], lw[2]);
                t5_split2(x1.z, x1.w, hw[3], mw[3], lw[3]);
                unsigned char *d = dst + udst[u];
                *reinterpret_cast<uint4 *>(d) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
                *reinterpret_cast<uint4 *>(d + kTsABytes) = make_uint4(mw[0], mw[1], mw[2], mw[3]);
                *reinterpret_cast<uint4 *>(d + 2 * kTsABytes) =
                    make_uint4(lw[0], lw[1], lw[2], lw[3]);
            }
            // slices visible to the tensor cores; the ring stage may be refilled
            t5_fence_proxy_async();
            __syncwarp();
            if (lane == 0) {
                t5_mbar_arrive(&sfull[b]);
                t5_mbar_arrive(&empty[q]);
            }
        }
        if (!ok && lane == 0) fail();
    } else if (warp < kQwLoadWarp) {
        // -------------------------------------------------------- epilogue
        const int quad = warp & 3;     // TMEM lanes 32 quad .. + 31
        const int r = 32 * quad + lane;  // row of the tile
        bool ok = true;
        for (int64_t tj = 0; tj < my_tiles; ++tj) {
            const int tb = (int)(tj & 1);
            bool w = t5_mbar_wait_or_abort(&afull[tb], (unsigned)((tj >> 1) & 1), abort_flag);
            if (w) w = t5_mbar_wait_or_abort(stfull, (unsigned)(tj & 1), abort_flag);
            if (!__all_sync(0xffffffffu, w)) {
                ok = false;
                break;
            }
            t5_fence_after();
            const unsigned tbase =
                tmem + ((unsigned)(32 * quad) << 16) + (unsigned)(tb * tmem_half);
#pragma unroll
            for (int c3 = 0; c3 < KS; ++c3) {
                unsigned char *rowp = stg + c3 * kQwBox + r * 128;
#pragma unroll
                for (int c8 = 0; c8 < 4; ++c8) {
                    if (32 * c3 + 8 * c8 >= K) break;
                    float v[8];
                    t5_ld8(tbase + (unsigned)(32 * c3 + 8 * c8), v);
                    float4 *p0 = reinterpret_cast<float4 *>(rowp + (((2 * c8) ^ (r & 7)) << 4));
                    float4 *p1 = reinterpret_cast<float4 *>(rowp + (((2 * c8 + 1) ^ (r & 7)) << 4));
                    const float4 a = *p0, bq = *p1;
                    *p0 = make_float4(a.x - v[0], a.y - v[1], a.z - v[2], a.w - v[3]);
                    *p1 = make_float4(bq.x - v[4], bq.y - v[5], bq.z - v[6], bq.w - v[7]);
                }
            }
            // accumulator read: the MMAs may reuse it; rows visible to the TMA store
            t5_fence_before();
            t5_fence_proxy_async();
            __syncwarp();
            if (lane == 0) {
                t5_mbar_arrive(&afree[tb]);
                const int y = tile_row0(tj) + 32 * quad;
                if (y < n) {  // a quadrant wholly past the last row has nothing to store
#pragma unroll
                    for (int c3 = 0; c3 < KS; ++c3)
                        tma_store_2d(&tmO, 32 * c3, y, stg + c3 * kQwBox + quad * 32 * 128);
                    tma_store_commit();
                    tma_store_wait_read();
                }
                t5_mbar_arrive(stfree);
            }
            __syncwarp();
        }
        if (lane == 0) {
            tma_store_wait_all();
            if (!ok) fail();
        }
    } else if (warp == kQwLoadWarp) {
        // ---------------------------------------------------- Q_in loader
        if (lane == 0) {
            int64_t issued = 0;
            for (int64_t j = 0; j < nsteps; ++j) {
                const int q = (int)(j % kQwStages);
                if (j >= kQwStages &&
                    !t5_mbar_wait_or_abort(&empty[q], (unsigned)(((j / kQwStages) - 1) & 1),
                                           abort_flag)) {
                    fail();
                    break;
                }
                tma_expect_tx(&full[q], kQwBox);
                tma_load_2d(ring + (size_t)q * kQwBox, &tmQ, (int)(j % KS) * kTsKT,
                            tile_row0(j / KS), &full[q]);
                issued = j + 1;
            }
            if (*abort_flag)  // the loads in flight land before the CTA exits (bounded)
                for (int64_t j = issued > kQwStages ? issued - kQwStages : 0; j < issued; ++j)
                    t5_mbar_wait(&full[j % kQwStages], (unsigned)((j / kQwStages) & 1));
        }
    } else if (warp == kQwMmaWarp) {
        // ---------------------------------------------------- MMA issuer
        if (lane == 0) {
            constexpr unsigned idesc = t5_idesc(kTsM, K);
            int64_t last = -1;
            for (int64_t j = 0; j < nsteps; ++j) {
                const int b = (int)(j & 1);
                const int64_t tj = j / KS;
                const int kc = (int)(j % KS);
                const int tb = (int)(tj & 1);
                if ((kc == 0 && tj >= 2 &&
                     !t5_mbar_wait_or_abort(&afree[tb], (unsigned)(((tj - 2) >> 1) & 1),
                                            abort_flag)) ||
                    !t5_mbar_wait_or_abort(&sfull[b], (unsigned)((j >> 1) & 1), abort_flag)) {
                    fail();
                    break;
                }
                t5_fence_after();
                const unsigned d = tmem + (unsigned)(tb * tmem_half);
                const unsigned abase = t5_smem_u32(asl + b * 3 * kTsABytes);
                const unsigned wbase = t5_smem_u32(wsl);
                unsigned accumulate = kc != 0;
                const int pa[6] = {2, 1, 0, 1, 0, 0}, pb[6] = {0, 1, 2, 0, 1, 0};
#pragma unroll
                for (int pr = 0; pr < 6; ++pr) {
#pragma unroll
                    for (int kk = 0; kk < kTsKT / 16; ++kk) {
                        if (kc * kTsKT + kk * 16 >= K) continue;  // K-padding half
                        const uint64_t ad = t5_desc(abase + pa[pr] * kTsABytes + kk * 256, 512);
                        const uint64_t bd = t5_desc(
                            wbase + pb[pr] * w_bytes + (kc * 4 + kk * 2) * 128, (Kp / 8) * 128);
                        t5_mma(d, ad, bd, idesc, accumulate);
                        accumulate = 1;
                    }
                }
                t5_commit(&sfree[b]);
                if (kc == KS - 1) t5_commit(&afull[tb]);
                last = j;
            }
            if (*abort_flag && last >= 0)  // committed MMAs finish before TMEM goes (bounded)
                t5_mbar_wait(&sfree[last & 1], (unsigned)((last >> 1) & 1));
        }
    } else {
        // ------------------------------------------------------- S loader
        if (lane == 0) {
            int64_t issued = 0;
            for (int64_t tj = 0; tj < my_tiles; ++tj) {
                if (tj >= 1 &&
                    !t5_mbar_wait_or_abort(stfree, (unsigned)((tj - 1) & 1), abort_flag)) {
                    fail();
                    break;
                }
                tma_expect_tx(stfull, KS * kQwBox);
#pragma unroll
                for (int c3 = 0; c3 < KS; ++c3)
                    tma_load_2d(stg + c3 * kQwBox, &tmS, 32 * c3, tile_row0(tj), stfull);
                issued = tj + 1;
            }
            if (*abort_flag && issued > 0)  // the last load lands (bounded)
                t5_mbar_wait(stfull, (unsigned)((issued - 1) & 1));
        }
    }
    t5_fence_before();
    __syncthreads();
    if (warp == 0) {
        t5_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem),
                     "r"(2 * tmem_half));
    }
}

// ---------------------------------------------------------------------------
// X += Q alpha, R -= AQ alpha (Q, AQ: n x k FP32, alpha: k x m FP64, X, R: n x m
// FP64), S0 = (float)R, R32 = (float)R, per-CTA partial ||R(:,c)||^2.
// Reference: dense_distributedMatL_localMatR_Mul_v1 (src/BLAS3.c:794-825) for
// Q alpha and AQ alpha, dense_mat_mat_add_TP (src/BLAS3.c:579-612) for the
// updates, norm2square_dist_denseMat_col_n (src/MatrixOperations.c:110-142).
// Same pipeline as the Q update; a tile takes 2 * KS steps (Q's K blocks, then
// AQ's), the MMAs accumulate Q alpha and AQ alpha into adjacent TMEM column
// ranges (N = 16 each, alpha zero-padded to 16 columns), and the epilogue
// thread of a row applies both updates in FP64.
constexpr int kXrN = 16;

__global__ void __launch_bounds__(kTsThreads, 1)
    tsm_xr_tc5_kernel(int64_t n, int K, int m, const float *__restrict__ Q,
                      const float *__restrict__ AQ, int64_t ldq,
                      const double *__restrict__ alpha, double *__restrict__ X,
                      double *__restrict__ R, float *__restrict__ S0, int64_t lds,
                      float *__restrict__ R32, double *__restrict__ part, int tmem_half,
                      int *__restrict__ status) {
    const int Kp = (K + 31) / 32 * 32;
    const int KS = Kp / kTsKT;
    const unsigned w_bytes = kXrN * Kp * 2;  // one slice of alpha^T (16 x Kp)
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *wsl = smem_raw;
    unsigned char *asl = smem_raw + ((3 * w_bytes + 1023) & ~1023u);
    float *ring = reinterpret_cast<float *>(asl + 2 * 3 * kTsABytes);
    uint64_t *mbar = reinterpret_cast<uint64_t *>(ring + kTsStages * kTsM * kTsRingLd);
    uint64_t *mma_done = mbar, *acc_full = mbar + 2, *acc_empty = mbar + 4;
    unsigned *tmem_slot = reinterpret_cast<unsigned *>(mbar + 6);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
    double *red = reinterpret_cast<double *>(mbar + 8);  // kTsEpi norm partials, then staging

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t ntiles = (n + kTsM - 1) / kTsM;
    const int64_t my_tiles =
        ntiles > blockIdx.x ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    const int SPT = 2 * KS;  // steps per tile
    const int64_t nsteps = my_tiles * SPT;

    // alpha^T slices: B row c (output column, zero for c >= m), K-major
    for (int pidx = tid; pidx < kXrN * Kp / 2; pidx += kTsThreads) {
        const int c = pidx / (Kp / 2), j = 2 * (pidx % (Kp / 2));
        const float w0 = (c < m && j < K) ? (float)alpha[(size_t)j * m + c] : 0.f;
        const float w1 = (c < m && j + 1 < K) ? (float)alpha[(size_t)(j + 1) * m + c] : 0.f;
        unsigned hw, mw, lw;
        t5_split2(w0, w1, hw, mw, lw);
        const unsigned off = (((c >> 3) * (Kp / 8) + (j >> 3)) * 64 + (c & 7) * 8 + (j & 7)) * 2;
        *reinterpret_cast<unsigned *>(wsl + off) = hw;
        *reinterpret_cast<unsigned *>(wsl + w_bytes + off) = mw;
        *reinterpret_cast<unsigned *>(wsl + 2 * w_bytes + off) = lw;
    }
    if (tid == 0) {
        for (int i = 0; i < 2; ++i) {
            t5_mbar_init(&mma_done[i], 1);
            t5_mbar_init(&acc_full[i], 1);
            t5_mbar_init(&acc_empty[i], kTsEpi / 32);
        }
        *abort_flag = 0;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                         t5_smem_u32(tmem_slot)),
                     "r"(2 * tmem_half));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    t5_fence_proxy_async();
    t5_fence_before();
    __syncthreads();
    t5_fence_after();
    const unsigned tmem = *tmem_slot;

    if (warp < kTsProd / 32) {
        // ================================ producers (as in the Q update)
        auto issue_loads = [&](int64_t j) {
            if (j < nsteps) {
                float *dst = ring + (int)(j % kTsStages) * kTsM * kTsRingLd;
                const int64_t tj = j / SPT;
                const int idx = (int)(j % SPT);
                const float *src = idx < KS ? Q : AQ;
                const int64_t r0 = (blockIdx.x + tj * gridDim.x) * (int64_t)kTsM;
                const int c0 = (idx % KS) * kTsKT;
#pragma unroll
                for (int v = 0; v < kTsM * kTsKT / 4 / kTsProd; ++v) {
                    const int id = tid + v * kTsProd;
                    const int r = id >> 3, c4 = id & 7;
                    const int64_t row = r0 + r;
                    const int col = c0 + 4 * c4;
                    const bool ok = row < n && col < K;
                    t5_cp16(dst + r * kTsRingLd + 4 * c4,
                            ok ? (const void *)(src + row * ldq + col) : src, ok ? 16 : 0);
                }
            }
            t5_cp_commit();
        };
        auto convert = [&](int stage, int buf) {
            const float *src = ring + stage * kTsM * kTsRingLd;
            unsigned char *dst = asl + buf * 3 * kTsABytes;
#pragma unroll
            for (int u = 0; u < kTsM * kTsKT / 8 / kTsProd; ++u) {
                const int id = tid + u * kTsProd;
                const int q = id & 7, o = (id >> 3) & 3, g = id >> 5;
                const int row = 8 * g + q;
                const float4 x0 = *reinterpret_cast<const float4 *>(src + row * kTsRingLd + 8 * o);
                const float4 x1 =
                    *reinterpret_cast<const float4 *>(src + row * kTsRingLd + 8 * o + 4);
                unsigned hw[4], mw[4], lw[4];
                t5_split2(x0.x, x0.y, hw[0], mw[0], lw[0]);
                t5_split2(x0.z, x0.w, hw[1], mw[1], lw[1]);
                t5_split2(x1.x, x1.y, hw[2], mw[2], lw[2]);
                t5_split2(x1.z, x1.w, hw[3], mw[3], lw[3]);
                const unsigned off = ((row >> 3) * (kTsKT / 8) + o) * 128 + (row & 7) * 16;
                *reinterpret_cast<uint4 *>(dst + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
                *reinterpret_cast<uint4 *>(dst + kTsABytes + off) =
                    make_uint4(mw[0], mw[1], mw[2], mw[3]);
                *reinterpret_cast<uint4 *>(dst + 2 * kTsABytes + off) =
                    make_uint4(lw[0], lw[1], lw[2], lw[3]);
            }
        };
        constexpr unsigned idesc = t5_idesc(kTsM, kXrN);
        auto issue_mma = [&](int64_t j) -> bool {
            const int buf = (int)(j & 1);
            const int64_t tj = j / SPT;
            const int idx = (int)(j % SPT);
            const int op = idx / KS, kc = idx % KS;
            const int tb = (int)(tj & 1);
            if (idx == 0 && tj >= 2) {
                if (!t5_mbar_wait(&acc_empty[tb], (unsigned)(((tj - 2) >> 1) & 1))) return false;
                t5_fence_after();
            }
            const unsigned d = tmem + (unsigned)(tb * tmem_half + op * kXrN);
            const unsigned abase = t5_smem_u32(asl + buf * 3 * kTsABytes);
            const unsigned wbase = t5_smem_u32(wsl);
            unsigned accumulate = kc != 0;
            const int pa[6] = {2, 1, 0, 1, 0, 0}, pb[6] = {0, 1, 2, 0, 1, 0};
#pragma unroll
            for (int pr = 0; pr < 6; ++pr) {
#pragma unroll
                for (int kk = 0; kk < kTsKT / 16; ++kk) {
                    if (kc * kTsKT + kk * 16 >= K) continue;  // K-padding half
                    const uint64_t ad = t5_desc(abase + pa[pr] * kTsABytes + kk * 256, 512);
                    const uint64_t bd = t5_desc(wbase + pb[pr] * w_bytes + (kc * 4 + kk * 2) * 128,
                                                (unsigned)(Kp / 8) * 128);
                    t5_mma(d, ad, bd, idesc, accumulate);
                    accumulate = 1;
                }
            }
            t5_commit(&mma_done[buf]);
            if (idx == SPT - 1) t5_commit(&acc_full[tb]);
            return true;
        };

        int timed_out = 0, aborted = 0;
        int64_t last_committed = -1;
        for (int j = 0; j < kTsStages - 1; ++j) issue_loads(j);
        for (int64_t i = 0; i <= nsteps; ++i) {
            if (i < nsteps) asm volatile("cp.async.wait_group %0;\n" ::"n"(kTsStages - 2));
            t5_fence_proxy_async();
            t5_fence_before();
            aborted = t5_bar_or(1, kTsProd, timed_out);
            t5_fence_after();
            if (aborted) break;
            if (i >= 1 && tid == 0) {
                if (issue_mma(i - 1)) {
                    last_committed = i - 1;
                } else {
                    atomicOr(status, kStatusTimeout);
                    timed_out = 1;
                }
            }
            if (i == nsteps) break;
            issue_loads(i + kTsStages - 1);
            if (i >= 2 && !__all_sync(0xffffffffu, t5_mbar_wait(&mma_done[i & 1],
                                                                (unsigned)(((i - 2) >> 1) & 1)))) {
                if (lane == 0) atomicOr(status, kStatusTimeout);
                timed_out = 1;
            }
            convert((int)(i % kTsStages), (int)(i & 1));
        }
        asm volatile("cp.async.wait_all;\n" ::: "memory");
        if (aborted && tid == 0) {
            *abort_flag = 1;
            if (last_committed >= 0)
                t5_mbar_wait(&mma_done[last_committed & 1], (unsigned)((last_committed >> 1) & 1));
        }
    } else {
        // ================================ epilogue: rows 32 * quad .. +31 of each tile.
        // Lane l reads TMEM row l (the tcgen05.ld lane rule), the warp stages its
        // 32 x m accumulator values in shared memory (row stride 17: conflict
        // free) and then walks the rows cooperatively: element e = it * 32 + l
        // is row e / m, column l % m (m divides 32), so X, R, S0, R32 accesses
        // are contiguous across the warp and a lane keeps one column's norm.
        const int quad = warp & 3, et = tid - kTsProd;
        float *stg = reinterpret_cast<float *>(red + kTsEpi) + (size_t)quad * 2 * 32 * 17;
        const int rpi = 32 / m;             // rows per warp step
        const int lr = lane / m, lc = lane % m;
        const bool lact = lr < rpi;          // lanes past rpi * m idle
        double sq = 0.0;
        for (int64_t tj = 0; tj < my_tiles; ++tj) {
            const int64_t row0 = (blockIdx.x + tj * gridDim.x) * (int64_t)kTsM + 32 * quad;
            double xv[kXrN], rw[kXrN];
#pragma unroll
            for (int it = 0; it < kXrN; ++it) {
                const int64_t row = row0 + it * rpi + lr;
                const bool ok = it < m && lact && row < n;
                xv[it] = ok ? X[row * m + lc] : 0.0;
                rw[it] = ok ? R[row * m + lc] : 0.0;
            }
            const int tb = (int)(tj & 1);
            const bool ok = __all_sync(0xffffffffu, t5_mbar_wait_or_abort(
                                                        &acc_full[tb], (unsigned)((tj >> 1) & 1),
                                                        abort_flag));
            if (!ok) {
                if (lane == 0) {
                    if (!*abort_flag) atomicOr(status, kStatusTimeout);
                    *abort_flag = 1;
                }
                break;
            }
            t5_fence_after();
            const unsigned tbase = tmem + ((unsigned)(32 * quad) << 16) + (unsigned)(tb * tmem_half);
#pragma unroll
            for (int h = 0; h < 4; ++h) {  // D1 cols 0-7, 8-15, D2 cols 0-7, 8-15
                float v[8];
                t5_ld8(tbase + 8 * h, v);
                float *dst = stg + (h >> 1) * 32 * 17 + lane * 17 + 8 * (h & 1);
#pragma unroll
                for (int q = 0; q < 8; ++q) dst[q] = v[q];
            }
            t5_fence_before();
            __syncwarp();
            if (lane == 0) t5_mbar_arrive(&acc_empty[tb]);
#pragma unroll
            for (int it = 0; it < kXrN; ++it) {
                const int r = it * rpi + lr;
                const int64_t row = row0 + r;
                if (it < m && lact && row < n) {
                    const double x = xv[it] + (double)stg[r * 17 + lc];
                    const double rr = rw[it] - (double)stg[32 * 17 + r * 17 + lc];
                    X[row * m + lc] = x;
                    R[row * m + lc] = rr;
                    const float rf = (float)rr;
                    if (S0) S0[row * lds + lc] = rf;
                    if (R32) R32[row * m + lc] = rf;
                    sq = fma(rr, rr, sq);
                }
            }
            __syncwarp();  // staging area reused by the next tile
        }
        // fixed-order per-CTA norm partials: column c sums the lanes holding it
        if (part) {
            red[et] = lact ? sq : 0.0;
            asm volatile("bar.sync 2, %0;\n" ::"n"(kTsEpi) : "memory");
            if (et < m) {
                double t = 0.0;
                for (int q = 0; q < kTsEpi; ++q)
                    if ((q & 31) < rpi * m && (q & 31) % m == et) t += red[q];
                part[(size_t)blockIdx.x * m + et] = t;
            }
        }
    }
    t5_fence_before();
    __syncthreads();
    if (warp == 0) {
        t5_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem),
                     "r"(2 * tmem_half));
    }
}

static size_t tsm_xr_smem(int k) {
    const int Kp = (k + 31) / 32 * 32;
    return (((size_t)3 * kXrN * Kp * 2 + 1023) & ~(size_t)1023) + 2 * 3 * (size_t)kTsABytes +
           (size_t)kTsStages * kTsM * kTsRingLd * 4 + 8 * 8 + (size_t)kTsEpi * 8 +
           (size_t)4 * 2 * 32 * 17 * 4;
}

bool tsm_xr_tc5_supported(int k, int m) {
    return k >= 4 && k % 4 == 0 && k <= 256 && m >= 1 && m <= kXrN && 32 % m == 0 &&
           tsm_xr_smem(k) <= max_smem_optin();
}

int launch_xrupdate_tc5(cudaStream_t st, int64_t n, int k, int m, const float *Q,
                        const float *AQ, int64_t ldq, const double *alpha, double *X, double *R,
                        float *S0, int64_t lds, float *R32, double *norms, double *ws,
                        int *status) {
    if (n < 0 || !alpha || !X || !R || !status || (norms && !ws)) return CACG_ERR_ARG;
    if (!tsm_xr_tc5_supported(k, m) || ldq % 4 || !aligned16(Q) || !aligned16(AQ))
        return CACG_ERR_UNSUPPORTED;
    if (n == 0) return CACG_OK;
    const size_t smem = tsm_xr_smem(k);
    set_smem_attr(tsm_xr_tc5_kernel, (int)max_smem_optin());
    const int64_t ntiles = (n + kTsM - 1) / kTsM;
    const int grid = (int)std::min<int64_t>(ntiles, sm_count());
    tsm_xr_tc5_kernel<<<grid, kTsThreads, smem, st>>>(n, k, m, Q, AQ, ldq, alpha, X, R, S0, lds,
                                                      R32, norms ? ws : nullptr, 32, status);
    int rc = check_launch();
    if (rc != CACG_OK || !norms) return rc;
    return launch_colsum(st, ws, grid, m, norms);
}
static size_t tsm_q_smem(int k) {
    const int Kp = (k + 31) / 32 * 32;
    return 3 * (size_t)k * Kp * 2 + 2 * 3 * (size_t)kTsABytes +
           (size_t)kTsStages * kTsM * kTsRingLd * 4 + 6 * 8 + 16;
}

bool tsm_q_tc5_supported(int k) {
    return k >= 16 && k % 16 == 0 && k / 16 <= kTsMaxNN && tsm_q_smem(k) <= max_smem_optin();
}

template <int NN>
static int launch_tsm_q(cudaStream_t st, int64_t n, float *Qout, int64_t ldo, const float *Qin,
                        int64_t ldq, const float *S, int64_t lds, const double *beta,
                        int *status) {
    const int k = 16 * NN;
    const size_t smem = tsm_q_smem(k);
    set_smem_attr(tsm_q_tc5_kernel<NN>, (int)max_smem_optin());
    int tmem_half = 32;
    while (tmem_half < k) tmem_half *= 2;
    const int64_t ntiles = (n + kTsM - 1) / kTsM;
    const int grid = (int)std::min<int64_t>(ntiles, sm_count());
    tsm_q_tc5_kernel<NN><<<grid, kTsThreads, smem, st>>>(n, Qout, ldo, Qin, ldq, S, lds, beta,
                                                         tmem_half, status);
    return check_launch();
}

template <int NN>
static int launch_tsm_qw(cudaStream_t st, int64_t n, float *Qout, int64_t ldo, const float *Qin,
                         int64_t ldq, const float *S, int64_t lds, const double *beta,
                         int *status) {
    constexpr int K = 16 * NN;
    constexpr QwLayout L = qw_layout(K);
    if ((size_t)L.total > (size_t)max_smem_optin() || n > (int64_t)INT32_MAX - kTsM)
        return CACG_ERR_UNSUPPORTED;
    CUtensorMap mq, ms, mo;
    if (!tma_encode_2d(&mq, Qin, K, (uint64_t)n, (uint64_t)ldq * 4, kTsKT, kTsM,
                       CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B) ||
        !tma_encode_2d(&ms, S, K, (uint64_t)n, (uint64_t)lds * 4, kTsKT, kTsM,
                       CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B) ||
        !tma_encode_2d(&mo, Qout, K, (uint64_t)n, (uint64_t)ldo * 4, kTsKT, 32,
                       CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_NONE))
        return CACG_ERR_UNSUPPORTED;
    set_smem_attr(tsm_q_tc5w_kernel<NN>, (int)qw_layout(16 * NN).total);
    int tmem_half = 32;
    while (tmem_half < K) tmem_half *= 2;
    const int64_t ntiles = (n + kTsM - 1) / kTsM;
    const int grid = (int)std::min<int64_t>(ntiles, sm_count());
    tsm_q_tc5w_kernel<NN><<<grid, kQwThreads, L.total, st>>>(mq, ms, mo, n, beta, tmem_half,
                                                              status);
    return check_launch();
}

int launch_qupdate_tc5(cudaStream_t st, int64_t n, int k, float *Qout, int64_t ldo,
                       const float *Qin, int64_t ldq, const float *S, int64_t lds,
                       const double *beta, int *status, bool allow_tma) {
    if (n < 0 || !beta || !status) return CACG_ERR_ARG;
    if (!tsm_q_tc5_supported(k) || ldq % 4 || ldo % 4 || lds % 4 || !aligned16(Qin) ||
        !aligned16(Qout) || !aligned16(S))
        return CACG_ERR_UNSUPPORTED;
    if (n == 0) return CACG_OK;
    if (allow_tma) {
        int rc = CACG_ERR_UNSUPPORTED;
        switch (k / 16) {
            case 1: rc = launch_tsm_qw<1>(st, n, Qout, ldo, Qin, ldq, S, lds, beta, status); break;
            case 2: rc = launch_tsm_qw<2>(st, n, Qout, ldo, Qin, ldq, S, lds, beta, status); break;
            case 3: rc = launch_tsm_qw<3>(st, n, Qout, ldo, Qin, ldq, S, lds, beta, status); break;
            case 4: rc = launch_tsm_qw<4>(st, n, Qout, ldo, Qin, ldq, S, lds, beta, status); break;
            case 5: rc = launch_tsm_qw<5>(st, n, Qout, ldo, Qin, ldq, S, lds, beta, status); break;
            case 6: rc = launch_tsm_qw<6>(st, n, Qout, ldo, Qin, ldq, S, lds, beta, status); break;
        }
        if (rc != CACG_ERR_UNSUPPORTED) return rc;
    }
    switch (k / 16) {
        case 1: return launch_tsm_q<1>(st, n, Qout, ldo, Qin, ldq, S, lds, beta, status);
        case 2: return launch_tsm_q<2>(st, n, Qout, ldo, Qin, ldq, S, lds, beta, status);
        case 3: return launch_tsm_q<3>(st, n, Qout, ldo, Qin, ldq, S, lds, beta, status);
        case 4: return launch_tsm_q<4>(st, n, Qout, ldo, Qin, ldq, S, lds, beta, status);
        case 5: return launch_tsm_q<5>(st, n, Qout, ldo, Qin, ldq, S, lds, beta, status);
        case 6: return launch_tsm_q<6>(st, n, Qout, ldo, Qin, ldq, S, lds, beta, status);
    }
    return CACG_ERR_UNSUPPORTED;
}

}  // namespace cacg
