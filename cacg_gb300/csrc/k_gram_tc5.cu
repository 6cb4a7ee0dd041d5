// k_gram_tc5.cu -- Gram products of FP32 blocks on the 5th-generation
// tensor cores (tcgen05, sm_103a), accumulators in tensor memory.
//
// Reference operations replaced (sclc/cacg): distributedMatLTransposeMatRMul
// (src/BLAS3.c:699-726) and distributedMatLTransposeMatRMul_updated
// (src/BLAS3.c:730-758), mixed-precision mode (L, R in FP32).
//
// C = L^T [R1 | R2] with L n x ka, R n x kb.  Each FP32 value is split exactly
// into three bf16 slices (x = x1 + x2 + x3, round-to-nearest at each split)
// and the six slice products of order <= 2^-16 are accumulated by tcgen05.mma
// (kind::f16, bf16 inputs, FP32 accumulator in TMEM).  The FP32 accumulator
// covers one group of kT5Flush = 2 K-steps (64 rows); the group's tile is
// then read from TMEM (tcgen05.ld) and added to float-float registers
// (TwoSum on packed FP32 pairs), one accumulator row per thread, and
// converted to FP64 once at the end.  Groups of 64 rows rather than 256 cost
// about 5 % more per Gram and take the 128^3, 16-RHS mixed solve from 32 to
// 30 outer iterations (29 in FP64).  Per-CTA FP64 partials go to the split-K workspace and the
// fixed-order reduction of k_gram.cu finishes the sum.
//
// Pipeline of one CTA (256 threads, one row chunk of the split-K, one output
// tile of at most 128 x 128), one barrier per K-step of 32 rows:
//   * raw FP32 rows of L and R stream into a 4-stage shared-memory ring with
//     cp.async (16-byte copies when rows are 16-byte aligned, zero fill past
//     the matrix edges), three steps ahead of the conversion;
//   * every thread converts fixed (column, 8 rows) units of the step from
//     the ring into the three slice tiles -- one 16-byte core-matrix row per
//     slice, K-major 8 x 16-byte core matrices without swizzle (LBO = 128 B
//     between K-adjacent core matrices, SBO = 512 B between 8-row groups),
//     so the 8 lanes of a store phase hit all 32 banks once;
//   * after the step's barrier, thread 0 issues the 12 MMAs of the previous
//     step (6 products x 2 halves of K = 32) and commits them to that slice
//     buffer's mbarrier, which guards its reuse two steps later;
//   * TMEM holds two group accumulators, so a finished group is read back
//     (two steps after its last MMAs) while the next group accumulates;
//   * every mbarrier wait is bounded: on expiry the thread records
//     kStatusTimeout in *status and the CTA leaves the loop at the next
//     barrier (__syncthreads_or, uniform), the issuer waits (bounded) for its
//     last committed MMAs, TMEM is freed and no partial is written.
#include <cuda_bf16.h>

#include <algorithm>

#include <atomic>

#include "cacg_internal.cuh"
#include "tc5_util.cuh"
#include "tma_util.cuh"

namespace cacg {

constexpr int kT5KT = 32;        // rows (K) per step: two K = 16 UMMAs per product
constexpr int kT5M = 128;        // UMMA M (output rows = columns of L, zero-padded)
constexpr int kT5Threads = 256;  // 8 warps
constexpr int kT5Flush = 2;      // K-steps (32 rows each) per FP32 accumulation group
constexpr int kT5Stages = 4;     // FP32 ring depth
constexpr int kT5MaxUnits = 4;   // (column, 8 rows) conversion units per thread per step
constexpr int kT5MaxN = 128;     // output tile columns (UMMA N)

// BB = 16 * NC8 output columns per tile; thread (warp w, lane) owns
// accumulator row 32 * (w % 4) + lane, columns [(w / 4) * BB / 2, +BB / 2).
template <int NC8>
__global__ void __launch_bounds__(kT5Threads, 1)
    gram_tc5_kernel(int64_t n, int64_t rows_per_chunk, const float *__restrict__ L, int64_t ldl,
                    int ka, const float *__restrict__ R1, int64_t ldr1, int kb1,
                    const float *__restrict__ R2, int64_t ldr2, int kb2, int BA, int tilesB,
                    int vec16, int tmem_half, double *__restrict__ part, int *__restrict__ status) {
    constexpr int BB = 16 * NC8;
    constexpr int HC = BB / 2;  // accumulator columns per thread
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    // [slices buf 0][slices buf 1][FP32 ring: kT5Stages x 32 x CW][mbar x2][tmem slot]
    constexpr unsigned a_bytes = kT5M * kT5KT * 2, b_bytes = BB * kT5KT * 2;
    constexpr unsigned buf_bytes = 3 * (a_bytes + b_bytes);
    const int CW = BA + BB;  // ring row: L columns then R columns
    float *ring = reinterpret_cast<float *>(smem_raw + 2 * buf_bytes);
    const int stage_floats = kT5KT * CW;
    uint64_t *mbar = reinterpret_cast<uint64_t *>(ring + kT5Stages * stage_floats);
    unsigned *tmem_slot = reinterpret_cast<unsigned *>(mbar + 2);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int tile_a = blockIdx.y / tilesB, tile_b = blockIdx.y % tilesB;
    const int a0 = tile_a * BA, b0 = tile_b * BB;
    const int64_t rbeg = (int64_t)blockIdx.x * rows_per_chunk;
    const int64_t rend = min(n, rbeg + rows_per_chunk);
    const int64_t nsteps = rend > rbeg ? (rend - rbeg + kT5KT - 1) / kT5KT : 0;

    // zero both slice buffers once (rows of A beyond BA stay zero)
    for (unsigned i = tid; i < 2 * buf_bytes / 16; i += kT5Threads)
        reinterpret_cast<uint4 *>(smem_raw)[i] = make_uint4(0, 0, 0, 0);
    if (tid == 0) {
        t5_mbar_init(&mbar[0], 1);
        t5_mbar_init(&mbar[1], 1);
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                         t5_smem_u32(tmem_slot)),
                     "r"(2 * tmem_half));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const unsigned tmem = *tmem_slot;

    // ---- loads: warp w stages ring rows w, w+8, w+16, w+24 of each step.
    // 16-byte path: lane copies chunks c4 = lane and lane + 32 of a row; the
    // column source of each chunk is fixed for the whole chunk of rows.
    const float *csrc[2];
    int64_t cld[2];
    int cbytes[2];
#pragma unroll
    for (int t = 0; t < 2; ++t) {
        const int c = 4 * (lane + 32 * t);
        csrc[t] = L;
        cld[t] = 0;
        cbytes[t] = -1;  // chunk outside the ring row
        if (c < CW) {
            cbytes[t] = 0;
            if (c < BA) {
                const int col = a0 + c;
                if (col < ka) csrc[t] = L + col, cld[t] = ldl, cbytes[t] = 4 * min(ka - col, 4);
            } else {
                const int cb = b0 + c - BA;
                if (cb < kb1)
                    csrc[t] = R1 + cb, cld[t] = ldr1, cbytes[t] = 4 * min(kb1 - cb, 4);
                else if (cb - kb1 < kb2)
                    csrc[t] = R2 + (cb - kb1), cld[t] = ldr2, cbytes[t] = 4 * min(kb2 - (cb - kb1), 4);
            }
        }
    }
    auto issue_loads = [&](int64_t j) {
        if (j < nsteps) {
            float *dst = ring + (int)(j % kT5Stages) * stage_floats;
            const int64_t r0 = rbeg + j * kT5KT;
            if (vec16) {
#pragma unroll
                for (int rr = 0; rr < kT5KT / 8; ++rr) {
                    const int r = warp + 8 * rr;
                    const int64_t row = r0 + r;
                    const bool rv = row < rend;
#pragma unroll
                    for (int t = 0; t < 2; ++t) {
                        if (cbytes[t] < 0) continue;
                        const int by = rv ? cbytes[t] : 0;
                        const float *src = by ? csrc[t] + row * cld[t] : L;
                        t5_cp16(dst + r * CW + 4 * (lane + 32 * t), src, by);
                    }
                }
            } else {
                for (int rr = 0; rr < kT5KT / 8; ++rr) {
                    const int r = warp + 8 * rr;
                    const int64_t row = r0 + r;
                    const bool rv = row < rend;
                    for (int c = lane; c < CW; c += 32) {
                        const float *src = L;
                        int by = 0;
                        if (rv) {
                            if (c < BA) {
                                if (a0 + c < ka) src = L + row * ldl + a0 + c, by = 4;
                            } else {
                                const int cb = b0 + c - BA;
                                if (cb < kb1)
                                    src = R1 + row * ldr1 + cb, by = 4;
                                else if (cb - kb1 < kb2)
                                    src = R2 + row * ldr2 + (cb - kb1), by = 4;
                            }
                        }
                        t5_cp4(dst + r * CW + c, src, by);
                    }
                }
            }
        }
        t5_cp_commit();  // one group per step, empty past the end
    };

    // ---- conversion units: (column c of the ring row, k-octet o)
    int usrc[kT5MaxUnits], udst[kT5MaxUnits], uslice[kT5MaxUnits];
#pragma unroll
    for (int u = 0; u < kT5MaxUnits; ++u) {
        const int id = tid + u * kT5Threads;
        usrc[u] = -1;
        udst[u] = 0;
        uslice[u] = 0;
        if (id < 4 * CW) {
            const int c = id % CW, o = id / CW;
            const bool isA = c < BA;
            const int row = isA ? c : c - BA;
            usrc[u] = 8 * o * CW + c;
            // byte offset of core-matrix row (row, k = 8o .. 8o+7) in slice 0
            udst[u] = (isA ? 0 : 3 * (int)a_bytes) + (((row >> 3) * (kT5KT / 8) + o) * 64 + (row & 7) * 8) * 2;
            uslice[u] = isA ? (int)a_bytes : (int)b_bytes;
        }
    }
    auto convert = [&](int stage, int buf) {
        const float *src = ring + stage * stage_floats;
        unsigned char *dbase = smem_raw + buf * buf_bytes;
#pragma unroll
        for (int u = 0; u < kT5MaxUnits; ++u) {
            if (usrc[u] < 0) continue;
            float x[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) x[j] = src[usrc[u] + j * CW];
            unsigned hw[4], mw[4], lw[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) t5_split2(x[2 * j], x[2 * j + 1], hw[j], mw[j], lw[j]);
            unsigned char *d = dbase + udst[u];
            *reinterpret_cast<uint4 *>(d) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
            *reinterpret_cast<uint4 *>(d + uslice[u]) = make_uint4(mw[0], mw[1], mw[2], mw[3]);
            *reinterpret_cast<uint4 *>(d + 2 * uslice[u]) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
        }
    };

    // ---- float-float accumulator row of this thread (hi + lo, about 48
    // significant bits), fed from TMEM once per group with TwoSum: FP32 adds
    // only, since the FP64 pipe of this part runs at 1/64 of the FP32 rate.
    const int quad = warp & 3, half = warp >> 2;
    const int row_t = 32 * quad + lane;
    float acc_hi[HC], acc_lo[HC];
#pragma unroll
    for (int q = 0; q < HC; ++q) acc_hi[q] = acc_lo[q] = 0.f;
    auto flush = [&](int64_t step) {  // group containing `step`
        const unsigned tb = (unsigned)(((step / kT5Flush) & 1) * tmem_half);
#pragma unroll
        for (int c8 = 0; c8 < NC8; ++c8) {
            float v[8];
            t5_ld8(tmem + ((unsigned)(32 * quad) << 16) + tb + (unsigned)(half * HC + 8 * c8), v);
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                float &hi = acc_hi[8 * c8 + q];
                const float s = hi + v[q];
                const float bp = s - hi;
                acc_lo[8 * c8 + q] += (hi - (s - bp)) + (v[q] - bp);
                hi = s;
            }
        }
    };
    auto group_end = [&](int64_t e) { return e % kT5Flush == kT5Flush - 1 || e == nsteps - 1; };

    const unsigned idesc = t5_idesc(kT5M, BB);
    auto issue_mma = [&](int64_t j) {  // thread 0: the 12 MMAs of step j
        const int buf = (int)(j & 1);
        const unsigned abase = t5_smem_u32(smem_raw + buf * buf_bytes);
        const unsigned bbase = abase + 3 * a_bytes;
        const unsigned d = tmem + (unsigned)(((j / kT5Flush) & 1) * tmem_half);
        unsigned accumulate = (j % kT5Flush) != 0;
        // products, small terms first: (3,1) (2,2) (1,3) (2,1) (1,2) (1,1)
        const int pa[6] = {2, 1, 0, 1, 0, 0}, pb[6] = {0, 1, 2, 0, 1, 0};
#pragma unroll
        for (int pr = 0; pr < 6; ++pr) {
#pragma unroll
            for (int kk = 0; kk < kT5KT / 16; ++kk) {
                const uint64_t ad = t5_desc(abase + pa[pr] * a_bytes + kk * 256, 512);
                const uint64_t bd = t5_desc(bbase + pb[pr] * b_bytes + kk * 256, 512);
                t5_mma(d, ad, bd, idesc, accumulate);
                accumulate = 1;
            }
        }
        t5_commit(&mbar[buf]);
    };

    int timed_out = 0, aborted = 0;
    int64_t last_committed = -1;  // thread 0
    for (int j = 0; j < kT5Stages - 1; ++j) issue_loads(j);
    for (int64_t i = 0; i <= nsteps; ++i) {
        if (i < nsteps) asm volatile("cp.async.wait_group %0;\n" ::"n"(kT5Stages - 2));
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        aborted = __syncthreads_or(timed_out);
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        if (aborted) break;
        if (i >= 1 && tid == 0) {
            issue_mma(i - 1);
            last_committed = i - 1;
        }
        if (i == nsteps) break;
        issue_loads(i + kT5Stages - 1);  // ring slot of step i-1, read before the barrier
        if (i >= 2) {
            // slice buffer i&1 and the TMEM group of step i-2 are complete
            // warp-uniform outcome: tcgen05.ld below is .sync.aligned
            if (!__all_sync(0xffffffffu, t5_mbar_wait(&mbar[i & 1], (unsigned)(((i - 2) >> 1) & 1)))) {
                if (lane == 0) atomicOr(status, kStatusTimeout);
                timed_out = 1;
            } else {
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                if (group_end(i - 2)) flush(i - 2);
            }
        }
        convert((int)(i % kT5Stages), (int)(i & 1));
    }
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    // drain: the commit of the last step covers every MMA of this CTA
    bool ok = !aborted;
    if (!aborted && nsteps > 0) {
        const int64_t last = nsteps - 1;
        ok = __all_sync(0xffffffffu, t5_mbar_wait(&mbar[last & 1], (unsigned)((last >> 1) & 1)));
        if (!ok && lane == 0) atomicOr(status, kStatusTimeout);
    } else if (aborted && tid == 0 && last_committed >= 0) {
        // bounded wait for the MMAs still in flight before TMEM is freed
        t5_mbar_wait(&mbar[last_committed & 1], (unsigned)((last_committed >> 1) & 1));
    }
    if (nsteps > 0) {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        if (!aborted) {
            // the two youngest groups were not flushed inside the loop
            if (ok && nsteps >= 2 && group_end(nsteps - 2)) flush(nsteps - 2);
            if (ok) flush(nsteps - 1);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    const int bad = __syncthreads_or(!ok);
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem),
                     "r"(2 * tmem_half));
    }
    if (bad || row_t >= BA) return;
    double *out = part + ((size_t)blockIdx.x * gridDim.y + blockIdx.y) * (size_t)BA * BB +
                  (size_t)row_t * BB + half * HC;
#pragma unroll
    for (int q = 0; q < HC; ++q) out[q] = (double)acc_hi[q] + (double)acc_lo[q];
}

// ---------------------------------------------------------------------------
// MN-major variant (the default where the operands allow TMA): raw FP32 rows
// arrive as 32 x 32 boxes (128 bytes a row, 128-byte swizzle) by 2-D TMA
// loads that one thread issues; the slices are stored MN-major (a core-matrix
// row = 8 consecutive columns of one input row), so a thread converts a unit
// (8 columns of one row) with two 16-byte shared loads, the split and three
// 16-byte stores, without the column gather a K-major tile needs.  The 128-B
// swizzle puts the 16-byte chunk c of row k at chunk c ^ (k & 7), so the 8
// rows a quarter warp reads fall on distinct banks; the MN-major core matrix
// rows (16 bytes at (k & 7) * 16) are conflict-free for the same 8 rows.
// Descriptors (no swizzle, MN-major): SBO = 128 B between 8-column groups,
// LBO = (MN / 8) * 128 B between 8-row (K) groups; instruction descriptor
// with the A and B transpose bits.
constexpr int kT5mBox = 32;                          // rows and FP32 columns of a box
constexpr unsigned kT5mBoxBytes = kT5mBox * kT5mBox * 4;  // 4 KB

constexpr int kT5wConvWarps = 16;                  // converter warps
constexpr int kT5wConv = 32 * kT5wConvWarps;          // converter threads
constexpr int kT5wThreads = kT5wConv + 64;            // + a loader warp and an MMA warp
constexpr int kT5wUnits = 2;                          // conversion units per converter thread
constexpr int kT5wNB = 2;                             // bf16 slice buffers

// Warp-specialised pipeline, no CTA-wide barrier per step:
//   loader (thread 512): waits empty[q], issues step j's TMA boxes into ring
//     stage q = j % stages, completing on full[q];
//   converters (warps 0-15): wait full[q] and sfree[b] (b = j % 2), split the
//     stage into slice buffer b, fence the stores to the async proxy, arrive
//     on sfull[b] and empty[q]; two steps after a group's last step they read
//     its FP32 sum from TMEM (gdone[g & 1]) into the float-float registers and
//     arrive on gfree[g & 1];
//   MMA issuer (thread 544): waits sfull[b] (and gfree before a group reuses
//     a TMEM buffer), issues the 12 MMAs, commits to sfree[b] and, at a
//     group's end, to gdone[g & 1].
// Every wait is bounded and also ends when another role has set the abort
// flag; a role that times out sets kStatusTimeout and the flag, the loader
// and the issuer then wait (bounded) for their own loads and MMAs in flight.
template <int NC8>
__global__ void __launch_bounds__(kT5wThreads, 1)
    gram_tc5m_kernel(const __grid_constant__ CUtensorMap tmL, const __grid_constant__ CUtensorMap tmR1,
                     const __grid_constant__ CUtensorMap tmR2, int64_t n, int64_t rows_per_chunk,
                     int ka, int kb1, int kb2, int BA, int tilesB, int tmem_half, int stages,
                     double *__restrict__ part, int *__restrict__ status, long long pipe_polls) {
    constexpr int BB = 16 * NC8;
    constexpr int HC = BB / 4;  // accumulator columns per converter thread (a quarter row)
    constexpr unsigned a_bytes = kT5M * kT5KT * 2, b_bytes = BB * kT5KT * 2;
    constexpr unsigned buf_bytes = 3 * (a_bytes + b_bytes);
    constexpr unsigned lbo_a = (kT5M / 8) * 128, lbo_b = (BB / 8) * 128;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    // [slice buffers][ring: stages x boxes x 4 KB, 1 KB aligned][mbarriers][tmem slot][abort]
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int tile_a = blockIdx.y / tilesB, tile_b = blockIdx.y % tilesB;
    const int a0 = tile_a * BA, b0 = tile_b * BB;
    const int nbl = (BA + kT5mBox - 1) / kT5mBox;
    const int r1end = min(b0 + BB, kb1);
    const int nbr1 = b0 < kb1 ? (r1end - b0 + kT5mBox - 1) / kT5mBox : 0;
    const int r2beg = max(b0, kb1), r2end = min(b0 + BB, kb1 + kb2);
    const int nbr2 = r2end > r2beg ? (r2end - r2beg + kT5mBox - 1) / kT5mBox : 0;
    const int c2 = r2beg - kb1;  // first R2 column of this tile's boxes
    const int nbox = nbl + nbr1 + nbr2;
    const unsigned ring_off = (kT5wNB * buf_bytes + 1023) / 1024 * 1024;
    unsigned char *ring = smem_raw + ring_off;
    const unsigned stage_bytes = (unsigned)nbox * kT5mBoxBytes;
    uint64_t *full = reinterpret_cast<uint64_t *>(ring + (size_t)stages * stage_bytes);
    uint64_t *empty = full + stages;
    uint64_t *sfull = empty + stages;
    uint64_t *sfree = sfull + kT5wNB;
    uint64_t *gdone = sfree + kT5wNB;
    uint64_t *gfree = gdone + 2;
    unsigned *tmem_slot = reinterpret_cast<unsigned *>(gfree + 2);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);

    const int64_t rbeg = (int64_t)blockIdx.x * rows_per_chunk;
    const int64_t rend = min(n, rbeg + rows_per_chunk);
    const int64_t nsteps = rend > rbeg ? (rend - rbeg + kT5KT - 1) / kT5KT : 0;

    for (unsigned i = tid; i < kT5wNB * buf_bytes / 16; i += kT5wThreads)
        reinterpret_cast<uint4 *>(smem_raw)[i] = make_uint4(0, 0, 0, 0);
    if (tid == 0) {
        for (int q = 0; q < stages; ++q) {
            t5_mbar_init(&full[q], 1);
            t5_mbar_init(&empty[q], kT5wConvWarps);
        }
        for (int b = 0; b < kT5wNB; ++b) {
            t5_mbar_init(&sfull[b], kT5wConvWarps);
            t5_mbar_init(&sfree[b], 1);
        }
        for (int x = 0; x < 2; ++x) {
            t5_mbar_init(&gdone[x], 1);
            t5_mbar_init(&gfree[x], kT5wConvWarps);
        }
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                         t5_smem_u32(tmem_slot)),
                     "r"(2 * tmem_half));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const unsigned tmem = *tmem_slot;
    auto fail = [&]() {
        *abort_flag = 1;
        atomicOr(status, kStatusTimeout);
    };
    auto group_end = [&](int64_t e) { return e % kT5Flush == kT5Flush - 1 || e == nsteps - 1; };

    float acc_hi[HC], acc_lo[HC];
#pragma unroll
    for (int q = 0; q < HC; ++q) acc_hi[q] = acc_lo[q] = 0.f;

    int64_t issued = 0;  // loader: TMA fills issued
    if (warp < kT5wConvWarps) {
        // ------------------------------------------------------ converters
        int usrc[kT5wUnits], uch[kT5wUnits], udst[kT5wUnits], uslice[kT5wUnits], urow[kT5wUnits];
        const int noct = (BA + BB) / 8;
#pragma unroll
        for (int u = 0; u < kT5wUnits; ++u) {
            const int id = tid + u * kT5wConv;
            usrc[u] = -1;
            uch[u] = 0;
            udst[u] = 0;
            uslice[u] = 0;
            urow[u] = 0;
            if (id < kT5KT * noct) {
                const int k = id % kT5KT, o = id / kT5KT;
                int box, col;
                if (o < BA / 8) {
                    box = (8 * o) / kT5mBox;
                    col = (8 * o) % kT5mBox;
                    udst[u] = o * 128 + (k / 8) * (int)lbo_a + (k % 8) * 16;
                    uslice[u] = (int)a_bytes;
                } else {
                    const int cb = 8 * (o - BA / 8);
                    if (b0 + cb < kb1) {
                        box = nbl + cb / kT5mBox;
                        col = cb % kT5mBox;
                    } else {
                        const int rel = b0 + cb - kb1 - c2;
                        box = nbl + nbr1 + rel / kT5mBox;
                        col = rel % kT5mBox;
                    }
                    udst[u] = 3 * (int)a_bytes + (o - BA / 8) * 128 + (k / 8) * (int)lbo_b +
                              (k % 8) * 16;
                    uslice[u] = (int)b_bytes;
                }
                // an octet past the operand's columns has no box: it converts zeros
                usrc[u] = box < nbox ? box * (int)kT5mBoxBytes + k * 128 : -2;
                uch[u] = col / 4;
                urow[u] = k;
            }
        }
        // warp w reads TMEM lanes 32 (w % 4) .. + 31 (its lane quadrant),
        // columns [(w / 4) HC, + HC)
        const int quad = warp & 3, quarter = warp >> 2;
        // TMEM loads of up to 16 columns go out together, then one wait
        auto flush = [&](int64_t step) {
            const unsigned tb = (unsigned)(((step / kT5Flush) & 1) * tmem_half);
            const unsigned ta = tmem + ((unsigned)(32 * quad) << 16) + tb + (unsigned)(quarter * HC);
#pragma unroll
            for (int h0 = 0; h0 < NC8; h0 += 4) {
                unsigned r[4][4];
#pragma unroll
                for (int c4 = 0; c4 < 4; ++c4)
                    if (h0 + c4 < NC8) t5_ld4_nowait(ta + 4 * (h0 + c4), r[c4]);
                t5_wait_ld();
#pragma unroll
                for (int c4 = 0; c4 < 4; ++c4) {
                    if (h0 + c4 >= NC8) break;
#pragma unroll
                    for (int q = 0; q < 4; q += 2) {
                        const int i = 4 * (h0 + c4) + q;
                        t5_twosum2(acc_hi[i], acc_hi[i + 1], acc_lo[i], acc_lo[i + 1],
                                   __uint_as_float(r[c4][q]), __uint_as_float(r[c4][q + 1]));
                    }
                }
            }
        };
        // flush of the group ending at step e; false if its MMAs never completed
        auto flush_group = [&](int64_t e) {
            const int64_t g = e / kT5Flush;
            const bool ok = __all_sync(0xffffffffu, t5_mbar_wait_or_abort(
                                                        &gdone[g & 1], (unsigned)((g >> 1) & 1),
                                                        abort_flag, pipe_polls));
            if (!ok) return false;
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            flush(e);
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
            __syncwarp();
            if (lane == 0) t5_mbar_arrive(&gfree[g & 1]);
            return true;
        };
        bool ok = true;
        // ring stage and its phase, stepped (no division by the runtime depth)
        int q = 0;
        unsigned qph = 0;
        for (int64_t j = 0; j < nsteps && ok; ++j) {
            const int b = (int)(j % kT5wNB);
            bool w = t5_mbar_wait_or_abort(&full[q], qph, abort_flag, pipe_polls);
            if (w && j >= kT5wNB)
                w = t5_mbar_wait_or_abort(&sfree[b], (unsigned)(((j / kT5wNB) - 1) & 1), abort_flag,
                                          pipe_polls);
            if (!__all_sync(0xffffffffu, w)) {
                ok = false;
                break;
            }
            const unsigned char *src = ring + (size_t)q * stage_bytes;
            unsigned char *dbase = smem_raw + b * buf_bytes;
            const int64_t r0 = rbeg + j * kT5KT;
#pragma unroll
            for (int u = 0; u < kT5wUnits; ++u) {
                if (usrc[u] == -1) continue;
                const int sw = urow[u] & 7;
                float4 v0 = make_float4(0.f, 0.f, 0.f, 0.f), v1 = v0;
                if (usrc[u] >= 0 && r0 + urow[u] < rend) {
                    v0 = *reinterpret_cast<const float4 *>(src + usrc[u] + ((uch[u] ^ sw) << 4));
                    v1 = *reinterpret_cast<const float4 *>(src + usrc[u] +
                                                           (((uch[u] + 1) ^ sw) << 4));
                }
                unsigned hw[4], mw[4], lw[4];
                t5_split2(v0.x, v0.y, hw[0], mw[0], lw[0]);
                t5_split2(v0.z, v0.w, hw[1], mw[1], lw[1]);
                t5_split2(v1.x, v1.y, hw[2], mw[2], lw[2]);
                t5_split2(v1.z, v1.w, hw[3], mw[3], lw[3]);
                unsigned char *d = dbase + udst[u];
                *reinterpret_cast<uint4 *>(d) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
                *reinterpret_cast<uint4 *>(d + uslice[u]) = make_uint4(mw[0], mw[1], mw[2], mw[3]);
                *reinterpret_cast<uint4 *>(d + 2 * uslice[u]) =
                    make_uint4(lw[0], lw[1], lw[2], lw[3]);
            }
            // slices visible to the tensor cores; the stage may be refilled
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            __syncwarp();
            if (lane == 0) {
                t5_mbar_arrive(&sfull[b]);
                t5_mbar_arrive(&empty[q]);
            }
            if (++q == stages) {
                q = 0;
                qph ^= 1u;
            }
            if (j >= 2 && group_end(j - 2)) ok = flush_group(j - 2);
        }
        // the last groups' sums
        for (int64_t e = nsteps - 2; ok && e < nsteps; ++e)
            if (e >= 0 && group_end(e)) ok = flush_group(e);
        if (!ok && lane == 0) fail();
    } else if (tid == kT5wConv) {
        // ---------------------------------------------------------- loader
        int q = 0;
        unsigned qph = 0;  // phase of stage q's current fill
        for (int64_t j = 0; j < nsteps; ++j) {
            if (j > 0 && q == 0) qph ^= 1u;
            if (j >= stages && !t5_mbar_wait_or_abort(&empty[q], qph ^ 1u, abort_flag, pipe_polls)) {
                fail();
                break;
            }
            unsigned char *dst = ring + (size_t)q * stage_bytes;
            const int row0 = (int)(rbeg + j * kT5KT);
            tma_expect_tx(&full[q], stage_bytes);
            for (int bx = 0; bx < nbl; ++bx)
                tma_load_2d(dst + bx * kT5mBoxBytes, &tmL, a0 + kT5mBox * bx, row0, &full[q]);
            for (int bx = 0; bx < nbr1; ++bx)
                tma_load_2d(dst + (nbl + bx) * kT5mBoxBytes, &tmR1, b0 + kT5mBox * bx, row0,
                            &full[q]);
            for (int bx = 0; bx < nbr2; ++bx)
                tma_load_2d(dst + (nbl + nbr1 + bx) * kT5mBoxBytes, &tmR2, c2 + kT5mBox * bx, row0,
                            &full[q]);
            issued = j + 1;
            if (++q == stages) q = 0;
        }
    } else if (tid == kT5wConv + 32) {
        // ---------------------------------------------------- MMA issuer
        const unsigned idesc = t5_idesc(kT5M, BB) | (1u << 15) | (1u << 16);  // A, B MN-major
        int64_t last = -1;
        for (int64_t j = 0; j < nsteps; ++j) {
            const int b = (int)(j % kT5wNB);
            const int64_t g = j / kT5Flush;
            if (!t5_mbar_wait_or_abort(&sfull[b], (unsigned)((j / kT5wNB) & 1), abort_flag,
                                       pipe_polls) ||
                (j % kT5Flush == 0 && g >= 2 &&
                 !t5_mbar_wait_or_abort(&gfree[g & 1], (unsigned)(((g >> 1) - 1) & 1),
                                        abort_flag, pipe_polls))) {
                fail();
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const unsigned abase = t5_smem_u32(smem_raw + b * buf_bytes);
            const unsigned bbase = abase + 3 * a_bytes;
            const unsigned dt = tmem + (unsigned)((g & 1) * tmem_half);
            unsigned accumulate = (j % kT5Flush) != 0;
            const int pa[6] = {2, 1, 0, 1, 0, 0}, pb[6] = {0, 1, 2, 0, 1, 0};
#pragma unroll
            for (int pr = 0; pr < 6; ++pr) {
#pragma unroll
                for (int kk = 0; kk < kT5KT / 16; ++kk) {
                    const uint64_t ad =
                        t5_desc_lbo(abase + pa[pr] * a_bytes + 2 * kk * lbo_a, lbo_a, 128);
                    const uint64_t bd =
                        t5_desc_lbo(bbase + pb[pr] * b_bytes + 2 * kk * lbo_b, lbo_b, 128);
                    t5_mma(dt, ad, bd, idesc, accumulate);
                    accumulate = 1;
                }
            }
            t5_commit(&sfree[b]);
            if (group_end(j)) t5_commit(&gdone[g & 1]);
            last = j;
        }
        // every committed MMA finishes before TMEM goes (bounded), whether or
        // not another role gave up after this loop ended
        if (last >= 0) {
            t5_mbar_wait(&sfree[last % kT5wNB], (unsigned)((last / kT5wNB) & 1));
            const int64_t g = last / kT5Flush;
            if (group_end(last)) t5_mbar_wait(&gdone[g & 1], (unsigned)((g >> 1) & 1));
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    const int bad = __syncthreads_or(*abort_flag);
    // after a give-up some fills may never have been consumed: the loader lets
    // its last `stages` fills land (bounded) before its thread, and so the
    // CTA and its shared memory, can retire
    if (bad && tid == kT5wConv)
        for (int64_t j = issued - stages > 0 ? issued - stages : 0; j < issued; ++j)
            t5_mbar_wait(&full[j % stages], (unsigned)((j / stages) & 1));
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem),
                     "r"(2 * tmem_half));
    }
    if (bad || warp >= kT5wConvWarps) return;
    const int row_t = 32 * (warp & 3) + lane, quarter = warp >> 2;
    if (row_t >= BA) return;
    double *out = part + ((size_t)blockIdx.x * gridDim.y + blockIdx.y) * (size_t)BA * BB +
                  (size_t)row_t * BB + quarter * HC;
#pragma unroll
    for (int q = 0; q < HC; ++q) out[q] = (double)acc_hi[q] + (double)acc_lo[q];
}


// Poll limit of the warp-specialised Gram's pipeline waits (the drain waits
// keep kT5SpinLimit): cacg_set_pipeline_wait_limit shortens it so a test can
// make those waits run out.
static std::atomic<long long> g_pipe_polls{kT5SpinLimit};

struct T5Plan {
    int BA, BB, tilesA, tilesB, nchunks, tmem_half;
    int64_t rows_per_chunk;
    size_t smem;
};

static T5Plan plan_tc5(int64_t n, int ka, int kb) {
    T5Plan p;
    auto ru = [](int x, int q) { return (x + q - 1) / q * q; };
    p.BA = std::min(ru(ka, 8), kT5M);
    p.BB = std::min(ru(kb, 16), kT5MaxN);
    p.tilesA = (ka + p.BA - 1) / p.BA;
    p.tilesB = (kb + p.BB - 1) / p.BB;
    p.tmem_half = 32;
    while (p.tmem_half < p.BB) p.tmem_half *= 2;
    const int tiles = p.tilesA * p.tilesB;
    int64_t nch = (sm_count() + tiles - 1) / tiles;
    int64_t maxch = std::max<int64_t>(1, (n + 4 * kT5KT - 1) / (4 * kT5KT));
    if (nch > maxch) nch = maxch;
    if (nch < 1) nch = 1;
    p.rows_per_chunk = (n + nch - 1) / nch;
    p.rows_per_chunk = (p.rows_per_chunk + kT5KT - 1) / kT5KT * kT5KT;
    if (p.rows_per_chunk < kT5KT) p.rows_per_chunk = kT5KT;
    p.nchunks = (int)((n + p.rows_per_chunk - 1) / p.rows_per_chunk);
    if (p.nchunks < 1) p.nchunks = 1;
    const size_t buf = 3 * ((size_t)kT5M * kT5KT * 2 + (size_t)p.BB * kT5KT * 2);
    p.smem = 2 * buf + (size_t)kT5Stages * kT5KT * (p.BA + p.BB) * 4 + 64;
    return p;
}

size_t gram_tc5_workspace_bytes(int64_t n, int ka, int kb) {
    // also the plan of an R1 part padded by 4 columns (see launch_gram_tc5)
    T5Plan p = plan_tc5(n, ka, kb), pp = plan_tc5(n, ka, kb + 4);
    return std::max((size_t)p.nchunks * p.tilesA * p.tilesB * p.BA * p.BB,
                    (size_t)pp.nchunks * pp.tilesA * pp.tilesB * pp.BA * pp.BB) *
           sizeof(double);
}

bool gram_tc5_supported(int ka, int kb) {
    // every tile shape fits: conversion units (KT/8) * (BA + BB) <= 256 * kT5MaxUnits,
    // shared memory <= 2 * 96 KiB slices + 128 KiB ring
    return ka > 0 && kb > 0;
}

template <int NC8>
static void t5_set_attr() {
    set_smem_attr(gram_tc5_kernel<NC8>, (int)max_smem_optin());
}

int launch_gram_reduce(cudaStream_t st, const double *part, int nchunks, int ntiles, int BA,
                       int BB, int tilesB, int ka, int kb, int kb1, double *C1, int ldc1,
                       double *C2, int ldc2, int gap = 0);

template <int NC8>
static void t5m_set_attr() {
    set_smem_attr(gram_tc5m_kernel<NC8>, (int)max_smem_optin());
}

// The MN-major / TMA kernel; CACG_ERR_UNSUPPORTED when the operands do not
// allow TMA boxes (16-byte aligned bases and row strides; an R1/R2 boundary
// on an 8-column octet) or the ring does not fit.
// kb1map <= kb1: R1's true width; columns [kb1map, kb1) of the kernel's R1
// part read as zeros (outside the tensor map), so an R1 width of 4 mod 8 can
// be padded to the converters' 8-column units.
static int launch_tc5m(cudaStream_t st, const T5Plan &p, int64_t n, const float *L, int64_t ldl,
                       int ka, const float *R1, int64_t ldr1, int kb1, const float *R2,
                       int64_t ldr2, int kb2, double *ws, int *status, int kb1map) {
    if (n <= 0 || n >= (1ll << 31) - 4096) return CACG_ERR_UNSUPPORTED;
    if (ldl % 4 || ldr1 % 4 || (kb2 > 0 && (ldr2 % 4 || kb1 % 8)) || !aligned16(L) ||
        !aligned16(R1) || (kb2 > 0 && !aligned16(R2)) || kb1map > kb1 || kb1map <= 0)
        return CACG_ERR_UNSUPPORTED;
    const CUtensorMapSwizzle sw = CU_TENSOR_MAP_SWIZZLE_128B;
    const CUtensorMapL2promotion pr = CU_TENSOR_MAP_L2_PROMOTION_L2_256B;
    CUtensorMap tmL, tmR1, tmR2;
    if (!tma_encode_2d(&tmL, L, (uint64_t)ka, (uint64_t)n, (uint64_t)ldl * 4, kT5mBox, kT5mBox,
                       sw, pr) ||
        !tma_encode_2d(&tmR1, R1, (uint64_t)kb1map, (uint64_t)n, (uint64_t)ldr1 * 4, kT5mBox,
                       kT5mBox, sw, pr))
        return CACG_ERR_UNSUPPORTED;
    if (kb2 > 0) {
        if (!tma_encode_2d(&tmR2, R2, (uint64_t)kb2, (uint64_t)n, (uint64_t)ldr2 * 4, kT5mBox,
                           kT5mBox, sw, pr))
            return CACG_ERR_UNSUPPORTED;
    } else {
        tmR2 = tmR1;  // never loaded
    }
    const size_t buf = 3 * ((size_t)kT5M * kT5KT * 2 + (size_t)p.BB * kT5KT * 2);
    const size_t ring_off = (kT5wNB * buf + 1023) / 1024 * 1024;
    const int nbox_max = (p.BA + kT5mBox - 1) / kT5mBox + (p.BB + kT5mBox - 1) / kT5mBox + 1;
    int stages = 4;
    size_t smem = 0;
    for (; stages >= 2; --stages) {
        smem = ring_off + (size_t)stages * nbox_max * kT5mBoxBytes +
               (2 * stages + 2 * kT5wNB + 4) * 8 + 16;
        if (smem <= max_smem_optin()) break;
    }
    if (stages < 2) return CACG_ERR_UNSUPPORTED;
    dim3 grid(p.nchunks, p.tilesA * p.tilesB);
#define T5M_CASE(NC)                                                                               \
    case NC:                                                                                       \
        t5m_set_attr<NC>();                                                                        \
        gram_tc5m_kernel<NC><<<grid, kT5wThreads, smem, st>>>(tmL, tmR1, tmR2, n, p.rows_per_chunk, \
                                                             ka, kb1, kb2, p.BA, p.tilesB,         \
                                                             p.tmem_half, stages, ws, status,      \
                                                             g_pipe_polls.load());                 \
        break;
    switch (p.BB / 16) {
        T5M_CASE(1)
        T5M_CASE(2)
        T5M_CASE(3)
        T5M_CASE(4)
        T5M_CASE(5)
        T5M_CASE(6)
        T5M_CASE(7)
        T5M_CASE(8)
        default:
            return CACG_ERR_UNSUPPORTED;
    }
#undef T5M_CASE
    return check_launch();
}

int launch_gram_tc5(cudaStream_t st, int64_t n, const float *L, int64_t ldl, int ka,
                    const float *R1, int64_t ldr1, int kb1, const float *R2, int64_t ldr2,
                    int kb2, double *C1, int ldc1, double *C2, int ldc2, double *ws,
                    size_t ws_bytes, int *status) {
    const int kb = kb1 + kb2;
    if (ka <= 0 || kb <= 0 || n < 0 || !C1 || (kb2 > 0 && !C2) || !status) return CACG_ERR_ARG;
    if (!gram_tc5_supported(ka, kb)) return CACG_ERR_UNSUPPORTED;
    T5Plan p = plan_tc5(n, ka, kb);
    const size_t need = (size_t)p.nchunks * p.tilesA * p.tilesB * p.BA * p.BB * sizeof(double);
    if (!ws || need > ws_bytes) return CACG_ERR_ARG;
    // Q^T [AQ | R] with k = 4 mod 8 (k = 4m, m odd): the TMA kernel's R1 part
    // padded by 4 zero columns, the reduction skipping them
    int gap = 0;
    int mrc = CACG_ERR_UNSUPPORTED;
    if (kb2 > 0 && kb1 % 8 == 4) {
        const int kb1p = kb1 + 4;
        T5Plan pp = plan_tc5(n, ka, kb1p + kb2);
        const size_t needp =
            (size_t)pp.nchunks * pp.tilesA * pp.tilesB * pp.BA * pp.BB * sizeof(double);
        if (needp <= ws_bytes) {
            mrc = launch_tc5m(st, pp, n, L, ldl, ka, R1, ldr1, kb1p, R2, ldr2, kb2, ws, status, kb1);
            if (mrc != CACG_ERR_UNSUPPORTED) {
                if (mrc != CACG_OK) return mrc;
                return launch_gram_reduce(st, ws, pp.nchunks, pp.tilesA * pp.tilesB, pp.BA, pp.BB,
                                          pp.tilesB, ka, kb, kb1, C1, ldc1, C2, ldc2, 4);
            }
        }
    }
    mrc = launch_tc5m(st, p, n, L, ldl, ka, R1, ldr1, kb1, R2, ldr2, kb2, ws, status, kb1);
    if (mrc != CACG_ERR_UNSUPPORTED) {
        if (mrc != CACG_OK) return mrc;
    } else if (n > 0) {
        if (p.smem > max_smem_optin()) return CACG_ERR_UNSUPPORTED;
        const int vec16 = (ldl % 4 == 0) && (ldr1 % 4 == 0) && (kb2 == 0 || ldr2 % 4 == 0) &&
                          (kb1 % 4 == 0) && aligned16(L) && aligned16(R1) &&
                          (kb2 == 0 || aligned16(R2));
        dim3 grid(p.nchunks, p.tilesA * p.tilesB);
#define T5_CASE(NC)                                                                               \
    case NC:                                                                                      \
        t5_set_attr<NC>();                                                                        \
        gram_tc5_kernel<NC><<<grid, kT5Threads, p.smem, st>>>(                                    \
            n, p.rows_per_chunk, L, ldl, ka, R1, ldr1, kb1, R2, ldr2, kb2, p.BA, p.tilesB, vec16, \
            p.tmem_half, ws, status);                                                             \
        break;
        switch (p.BB / 16) {
            T5_CASE(1)
            T5_CASE(2)
            T5_CASE(3)
            T5_CASE(4)
            T5_CASE(5)
            T5_CASE(6)
            T5_CASE(7)
            T5_CASE(8)
            default:
                return CACG_ERR_UNSUPPORTED;
        }
#undef T5_CASE
        int rc = check_launch();
        if (rc != CACG_OK) return rc;
    } else {
        if (cudaMemsetAsync(ws, 0, need, st) != cudaSuccess) return CACG_ERR_CUDA;
    }
    return launch_gram_reduce(st, ws, n > 0 ? p.nchunks : 1, p.tilesA * p.tilesB, p.BA, p.BB,
                              p.tilesB, ka, kb, kb1, C1, ldc1, C2, ldc2, gap);
}

}  // namespace cacg

extern "C" int cacg_set_pipeline_wait_limit(int64_t polls) {
    cacg::g_pipe_polls.store(polls >= 0 ? (long long)polls : cacg::kT5SpinLimit);
    return CACG_OK;
}
