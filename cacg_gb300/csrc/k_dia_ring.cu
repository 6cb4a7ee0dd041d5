// k_dia_ring.cu -- DIA SpMM (FP32, 16-column tiles) with the X rows staged in
// shared memory by TMA: Y = ca A X + cb Z1 + cc Z2, the mixed mode's
// Chebyshev basis step (src/common.c:182-256: Y = T_{j+1}, X = Z1 = T_j,
// Z2 = T_{j-1}) and A Q (src/bcbcgKernel.c, the AQ product), A in the DIA
// view of k_dia.cu.
//
// Bands.  The diagonals (ascending offsets) are cut into bands of nearby
// offsets; the 27-point stencil on an N^3 grid gives three bands (dz = -1, 0,
// +1), each 2N + 2 offsets wide.  A block of BR = 96 output rows starting at
// r0 reads the X rows [r0 + lo_b, r0 + hi_b + BR) of band b.  A CTA walks an
// item of consecutive blocks, so band b is a ring of K_b + 1 chunks of BR rows
// in shared memory: K_b = ceil((hi_b - lo_b) / BR) + 1 chunks in use, one more
// being loaded for the next block.  Each X row crosses L2 -> shared memory
// once per band and item (plus the item's K_b - 1 start-up chunks), one 2-D
// TMA load per chunk, and the FMAs read it from shared memory.  The block's
// DIA values (ndiag x BR FP32) come by one more TMA load into a double buffer.
//
// Threads.  128 compute threads and a producer warp (one thread issues the
// TMA loads); the producer refills block u - 1's slot and value buffer as
// soon as the four compute warps have arrived on that block's "done"
// mbarrier, so the warps run independently (no CTA-wide barrier per block).
// Thread (lr, c) = (tid / 4, tid % 4) computes rows
// r0 + 3 lr + i (i < 3) of columns 4c .. 4c + 3.  Three rows per thread (an
// odd count) puts the two rows that a quarter warp's 16-byte loads touch in
// 64-byte slots of different parity, i.e. on disjoint banks.  Each output
// sums its diagonals in ascending offset order with one FMA chain, as the
// other DIA kernels and the CSR kernels do, so the results are bit-identical
// to theirs.
//
// Items (sb consecutive blocks of one 16-column tile) go round-robin to the
// CTAs, so at any time the CTAs work on neighbouring rows, and an X row that
// the three bands read (N^2 rows apart) is an L2 hit after its first read.
// The waits on the TMA barriers are bounded: on expiry the CTA sets
// kStatusTimeout, waits (bounded) for the loads it has in flight and returns.
#include <algorithm>
#include <vector>

#include "cacg_internal.cuh"
#include "cacg_solver.h"
#include "tc5_util.cuh"
#include "tma_util.cuh"

namespace cacg {

namespace {

constexpr int kRingThreads = 128;
constexpr int kRingCpr = 4;                                // threads per row (float4 each)
constexpr int kRingR = 3;                                  // rows per thread (odd)
constexpr int kRingBR = kRingThreads / kRingCpr * kRingR;  // 96 rows per block
constexpr int kRingCols = 16;                              // columns per tile
constexpr int kRingRowBytes = kRingCols * 4;               // 64 bytes of a staged row
constexpr int kRingBandMax = 4;
constexpr int kRingMirror = 8;  // rows of slot 0 repeated after a ring's end
constexpr int kRingItemsPerCta = 8;
constexpr int kRingSmemMax = 227 * 1024;

struct RingDesc {
    int nb;                        // bands
    int lo[kRingBandMax];          // lowest offset of band b
    int K[kRingBandMax];           // chunks one block reads from band b
    int cap[kRingBandMax];         // ring rows, (K + 1) * BR (plus kRingMirror rows)
    int soff[kRingBandMax];        // byte offset of the ring in shared memory
    int gfirst[kRingBandMax + 1];  // groups of band b: [gfirst[b], gfirst[b + 1])
    int voff;                      // byte offset of the two value buffers
    int vbytes;                    // bytes of one value buffer (ndiag x BR x 4, rounded up)
    int vtx;                       // bytes one value load delivers (ndiag x BR x 4)
    int boff;                      // byte offset of the two mbarriers
    int z1band, z1rel;             // Z1 == X: band whose ring holds rows r0 .. r0+BR-1
    int sb;                        // blocks per item
    int tiles;                     // 16-column tiles
    int grel[kDiaMax];             // group g: first offset - lo of its band
    int gdg[kDiaMax];              // group g: first diagonal | diagonals << 8
};

// Loads of block t of an item (first: the K_b start-up chunks of every band)
// and its values, completing on *bar.  A chunk that goes to slot 0 also
// fills the ring's mirror rows (its first kRingMirror rows, after the last
// slot), so a window of consecutive ring rows never wraps.
__device__ __forceinline__ void ring_issue(unsigned char *sm, const RingDesc &rd,
                                           const CUtensorMap *tmx, const CUtensorMap *tmm,
                                           const CUtensorMap *tmv, int64_t R0, int col0, int t,
                                           bool first, void *vdst, uint64_t *bar) {
    unsigned bytes = (unsigned)rd.vtx;
    for (int b = 0; b < rd.nb; ++b) {
        const int j0 = first ? 0 : t + rd.K[b] - 1, j1 = first ? rd.K[b] : j0 + 1;
        for (int j = j0; j < j1; ++j)
            bytes += kRingBR * kRingRowBytes +
                     (j % (rd.K[b] + 1) == 0 ? kRingMirror * kRingRowBytes : 0);
    }
    tma_expect_tx(bar, bytes);
    for (int b = 0; b < rd.nb; ++b) {
        const int j0 = first ? 0 : t + rd.K[b] - 1, j1 = first ? rd.K[b] : j0 + 1;
        for (int j = j0; j < j1; ++j) {
            const int slot = j % (rd.K[b] + 1);
            const int y = (int)(R0 + rd.lo[b] + (int64_t)j * kRingBR);
            tma_load_2d(sm + rd.soff[b] + slot * (kRingBR * kRingRowBytes), tmx, col0, y, bar);
            if (slot == 0)
                tma_load_2d(sm + rd.soff[b] + rd.cap[b] * kRingRowBytes, tmm, col0, y, bar);
        }
    }
    tma_load_2d(vdst, tmv, (int)(R0 + (int64_t)t * kRingBR), 0, bar);
}

// One group of G adjacent diagonals: the window of R + G - 1 staged rows
// starting at ring row q < cap (the mirror rows continue the ring past cap),
// G x R values from vp (stride BR per diagonal), FMAs into acc in diagonal
// order.
template <int G>
__device__ __forceinline__ void ring_group(const unsigned char *ring, int q, const float *vp,
                                           float4 (&acc)[kRingR]) {
    constexpr int W = kRingR + G - 1;
    static_assert(W - 1 <= kRingMirror, "window longer than the mirror");
    float4 win[W];
    const unsigned char *p = ring + q * kRingRowBytes;
#pragma unroll
    for (int w = 0; w < W; ++w) win[w] = *reinterpret_cast<const float4 *>(p + w * kRingRowBytes);
#pragma unroll
    for (int j = 0; j < G; ++j) {
        float v[kRingR];
#pragma unroll
        for (int i = 0; i < kRingR; ++i) v[i] = vp[j * kRingBR + i];
#pragma unroll
        for (int i = 0; i < kRingR; ++i) {
            acc[i].x = fmaf(v[i], win[i + j].x, acc[i].x);
            acc[i].y = fmaf(v[i], win[i + j].y, acc[i].y);
            acc[i].z = fmaf(v[i], win[i + j].z, acc[i].z);
            acc[i].w = fmaf(v[i], win[i + j].w, acc[i].w);
        }
    }
}

// NB > 0: NB bands of GPB groups of G diagonals each (the 27-point stencil's
// 3 x 3 x 3), loops unrolled so the window loads of later groups can be
// issued ahead of earlier groups' FMAs; NB = 0: any layout, read from rd.
template <int NB, int GPB, int G>
__global__ void __launch_bounds__(kRingThreads + 32, 2)
    dia_ring_kernel(const __grid_constant__ CUtensorMap tmx, const __grid_constant__ CUtensorMap tmm,
                    const __grid_constant__ CUtensorMap tmv,
                    int64_t n, int64_t nitems, const DiaDesc desc, const __grid_constant__ RingDesc rd,
                    float *__restrict__ Y, int64_t ldy, const float *__restrict__ Z1, int64_t ldz1,
                    const float *__restrict__ Z2, int64_t ldz2, float ca, float cb, float cc,
                    int *__restrict__ status) {
    extern __shared__ __align__(128) unsigned char ring_smem[];
    // full[2]: block u's loads landed (TMA); done[2]: all 128 compute threads
    // finished block u (its ring slots and value buffer may be refilled)
    uint64_t *full = reinterpret_cast<uint64_t *>(ring_smem + rd.boff);
    uint64_t *done = full + 2;
    volatile int *abort_flag = reinterpret_cast<volatile int *>(done + 2);
    const int tid = threadIdx.x, lr = tid / kRingCpr, c = tid % kRingCpr;
    const int rowoff = lr * kRingR;
    if (tid == 0) {
        t5_mbar_init(&full[0], 1);
        t5_mbar_init(&full[1], 1);
        t5_mbar_init(&done[0], kRingThreads);  // every compute thread releases
        t5_mbar_init(&done[1], kRingThreads);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        t5_fence_proxy_async();
    }
    __syncthreads();

    const int64_t nblk = (n + kRingBR - 1) / kRingBR;
    if (tid >= kRingThreads) {
        // ------------------------------------------------ producer (one thread)
        if (tid != kRingThreads) return;
        unsigned u = 0, issued = 0;
        bool stop = false;
        // false (and the abort flag set) if block v did not finish in time
        auto wait_done = [&](unsigned v) {
            if (t5_mbar_wait_or_abort(&done[v & 1], (v >> 1) & 1, abort_flag)) return true;
            if (!*abort_flag) atomicOr(status, kStatusTimeout);
            *abort_flag = 1;
            return false;
        };
        for (int64_t it = blockIdx.x; it < nitems && !stop; it += gridDim.x) {
            const int64_t ri = it / rd.tiles;
            const int col0 = (int)(it % rd.tiles) * kRingCols;
            const int64_t b0 = ri * rd.sb;
            const int nbk = (int)std::min<int64_t>(rd.sb, nblk - b0);
            const int64_t R0 = b0 * kRingBR;
            // the item's start-up chunks take every slot: block u - 1 must be done
            if (u >= 1 && !wait_done(u - 1)) break;
            t5_fence_proxy_async();
            ring_issue(ring_smem, rd, &tmx, &tmm, &tmv, R0, col0, 0, true,
                       ring_smem + rd.voff + (u & 1) * rd.vbytes, &full[u & 1]);
            ++issued;
            for (int t = 0; t < nbk; ++t, ++u) {
                if (t + 1 >= nbk) continue;
                // block t + 1 takes the slot of block t - 1's first chunk and the
                // value buffer of block t - 1 (t = 0: waited for above)
                if (t >= 1 && !wait_done(u - 1)) {
                    stop = true;
                    break;
                }
                t5_fence_proxy_async();
                ring_issue(ring_smem, rd, &tmx, &tmm, &tmv, R0, col0, t + 1, false,
                           ring_smem + rd.voff + ((u + 1) & 1) * rd.vbytes, &full[(u + 1) & 1]);
                ++issued;
            }
        }
        if (*abort_flag)  // let the loads in flight land before the CTA exits (bounded)
            for (unsigned v = issued >= 2 ? issued - 2 : 0; v < issued; ++v)
                t5_mbar_wait(&full[v & 1], (v >> 1) & 1);
        return;
    }
    // ------------------------------------------------------ compute warps
    unsigned u = 0;  // blocks computed (barrier stage and parity)
    bool timeout = false;
    for (int64_t it = blockIdx.x; it < nitems && !timeout; it += gridDim.x) {
        const int64_t ri = it / rd.tiles;
        const int col0 = (int)(it % rd.tiles) * kRingCols;
        const int64_t b0 = ri * rd.sb;
        const int nbk = (int)std::min<int64_t>(rd.sb, nblk - b0);
        const int64_t R0 = b0 * kRingBR;
        int base[kRingBandMax];  // ring row of the block's first row, band b: t BR mod cap
#pragma unroll
        for (int b = 0; b < kRingBandMax; ++b) base[b] = 0;
        const int col = col0 + 4 * c;
        // Z2 (the recurrence's T_{j-1}) from global memory is software-
        // pipelined one block ahead: block t + 1's rows are requested while
        // block t waits and computes, so their latency is hidden behind a
        // whole block instead of the (short) barrier wait
        float4 z2v[kRingR], z2n[kRingR];
        auto load_z2 = [&](int tt, float4(&dst)[kRingR]) {
            const int64_t rb = R0 + (int64_t)tt * kRingBR + rowoff;
#pragma unroll
            for (int i = 0; i < kRingR; ++i)
                dst[i] = Z2 && tt < nbk && rb + i < n
                             ? *reinterpret_cast<const float4 *>(Z2 + (rb + i) * ldz2 + col)
                             : make_float4(0.f, 0.f, 0.f, 0.f);
        };
        load_z2(0, z2v);
        for (int t = 0; t < nbk; ++t, ++u) {
            const int64_t rbase = R0 + (int64_t)t * kRingBR + rowoff;
            load_z2(t + 1, z2n);
            // Z1 from global memory (when the ring does not hold it) goes out
            // before the barrier wait
            const bool z1g = Z1 && rd.z1band < 0;
            float4 z1v[kRingR];
#pragma unroll
            for (int i = 0; i < kRingR; ++i) {
                const bool in = rbase + i < n;
                z1v[i] = z1g && in ? *reinterpret_cast<const float4 *>(Z1 + (rbase + i) * ldz1 + col)
                                   : make_float4(0.f, 0.f, 0.f, 0.f);
            }
            const bool ok = __all_sync(0xffffffffu, t5_mbar_wait_or_abort(
                                                        &full[u & 1], (u >> 1) & 1, abort_flag));
            if (!ok) {
                if ((tid & 31) == 0) {
                    if (!*abort_flag) atomicOr(status, kStatusTimeout);
                    *abort_flag = 1;
                }
                timeout = true;
                break;
            }
            const float *vb =
                reinterpret_cast<const float *>(ring_smem + rd.voff + (u & 1) * rd.vbytes) + rowoff;
            float4 acc[kRingR];
#pragma unroll
            for (int i = 0; i < kRingR; ++i) acc[i] = make_float4(0.f, 0.f, 0.f, 0.f);
            int zq = -1;  // ring row of the thread's first row in the Z1 band
#pragma unroll
            for (int b = 0; b < (NB > 0 ? NB : kRingBandMax); ++b) {
                if (NB > 0 || b < rd.nb) {
                    const unsigned char *ring = ring_smem + rd.soff[b] + c * 16;
                    const int cap = rd.cap[b];
                    const int qb = base[b] + rowoff;
                    if (b == rd.z1band) {
                        zq = qb + rd.z1rel;
                        if (zq >= cap) zq -= cap;
                    }
                    if constexpr (NB > 0) {
#pragma unroll
                        for (int gg = 0; gg < GPB; ++gg) {
                            const int g = b * GPB + gg;
                            int q = qb + rd.grel[g];
                            if (q >= cap) q -= cap;
                            ring_group<G>(ring, q, vb + (rd.gdg[g] & 0xFF) * kRingBR, acc);
                        }
                    } else {
                        for (int g = rd.gfirst[b]; g < rd.gfirst[b + 1]; ++g) {
                            int q = qb + rd.grel[g];
                            if (q >= cap) q -= cap;
                            const int dg = rd.gdg[g];
                            const float *vp = vb + (dg & 0xFF) * kRingBR;
                            switch (dg >> 8) {
                                case 1: ring_group<1>(ring, q, vp, acc); break;
                                case 2: ring_group<2>(ring, q, vp, acc); break;
                                case 3: ring_group<3>(ring, q, vp, acc); break;
                                default: ring_group<4>(ring, q, vp, acc); break;
                            }
                        }
                    }
                }
            }
            float *yp = Y + rbase * ldy + col;
#pragma unroll
            for (int i = 0; i < kRingR; ++i) {
                if (rbase + i >= n) break;
                float4 y = make_float4(ca * acc[i].x, ca * acc[i].y, ca * acc[i].z, ca * acc[i].w);
                if (Z1) {
                    float4 z;
                    if (zq >= 0) {
                        z = *reinterpret_cast<const float4 *>(ring_smem + rd.soff[rd.z1band] +
                                                              c * 16 + (zq + i) * kRingRowBytes);
                    } else {
                        z = z1v[i];
                    }
                    y.x = fmaf(cb, z.x, y.x);
                    y.y = fmaf(cb, z.y, y.y);
                    y.z = fmaf(cb, z.z, y.z);
                    y.w = fmaf(cb, z.w, y.w);
                }
                if (Z2) {
                    const float4 z = z2v[i];
                    y.x = fmaf(cc, z.x, y.x);
                    y.y = fmaf(cc, z.y, y.y);
                    y.z = fmaf(cc, z.z, y.z);
                    y.w = fmaf(cc, z.w, y.w);
                }
                *reinterpret_cast<float4 *>(yp + i * ldy) = y;
            }
#pragma unroll
            for (int b = 0; b < (NB > 0 ? NB : kRingBandMax); ++b) {
                if (NB > 0 || b < rd.nb) {
                    base[b] += kRingBR;
                    if (base[b] >= rd.cap[b]) base[b] -= rd.cap[b];
                }
            }
            // this thread is done with the block's ring slots and values: each
            // thread orders its own shared-memory reads before the producer's
            // next TMA fill of these slots (proxy fence, then its arrive)
            t5_fence_proxy_async();
            t5_mbar_arrive(&done[u & 1]);
#pragma unroll
            for (int i = 0; i < kRingR; ++i) z2v[i] = z2n[i];
        }
    }
}

// Bands, rings and shared-memory layout for the matrix's diagonals; false
// when they do not fit.
bool ring_plan(const DiaDesc &D, RingDesc *rd, size_t *smem) {
    std::vector<int> gfirst;
    std::vector<int64_t> lo, hi;
    for (int g = 0; g < D.ngroups; ++g) {
        const int64_t a = D.off[D.gstart[g]], e = D.off[D.gstart[g + 1] - 1];
        if (!lo.empty() && a - hi.back() < 2 * kRingBR) {
            hi.back() = e;  // a gap this small costs less than a ring of its own
            continue;
        }
        gfirst.push_back(g);
        lo.push_back(a);
        hi.push_back(e);
    }
    const int nb = (int)lo.size();
    if (nb == 0 || nb > kRingBandMax) return false;
    *rd = RingDesc{};
    rd->nb = nb;
    rd->z1band = -1;
    size_t off = 0;
    for (int b = 0; b < nb; ++b) {
        const int64_t span = hi[b] - lo[b];
        rd->lo[b] = (int)lo[b];
        rd->K[b] = (int)((span + kRingBR - 1) / kRingBR) + 1;
        rd->cap[b] = (rd->K[b] + 1) * kRingBR;
        rd->soff[b] = (int)off;
        rd->gfirst[b] = gfirst[b];
        off += (size_t)(rd->cap[b] + kRingMirror) * kRingRowBytes;
        if (lo[b] <= 0 && hi[b] >= 0) {
            rd->z1band = b;
            rd->z1rel = (int)-lo[b];
        }
    }
    rd->gfirst[nb] = D.ngroups;
    for (int b = 0; b < nb; ++b)
        for (int g = rd->gfirst[b]; g < rd->gfirst[b + 1]; ++g) {
            rd->grel[g] = (int)(D.off[D.gstart[g]] - lo[b]);
            rd->gdg[g] = D.gstart[g] | ((D.gstart[g + 1] - D.gstart[g]) << 8);
        }
    rd->voff = (int)off;
    rd->vtx = D.ndiag * kRingBR * 4;
    rd->vbytes = (rd->vtx + 127) / 128 * 128;
    off += 2 * (size_t)rd->vbytes;
    rd->boff = (int)off;
    off += 48;  // full[2], done[2], abort flag
    *smem = off;
    return off <= (size_t)kRingSmemMax;
}

template <int NB, int GPB, int G>
int ring_launch(cudaStream_t st, const CUtensorMap &tmx, const CUtensorMap &tmm,
                const CUtensorMap &tmv, int64_t n, const DiaDesc &desc, RingDesc &rd, size_t smem,
                float *Y, int64_t ldy, const float *Z1, int64_t ldz1, const float *Z2, int64_t ldz2,
                float ca, float cb, float cc, int *status) {
    set_smem_attr(dia_ring_kernel<NB, GPB, G>, kRingSmemMax);
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, dia_ring_kernel<NB, GPB, G>,
                                                      kRingThreads + 32, smem) != cudaSuccess ||
        occ < 1) {
        cudaGetLastError();
        return CACG_ERR_UNSUPPORTED;
    }
    const int64_t grid0 = (int64_t)sm_count() * std::min(occ, 2);
    const int64_t nblk = (n + kRingBR - 1) / kRingBR;
    int kmax = 1;
    for (int b = 0; b < rd.nb; ++b) kmax = std::max(kmax, rd.K[b]);
    // about kRingItemsPerCta items per CTA; an item at least 2 K blocks long
    const int64_t want = std::max<int64_t>(1, grid0 * kRingItemsPerCta / rd.tiles);
    rd.sb = (int)std::max<int64_t>(2 * kmax, (nblk + want - 1) / want);
    const int64_t nitems = (nblk + rd.sb - 1) / rd.sb * rd.tiles;
    const int64_t grid = std::min<int64_t>(grid0, nitems);
    dia_ring_kernel<NB, GPB, G><<<(unsigned)grid, kRingThreads + 32, smem, st>>>(
        tmx, tmm, tmv, n, nitems, desc, rd, Y, ldy, Z1, ldz1, Z2, ldz2, ca, cb, cc, status);
    return check_launch();
}

}  // namespace

int launch_dia_ring(cudaStream_t st, const DevMatrix *A, int w, const float *X, int64_t ldx,
                    float *Y, int64_t ldy, const float *Z1, int64_t ldz1, const float *Z2,
                    int64_t ldz2, double ca, double cb, double cc, int *status) {
    if (!A || !A->dia32 || A->dia_ndiag <= 0 || !status) return CACG_ERR_UNSUPPORTED;
    const int64_t n = A->n;
    // one 16-column tile: wider blocks (A Q) keep the unstaged kernel, which
    // shares each row's values and window addressing over all columns (six
    // staged tiles measured 0.93 ms against its 0.83 ms at 128^3, k = 96)
    if (n <= 0 || n >= (1ll << 30) || w != kRingCols) return CACG_ERR_UNSUPPORTED;
    if (!aligned16(X) || !aligned16(Y) || ldx % 4 || ldy % 4 || ldx < w || ldy < w)
        return CACG_ERR_UNSUPPORTED;
    if (Z1 && (!aligned16(Z1) || ldz1 % 4)) return CACG_ERR_UNSUPPORTED;
    if (Z2 && (!aligned16(Z2) || ldz2 % 4)) return CACG_ERR_UNSUPPORTED;
    if (A->dia_npad % 4 || !aligned16(A->dia32)) return CACG_ERR_UNSUPPORTED;
    RingDesc rd;
    size_t smem = 0;
    if (!ring_plan(A->dia, &rd, &smem)) return CACG_ERR_UNSUPPORTED;
    if (!(Z1 == X && ldz1 == ldx)) rd.z1band = -1;  // Z1 read from global memory
    rd.tiles = w / kRingCols;
    CUtensorMap tmx, tmm, tmv;
    const CUtensorMapSwizzle nosw = CU_TENSOR_MAP_SWIZZLE_NONE;
    if (!tma_encode_2d(&tmx, X, (uint64_t)w, (uint64_t)n, (uint64_t)ldx * 4, kRingCols, kRingBR,
                       nosw, CU_TENSOR_MAP_L2_PROMOTION_NONE) ||
        !tma_encode_2d(&tmm, X, (uint64_t)w, (uint64_t)n, (uint64_t)ldx * 4, kRingCols,
                       kRingMirror, nosw, CU_TENSOR_MAP_L2_PROMOTION_NONE) ||
        !tma_encode_2d(&tmv, A->dia32, (uint64_t)A->dia_npad, (uint64_t)A->dia_ndiag,
                       (uint64_t)A->dia_npad * 4, kRingBR, (uint32_t)A->dia_ndiag, nosw,
                       CU_TENSOR_MAP_L2_PROMOTION_L2_256B))
        return CACG_ERR_UNSUPPORTED;
    bool box333 = rd.nb == 3 && A->dia.ngroups == 9;
    for (int b = 0; box333 && b < 3; ++b) box333 = rd.gfirst[b] == 3 * b;
    for (int g = 0; box333 && g < 9; ++g) box333 = (rd.gdg[g] >> 8) == 3;
    if (box333)
        return ring_launch<3, 3, 3>(st, tmx, tmm, tmv, n, A->dia, rd, smem, Y, ldy, Z1, ldz1, Z2,
                                    ldz2, (float)ca, (float)cb, (float)cc, status);
    return ring_launch<0, 0, 0>(st, tmx, tmm, tmv, n, A->dia, rd, smem, Y, ldy, Z1, ldz1, Z2,
                                ldz2, (float)ca, (float)cb, (float)cc, status);
}

}  // namespace cacg
