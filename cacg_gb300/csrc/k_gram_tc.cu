// k_gram_tc.cu -- Gram products of FP32 blocks on the tensor cores.
//
// Reference operations replaced (sclc/cacg): distributedMatLTransposeMatRMul
// (src/BLAS3.c:699-726) and distributedMatLTransposeMatRMul_updated
// (src/BLAS3.c:730-758) in the mixed-precision mode, where L, R are FP32.
//
// C = L^T [R1 | R2], L n x ka, R n x kb.  Each FP32 value x is split exactly
// into three bf16 slices, x = x1 + x2 + x3 (x1 = bf16(x), x2 = bf16(x - x1),
// x3 = bf16(x - x1 - x2); every difference is exact in FP32), and the product
// is assembled from the six slice products whose order is <= 2^-16 of the
// leading one: L1R1, L1R2, L2R1, L1R3, L2R2, L3R1.  bf16 x bf16 products are
// exact in the FP32 accumulator; FP32 accumulation runs over 256-row groups,
// after which the group sums are added into FP64 accumulators in shared
// memory, and the per-CTA FP64 partials are summed in a fixed order by the
// split-K reduction (gram_reduce in k_gram.cu).
//
// Layout: per K-step of 32 rows the FP32 tiles are staged by cp.async
// (double-buffered) and converted into slice tiles in the 8x8 "core matrix"
// layout (8 rows x 16 bytes contiguous, K-major for both operands), read by
// ldmatrix and consumed by mma.sync m16n8k16 (bf16 in, FP32 accumulate).
#include <cuda_bf16.h>

#include <algorithm>

#include "cacg_internal.cuh"

namespace cacg {

constexpr int kTcKT = 32;         // rows per K-step
constexpr int kTcFlush = 8;       // K-steps per FP32 accumulation group (256 rows)
constexpr int kTcWarpM = 32;      // warp tile rows (2 x m16)
constexpr int kTcWarpN = 16;      // warp tile cols (2 x n8)
constexpr int kTcMaxThreads = 768;

__device__ __forceinline__ unsigned smem_u32(const void *p) {
    return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void tc_cp_async4(void *smem, const void *g) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(smem_u32(smem)), "l"(g));
}
__device__ __forceinline__ void tc_cp_async16(void *smem, const void *g) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_u32(smem)), "l"(g));
}
__device__ __forceinline__ void tc_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void tc_wait1() { asm volatile("cp.async.wait_group 1;\n" ::); }
__device__ __forceinline__ void tc_wait0() { asm volatile("cp.async.wait_group 0;\n" ::); }

__device__ __forceinline__ void ldsm_x4(unsigned (&r)[4], unsigned addr) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(addr));
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const unsigned (&a)[4], unsigned b0,
                                         unsigned b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
        "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// offset (in bf16 elements) of element (row, k) in a core-matrix tile whose
// K extent is kTcKT: core (row/8, k/8) at ((row/8)*(KT/8) + k/8)*64,
// inside: (row%8)*8 + k%8.
__device__ __forceinline__ int core_off(int row, int k) {
    return ((row >> 3) * (kTcKT / 8) + (k >> 3)) * 64 + (row & 7) * 8 + (k & 7);
}

// split x into three bf16 slices (exact: x == s1 + s2 + s3 up to FP32's 24 bits)
__device__ __forceinline__ void split3(float x, __nv_bfloat16 &s1, __nv_bfloat16 &s2,
                                       __nv_bfloat16 &s3) {
    s1 = __float2bfloat16_rn(x);
    float r1 = x - __bfloat162float(s1);
    s2 = __float2bfloat16_rn(r1);
    float r2 = r1 - __bfloat162float(s2);
    s3 = __float2bfloat16_rn(r2);
}

struct TcSmem {
    float *stL[2], *stR[2];  // FP32 staging [KT][BA], [KT][BB]
    __nv_bfloat16 *sl[3];    // L slices, core layout, BA x KT each
    __nv_bfloat16 *sr[3];    // R slices, core layout, BB x KT each
    double *acc;             // BA x BB FP64
};

__global__ void __launch_bounds__(kTcMaxThreads)
    gram_tc_kernel(int64_t n, int64_t rows_per_chunk, const float *__restrict__ L, int64_t ldl,
                   int ka, const float *__restrict__ R1, int64_t ldr1, int kb1,
                   const float *__restrict__ R2, int64_t ldr2, int kb2, int BA, int BB,
                   int tilesB, int vec16, double *__restrict__ part) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    TcSmem sm;
    {
        unsigned char *p = smem_raw;
        for (int b = 0; b < 2; ++b) {
            sm.stL[b] = reinterpret_cast<float *>(p);
            p += (size_t)kTcKT * BA * 4;
            sm.stR[b] = reinterpret_cast<float *>(p);
            p += (size_t)kTcKT * BB * 4;
        }
        for (int s = 0; s < 3; ++s) {
            sm.sl[s] = reinterpret_cast<__nv_bfloat16 *>(p);
            p += (size_t)BA * kTcKT * 2;
        }
        for (int s = 0; s < 3; ++s) {
            sm.sr[s] = reinterpret_cast<__nv_bfloat16 *>(p);
            p += (size_t)BB * kTcKT * 2;
        }
        sm.acc = reinterpret_cast<double *>(p);
    }
    const int tid = threadIdx.x, nthr = blockDim.x;
    const int tile_a = blockIdx.y / tilesB, tile_b = blockIdx.y % tilesB;
    const int a0 = tile_a * BA, b0 = tile_b * BB;
    const int warp = tid >> 5, lane = tid & 31;
    const int wn_count = BB / kTcWarpN;
    const int wm = warp / wn_count, wn = warp % wn_count;
    const bool wactive = wm < BA / kTcWarpM;
    const int64_t rbeg = (int64_t)blockIdx.x * rows_per_chunk;
    const int64_t rend = min(n, rbeg + rows_per_chunk);

    for (int i = tid; i < BA * BB; i += nthr) sm.acc[i] = 0.0;

    // ---- staging of one K-step (rows r0 .. r0+KT) into buffer b
    auto stage = [&](int b, int64_t r0) {
        float *dL = sm.stL[b], *dR = sm.stR[b];
        if (vec16) {
            const int qa = BA / 4, qb = BB / 4;
            for (int idx = tid; idx < kTcKT * qa; idx += nthr) {
                int r = idx / qa, c = (idx % qa) * 4;
                int64_t row = r0 + r;
                float *dst = dL + r * BA + c;
                if (row < rend && a0 + c < ka)
                    tc_cp_async16(dst, L + row * ldl + a0 + c);
                else
                    *reinterpret_cast<float4 *>(dst) = make_float4(0.f, 0.f, 0.f, 0.f);
            }
            for (int idx = tid; idx < kTcKT * qb; idx += nthr) {
                int r = idx / qb, c = (idx % qb) * 4;
                int64_t row = r0 + r;
                int gb = b0 + c;
                float *dst = dR + r * BB + c;
                if (row < rend && gb < kb1)
                    tc_cp_async16(dst, R1 + row * ldr1 + gb);
                else if (row < rend && gb >= kb1 && gb - kb1 < kb2)
                    tc_cp_async16(dst, R2 + row * ldr2 + (gb - kb1));
                else
                    *reinterpret_cast<float4 *>(dst) = make_float4(0.f, 0.f, 0.f, 0.f);
            }
        } else {
            for (int idx = tid; idx < kTcKT * BA; idx += nthr) {
                int r = idx / BA, c = idx % BA;
                int64_t row = r0 + r;
                float *dst = dL + r * BA + c;
                if (row < rend && a0 + c < ka)
                    tc_cp_async4(dst, L + row * ldl + a0 + c);
                else
                    *dst = 0.f;
            }
            for (int idx = tid; idx < kTcKT * BB; idx += nthr) {
                int r = idx / BB, c = idx % BB;
                int64_t row = r0 + r;
                int gb = b0 + c;
                float *dst = dR + r * BB + c;
                if (row < rend && gb < kb1)
                    tc_cp_async4(dst, R1 + row * ldr1 + gb);
                else if (row < rend && gb >= kb1 && gb - kb1 < kb2)
                    tc_cp_async4(dst, R2 + row * ldr2 + (gb - kb1));
                else
                    *dst = 0.f;
            }
        }
    };

    // ---- convert staging buffer b into the slice tiles (pairs of K rows)
    auto convert = [&](int b) {
        const float *sL = sm.stL[b], *sR = sm.stR[b];
        const int pairsL = BA * (kTcKT / 2), pairsR = BB * (kTcKT / 2);
        for (int idx = tid; idx < pairsL + pairsR; idx += nthr) {
            const bool isL = idx < pairsL;
            const int q = isL ? idx : idx - pairsL;
            const int W = isL ? BA : BB;
            const int col = q % W, k = (q / W) * 2;
            const float *src = isL ? sL : sR;
            float x0 = src[k * W + col], x1 = src[(k + 1) * W + col];
            __nv_bfloat16 h0, m0, l0, h1, m1, l1;
            split3(x0, h0, m0, l0);
            split3(x1, h1, m1, l1);
            const int off = core_off(col, k);
            __nv_bfloat16 **dst = isL ? sm.sl : sm.sr;
            *reinterpret_cast<__nv_bfloat162 *>(dst[0] + off) = __halves2bfloat162(h0, h1);
            *reinterpret_cast<__nv_bfloat162 *>(dst[1] + off) = __halves2bfloat162(m0, m1);
            *reinterpret_cast<__nv_bfloat162 *>(dst[2] + off) = __halves2bfloat162(l0, l1);
        }
    };

    float c[2][2][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j)
#pragma unroll
            for (int q = 0; q < 4; ++q) c[i][j][q] = 0.f;

    auto flush = [&]() {
        if (!wactive) return;
        const int g = lane >> 2, t = lane & 3;
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const int ra = wm * kTcWarpM + i * 16 + g;
                const int cb = wn * kTcWarpN + j * 8 + 2 * t;
                sm.acc[ra * BB + cb] += (double)c[i][j][0];
                sm.acc[ra * BB + cb + 1] += (double)c[i][j][1];
                sm.acc[(ra + 8) * BB + cb] += (double)c[i][j][2];
                sm.acc[(ra + 8) * BB + cb + 1] += (double)c[i][j][3];
#pragma unroll
                for (int q = 0; q < 4; ++q) c[i][j][q] = 0.f;
            }
    };

    int64_t r0 = rbeg;
    if (r0 < rend) stage(0, r0);
    tc_commit();
    int buf = 0, step = 0;
    for (; r0 < rend; r0 += kTcKT) {
        if (r0 + kTcKT < rend) stage(buf ^ 1, r0 + kTcKT);
        tc_commit();
        tc_wait1();
        __syncthreads();  // staging[buf] complete; previous MMAs done with slices
        convert(buf);
        __syncthreads();
        if (wactive) {
#pragma unroll
            for (int ks = 0; ks < kTcKT / 16; ++ks) {
                // A fragments (3 slices x 2 m-tiles), B fragments (3 slices x 2 n-tiles)
                unsigned af[3][2][4], bf[3][4];
#pragma unroll
                for (int s = 0; s < 3; ++s) {
#pragma unroll
                    for (int i = 0; i < 2; ++i) {
                        const int row = wm * kTcWarpM + i * 16 + ((lane >> 3) & 1) * 8 + (lane & 7);
                        const int k = ks * 16 + (lane >> 4) * 8;
                        ldsm_x4(af[s][i], smem_u32(sm.sl[s] + core_off(row, k)));
                    }
                    const int col = wn * kTcWarpN + (lane >> 4) * 8 + (lane & 7);
                    const int k = ks * 16 + ((lane >> 3) & 1) * 8;
                    ldsm_x4(bf[s], smem_u32(sm.sr[s] + core_off(col, k)));
                }
#pragma unroll
                for (int i = 0; i < 2; ++i)
#pragma unroll
                    for (int j = 0; j < 2; ++j) {
                        // small terms first
                        mma_bf16(c[i][j], af[2][i], bf[0][2 * j], bf[0][2 * j + 1]);
                        mma_bf16(c[i][j], af[1][i], bf[1][2 * j], bf[1][2 * j + 1]);
                        mma_bf16(c[i][j], af[0][i], bf[2][2 * j], bf[2][2 * j + 1]);
                        mma_bf16(c[i][j], af[1][i], bf[0][2 * j], bf[0][2 * j + 1]);
                        mma_bf16(c[i][j], af[0][i], bf[1][2 * j], bf[1][2 * j + 1]);
                        mma_bf16(c[i][j], af[0][i], bf[0][2 * j], bf[0][2 * j + 1]);
                    }
            }
        }
        if (++step == kTcFlush) {
            flush();
            step = 0;
        }
        buf ^= 1;
    }
    tc_wait0();
    flush();
    __syncthreads();
    double *out = part + ((size_t)blockIdx.x * gridDim.y + blockIdx.y) * (size_t)BA * BB;
    for (int i = tid; i < BA * BB; i += nthr) out[i] = sm.acc[i];
}

struct TcPlan {
    int BA, BB, tilesA, tilesB, nchunks, threads;
    int64_t rows_per_chunk;
    size_t smem;
};

static size_t tc_smem(int BA, int BB) {
    return (size_t)2 * kTcKT * (BA + BB) * 4 + (size_t)3 * (BA + BB) * kTcKT * 2 +
           (size_t)BA * BB * 8;
}

static TcPlan plan_tc(int64_t n, int ka, int kb) {
    TcPlan p;
    auto ru = [](int x, int q) { return (x + q - 1) / q * q; };
    p.BA = std::min(ru(ka, kTcWarpM), 128);
    p.BB = std::min(ru(kb, kTcWarpN), 128);
    const size_t budget = max_smem_optin() - 1024;
    while (tc_smem(p.BA, p.BB) > budget && p.BB > kTcWarpN) p.BB -= kTcWarpN;
    while (tc_smem(p.BA, p.BB) > budget && p.BA > kTcWarpM) p.BA -= kTcWarpM;
    while ((p.BA / kTcWarpM) * (p.BB / kTcWarpN) * 32 > kTcMaxThreads && p.BB > kTcWarpN)
        p.BB -= kTcWarpN;
    p.tilesA = (ka + p.BA - 1) / p.BA;
    p.tilesB = (kb + p.BB - 1) / p.BB;
    p.threads = (p.BA / kTcWarpM) * (p.BB / kTcWarpN) * 32;
    const int tiles = p.tilesA * p.tilesB;
    int64_t nch = (sm_count() + tiles - 1) / tiles;
    int64_t maxch = std::max<int64_t>(1, (n + 4 * kTcKT - 1) / (4 * kTcKT));
    if (nch > maxch) nch = maxch;
    if (nch < 1) nch = 1;
    p.rows_per_chunk = (n + nch - 1) / nch;
    p.rows_per_chunk = (p.rows_per_chunk + kTcKT - 1) / kTcKT * kTcKT;
    if (p.rows_per_chunk < kTcKT) p.rows_per_chunk = kTcKT;
    p.nchunks = (int)((n + p.rows_per_chunk - 1) / p.rows_per_chunk);
    if (p.nchunks < 1) p.nchunks = 1;
    p.smem = tc_smem(p.BA, p.BB);
    return p;
}

size_t gram_tc_workspace_bytes(int64_t n, int ka, int kb) {
    TcPlan p = plan_tc(n, ka, kb);
    return (size_t)p.nchunks * p.tilesA * p.tilesB * p.BA * p.BB * sizeof(double);
}

// the fixed-order reduction kernel of k_gram.cu
int launch_gram_reduce(cudaStream_t st, const double *part, int nchunks, int ntiles, int BA,
                       int BB, int tilesB, int ka, int kb, int kb1, double *C1, int ldc1,
                       double *C2, int ldc2, int gap = 0);

int launch_gram_tc(cudaStream_t st, int64_t n, const float *L, int64_t ldl, int ka,
                   const float *R1, int64_t ldr1, int kb1, const float *R2, int64_t ldr2, int kb2,
                   double *C1, int ldc1, double *C2, int ldc2, double *ws, size_t ws_bytes) {
    const int kb = kb1 + kb2;
    if (ka <= 0 || kb <= 0 || n < 0 || !C1 || (kb2 > 0 && !C2)) return CACG_ERR_ARG;
    TcPlan p = plan_tc(n, ka, kb);
    const size_t need = (size_t)p.nchunks * p.tilesA * p.tilesB * p.BA * p.BB * sizeof(double);
    if (!ws || need > ws_bytes || p.threads > kTcMaxThreads) return CACG_ERR_ARG;
    const int vec16 = (ldl % 4 == 0) && (ldr1 % 4 == 0) && (kb2 == 0 || ldr2 % 4 == 0) &&
                      (ka % 4 == 0) && (kb1 % 4 == 0) && (kb2 % 4 == 0) && aligned16(L) &&
                      aligned16(R1) && (kb2 == 0 || aligned16(R2));
    if (n > 0) {
        set_smem_attr(gram_tc_kernel, (int)max_smem_optin());
        dim3 grid(p.nchunks, p.tilesA * p.tilesB);
        gram_tc_kernel<<<grid, p.threads, p.smem, st>>>(n, p.rows_per_chunk, L, ldl, ka, R1, ldr1,
                                                        kb1, R2, ldr2, kb2, p.BA, p.BB, p.tilesB,
                                                        vec16, ws);
        int rc = check_launch();
        if (rc != CACG_OK) return rc;
    } else {
        if (cudaMemsetAsync(ws, 0, need, st) != cudaSuccess) return CACG_ERR_CUDA;
    }
    return launch_gram_reduce(st, ws, n > 0 ? p.nchunks : 1, p.tilesA * p.tilesB, p.BA, p.BB,
                              p.tilesB, ka, kb, kb1, C1, ldc1, C2, ldc2);
}

}  // namespace cacg

// ---------------------------------------------------------------------------
// Gram from precomputed slice planes.  The producers of L and R (SpMM, Q
// update, X/R update, residual) write the three bf16 slices of every FP32
// value next to it, so this kernel only streams bf16 tiles (cp.async ring of
// STAGES K-steps, rows padded by 8 elements so ldmatrix rows hit distinct
// banks), reads fragments with ldmatrix.trans (the tiles are row-major in the
// K dimension, i.e. MN-major for both operands) and issues the six slice
// products per tile on the tensor cores.  Accumulation as in gram_tc_kernel.
// ---------------------------------------------------------------------------
namespace cacg {

__device__ __forceinline__ void ldsm_x4_t(unsigned (&r)[4], unsigned addr) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(addr));
}

template <int STAGES>
__device__ __forceinline__ void tcs_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(STAGES - 2));
}

template <int STAGES>
__global__ void __launch_bounds__(kTcMaxThreads)
    gram_tcs_kernel(int64_t n, int64_t rows_per_chunk, const __nv_bfloat16 *__restrict__ Lp,
                    int64_t lpl, int64_t ldl, int ka, const __nv_bfloat16 *__restrict__ R1p,
                    int64_t r1pl, int64_t ldr1, int kb1, const __nv_bfloat16 *__restrict__ R2p,
                    int64_t r2pl, int64_t ldr2, int kb2, int BA, int BB, int tilesB,
                    double *__restrict__ part) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int la = BA + 8, lb = BB + 8;  // padded row lengths (elements)
    const size_t stage_elems = (size_t)3 * kTcKT * (la + lb);
    __nv_bfloat16 *ring = reinterpret_cast<__nv_bfloat16 *>(smem_raw);
    double *acc = reinterpret_cast<double *>(smem_raw + STAGES * stage_elems * 2);
    const int tid = threadIdx.x, nthr = blockDim.x;
    const int tile_a = blockIdx.y / tilesB, tile_b = blockIdx.y % tilesB;
    const int a0 = tile_a * BA, b0 = tile_b * BB;
    const int warp = tid >> 5, lane = tid & 31;
    const int wn_count = BB / kTcWarpN;
    const int wm = warp / wn_count, wn = warp % wn_count;
    const bool wactive = wm < BA / kTcWarpM;
    const int64_t rbeg = (int64_t)blockIdx.x * rows_per_chunk;
    const int64_t rend = min(n, rbeg + rows_per_chunk);
    const int64_t nsteps = (rend - rbeg + kTcKT - 1) / kTcKT;

    for (int i = tid; i < BA * BB; i += nthr) acc[i] = 0.0;

    auto Ltile = [&](int st, int s) { return ring + st * stage_elems + (size_t)s * kTcKT * la; };
    auto Rtile = [&](int st, int s) {
        return ring + st * stage_elems + (size_t)3 * kTcKT * la + (size_t)s * kTcKT * lb;
    };

    auto load = [&](int st, int64_t r0) {
        const int ca = BA / 8, cb = BB / 8;
        const int per_plane = kTcKT * (ca + cb);
        for (int idx = tid; idx < 3 * per_plane; idx += nthr) {
            const int s = idx / per_plane, q = idx % per_plane;
            const int r = q / (ca + cb), c = q % (ca + cb);
            const int64_t row = r0 + r;
            if (c < ca) {
                __nv_bfloat16 *dst = Ltile(st, s) + r * la + c * 8;
                const int col = a0 + c * 8;
                if (row < rend && col < ka)
                    tc_cp_async16(dst, Lp + s * lpl + row * ldl + col);
                else
                    *reinterpret_cast<uint4 *>(dst) = make_uint4(0, 0, 0, 0);
            } else {
                const int cc = c - ca;
                __nv_bfloat16 *dst = Rtile(st, s) + r * lb + cc * 8;
                const int gb = b0 + cc * 8;
                if (row < rend && gb < kb1)
                    tc_cp_async16(dst, R1p + s * r1pl + row * ldr1 + gb);
                else if (row < rend && gb >= kb1 && gb - kb1 < kb2)
                    tc_cp_async16(dst, R2p + s * r2pl + row * ldr2 + (gb - kb1));
                else
                    *reinterpret_cast<uint4 *>(dst) = make_uint4(0, 0, 0, 0);
            }
        }
    };

    float c[2][2][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j)
#pragma unroll
            for (int q = 0; q < 4; ++q) c[i][j][q] = 0.f;

    auto flush = [&]() {
        if (!wactive) return;
        const int g = lane >> 2, t = lane & 3;
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const int ra = wm * kTcWarpM + i * 16 + g;
                const int cbb = wn * kTcWarpN + j * 8 + 2 * t;
                acc[ra * BB + cbb] += (double)c[i][j][0];
                acc[ra * BB + cbb + 1] += (double)c[i][j][1];
                acc[(ra + 8) * BB + cbb] += (double)c[i][j][2];
                acc[(ra + 8) * BB + cbb + 1] += (double)c[i][j][3];
#pragma unroll
                for (int q = 0; q < 4; ++q) c[i][j][q] = 0.f;
            }
    };

#pragma unroll
    for (int s = 0; s < STAGES - 1; ++s) {
        if (s < nsteps) load(s, rbeg + (int64_t)s * kTcKT);
        tc_commit();
    }
    int fl = 0;
    for (int64_t i = 0; i < nsteps; ++i) {
        tcs_wait<STAGES>();
        __syncthreads();
        const int64_t nxt = i + STAGES - 1;
        if (nxt < nsteps) load((int)(nxt % STAGES), rbeg + nxt * kTcKT);
        tc_commit();
        const int cur = (int)(i % STAGES);
        if (wactive) {
#pragma unroll
            for (int ks = 0; ks < kTcKT / 16; ++ks) {
                unsigned af[3][2][4], bf[3][4];
#pragma unroll
                for (int s = 0; s < 3; ++s) {
                    const __nv_bfloat16 *Lt = Ltile(cur, s), *Rt = Rtile(cur, s);
                    const int mi = lane >> 3;
#pragma unroll
                    for (int ii = 0; ii < 2; ++ii) {
                        const int r = ks * 16 + (mi >> 1) * 8 + (lane & 7);
                        const int a = wm * kTcWarpM + ii * 16 + (mi & 1) * 8;
                        ldsm_x4_t(af[s][ii], smem_u32(Lt + r * la + a));
                    }
                    const int r = ks * 16 + (mi & 1) * 8 + (lane & 7);
                    const int b = wn * kTcWarpN + (mi >> 1) * 8;
                    ldsm_x4_t(bf[s], smem_u32(Rt + r * lb + b));
                }
#pragma unroll
                for (int ii = 0; ii < 2; ++ii)
#pragma unroll
                    for (int j = 0; j < 2; ++j) {
                        mma_bf16(c[ii][j], af[2][ii], bf[0][2 * j], bf[0][2 * j + 1]);
                        mma_bf16(c[ii][j], af[1][ii], bf[1][2 * j], bf[1][2 * j + 1]);
                        mma_bf16(c[ii][j], af[0][ii], bf[2][2 * j], bf[2][2 * j + 1]);
                        mma_bf16(c[ii][j], af[1][ii], bf[0][2 * j], bf[0][2 * j + 1]);
                        mma_bf16(c[ii][j], af[0][ii], bf[1][2 * j], bf[1][2 * j + 1]);
                        mma_bf16(c[ii][j], af[0][ii], bf[0][2 * j], bf[0][2 * j + 1]);
                    }
            }
        }
        if (++fl == kTcFlush) {
            flush();
            fl = 0;
        }
    }
    tc_wait0();
    flush();
    __syncthreads();
    double *out = part + ((size_t)blockIdx.x * gridDim.y + blockIdx.y) * (size_t)BA * BB;
    for (int i = tid; i < BA * BB; i += nthr) out[i] = acc[i];
}

struct TcsPlan {
    int BA, BB, tilesA, tilesB, nchunks, threads, stages;
    int64_t rows_per_chunk;
    size_t smem;
};

static size_t tcs_smem(int BA, int BB, int stages) {
    return (size_t)stages * 3 * kTcKT * ((BA + 8) + (BB + 8)) * 2 + (size_t)BA * BB * 8;
}

static TcsPlan plan_tcs(int64_t n, int ka, int kb) {
    TcsPlan p;
    auto ru = [](int x, int q) { return (x + q - 1) / q * q; };
    p.BA = std::min(ru(ka, kTcWarpM), 128);
    p.BB = std::min(ru(kb, kTcWarpN), 128);
    const size_t budget = max_smem_optin() - 1024;
    while ((p.BA / kTcWarpM) * (p.BB / kTcWarpN) * 32 > kTcMaxThreads && p.BB > kTcWarpN)
        p.BB -= kTcWarpN;
    p.stages = 3;
    if (tcs_smem(p.BA, p.BB, 3) > budget) p.stages = 2;
    while (tcs_smem(p.BA, p.BB, p.stages) > budget && p.BB > kTcWarpN) p.BB -= kTcWarpN;
    p.tilesA = (ka + p.BA - 1) / p.BA;
    p.tilesB = (kb + p.BB - 1) / p.BB;
    p.threads = (p.BA / kTcWarpM) * (p.BB / kTcWarpN) * 32;
    const int tiles = p.tilesA * p.tilesB;
    int64_t nch = (sm_count() + tiles - 1) / tiles;
    int64_t maxch = std::max<int64_t>(1, (n + 4 * kTcKT - 1) / (4 * kTcKT));
    if (nch > maxch) nch = maxch;
    if (nch < 1) nch = 1;
    p.rows_per_chunk = (n + nch - 1) / nch;
    p.rows_per_chunk = (p.rows_per_chunk + kTcKT - 1) / kTcKT * kTcKT;
    if (p.rows_per_chunk < kTcKT) p.rows_per_chunk = kTcKT;
    p.nchunks = (int)((n + p.rows_per_chunk - 1) / p.rows_per_chunk);
    if (p.nchunks < 1) p.nchunks = 1;
    p.smem = tcs_smem(p.BA, p.BB, p.stages);
    return p;
}

size_t gram_tcs_workspace_bytes(int64_t n, int ka, int kb) {
    TcsPlan p = plan_tcs(n, ka, kb);
    return (size_t)p.nchunks * p.tilesA * p.tilesB * p.BA * p.BB * sizeof(double);
}

bool gram_tcs_supported(int ka, int kb1, int kb2, int64_t ldl, int64_t ldr1, int64_t ldr2) {
    return ka % 8 == 0 && kb1 % 8 == 0 && kb2 % 8 == 0 && ldl % 8 == 0 && ldr1 % 8 == 0 &&
           (kb2 == 0 || ldr2 % 8 == 0);
}

int launch_gram_tcs(cudaStream_t st, int64_t n, Slices L, int64_t ldl, int ka, Slices R1,
                    int64_t ldr1, int kb1, Slices R2, int64_t ldr2, int kb2, double *C1,
                    int ldc1, double *C2, int ldc2, double *ws, size_t ws_bytes) {
    const int kb = kb1 + kb2;
    if (ka <= 0 || kb <= 0 || n < 0 || !C1 || (kb2 > 0 && !C2) || !L.p || !R1.p ||
        (kb2 > 0 && !R2.p))
        return CACG_ERR_ARG;
    if (!gram_tcs_supported(ka, kb1, kb2, ldl, ldr1, ldr2) || L.plane % 8 || R1.plane % 8 ||
        (kb2 > 0 && R2.plane % 8) || !aligned16(L.p) || !aligned16(R1.p) ||
        (kb2 > 0 && !aligned16(R2.p)))
        return CACG_ERR_ARG;
    TcsPlan p = plan_tcs(n, ka, kb);
    const size_t need = (size_t)p.nchunks * p.tilesA * p.tilesB * p.BA * p.BB * sizeof(double);
    if (!ws || need > ws_bytes || p.threads > kTcMaxThreads) return CACG_ERR_ARG;
    if (n > 0) {
        set_smem_attr(gram_tcs_kernel<2>, (int)max_smem_optin());
        set_smem_attr(gram_tcs_kernel<3>, (int)max_smem_optin());
        dim3 grid(p.nchunks, p.tilesA * p.tilesB);
        if (p.stages == 3)
            gram_tcs_kernel<3><<<grid, p.threads, p.smem, st>>>(
                n, p.rows_per_chunk, L.p, L.plane, ldl, ka, R1.p, R1.plane, ldr1, kb1, R2.p,
                R2.plane, ldr2, kb2, p.BA, p.BB, p.tilesB, ws);
        else
            gram_tcs_kernel<2><<<grid, p.threads, p.smem, st>>>(
                n, p.rows_per_chunk, L.p, L.plane, ldl, ka, R1.p, R1.plane, ldr1, kb1, R2.p,
                R2.plane, ldr2, kb2, p.BA, p.BB, p.tilesB, ws);
        int rc = check_launch();
        if (rc != CACG_OK) return rc;
    } else {
        if (cudaMemsetAsync(ws, 0, need, st) != cudaSuccess) return CACG_ERR_CUDA;
    }
    return launch_gram_reduce(st, ws, n > 0 ? p.nchunks : 1, p.tilesA * p.tilesB, p.BA, p.BB,
                              p.tilesB, ka, kb, kb1, C1, ldc1, C2, ldc2);
}

}  // namespace cacg

namespace cacg {

// slice planes of an FP32 block (n x w, row stride ld, planes n*ld apart)
__global__ void split_planes_kernel(int64_t n, int w, const float *__restrict__ X, int64_t ld,
                                    Slices out) {
    const int64_t tot = n * w;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < tot;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = q / w;
        const int c = (int)(q % w);
        store_slices1(out, i * ld + c, X[i * ld + c]);
    }
}

int launch_split_planes(cudaStream_t st, int64_t n, int w, const float *X, int64_t ld,
                        Slices out) {
    if (n <= 0 || w <= 0) return CACG_OK;
    int64_t blocks = (n * w + 255) / 256;
    int64_t cap = (int64_t)sm_count() * 8;
    split_planes_kernel<<<(unsigned)(blocks < cap ? blocks : cap), 256, 0, st>>>(n, w, X, ld, out);
    return check_launch();
}

}  // namespace cacg
