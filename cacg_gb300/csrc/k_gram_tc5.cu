// k_gram_tc5.cu -- Gram products of FP32 blocks on the 5th-generation
// tensor cores (tcgen05, sm_103a), accumulators in tensor memory.
//
// Reference operations replaced (sclc/cacg): distributedMatLTransposeMatRMul
// (src/BLAS3.c:699-726) and distributedMatLTransposeMatRMul_updated
// (src/BLAS3.c:730-758), mixed-precision mode (L, R in FP32).
//
// C = L^T [R1 | R2] with L n x ka, R n x kb.  Each FP32 value is split exactly
// into three bf16 slices (x = x1 + x2 + x3) and the six slice products of
// order <= 2^-16 are accumulated by tcgen05.mma (kind::f16, bf16 inputs, FP32
// accumulator in TMEM).  The FP32 accumulator covers 8 K-steps (256 rows);
// then every warp reads its part of the tile from TMEM (tcgen05.ld) and adds it
// to FP64 registers.  Per-CTA FP64 partials go to the split-K workspace and
// the fixed-order reduction of k_gram.cu finishes the sum.
//
// Work split per CTA (256 threads, one row chunk of the split-K, one output
// tile of at most 128 x 256):
//   * every thread owns fixed (row pair, 4 columns) units of the K-step's FP32
//     tile: it loads them into registers one step ahead and converts them into
//     the three slice tiles, stored in the K-major 8 x 16-byte core-matrix
//     layout the UMMA shared-memory descriptors describe (no swizzle,
//     LBO = 128 B between K-adjacent core matrices, SBO = 512 B between
//     8-row groups);
//   * one barrier per K-step publishes the slices (after a proxy fence);
//     thread 0 issues the 12 MMAs (6 products x 2 halves of K = 32) and
//     commits them to the step's mbarrier, which guards reuse of that slice
//     buffer two steps later;
//   * all mbarrier waits are bounded: on expiry the kernel records
//     kStatusTimeout in *status, all threads leave the K loop together at
//     the next barrier, the issuer waits (bounded) for its last committed
//     MMAs, TMEM is freed and the CTA returns without writing its partial.
#include <cuda_bf16.h>

#include <algorithm>

#include "cacg_internal.cuh"

namespace cacg {

constexpr int kT5KT = 32;        // rows (K) per step: two K = 16 UMMAs per product
constexpr int kT5M = 128;        // UMMA M (output rows = columns of L, zero-padded)
constexpr int kT5Threads = 256;  // 8 warps
constexpr int kT5Flush = 8;      // K-steps per FP32 accumulation group
constexpr int kT5MaxUnits = 4;   // (row pair, 4 columns) units per thread per step
constexpr int kT5MaxN = 128;     // output tile columns (UMMA N)
constexpr long long kT5SpinLimit = 1ll << 22;  // bounded mbarrier polls

__device__ __forceinline__ unsigned t5_smem_u32(const void *p) {
    return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ int t5_core_off(int row, int k) {
    return ((row >> 3) * (kT5KT / 8) + (k >> 3)) * 64 + (row & 7) * 8 + (k & 7);
}

// UMMA shared-memory descriptor: start address, LBO, SBO (bytes >> 4),
// version bits 46-47 = 1, no swizzle.
__device__ __forceinline__ uint64_t t5_desc(unsigned saddr) {
    const uint64_t lbo = 128, sbo = (kT5KT / 8) * 128;
    return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

__device__ __forceinline__ void t5_mma(unsigned tmem_d, uint64_t adesc, uint64_t bdesc,
                                       unsigned idesc, unsigned accumulate) {
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "setp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
        "}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void t5_commit(uint64_t *bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
            t5_smem_u32(bar)));
}

__device__ __forceinline__ void t5_mbar_init(uint64_t *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(t5_smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ bool t5_mbar_try(uint64_t *bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(ok)
        : "r"(t5_smem_u32(bar)), "r"(parity));
    return ok != 0;
}

// bounded wait; false on expiry
__device__ __forceinline__ bool t5_mbar_wait(uint64_t *bar, unsigned parity) {
    for (long long i = 0; i < kT5SpinLimit; ++i)
        if (t5_mbar_try(bar, parity)) return true;
    return false;
}

__device__ __forceinline__ void t5_ld8(unsigned taddr, float (&v)[8]) {
    unsigned r[8];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int q = 0; q < 8; ++q) v[q] = __uint_as_float(r[q]);
}

__global__ void __launch_bounds__(kT5Threads, 1)
    gram_tc5_kernel(int64_t n, int64_t rows_per_chunk, const float *__restrict__ L, int64_t ldl,
                    int ka, const float *__restrict__ R1, int64_t ldr1, int kb1,
                    const float *__restrict__ R2, int64_t ldr2, int kb2, int BA, int BB,
                    int tilesB, int vec16, int tmem_cols, double *__restrict__ part,
                    int *__restrict__ status) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    // [slices buf 0][slices buf 1][FP64 acc BA x (BB+1)][mbar x2][tmem slot][abort]
    const size_t a_bytes = (size_t)kT5M * kT5KT * 2, b_bytes = (size_t)BB * kT5KT * 2;
    const size_t buf_bytes = 3 * (a_bytes + b_bytes);
    const int lda = BB + 1;  // padded FP64 accumulator row (bank spread)
    double *acc = reinterpret_cast<double *>(smem_raw + 2 * buf_bytes);
    uint64_t *mbar = reinterpret_cast<uint64_t *>(acc + (size_t)BA * lda);
    unsigned *tmem_slot = reinterpret_cast<unsigned *>(mbar + 2);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
    auto sliceA = [&](int buf, int s) {
        return reinterpret_cast<__nv_bfloat16 *>(smem_raw + buf * buf_bytes + s * a_bytes);
    };
    auto sliceB = [&](int buf, int s) {
        return reinterpret_cast<__nv_bfloat16 *>(smem_raw + buf * buf_bytes + 3 * a_bytes +
                                                 s * b_bytes);
    };

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int tile_a = blockIdx.y / tilesB, tile_b = blockIdx.y % tilesB;
    const int a0 = tile_a * BA, b0 = tile_b * BB;
    const int64_t rbeg = (int64_t)blockIdx.x * rows_per_chunk;
    const int64_t rend = min(n, rbeg + rows_per_chunk);
    const int64_t nsteps = (rend - rbeg + kT5KT - 1) / kT5KT;

    // zero both slice buffers once (rows beyond BA / BB stay zero) and the acc
    for (size_t i = tid; i < 2 * buf_bytes / 16; i += kT5Threads)
        reinterpret_cast<uint4 *>(smem_raw)[i] = make_uint4(0, 0, 0, 0);
    for (int i = tid; i < BA * lda; i += kT5Threads) acc[i] = 0.0;
    if (tid == 0) {
        t5_mbar_init(&mbar[0], 1);
        t5_mbar_init(&mbar[1], 1);
        *abort_flag = 0;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                         t5_smem_u32(tmem_slot)),
                     "r"(tmem_cols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const unsigned tmem = *tmem_slot;

    // ---- work units: (row pair p in [0, KT/2), column group g of 4 columns)
    const int ga = BA / 4, gb = BB / 4, groups = ga + gb;
    const int units = (kT5KT / 2) * groups;

    float4 rx[kT5MaxUnits][2];  // prefetched rows of the next step
    auto fetch = [&](int64_t r0) {
#pragma unroll
        for (int u = 0; u < kT5MaxUnits; ++u) {
            const int id = tid + u * kT5Threads;
            rx[u][0] = rx[u][1] = make_float4(0.f, 0.f, 0.f, 0.f);
            if (id >= units) continue;
            const int p = id / groups, g = id % groups;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int64_t row = r0 + 2 * p + h;
                if (row >= rend) continue;
                float v[4] = {0.f, 0.f, 0.f, 0.f};
                if (g < ga) {
                    const int col = a0 + 4 * g;
                    const float *src = L + row * ldl + col;
                    if (vec16 && col + 3 < ka) {
                        float4 t = __ldg(reinterpret_cast<const float4 *>(src));
                        v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
                    } else {
#pragma unroll
                        for (int q = 0; q < 4; ++q)
                            if (col + q < ka) v[q] = __ldg(src + q);
                    }
                } else {
                    const int cb = b0 + 4 * (g - ga);
                    if (vec16 && cb + 3 < kb1) {
                        float4 t = __ldg(reinterpret_cast<const float4 *>(R1 + row * ldr1 + cb));
                        v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
                    } else if (vec16 && cb >= kb1 && cb - kb1 + 3 < kb2) {
                        float4 t = __ldg(
                            reinterpret_cast<const float4 *>(R2 + row * ldr2 + (cb - kb1)));
                        v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
                    } else {
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            const int c = cb + q;
                            if (c < kb1)
                                v[q] = __ldg(R1 + row * ldr1 + c);
                            else if (c - kb1 < kb2)
                                v[q] = __ldg(R2 + row * ldr2 + (c - kb1));
                        }
                    }
                }
                rx[u][h] = make_float4(v[0], v[1], v[2], v[3]);
            }
        }
    };
    auto convert = [&](int buf) {
#pragma unroll
        for (int u = 0; u < kT5MaxUnits; ++u) {
            const int id = tid + u * kT5Threads;
            if (id >= units) continue;
            const int p = id / groups, g = id % groups;
            const bool isA = g < ga;
            const int col0 = isA ? 4 * g : 4 * (g - ga);
            const float x0[4] = {rx[u][0].x, rx[u][0].y, rx[u][0].z, rx[u][0].w};
            const float x1[4] = {rx[u][1].x, rx[u][1].y, rx[u][1].z, rx[u][1].w};
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                float2 x = make_float2(x0[q], x1[q]);
                __nv_bfloat162 h = __float22bfloat162_rn(x);
                float2 hf = __bfloat1622float2(h);
                float2 r1 = make_float2(x.x - hf.x, x.y - hf.y);
                __nv_bfloat162 m = __float22bfloat162_rn(r1);
                float2 mf = __bfloat1622float2(m);
                __nv_bfloat162 l = __float22bfloat162_rn(make_float2(r1.x - mf.x, r1.y - mf.y));
                const int off = t5_core_off(col0 + q, 2 * p);
                __nv_bfloat16 *d0 = isA ? sliceA(buf, 0) : sliceB(buf, 0);
                __nv_bfloat16 *d1 = isA ? sliceA(buf, 1) : sliceB(buf, 1);
                __nv_bfloat16 *d2 = isA ? sliceA(buf, 2) : sliceB(buf, 2);
                *reinterpret_cast<__nv_bfloat162 *>(d0 + off) = h;
                *reinterpret_cast<__nv_bfloat162 *>(d1 + off) = m;
                *reinterpret_cast<__nv_bfloat162 *>(d2 + off) = l;
            }
        }
    };

    // TMEM -> FP64: warp w reads lanes 32*(w%4).. (tile rows) of column half w/4
    const int quad = warp & 3, half = warp >> 2;
    const int hcols = BB / 2;  // multiple of 8
    const int row_t = 32 * quad + lane;
    auto flush = [&]() {
        for (int c8 = 0; c8 < hcols; c8 += 8) {
            float v[8];
            t5_ld8(tmem + ((unsigned)(32 * quad) << 16) + (unsigned)(half * hcols + c8), v);
            if (row_t < BA) {
                double *arow = acc + (size_t)row_t * lda + half * hcols + c8;
#pragma unroll
                for (int q = 0; q < 8; ++q) arow[q] += (double)v[q];
            }
        }
    };

    const unsigned idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(BB >> 3) << 17) |
                           ((unsigned)(kT5M >> 4) << 24);

    if (nsteps > 0) {
        fetch(rbeg);
        convert(0);
        if (nsteps > 1) fetch(rbeg + kT5KT);
    }
    unsigned accumulate = 0;
    int in_group = 0;
    int64_t last_committed = -1;
    for (int64_t i = 0; i < nsteps; ++i) {
        const int buf = (int)(i & 1);
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        if (*abort_flag) break;  // uniform: read after the barrier
        if (tid == 0) {
            const unsigned abase = t5_smem_u32(sliceA(buf, 0)), bbase = t5_smem_u32(sliceB(buf, 0));
            // products, small terms first: (3,1) (2,2) (1,3) (2,1) (1,2) (1,1)
            const int pa[6] = {2, 1, 0, 1, 0, 0}, pb[6] = {0, 1, 2, 0, 1, 0};
#pragma unroll
            for (int pr = 0; pr < 6; ++pr) {
#pragma unroll
                for (int kk = 0; kk < kT5KT / 16; ++kk) {
                    const uint64_t ad = t5_desc(abase + pa[pr] * (unsigned)a_bytes + kk * 256);
                    const uint64_t bd = t5_desc(bbase + pb[pr] * (unsigned)b_bytes + kk * 256);
                    t5_mma(tmem, ad, bd, idesc, accumulate);
                    accumulate = 1;
                }
            }
            t5_commit(&mbar[buf]);
        }
        last_committed = i;
        ++in_group;
        bool good = true;
        // next step: its slice buffer was read by the MMAs of step i-1
        if (i + 1 < nsteps) {
            if (i >= 1 && !t5_mbar_wait(&mbar[buf ^ 1], (unsigned)(((i - 1) >> 1) & 1))) {
                atomicOr(status, kStatusTimeout);
                *abort_flag = 1;
                good = false;
            }
            if (good) {
                convert(buf ^ 1);
                if (i + 2 < nsteps) fetch(rbeg + (i + 2) * kT5KT);
            }
        }
        if (in_group == kT5Flush || i + 1 == nsteps) {
            // all MMAs of the group done -> add the FP32 accumulator into FP64
            if (good && !t5_mbar_wait(&mbar[buf], (unsigned)((i >> 1) & 1))) {
                atomicOr(status, kStatusTimeout);
                *abort_flag = 1;
                good = false;
            }
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            if (good && !*abort_flag) flush();
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
            __syncthreads();  // TMEM reads done before the next group overwrites it
            accumulate = 0;
            in_group = 0;
        }
    }
    // drain: MMAs committed last must be complete before TMEM is freed
    if (tid == 0 && last_committed >= 0)
        t5_mbar_wait(&mbar[last_committed & 1], (unsigned)((last_committed >> 1) & 1));
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem),
                     "r"(tmem_cols));
    }
    if (*abort_flag) return;
    double *out = part + ((size_t)blockIdx.x * gridDim.y + blockIdx.y) * (size_t)BA * BB;
    for (int i = tid; i < BA * BB; i += kT5Threads) out[i] = acc[(size_t)(i / BB) * lda + i % BB];
}

struct T5Plan {
    int BA, BB, tilesA, tilesB, nchunks, tmem_cols;
    int64_t rows_per_chunk;
    size_t smem;
};

static T5Plan plan_tc5(int64_t n, int ka, int kb) {
    T5Plan p;
    auto ru = [](int x, int q) { return (x + q - 1) / q * q; };
    p.BA = std::min(ru(ka, 4), kT5M);
    p.BB = std::min(ru(kb, 16), kT5MaxN);
    p.tilesA = (ka + p.BA - 1) / p.BA;
    p.tilesB = (kb + p.BB - 1) / p.BB;
    p.tmem_cols = 32;
    while (p.tmem_cols < p.BB) p.tmem_cols *= 2;
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
    p.smem = 2 * buf + (size_t)p.BA * (p.BB + 1) * 8 + 64;
    return p;
}

size_t gram_tc5_workspace_bytes(int64_t n, int ka, int kb) {
    T5Plan p = plan_tc5(n, ka, kb);
    return (size_t)p.nchunks * p.tilesA * p.tilesB * p.BA * p.BB * sizeof(double);
}

bool gram_tc5_supported(int ka, int kb) {
    (void)ka;
    // units per thread per step: (KT/2) * (BA + BB)/4 <= 256 * kT5MaxUnits
    const int BA = std::min((ka + 3) / 4 * 4, kT5M);
    const int BB = std::min((kb + 15) / 16 * 16, kT5MaxN);
    return (kT5KT / 2) * ((BA + BB) / 4) <= kT5Threads * kT5MaxUnits;
}

int launch_gram_reduce(cudaStream_t st, const double *part, int nchunks, int ntiles, int BA,
                       int BB, int tilesB, int ka, int kb, int kb1, double *C1, int ldc1,
                       double *C2, int ldc2);

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
    const int vec16 = (ldl % 4 == 0) && (ldr1 % 4 == 0) && (kb2 == 0 || ldr2 % 4 == 0) &&
                      (kb1 % 4 == 0) && aligned16(L) && aligned16(R1) &&
                      (kb2 == 0 || aligned16(R2));
    if (n > 0) {
        static const bool attr = [] {
            cudaFuncSetAttribute(gram_tc5_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)max_smem_optin());
            return true;
        }();
        (void)attr;
        dim3 grid(p.nchunks, p.tilesA * p.tilesB);
        gram_tc5_kernel<<<grid, kT5Threads, p.smem, st>>>(n, p.rows_per_chunk, L, ldl, ka, R1,
                                                          ldr1, kb1, R2, ldr2, kb2, p.BA, p.BB,
                                                          p.tilesB, vec16, p.tmem_cols, ws,
                                                          status);
        int rc = check_launch();
        if (rc != CACG_OK) return rc;
    } else {
        if (cudaMemsetAsync(ws, 0, need, st) != cudaSuccess) return CACG_ERR_CUDA;
    }
    return launch_gram_reduce(st, ws, n > 0 ? p.nchunks : 1, p.tilesA * p.tilesB, p.BA, p.BB,
                              p.tilesB, ka, kb, kb1, C1, ldc1, C2, ldc2);
}

}  // namespace cacg
