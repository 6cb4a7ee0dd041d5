// k_gram.cu -- tall-skinny Gram products C = L^T [R1 | R2] with split-K.
//
// Reference operations replaced (sclc/cacg):
//   distributedMatLTransposeMatRMul          src/BLAS3.c:699-726  Q^T AQ
//   distributedMatLTransposeMatRMul_updated  src/BLAS3.c:730-758  (AQ)^T S, Q^T R
// and the MPI_Allreduce(SUM) that follows each (src/BLAS3.c:721-722, 753-754):
// on one GPU the cross-rank sum becomes the split-K reduction below.
//
// The K dimension is the row count n (millions), the output is k x (k+m)
// (k = s*m <= 256).  Grid: blockIdx.x = split-K chunk of rows, blockIdx.y =
// output tile (<= 128 x 128).  Each CTA stages KT-row slabs of L and R in
// shared memory (cp.async, double-buffered) and every thread accumulates a
// 4 x 4 micro-tile; partial tiles go to a workspace and a second kernel sums
// them in a fixed chunk order, so the result is deterministic and depends only
// on the problem's own shape (never on other work sharing the GPU).
//
// Accumulation:
//   FP64 inputs  -- FP64 FMA (variant FMA) or FP64 tensor core mma.sync
//                   m8n8k4 (variant DMMA);
//   FP32 inputs  -- error-free products (p = a*b, e = fma(a,b,-p)) summed in
//                   float-float with TwoSum, converted to FP64 per CTA chunk:
//                   an FP64-accurate Gram of the FP32 basis without using the
//                   FP64 pipe in the inner loop.
#include <algorithm>

#include "cacg_internal.cuh"

namespace cacg {

constexpr int kMA = 4, kMB = 4;  // micro-tile per thread
constexpr int kMaxTile = 128;    // output tile edge

template <typename T> struct GramKT;
template <> struct GramKT<double> { static constexpr int value = 16; };
template <> struct GramKT<float> { static constexpr int value = 32; };

struct FF {  // float-float accumulator
    float s, c;
};

__device__ __forceinline__ void acc_init(double &a) { a = 0.0; }
__device__ __forceinline__ void acc_init(FF &a) { a.s = 0.f; a.c = 0.f; }
__device__ __forceinline__ void acc_mac(double &acc, double l, double r) { acc = fma(l, r, acc); }
__device__ __forceinline__ void acc_mac(FF &acc, float l, float r) {
    float p = l * r;
    float e = fmaf(l, r, -p);  // l*r == p + e exactly
    float t = acc.s + p;       // TwoSum(acc.s, p)
    float bp = t - acc.s;
    float err = (acc.s - (t - bp)) + (p - bp);
    acc.s = t;
    acc.c += err + e;
}
__device__ __forceinline__ double acc_val(double a) { return a; }
__device__ __forceinline__ double acc_val(FF a) { return (double)a.s + (double)a.c; }

template <typename T> struct AccOf;
template <> struct AccOf<double> { using type = double; };
template <> struct AccOf<float> { using type = FF; };

__device__ __forceinline__ void cp_async4(void *smem, const void *g) {
    unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(g));
}
__device__ __forceinline__ void cp_async8(void *smem, const void *g) {
    unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(g));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::); }
__device__ __forceinline__ void cp_async_wait_1() { asm volatile("cp.async.wait_group 1;\n" ::); }

template <typename T>
__device__ __forceinline__ void cp_elem(T *smem, const T *g) {
    if constexpr (sizeof(T) == 8)
        cp_async8(smem, g);
    else
        cp_async4(smem, g);
}

// Stage rows [r0, r0+KT) of the L tile (cols a0..a0+BA) and R tile into smem.
template <typename T, int KT>
__device__ __forceinline__ void stage_slab(T *Ls, T *Rs, int BA, int BB, int64_t r0,
                                           int64_t rend, const T *L, int64_t ldl, int ka,
                                           int a0, const T *R1, int64_t ldr1, int kb1,
                                           const T *R2, int64_t ldr2, int kb2, int b0) {
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int idx = tid; idx < KT * BA; idx += nt) {
        int r = idx / BA, a = idx % BA;
        int64_t row = r0 + r;
        T *dst = Ls + r * BA + a;
        if (row < rend && a0 + a < ka)
            cp_elem(dst, L + row * ldl + a0 + a);
        else
            *dst = T(0);
    }
    for (int idx = tid; idx < KT * BB; idx += nt) {
        int r = idx / BB, b = idx % BB;
        int64_t row = r0 + r;
        int gb = b0 + b;
        T *dst = Rs + r * BB + b;
        if (row < rend && gb < kb1)
            cp_elem(dst, R1 + row * ldr1 + gb);
        else if (row < rend && gb - kb1 < kb2)
            cp_elem(dst, R2 + row * ldr2 + (gb - kb1));
        else
            *dst = T(0);
    }
}

constexpr int kGramMaxThreads = 768;

template <typename T>
__global__ void __launch_bounds__(kGramMaxThreads)
    gram_fma_kernel(int64_t n, int64_t rows_per_chunk, const T *__restrict__ L, int64_t ldl,
                    int ka, const T *__restrict__ R1, int64_t ldr1, int kb1,
                    const T *__restrict__ R2, int64_t ldr2, int kb2, int BA, int BB,
                    int tilesB, double *__restrict__ part, int sym) {
    constexpr int KT = GramKT<T>::value;
    using A = typename AccOf<T>::type;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *Ls0 = reinterpret_cast<T *>(smem_raw);
    T *Rs0 = Ls0 + KT * BA;
    T *Ls1 = Rs0 + KT * BB;
    T *Rs1 = Ls1 + KT * BA;

    const int tile_a = blockIdx.y / tilesB, tile_b = blockIdx.y % tilesB;
    const int a0 = tile_a * BA, b0 = tile_b * BB;
    const int kb = kb1 + kb2;
    const int nb = BB / kMB, na = BA / kMA;
    int ta, tb;
    bool active;
    if (!sym) {
        ta = threadIdx.x / nb;
        tb = threadIdx.x % nb;
        active = ta < na;
    } else {
        // symmetric leading block (one tile, L^T R1 with R1 = A L): the
        // threads take its upper-triangular micro-tiles (tb >= ta), then the
        // micro-tiles of the columns past it; the reduction mirrors the rest
        const int ntri = na * (na + 1) / 2, nrest = na * (nb - na);
        int t = threadIdx.x;
        ta = 0;
        tb = 0;
        active = true;
        if (t < ntri) {
            while (t >= na - ta) {
                t -= na - ta;
                ++ta;
            }
            tb = ta + t;
        } else if (t - ntri < nrest) {
            t -= ntri;
            ta = t / (nb - na);
            tb = na + t % (nb - na);
        } else {
            active = false;
        }
    }

    const int64_t rbeg = (int64_t)blockIdx.x * rows_per_chunk;
    const int64_t rend = min(n, rbeg + rows_per_chunk);

    A acc[kMA][kMB];
#pragma unroll
    for (int i = 0; i < kMA; ++i)
#pragma unroll
        for (int j = 0; j < kMB; ++j) acc_init(acc[i][j]);

    int64_t r0 = rbeg;
    if (r0 < rend) {
        stage_slab<T, KT>(Ls0, Rs0, BA, BB, r0, rend, L, ldl, ka, a0, R1, ldr1, kb1, R2, ldr2,
                          kb2, b0);
    }
    cp_async_commit();
    int buf = 0;
    for (; r0 < rend; r0 += KT) {
        T *Ls = buf ? Ls1 : Ls0;
        T *Rs = buf ? Rs1 : Rs0;
        if (r0 + KT < rend) {
            stage_slab<T, KT>(buf ? Ls0 : Ls1, buf ? Rs0 : Rs1, BA, BB, r0 + KT, rend, L, ldl,
                              ka, a0, R1, ldr1, kb1, R2, ldr2, kb2, b0);
        }
        cp_async_commit();
        cp_async_wait_1();
        __syncthreads();
        if (active) {
#pragma unroll 4
            for (int r = 0; r < KT; ++r) {
                T lv[kMA], rv[kMB];
#pragma unroll
                for (int i = 0; i < kMA; ++i) lv[i] = Ls[r * BA + ta * kMA + i];
#pragma unroll
                for (int j = 0; j < kMB; ++j) rv[j] = Rs[r * BB + tb * kMB + j];
#pragma unroll
                for (int i = 0; i < kMA; ++i)
#pragma unroll
                    for (int j = 0; j < kMB; ++j) acc_mac(acc[i][j], lv[i], rv[j]);
            }
        }
        __syncthreads();
        buf ^= 1;
    }
    cp_async_wait_all();
    if (active) {
        double *out = part + ((size_t)blockIdx.x * gridDim.y + blockIdx.y) * (size_t)BA * BB;
#pragma unroll
        for (int i = 0; i < kMA; ++i)
#pragma unroll
            for (int j = 0; j < kMB; ++j)
                out[(ta * kMA + i) * BB + tb * kMB + j] = acc_val(acc[i][j]);
    }
    (void)kb;
}

// ------------------------------------------------------------ DMMA variant
// FP64 tensor core: mma.sync.aligned.m8n8k4.row.col.f64.  A = L^T (8 x 4 per
// step), B = R (4 x 8).  Each warp owns a list of 8x8 output tiles.
constexpr int kDmmaMaxTilesPerWarp = 16;

__global__ void __launch_bounds__(512)
    gram_dmma_kernel(int64_t n, int64_t rows_per_chunk, const double *__restrict__ L,
                     int64_t ldl, int ka, const double *__restrict__ R1, int64_t ldr1, int kb1,
                     const double *__restrict__ R2, int64_t ldr2, int kb2, int BA, int BB,
                     int tilesB, double *__restrict__ part) {
    constexpr int KT = 16;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    // padded strides (BA + 4, BB + 4 with BA, BB multiples of 8) keep the
    // 4-row x 8-column fragment reads free of bank conflicts
    const int sa = BA + 4, sb = BB + 4;
    double *Ls0 = reinterpret_cast<double *>(smem_raw);
    double *Rs0 = Ls0 + KT * sa;
    double *Ls1 = Rs0 + KT * sb;
    double *Rs1 = Ls1 + KT * sa;

    const int tile_a = blockIdx.y / tilesB, tile_b = blockIdx.y % tilesB;
    const int a0 = tile_a * BA, b0 = tile_b * BB;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nwarps = blockDim.x >> 5;
    const int ta8 = BA / 8, tb8 = BB / 8, ntiles = ta8 * tb8;
    const int g = lane >> 2, t4 = lane & 3;

    const int64_t rbeg = (int64_t)blockIdx.x * rows_per_chunk;
    const int64_t rend = min(n, rbeg + rows_per_chunk);

    double c[kDmmaMaxTilesPerWarp][2];
#pragma unroll
    for (int t = 0; t < kDmmaMaxTilesPerWarp; ++t) c[t][0] = c[t][1] = 0.0;

    auto stage = [&](double *Ls, double *Rs, int64_t r0) {
        for (int idx = threadIdx.x; idx < KT * BA; idx += blockDim.x) {
            int r = idx / BA, a = idx % BA;
            int64_t row = r0 + r;
            double *dst = Ls + r * sa + a;
            if (row < rend && a0 + a < ka)
                cp_async8(dst, L + row * ldl + a0 + a);
            else
                *dst = 0.0;
        }
        for (int idx = threadIdx.x; idx < KT * BB; idx += blockDim.x) {
            int r = idx / BB, b = idx % BB;
            int64_t row = r0 + r;
            int gb = b0 + b;
            double *dst = Rs + r * sb + b;
            if (row < rend && gb < kb1)
                cp_async8(dst, R1 + row * ldr1 + gb);
            else if (row < rend && gb - kb1 < kb2)
                cp_async8(dst, R2 + row * ldr2 + (gb - kb1));
            else
                *dst = 0.0;
        }
    };

    int64_t r0 = rbeg;
    if (r0 < rend) stage(Ls0, Rs0, r0);
    cp_async_commit();
    int buf = 0;
    for (; r0 < rend; r0 += KT) {
        double *Ls = buf ? Ls1 : Ls0;
        double *Rs = buf ? Rs1 : Rs0;
        if (r0 + KT < rend) stage(buf ? Ls0 : Ls1, buf ? Rs0 : Rs1, r0 + KT);
        cp_async_commit();
        cp_async_wait_1();
        __syncthreads();
#pragma unroll
        for (int ks = 0; ks < KT; ks += 4) {
#pragma unroll
            for (int t = 0; t < kDmmaMaxTilesPerWarp; ++t) {
                int tile = warp + t * nwarps;
                if (tile < ntiles) {
                    int ia = tile / tb8, ib = tile % tb8;
                    double av = Ls[(ks + t4) * sa + ia * 8 + g];
                    double bv = Rs[(ks + t4) * sb + ib * 8 + g];
                    asm volatile(
                        "mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 "
                        "{%0, %1}, {%2}, {%3}, {%0, %1};\n"
                        : "+d"(c[t][0]), "+d"(c[t][1])
                        : "d"(av), "d"(bv));
                }
            }
        }
        __syncthreads();
        buf ^= 1;
    }
    cp_async_wait_all();
    double *out = part + ((size_t)blockIdx.x * gridDim.y + blockIdx.y) * (size_t)BA * BB;
#pragma unroll
    for (int t = 0; t < kDmmaMaxTilesPerWarp; ++t) {
        int tile = warp + t * nwarps;
        if (tile < ntiles) {
            int ia = tile / tb8, ib = tile % tb8;
            out[(ia * 8 + g) * BB + ib * 8 + 2 * t4] = c[t][0];
            out[(ia * 8 + g) * BB + ib * 8 + 2 * t4 + 1] = c[t][1];
        }
    }
}

// C[a][b] = sum over chunks p (in order) of part[p][tile(a,b)][a%BA][b%BB]
// C = sum over chunks of the per-chunk partial tiles.  Four threads share one
// output element: thread quarter q sums its contiguous quarter of the chunks
// in chunk order (loads issued 8 at a time, coalesced across elements), then
// quarter 0 adds the four quarter sums in quarter order -- a fixed order
// that depends only on the shape.
constexpr int kRedElems = 64;  // output elements per block (x 4 quarters = 256 threads)

__global__ void __launch_bounds__(4 * kRedElems)
    gram_reduce_kernel(const double *__restrict__ part, int nchunks, int ntiles, int BA, int BB,
                       int tilesB, int ka, int kb, int kb1, double *__restrict__ C1, int ldc1,
                       double *__restrict__ C2, int ldc2, int sym, int gap = 0) {
    __shared__ double qs[4][kRedElems];
    const int el = threadIdx.x % kRedElems, q = threadIdx.x / kRedElems;
    const int idx = blockIdx.x * kRedElems + el;
    const bool active = idx < ka * kb;
    const int a = active ? idx / kb : 0, b = active ? idx % kb : 0;
    // symmetric leading block: the lower triangle reads its mirror image
    const bool mirror = sym && b < kb1 && a > b;
    // gap: the partial tiles hold `gap` zero columns between the R1 and R2
    // parts (an R1 width padded to the tensor-core kernel's 8-column units)
    const int pa = mirror ? b : a, pb = mirror ? a : (b < kb1 ? b : b + gap);
    const int tile = (pa / BA) * tilesB + (pb / BB);
    const size_t off = (size_t)tile * BA * BB + (size_t)(pa % BA) * BB + (pb % BB);
    const size_t stride = (size_t)ntiles * BA * BB;
    const int per = (nchunks + 3) / 4;
    const int p0 = q * per, p1 = min(nchunks, p0 + per);
    double s = 0.0;
    if (active) {
        int p = p0;
        for (; p + 8 <= p1; p += 8) {
            double v[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) v[u] = part[off + (size_t)(p + u) * stride];
#pragma unroll
            for (int u = 0; u < 8; ++u) s += v[u];
        }
        for (; p < p1; ++p) s += part[off + (size_t)p * stride];
    }
    qs[q][el] = s;
    __syncthreads();
    if (q == 0 && active) {
        const double t = ((qs[0][el] + qs[1][el]) + qs[2][el]) + qs[3][el];
        if (b < kb1)
            C1[(size_t)a * ldc1 + b] = t;
        else
            C2[(size_t)a * ldc2 + (b - kb1)] = t;
    }
}

struct GramPlan {
    int BA, BB, tilesA, tilesB, nchunks;
    int64_t rows_per_chunk;
    size_t smem;
    int threads;
};

static int round_up(int x, int q) { return (x + q - 1) / q * q; }

template <typename T>
static GramPlan plan_gram(int variant, int64_t n, int ka, int kb) {
    GramPlan p;
    const int q = (variant == CACG_GRAM_DMMA) ? 8 : 4;
    p.BA = std::min(round_up(ka, q), kMaxTile);
    // FMA variant: (BA/4) * (BB/4) threads, at most kGramMaxThreads
    int maxBB = variant == CACG_GRAM_DMMA ? kMaxTile
                                          : std::min(kMaxTile, (kGramMaxThreads * kMA * kMB / p.BA) / q * q);
    p.BB = std::min(round_up(kb, q), maxBB);
    p.tilesA = (ka + p.BA - 1) / p.BA;
    p.tilesB = (kb + p.BB - 1) / p.BB;
    int tiles = p.tilesA * p.tilesB;
    int target = 2 * sm_count();
    int64_t nchunks = (target + tiles - 1) / tiles;
    const int KT = (variant == CACG_GRAM_DMMA) ? 16 : GramKT<T>::value;
    int64_t maxchunks = std::max<int64_t>(1, (n + 4 * KT - 1) / (4 * KT));
    if (nchunks > maxchunks) nchunks = maxchunks;
    if (nchunks < 1) nchunks = 1;
    p.rows_per_chunk = (n + nchunks - 1) / nchunks;
    p.rows_per_chunk = (p.rows_per_chunk + KT - 1) / KT * KT;
    if (p.rows_per_chunk < KT) p.rows_per_chunk = KT;  // n == 0
    p.nchunks = (int)((n + p.rows_per_chunk - 1) / p.rows_per_chunk);
    if (p.nchunks < 1) p.nchunks = 1;
    if (variant == CACG_GRAM_DMMA) {
        int ntiles = (p.BA / 8) * (p.BB / 8);
        int warps = (ntiles + kDmmaMaxTilesPerWarp - 1) / kDmmaMaxTilesPerWarp;
        p.threads = 32 * std::max(1, std::min(16, warps));
        p.smem = (size_t)2 * KT * ((p.BA + 4) + (p.BB + 4)) * sizeof(double);
    } else {
        p.threads = (p.BA / kMA) * (p.BB / kMB);
        p.threads = round_up(p.threads, 32);
        p.smem = (size_t)2 * KT * (p.BA + p.BB) * sizeof(T);
    }
    return p;
}

size_t gram_workspace_bytes(int64_t n, int ka, int kb) {
    size_t best = 0;
    for (int v = 1; v <= 2; ++v) {
        GramPlan p = plan_gram<double>(v, n, ka, kb);
        GramPlan q = plan_gram<float>(v, n, ka, kb);
        size_t b1 = (size_t)p.nchunks * p.tilesA * p.tilesB * p.BA * p.BB * sizeof(double);
        size_t b2 = (size_t)q.nchunks * q.tilesA * q.tilesB * q.BA * q.BB * sizeof(double);
        best = std::max(best, std::max(b1, b2));
    }
    return best;
}

template <typename T>
int launch_gram(cudaStream_t st, int variant, int64_t n, const T *L, int64_t ldl, int ka,
                const T *R1, int64_t ldr1, int kb1, const T *R2, int64_t ldr2, int kb2,
                double *C1, int ldc1, double *C2, int ldc2, double *ws, size_t ws_bytes,
                bool symmetric) {
    const int kb = kb1 + kb2;
    if (ka <= 0 || kb <= 0 || n < 0 || !C1 || (kb2 > 0 && !C2)) return CACG_ERR_ARG;
    if (variant != CACG_GRAM_AUTO && variant != CACG_GRAM_FMA && variant != CACG_GRAM_DMMA)
        return CACG_ERR_UNSUPPORTED;
    if (variant == CACG_GRAM_AUTO) variant = CACG_GRAM_FMA;
    if (!std::is_same<T, double>::value) variant = CACG_GRAM_FMA;
    if (variant == CACG_GRAM_DMMA) {
        // each warp holds at most kDmmaMaxTilesPerWarp 8x8 tiles
        int BA = std::min(round_up(ka, 8), kMaxTile), BB = std::min(round_up(kb, 8), kMaxTile);
        if ((BA / 8) * (BB / 8) > 16 * kDmmaMaxTilesPerWarp) variant = CACG_GRAM_FMA;
    }
    GramPlan p = plan_gram<T>(variant, n, ka, kb);
    size_t need = (size_t)p.nchunks * p.tilesA * p.tilesB * p.BA * p.BB * sizeof(double);
    if (need > ws_bytes || !ws) return CACG_ERR_ARG;
    // L^T R1 symmetric (R1 = A L, A symmetric): one tile, square leading block
    const int sym = symmetric && variant == CACG_GRAM_FMA && p.tilesA == 1 && p.tilesB == 1 &&
                    ka == kb1 && ka % kMA == 0 && p.BA == ka;
    if (sym) {
        const int na = p.BA / kMA, nb = p.BB / kMB;
        p.threads = round_up(na * (na + 1) / 2 + na * (nb - na), 32);
    }
    dim3 grid(p.nchunks, p.tilesA * p.tilesB);
    if (n > 0) {
        if (variant == CACG_GRAM_DMMA) {
            if constexpr (std::is_same<T, double>::value) {
                set_smem_attr(gram_dmma_kernel, (int)max_smem_optin());
                gram_dmma_kernel<<<grid, p.threads, p.smem, st>>>(n, p.rows_per_chunk, L, ldl,
                                                                  ka, R1, ldr1, kb1, R2, ldr2,
                                                                  kb2, p.BA, p.BB, p.tilesB,
                                                                  ws);
            }
        } else {
            set_smem_attr(gram_fma_kernel<T>, (int)max_smem_optin());
            gram_fma_kernel<T><<<grid, p.threads, p.smem, st>>>(n, p.rows_per_chunk, L, ldl,
                                                                ka, R1, ldr1, kb1, R2, ldr2,
                                                                kb2, p.BA, p.BB, p.tilesB, ws,
                                                                sym);
        }
        int rc = check_launch();
        if (rc != CACG_OK) return rc;
    } else {
        cudaMemsetAsync(ws, 0, need, st);
    }
    int tot = ka * kb;
    gram_reduce_kernel<<<(tot + kRedElems - 1) / kRedElems, 4 * kRedElems, 0, st>>>(ws, n > 0 ? p.nchunks : 1,
                                                          p.tilesA * p.tilesB, p.BA, p.BB,
                                                          p.tilesB, ka, kb, kb1, C1, ldc1,
                                                          C2, ldc2, sym && n > 0);
    return check_launch();
}

int launch_gram_reduce(cudaStream_t st, const double *part, int nchunks, int ntiles, int BA,
                       int BB, int tilesB, int ka, int kb, int kb1, double *C1, int ldc1,
                       double *C2, int ldc2, int gap) {
    int tot = ka * kb;
    gram_reduce_kernel<<<(tot + kRedElems - 1) / kRedElems, 4 * kRedElems, 0, st>>>(
        part, nchunks, ntiles, BA, BB, tilesB, ka, kb, kb1, C1, ldc1, C2, ldc2, 0, gap);
    return check_launch();
}

template int launch_gram<double>(cudaStream_t, int, int64_t, const double *, int64_t, int,
                                 const double *, int64_t, int, const double *, int64_t, int,
                                 double *, int, double *, int, double *, size_t, bool);
template int launch_gram<float>(cudaStream_t, int, int64_t, const float *, int64_t, int,
                                const float *, int64_t, int, const float *, int64_t, int,
                                double *, int, double *, int, double *, size_t, bool);

}  // namespace cacg

using namespace cacg;

extern "C" int cacg_k_gram(int32_t vtype, int32_t variant, int64_t n, const void *L,
                           int64_t ldl, int32_t ka, const void *R1, int64_t ldr1, int32_t kb1,
                           const void *R2, int64_t ldr2, int32_t kb2, double *C, int32_t ldc,
                           void *stream) {
    cudaStream_t st = (cudaStream_t)stream;
    if (kb2 > 0 && !R2) return CACG_ERR_ARG;
    if (variant == CACG_GRAM_TC5) {
        if (vtype != CACG_VAL_F32) return CACG_ERR_ARG;
        if (!gram_tc5_supported(ka, kb1 + kb2)) return CACG_ERR_UNSUPPORTED;
        size_t wsb = gram_tc5_workspace_bytes(n, ka, kb1 + kb2);
        char *buf = nullptr;
        if (cudaMallocAsync((void **)&buf, wsb + 256, st) != cudaSuccess) return CACG_ERR_OOM;
        int *status = (int *)(buf + wsb);
        cudaMemsetAsync(status, 0, sizeof(int), st);
        int rc = launch_gram_tc5(st, n, (const float *)L, ldl, ka, (const float *)R1, ldr1, kb1,
                                 (const float *)R2, ldr2, kb2, C, ldc, C + kb1, ldc, (double *)buf,
                                 wsb, status);
        int hs = 0;
        if (rc == CACG_OK) {
            cudaMemcpyAsync(&hs, status, sizeof(int), cudaMemcpyDeviceToHost, st);
            if (cudaStreamSynchronize(st) != cudaSuccess) rc = CACG_ERR_CUDA;
        }
        cudaFreeAsync(buf, st);
        if (rc == CACG_OK && (hs & kStatusTimeout)) rc = CACG_ERR_TIMEOUT;
        return rc;
    }
    if (variant == CACG_GRAM_TC_SLICES) {
        // split the FP32 inputs into slice planes, then the slice-plane kernel
        if (vtype != CACG_VAL_F32) return CACG_ERR_ARG;
        const int kb = kb1 + kb2;
        if (!gram_tcs_supported(ka, kb1, kb2, ldl, ldr1, ldr2)) return CACG_ERR_ARG;
        const size_t pl_l = (size_t)n * ldl, pl_1 = (size_t)n * ldr1,
                     pl_2 = kb2 > 0 ? (size_t)n * ldr2 : 0;
        size_t wsb = gram_tcs_workspace_bytes(n, ka, kb);
        size_t tot = ((3 * (pl_l + pl_1 + pl_2) * 2 + 255) / 256) * 256 + wsb + 256;
        char *buf = nullptr;
        if (cudaMallocAsync((void **)&buf, tot, st) != cudaSuccess) return CACG_ERR_OOM;
        Slices sL{(__nv_bfloat16 *)buf, (int64_t)pl_l};
        Slices s1{sL.p + 3 * pl_l, (int64_t)pl_1};
        Slices s2{s1.p + 3 * pl_1, (int64_t)pl_2};
        double *w = (double *)(buf + ((3 * (pl_l + pl_1 + pl_2) * 2 + 255) / 256) * 256);
        int rc = launch_split_planes(st, n, ka, (const float *)L, ldl, sL);
        if (rc == CACG_OK) rc = launch_split_planes(st, n, kb1, (const float *)R1, ldr1, s1);
        if (rc == CACG_OK && kb2 > 0)
            rc = launch_split_planes(st, n, kb2, (const float *)R2, ldr2, s2);
        if (rc == CACG_OK)
            rc = launch_gram_tcs(st, n, sL, ldl, ka, s1, ldr1, kb1, s2, ldr2, kb2, C, ldc, C + kb1,
                                 ldc, w, wsb);
        cudaFreeAsync(buf, st);
        return rc;
    }
    if (variant == CACG_GRAM_TC) {
        if (vtype != CACG_VAL_F32) return CACG_ERR_ARG;
        size_t wsb = gram_tc_workspace_bytes(n, ka, kb1 + kb2);
        double *w = nullptr;
        if (cudaMallocAsync((void **)&w, wsb > 0 ? wsb : 16, st) != cudaSuccess) return CACG_ERR_OOM;
        int rc = launch_gram_tc(st, n, (const float *)L, ldl, ka, (const float *)R1, ldr1, kb1,
                                (const float *)R2, ldr2, kb2, C, ldc, C + kb1, ldc, w, wsb);
        cudaFreeAsync(w, st);
        return rc;
    }
    size_t ws_bytes = gram_workspace_bytes(n, ka, kb1 + kb2);
    double *ws = nullptr;
    if (cudaMallocAsync((void **)&ws, ws_bytes, st) != cudaSuccess) return CACG_ERR_OOM;
    int rc;
    if (vtype == CACG_VAL_F64)
        rc = launch_gram<double>(st, variant, n, (const double *)L, ldl, ka,
                                 (const double *)R1, ldr1, kb1, (const double *)R2, ldr2, kb2,
                                 C, ldc, C + kb1, ldc, ws, ws_bytes);
    else if (vtype == CACG_VAL_F32)
        rc = launch_gram<float>(st, variant, n, (const float *)L, ldl, ka, (const float *)R1,
                                ldr1, kb1, (const float *)R2, ldr2, kb2, C, ldc, C + kb1, ldc, ws,
                                ws_bytes);
    else
        rc = CACG_ERR_ARG;
    cudaFreeAsync(ws, st);
    return rc;
}

// ---------------------------------------------------------------------------
// Gram without device allocation.
//
// Some callers cannot let a library call cudaMalloc/cudaMallocAsync: processes
// whose device memory is handed out by their own allocator (the whole pool
// reserved up front, so a third-party allocation fails or breaks the budget),
// and latency-critical loops where an allocation or free may synchronise the
// device.  For them, cacg_k_gram_noalloc computes the same product as
// cacg_k_gram, but its split-K partial tiles live in the fixed device array
// below instead of a per-call workspace.
//
// * The array is 16 MiB, file-scope, and every GPU that loads libcacg.so holds
//   it until the process exits.
// * Shapes whose smallest split (one row chunk: tilesA*tilesB*BA*BB doubles)
//   does not fit in it are rejected with CACG_ERR_ARG and a message; shapes
//   that fit use as many row chunks as the array holds (fewer than
//   cacg_k_gram may use, so the summation order, not the accuracy class,
//   differs).
// * All calls share the array and each call leaves its partial tiles in it.
//   Every partial tile is fully overwritten by its CTA when n > 0; for n == 0
//   the tiles are cleared with cudaMemsetAsync before the reduction.  Calls
//   that overlap on the GPU (different streams, or different host threads)
//   race on the array: serialise them.
// * Device addresses: the host-side name of the array is not a device
//   address.  The first call on each device (that device current) looks the
//   address up once with cudaGetSymbolAddress and caches it under the
//   device's current context ID, so a context re-created after
//   cudaDeviceReset gets a fresh lookup; make the first call in each context
//   before any stream capture.
// * variant: CACG_GRAM_AUTO, CACG_GRAM_FMA or CACG_GRAM_DMMA (FP64 inputs);
//   the tensor-core variants of cacg_k_gram need their own workspace and are
//   refused with CACG_ERR_UNSUPPORTED.  FP32 inputs take the FP64-accurate
//   CUDA-core product whatever the variant.
// ---------------------------------------------------------------------------
#include <cuda.h>

#include <cstdio>
#include <mutex>

namespace cacg {

constexpr size_t kGramNoAllocScratchBytes = size_t(16) << 20;
static __device__ __align__(256) double
    g_gram_noalloc_scratch[kGramNoAllocScratchBytes / sizeof(double)];

static std::mutex g_noalloc_mu;
struct NoAllocEntry {
    unsigned long long ctx_id;  // 0: not looked up yet
    double *ptr;
};
static NoAllocEntry g_noalloc[64];

// ID of the current context (unique for the process's lifetime, unlike the
// context handle); 0 when the driver does not provide it.
static unsigned long long current_context_id() {
    using GetCurrent = CUresult (*)(CUcontext *);
    using GetId = CUresult (*)(CUcontext, unsigned long long *);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr, *q = nullptr;
        cudaDriverEntryPointQueryResult r1 = cudaDriverEntryPointSymbolNotFound, r2 = r1;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault,
                                             &r1) == cudaSuccess &&
            r1 == cudaDriverEntryPointSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &q, 12000, cudaEnableDefault, &r2) ==
                cudaSuccess &&
            r2 == cudaDriverEntryPointSuccess) {
            get_current = reinterpret_cast<GetCurrent>(p);
            get_id = reinterpret_cast<GetId>(q);
        }
        cudaGetLastError();
    });
    CUcontext c = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&c) != CUDA_SUCCESS || !c ||
        get_id(c, &id) != CUDA_SUCCESS)
        return 0;
    return id;
}

static int noalloc_scratch(double **out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        return CACG_ERR_CUDA;
    }
    // cudaSetDevice initialises the device's primary context and makes it
    // current on this thread, so the context ID below is the one the kernels
    // will run in
    if (cudaSetDevice(dev) != cudaSuccess) {
        cudaGetLastError();
        return CACG_ERR_CUDA;
    }
    const unsigned long long id = current_context_id();
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    NoAllocEntry &e = g_noalloc[dev];
    if (id == 0 || e.ctx_id != id) {
        double *p = nullptr;
        cudaError_t rc = cudaGetSymbolAddress((void **)&p, g_gram_noalloc_scratch);
        if (rc != cudaSuccess || !p) {
            record_cuda_error(rc, "cudaGetSymbolAddress(g_gram_noalloc_scratch)", __FILE__,
                              __LINE__);
            cudaGetLastError();
            return CACG_ERR_CUDA;
        }
        e.ctx_id = id;
        e.ptr = p;
    }
    *out = e.ptr;
    return CACG_OK;
}

template <typename T>
static int gram_fixed_scratch(cudaStream_t st, int variant, int64_t n, const T *L, int64_t ldl,
                              int ka, const T *R1, int64_t ldr1, int kb1, const T *R2,
                              int64_t ldr2, int kb2, double *C1, int ldc1, double *C2, int ldc2,
                              double *ws, size_t ws_bytes) {
    const int kb = kb1 + kb2;
    if (ka <= 0 || kb <= 0 || n < 0 || !C1 || (kb2 > 0 && !C2)) return CACG_ERR_ARG;
    if (variant != CACG_GRAM_AUTO && variant != CACG_GRAM_FMA && variant != CACG_GRAM_DMMA)
        return CACG_ERR_UNSUPPORTED;
    if (variant == CACG_GRAM_AUTO) variant = CACG_GRAM_FMA;
    if (!std::is_same<T, double>::value) variant = CACG_GRAM_FMA;
    if (variant == CACG_GRAM_DMMA) {
        int BA = std::min(round_up(ka, 8), kMaxTile), BB = std::min(round_up(kb, 8), kMaxTile);
        if ((BA / 8) * (BB / 8) > 16 * kDmmaMaxTilesPerWarp) variant = CACG_GRAM_FMA;
    }
    GramPlan p = plan_gram<T>(variant, n, ka, kb);
    const size_t per_chunk = (size_t)p.tilesA * p.tilesB * p.BA * p.BB * sizeof(double);
    if (per_chunk > ws_bytes) {
        fprintf(stderr,
                "cacg_k_gram_noalloc: a %d x %d Gram needs %zu bytes of scratch per row chunk; "
                "the fixed scratch holds %zu bytes\n",
                ka, kb, per_chunk, ws_bytes);
        return CACG_ERR_ARG;
    }
    const int64_t max_chunks = (int64_t)(ws_bytes / per_chunk);
    if (p.nchunks > max_chunks) {
        const int KT = (variant == CACG_GRAM_DMMA) ? 16 : GramKT<T>::value;
        p.rows_per_chunk = (n + max_chunks - 1) / max_chunks;
        p.rows_per_chunk = (p.rows_per_chunk + KT - 1) / KT * KT;
        p.nchunks = (int)((n + p.rows_per_chunk - 1) / p.rows_per_chunk);
        if (p.nchunks < 1) p.nchunks = 1;
    }
    const size_t need = (size_t)p.nchunks * per_chunk;
    dim3 grid(p.nchunks, p.tilesA * p.tilesB);
    if (n > 0) {
        if (variant == CACG_GRAM_DMMA) {
            if constexpr (std::is_same<T, double>::value) {
                set_smem_attr(gram_dmma_kernel, (int)max_smem_optin());
                gram_dmma_kernel<<<grid, p.threads, p.smem, st>>>(n, p.rows_per_chunk, L, ldl,
                                                                  ka, R1, ldr1, kb1, R2, ldr2,
                                                                  kb2, p.BA, p.BB, p.tilesB,
                                                                  ws);
            }
        } else {
            set_smem_attr(gram_fma_kernel<T>, (int)max_smem_optin());
            gram_fma_kernel<T><<<grid, p.threads, p.smem, st>>>(n, p.rows_per_chunk, L, ldl,
                                                                ka, R1, ldr1, kb1, R2, ldr2,
                                                                kb2, p.BA, p.BB, p.tilesB, ws, 0);
        }
        int rc = check_launch();
        if (rc != CACG_OK) return rc;
    } else {
        if (cudaMemsetAsync(ws, 0, need, st) != cudaSuccess) return CACG_ERR_CUDA;
    }
    int tot = ka * kb;
    gram_reduce_kernel<<<(tot + kRedElems - 1) / kRedElems, 4 * kRedElems, 0, st>>>(ws, n > 0 ? p.nchunks : 1,
                                                          p.tilesA * p.tilesB, p.BA, p.BB,
                                                          p.tilesB, ka, kb, kb1, C1, ldc1,
                                                          C2, ldc2, 0);
    return check_launch();
}

}  // namespace cacg

extern "C" int cacg_k_gram_noalloc(int32_t vtype, int32_t variant, int64_t n, const void *L,
                                   int64_t ldl, int32_t ka, const void *R1, int64_t ldr1,
                                   int32_t kb1, const void *R2, int64_t ldr2, int32_t kb2,
                                   double *C, int32_t ldc, void *stream) {
    cudaStream_t st = (cudaStream_t)stream;
    if (kb2 > 0 && !R2) return CACG_ERR_ARG;
    double *ws = nullptr;
    int rc = noalloc_scratch(&ws);
    if (rc != CACG_OK) return rc;
    const size_t wsb = kGramNoAllocScratchBytes;
    if (vtype == CACG_VAL_F64)
        return gram_fixed_scratch<double>(st, variant, n, (const double *)L, ldl, ka,
                                          (const double *)R1, ldr1, kb1, (const double *)R2,
                                          ldr2, kb2, C, ldc, C + kb1, ldc, ws, wsb);
    if (vtype == CACG_VAL_F32)
        return gram_fixed_scratch<float>(st, variant, n, (const float *)L, ldl, ka,
                                         (const float *)R1, ldr1, kb1, (const float *)R2, ldr2,
                                         kb2, C, ldc, C + kb1, ldc, ws, wsb);
    return CACG_ERR_ARG;
}
