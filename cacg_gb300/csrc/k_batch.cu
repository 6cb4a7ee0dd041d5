// k_batch.cu -- the serving engine's batched kernels (no reference
// counterpart: sclc/cacg solves one system per process, src/main.c:22-221).
//
// One launch per phase covers every admitted request of a precision class.
// Blocks stride over the class's tile table (batch.h): a row tile is kBRows
// consecutive rows of one request, a Gram piece bpiece<T>() rows.  The work
// of a tile depends only on its own request's data, and every sum runs in a
// fixed order inside the tile (SpMM: the CSR row order; Gram: a fixed
// row-group split inside a piece, then pieces in order; norms: a fixed
// thread and warp order inside a tile, then tiles in order), so results do
// not depend on the grid size or on which other requests share the launch.
//
// The operations are the reference iteration's (src/bcbcgKernel.c:172-526):
//   basis step j  T_j = 2a A T_{j-1} + 2b T_{j-1} - T_{j-2}   (src/common.c:182-249)
//   Gram          C = L^T [R1 | R2]                            (src/BLAS3.c:699-758)
//   LU            Crout, unit-diagonal U, no pivoting           (src/DLSsolvers.c:106-208)
//   Q update      Q = S - Q_old beta                            (src/BLAS3.c:794-825, 579-612)
//   X/R update    X += Q alpha, R -= AQ alpha, ||R(:,c)||^2     (src/bcbcgKernel.c:376-447)
//   residual      R = B - A X                                   (src/bcbcgKernel.c:136-154)
// FP64 class: every operand FP64.  FP32 class (the mixed mode): A, the basis,
// Q and AQ in FP32; the SpMMs, the Q update, the Gram sums inside a piece and
// the X/R products in FP32; Gram partials, LU, X and R in FP64; residuals in
// FP64.  GB300's FP64 pipe runs at about 1/58 of the FP32 rate, so the FP32
// class keeps FP64 to the small dense work and the additions into X and R.
//
// Dense tiles go through shared memory with a row pitch of an odd number of
// 16-byte units (bpitch), so a warp's 16-byte loads from up to eight rows
// fall in distinct bank groups; a thread owns 4 consecutive output columns
// (and, in the Q update, two rows) and reads 16-byte pieces, 2-3 shared loads
// per 8 FMAs.
//
// No kernel here waits on another block; the only waits are for a block's
// own asynchronous copies into its shared memory (cp.async.wait_group).
#include <type_traits>

#include "batch.h"
#include "cacg_internal.cuh"

namespace cacg {

// request r with start[r] <= t < start[r + 1] (start[0] = 0, nr >= 1)
__device__ __forceinline__ int bfind(const int *__restrict__ start, int nr, int t) {
    int lo = 0, hi = nr;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (start[mid] <= t)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

template <typename T>
__device__ __forceinline__ const T *bvals(const BDesc &d);
template <>
__device__ __forceinline__ const double *bvals<double>(const BDesc &d) {
    return d.val;
}
template <>
__device__ __forceinline__ const float *bvals<float>(const BDesc &d) {
    return d.val32;
}

// ------------------------------------------------------------ helpers
// floor(i / d) for 0 <= i < 2^32 / d: i itself for d = 1, else the high word
// of i * ceil(2^32 / d) (mg = bdiv_magic(d)), exact in that range
__device__ __forceinline__ uint32_t bdiv_magic(int d) {
    return d > 1 ? 0xFFFFFFFFu / (uint32_t)d + 1u : 0u;
}
__device__ __forceinline__ int bdiv(int i, int d, uint32_t mg) {
    return d > 1 ? (int)__umulhi((uint32_t)i, mg) : i;
}

// log2 of the smallest power of two >= x (x >= 1)
__device__ __forceinline__ int blog2_ceil(int x) {
    int l = 0;
    while ((1 << l) < x) ++l;
    return l;
}

// shared-memory row pitch (elements) of `cols` values read as 16-byte
// pieces: a multiple of 4 elements and an odd number of 16-byte units
template <typename T>
__host__ __device__ constexpr int bpitch(int cols) {
    return ((((cols + 3) & ~3) / (16 / (int)sizeof(T))) & 1) ? ((cols + 3) & ~3)
                                                             : ((cols + 3) & ~3) + 16 / (int)sizeof(T);
}
constexpr int kBPitchK = kBMaxK + 4;  // >= bpitch<T>(k), k <= kBMaxK
constexpr int kBPitchM = kBMaxM + 4;  // >= bpitch<T>(m), m <= kBMaxM
static_assert(bpitch<float>(kBMaxK) <= kBPitchK && bpitch<double>(kBMaxK) <= kBPitchK, "pitch");
static_assert(bpitch<float>(kBMaxM) <= kBPitchM && bpitch<double>(kBMaxM) <= kBPitchM, "pitch");

// rows of the X/R and Q update's shared-memory sub-tiles
template <typename T>
__host__ __device__ constexpr int bxsub() {
    return sizeof(T) == 4 ? 64 : 32;
}

__device__ __forceinline__ void ld4(const float *p, float v[4]) {
    const float4 t = *reinterpret_cast<const float4 *>(p);
    v[0] = t.x;
    v[1] = t.y;
    v[2] = t.z;
    v[3] = t.w;
}
__device__ __forceinline__ void ld4(const double *p, double v[4]) {
    const double2 a = *reinterpret_cast<const double2 *>(p);
    const double2 c = *reinterpret_cast<const double2 *>(p + 2);
    v[0] = a.x;
    v[1] = a.y;
    v[2] = c.x;
    v[3] = c.y;
}

// rows x cols values, contiguous in global memory (row stride cols), into
// shared memory rows of `pitch` by asynchronous copies (cp.async): 16-byte
// pieces when a row is a whole number of them, else one copy a value.  Every
// copy of the block is in flight at once; bstage_wait() completes them.
__device__ __forceinline__ void bcp_async(void *dst, const void *src, int bytes) {
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst);
    if (bytes == 16)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
    else if (bytes == 8)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}

template <typename T>
__device__ __forceinline__ void bstage(T *__restrict__ dst, int pitch, const T *__restrict__ src,
                                       int rows, int cols, uint32_t mg) {
    constexpr int V = 16 / (int)sizeof(T);
    if (cols % V == 0 && ((uintptr_t)src & 15) == 0) {
        const int cv = cols / V;
        const uint32_t mgv = bdiv_magic(cv);
        for (int g = threadIdx.x; g < rows * cv; g += kBThreads) {
            const int i = bdiv(g, cv, mgv);
            bcp_async(dst + i * pitch + (g - i * cv) * V, src + (size_t)g * V, 16);
        }
    } else {
        for (int idx = threadIdx.x; idx < rows * cols; idx += kBThreads) {
            const int i = bdiv(idx, cols, mg);
            bcp_async(dst + i * pitch + (idx - i * cols), src + idx, (int)sizeof(T));
        }
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}

__device__ __forceinline__ void bstage_wait() {
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

// zero columns [cols, cols rounded up to 4) of `rows` shared-memory rows
template <typename T>
__device__ __forceinline__ void bzero_pad(T *dst, int pitch, int rows, int cols) {
    const int w = ((cols + 3) & ~3) - cols;
    if (w == 0) return;
    for (int idx = threadIdx.x; idx < rows * w; idx += kBThreads) {
        const int i = idx / w;
        dst[i * pitch + cols + (idx - i * w)] = (T)0;
    }
}

// A row tile's CSR rows in shared memory: row pointers, and the column
// indices and values when the tile's entries fit kBSpCap (otherwise they are
// read from global memory; the sums are the same either way).
constexpr int kBSpCap = 2048;

template <typename V>
struct BCsrTile {
    int rps[kBRows + 1];
    int cis[kBSpCap];
    V vs[kBSpCap];
};

// stages the tile; returns whether the entries are in shared memory
template <typename V>
__device__ __forceinline__ bool bstage_csr(BCsrTile<V> &sh, const int32_t *__restrict__ rp,
                                           const int32_t *__restrict__ ci,
                                           const V *__restrict__ val, int64_t row0, int rows) {
    __syncthreads();  // the previous tile's readers are done
    for (int i = threadIdx.x; i <= rows; i += kBThreads) sh.rps[i] = rp[row0 + i];
    __syncthreads();
    const int p0 = sh.rps[0], np = sh.rps[rows] - p0;
    const bool staged = np <= kBSpCap;
    if (staged)
        for (int i = threadIdx.x; i < np; i += kBThreads) {
            sh.cis[i] = ci[p0 + i];
            sh.vs[i] = val[p0 + i];
        }
    __syncthreads();
    return staged;
}

// column sums of a tile: thread partials for columns 4 cg .. 4 cg + 3 (cg =
// lane mod G, G a power of two <= 8) are combined over the lanes by a fixed
// butterfly, then over the warps in order; npart[c] for c < m
__device__ __forceinline__ void bcolsum_store(double nsq[4], int G, int m,
                                              double (*Ws)[32], double *__restrict__ npart) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int v = 0; v < 4; ++v)
        for (int o = G; o < 32; o <<= 1) nsq[v] += __shfl_xor_sync(0xffffffffu, nsq[v], o);
    if (lane < G)
#pragma unroll
        for (int v = 0; v < 4; ++v) Ws[warp][4 * lane + v] = nsq[v];
    __syncthreads();
    if ((int)threadIdx.x < m) {
        double s = 0.0;
#pragma unroll
        for (int w = 0; w < kBThreads / 32; ++w) s += Ws[w][threadIdx.x];
        npart[threadIdx.x] = s;
    }
}

// ------------------------------------------------------------ SpMM
// MODE 0: basis step j, Y = T_j (width m).  MODE 1: AQ = A Q (width k).
// A thread owns one row x 4 consecutive columns: one CSR entry per 4 FMAs.
template <typename T, int MODE>
__global__ void __launch_bounds__(kBThreads) bk_spmm(const BBatch *__restrict__ b, int j) {
    __shared__ __align__(16) BCsrTile<T> sh;
    const int nr = b->nr, total = b->total_tiles;
    for (int t = blockIdx.x; t < total; t += gridDim.x) {
        const int r = bfind(b->tile_start, nr, t);
        const BDesc &d = b->d[r];
        if (!(d.flags & kBActive)) continue;
        if (MODE == 0 && j >= d.s) continue;
        const int k = d.k, m = d.m;
        const int64_t row0 = (int64_t)(t - b->tile_start[r]) * kBRows;
        const int rows = (int)min((int64_t)kBRows, d.n - row0);
        T *S = (T *)d.S;
        const T *X;
        const T *Z2 = nullptr;
        T *Y;
        int w;
        T ca, cb, cc;
        if (MODE == 0) {
            X = S + (size_t)(j - 1) * m;
            Y = S + (size_t)j * m;
            if (j >= 2) Z2 = S + (size_t)(j - 2) * m;
            ca = (T)(j == 1 ? d.sa : 2.0 * d.sa);
            cb = (T)(j == 1 ? d.sb : 2.0 * d.sb);
            cc = (T)(-1.0);
            w = m;
        } else {
            X = S;
            Y = (T *)d.AQ;
            ca = (T)1.0;
            cb = cc = (T)0.0;
            w = k;
        }
        const T *val = bvals<T>(d);
        const int32_t *ci = d.ci;
        const bool staged = bstage_csr(sh, d.rp, ci, val, row0, rows);
        const int p0 = sh.rps[0];
        const int ng = (w + 3) >> 2;
        const uint32_t mg = bdiv_magic(ng);
        // a row's 4-column piece of Q is 16-byte aligned (FP64: 32 bytes, two loads)
        const bool vec = ((uintptr_t)X & 15) == 0 && (k & 3) == 0;
        for (int e = threadIdx.x; e < rows * ng; e += kBThreads) {
            const int lr = bdiv(e, ng, mg), c0 = 4 * (e - lr * ng), nc = min(4, w - c0);
            const int64_t row = row0 + lr;
            const int q0 = sh.rps[lr] - p0, q1 = sh.rps[lr + 1] - p0;
            T acc[4] = {(T)0.0, (T)0.0, (T)0.0, (T)0.0};
            if (MODE == 1 && staged && vec && nc == 4) {
                // A Q: 16-byte gathers of the 4 columns (same FMAs, same order)
#pragma unroll 4
                for (int q = q0; q < q1; ++q) {
                    const T v = sh.vs[q];
                    T xv[4];
                    ld4(X + (int64_t)sh.cis[q] * k + c0, xv);
#pragma unroll
                    for (int u = 0; u < 4; ++u) acc[u] = fma(v, xv[u], acc[u]);
                }
            } else if (staged) {
#pragma unroll 2
                for (int q = q0; q < q1; ++q) {
                    const T v = sh.vs[q];
                    const T *xr = X + (int64_t)sh.cis[q] * k + c0;
#pragma unroll
                    for (int u = 0; u < 4; ++u)
                        if (u < nc) acc[u] = fma(v, xr[u], acc[u]);
                }
            } else {
                for (int q = q0; q < q1; ++q) {
                    const T v = val[p0 + q];
                    const T *xr = X + (int64_t)ci[p0 + q] * k + c0;
#pragma unroll
                    for (int u = 0; u < 4; ++u)
                        if (u < nc) acc[u] = fma(v, xr[u], acc[u]);
                }
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                if (u >= nc) break;
                const int c = c0 + u;
                T y = ca * acc[u];
                if (MODE == 0) {
                    y = fma(cb, X[row * k + c], y);
                    if (Z2) y = fma(cc, Z2[row * k + c], y);
                }
                Y[row * k + c] = y;
            }
        }
    }
}

// R = B - A X (FP64) for requests flagged kBResid; T_0 = R into S (and R32);
// per-tile squared column norms into npart.
template <typename T>
__global__ void __launch_bounds__(kBThreads) bk_residual(const BBatch *__restrict__ b) {
    __shared__ __align__(16) BCsrTile<double> sh;
    __shared__ double Ws[kBThreads / 32][32];
    const int nr = b->nr, total = b->total_tiles;
    const int tid = threadIdx.x;
    for (int t = blockIdx.x; t < total; t += gridDim.x) {
        const int r = bfind(b->tile_start, nr, t);
        const BDesc &d = b->d[r];
        if (!(d.flags & kBResid)) continue;
        const int k = d.k, m = d.m;
        const int lt = t - b->tile_start[r];
        const int64_t row0 = (int64_t)lt * kBRows;
        const int rows = (int)min((int64_t)kBRows, d.n - row0);
        const int32_t *ci = d.ci;
        const double *val = d.val, *X = d.X, *B = d.B;
        double *R = d.R;
        T *S = (T *)d.S;
        float *R32 = d.R32;
        const bool staged = bstage_csr(sh, d.rp, ci, val, row0, rows);
        const int p0 = sh.rps[0];
        const int lgG = blog2_ceil((m + 3) >> 2), G = 1 << lgG;
        const int cg = tid & (G - 1), c0 = 4 * cg;
        double nsq[4] = {0.0, 0.0, 0.0, 0.0};
        for (int lr = tid >> lgG; lr < rows; lr += kBThreads >> lgG) {
            const int64_t row = row0 + lr;
            const int q0 = sh.rps[lr] - p0, q1 = sh.rps[lr + 1] - p0;
            double acc[4] = {0.0, 0.0, 0.0, 0.0};
            for (int q = q0; q < q1; ++q) {
                const double v = staged ? sh.vs[q] : val[p0 + q];
                const double *xr = X + (int64_t)(staged ? sh.cis[q] : ci[p0 + q]) * m + c0;
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    if (c0 + u < m) acc[u] = fma(v, xr[u], acc[u]);
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int c = c0 + u;
                if (c >= m) break;
                const double rv = B[row * m + c] - acc[u];
                R[row * m + c] = rv;
                S[row * k + c] = (T)rv;
                if (R32) R32[row * m + c] = (float)rv;
                nsq[u] = fma(rv, rv, nsq[u]);
            }
        }
        bcolsum_store(nsq, G, m, Ws, d.npart + (size_t)lt * m);
    }
}

// ------------------------------------------------------------ Gram
// WHICH 0: QtAS = AQ^T S (requests past their first iteration).
// WHICH 1: [QtAQ | QtR] = Q^T [AQ | R] (Q is the S buffer after the update);
// Q^T A Q is symmetric, so only its upper triangle is computed and the
// reduction mirrors it.
// A block takes one piece: its rows are copied chunk by chunk into shared
// memory (coalesced, two barriers a chunk) and threads own 4 x 4 tiles of the
// product, summed in registers over the whole piece; when the product has
// few tiles, G row groups (rows i = g mod G) run side by side and their sums
// are added in group order.  The piece sums in the operands' precision (FP64
// class: FP64; FP32 class: FP32 over the piece's 256 rows); the piece
// partials are summed in FP64, piece by piece.
__device__ __forceinline__ int bk_gram_groups(int ntiles) {
    int G = 1;
    while (G < 8 && ntiles * G * 2 <= kBThreads) G *= 2;
    return G;
}

// tile w's first row a0 and first virtual column b0 (R1 columns [0, k4), R2
// columns from k4 on)
template <int WHICH>
__device__ __forceinline__ void bgram_tile(int w, int nta, int ntb2, int k4, int &a0, int &b0) {
    if (WHICH == 0) {
        const int at = w / nta;
        a0 = 4 * at;
        b0 = 4 * (w - at * nta);
        return;
    }
    const int ntri = nta * (nta + 1) / 2;
    if (w < ntri) {  // upper triangle, column by column: (at, bt), at <= bt
        int bt = (int)((sqrtf(8.f * (float)w + 1.f) - 1.f) * 0.5f);
        while (bt * (bt + 1) / 2 > w) --bt;
        while ((bt + 1) * (bt + 2) / 2 <= w) ++bt;
        a0 = 4 * (w - bt * (bt + 1) / 2);
        b0 = 4 * bt;
    } else {
        const int w2 = w - ntri, at = w2 / ntb2;
        a0 = 4 * at;
        b0 = k4 + 4 * (w2 - at * ntb2);
    }
}

// stores entry (a, virtual column bv) of a piece's partial when it is one
// the reduction reads
template <int WHICH>
__device__ __forceinline__ void bgram_put(double *gp, int k, int kb, int k4, int a, int bv,
                                          double v) {
    if (a >= k) return;
    if (bv < k4) {
        if (bv >= k || (WHICH == 1 && a > bv)) return;
        gp[a * kb + bv] = v;
    } else {
        const int bb = k + (bv - k4);
        if (bb < kb) gp[a * kb + bb] = v;
    }
}

template <typename T, int WHICH>
__global__ void __launch_bounds__(kBThreads) bk_gram(const BBatch *__restrict__ b) {
    extern __shared__ __align__(16) unsigned char bg_smem[];
    constexpr int CH = bgchunk<T>(), PR = bpiece<T>();
    T *Ls = reinterpret_cast<T *>(bg_smem);  // CH x pk
    T *R1s = Ls + CH * kBPitchK;               // CH x pk
    T *R2s = R1s + CH * kBPitchK;              // CH x pm
    T *Sc = Ls;  // after the piece's last chunk: group sums, G x ntiles x 16
    const int nr = b->nr, total = b->total_pieces;
    const int tid = threadIdx.x;
    for (int t = blockIdx.x; t < total; t += gridDim.x) {
        const int r = bfind(b->piece_start, nr, t);
        const BDesc &d = b->d[r];
        if (!(d.flags & kBActive)) continue;
        if (WHICH == 0 && d.it == 0) continue;
        const int k = d.k, m = WHICH ? d.m : 0, kb = k + m, k4 = (k + 3) & ~3;
        const int pk = bpitch<T>(k), pm = bpitch<T>(WHICH ? m : 1);
        const int lp = t - b->piece_start[r];
        const int64_t prow0 = (int64_t)lp * PR;
        const int prows = (int)min((int64_t)PR, d.n - prow0);
        const T *L = (const T *)(WHICH == 0 ? d.AQ : d.S);
        const T *R1 = (const T *)(WHICH == 0 ? d.S : d.AQ);
        const T *R2 = nullptr;
        if (WHICH == 1) R2 = std::is_same<T, float>::value ? (const T *)(const void *)d.R32
                                                             : (const T *)(const void *)d.R;
        const int nta = k4 >> 2, ntb2 = (m + 3) >> 2;
        const int ntiles = WHICH ? nta * (nta + 1) / 2 + nta * ntb2 : nta * nta;
        const int G = bk_gram_groups(ntiles);
        const int nwork = ntiles * G;
        const uint32_t mgk = bdiv_magic(k), mgm = bdiv_magic(m);
        double *gp = d.gpart + (size_t)lp * k * kb;
        // one pass, unless a product of more than kBThreads tiles (G = 1)
        // takes a second pass over the piece
        for (int w0 = 0; w0 < nwork; w0 += kBThreads) {
            const int w = w0 + tid;
            const bool has = w < nwork;
            const int grp = has ? w / ntiles : 0;
            int a0 = 0, b0 = 0;
            if (has) bgram_tile<WHICH>(w - grp * ntiles, nta, ntb2, k4, a0, b0);
            const bool r1 = b0 < k4;
            const T *lb = Ls + a0;
            const T *rb = r1 ? R1s + b0 : R2s + (b0 - k4);
            const int rpch = r1 ? pk : pm;
            T acc[4][4];
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v) acc[u][v] = (T)0.0;
            for (int crow = 0; crow < prows; crow += CH) {
                const int rows = min(CH, prows - crow);
                const int64_t g0 = prow0 + crow;
                __syncthreads();  // the previous chunk's readers are done
                bstage(Ls, pk, L + g0 * k, rows, k, mgk);
                bstage(R1s, pk, R1 + g0 * k, rows, k, mgk);
                if (WHICH == 1) bstage(R2s, pm, R2 + g0 * m, rows, m, mgm);
                bstage_wait();
                __syncthreads();
                if (has)
                    for (int i = grp; i < rows; i += G) {
                        T lv[4], rv[4];
                        ld4(lb + i * pk, lv);
                        ld4(rb + i * rpch, rv);
#pragma unroll
                        for (int u = 0; u < 4; ++u)
#pragma unroll
                            for (int v = 0; v < 4; ++v) acc[u][v] = fma(lv[u], rv[v], acc[u][v]);
                    }
            }
            if (G == 1) {
                if (has)
#pragma unroll
                    for (int u = 0; u < 4; ++u)
#pragma unroll
                        for (int v = 0; v < 4; ++v)
                            bgram_put<WHICH>(gp, k, kb, k4, a0 + u, b0 + v, (double)acc[u][v]);
            } else {
                __syncthreads();  // the staging area becomes the group scratch
                if (has)
#pragma unroll
                    for (int u = 0; u < 4; ++u)
#pragma unroll
                        for (int v = 0; v < 4; ++v) Sc[(tid * 4 + u) * 4 + v] = acc[u][v];
                __syncthreads();
                for (int e = tid; e < ntiles * 16; e += kBThreads) {
                    const int tile = e >> 4, uv = e & 15;
                    T sum = Sc[e];
                    for (int g = 1; g < G; ++g) sum += Sc[(size_t)g * ntiles * 16 + e];
                    int ta, tb;
                    bgram_tile<WHICH>(tile, nta, ntb2, k4, ta, tb);
                    bgram_put<WHICH>(gp, k, kb, k4, ta + (uv >> 2), tb + (uv & 3), (double)sum);
                }
            }
        }
    }
}

// request r's piece partials: a block takes 32 entries; slice q (warp q of
// kBRedSlices) sums pieces q, q + kBRedSlices, ... in order, then the slices
// are added in order; grid (kBMax, entries / 32)
constexpr int kBRedSlices = kBThreads / 32;

template <int WHICH>
__global__ void __launch_bounds__(kBThreads) bk_gram_reduce(const BBatch *__restrict__ b) {
    __shared__ double part[kBRedSlices][32];
    const int r = blockIdx.x;
    if (r >= b->nr) return;
    const BDesc &d = b->d[r];
    if (!(d.flags & kBActive) || (WHICH == 0 && d.it == 0)) return;
    const int k = d.k, m = d.m, kb = k + (WHICH ? m : 0), tot = k * kb;
    const int e0 = blockIdx.y * 32;
    if (e0 >= tot) return;
    const int lane = threadIdx.x & 31, q = threadIdx.x >> 5;
    const int e = e0 + lane;
    const int a = e / kb, bb = e - a * kb;
    // upper triangle of the symmetric part only: the lower entries mirror it
    const bool want = e < tot && !(WHICH == 1 && bb < k && a > bb);
    double s = 0.0;
    if (want) {
        const double *p = d.gpart + e;
        const int np = d.npiece;
        int c = q;
        for (; c + 3 * kBRedSlices < np; c += 4 * kBRedSlices) {
            double v[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) v[u] = p[(size_t)(c + u * kBRedSlices) * tot];
#pragma unroll
            for (int u = 0; u < 4; ++u) s += v[u];
        }
        for (; c < np; c += kBRedSlices) s += p[(size_t)c * tot];
    }
    part[q][lane] = s;
    __syncthreads();
    if (q != 0 || !want) return;
    s = part[0][lane];
#pragma unroll
    for (int u = 1; u < kBRedSlices; ++u) s += part[u][lane];
    if (WHICH == 0) {
        d.QtAS[a * k + bb] = s;
    } else if (bb < k) {
        d.QtAQ[a * k + bb] = s;
        d.QtAQ[bb * k + a] = s;
    } else {
        d.QtR[a * m + (bb - k)] = s;
    }
}

// ------------------------------------------------------------ LU
// Crout factor of QtAQ, unit-diagonal U, no pivoting (src/DLSsolvers.c:125-145):
// F = the factors (k x k), the reciprocals of L's diagonal (k), the factors
// transposed (k x k, for the solves' column sweeps).  Step dd: warp 0 updates
// row dd + 1 and at once takes its pivot and scales it into U's row (the next
// step's critical path), while warps 1-7 update rows dd + 2 .. k - 1 as one
// flat range of (row, column) entries, so every FP64 instruction of the
// trailing update carries 32 useful lanes; one barrier a step.
__device__ __forceinline__ void blu_pivot_row(double *W, int k, int i, double *Dinv, int lane,
                                              int &bad) {
    double inv = 0.0;
    if (lane == 0) {
        const double piv = W[i * k + i];
        if (piv == 0.0 || !isfinite(piv)) bad = 1;
        inv = 1.0 / piv;
        Dinv[i] = inv;
    }
    inv = __shfl_sync(0xffffffffu, inv, 0);
    for (int c = i + 1 + lane; c < k; c += 32) W[i * k + c] *= inv;
}

__global__ void __launch_bounds__(kBThreads) bk_lu_factor(const BBatch *__restrict__ b) {
    __shared__ double W[kBMaxK * kBMaxK];
    const int r = blockIdx.x;
    if (r >= b->nr) return;
    const BDesc &d = b->d[r];
    if (!(d.flags & kBActive)) return;
    const int k = d.k, kk = k * k;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    for (int i = tid; i < kk; i += blockDim.x) W[i] = d.QtAQ[i];
    __syncthreads();
    double *Dinv = d.F + kk, *FT = d.F + kk + k;
    int bad = 0;
    if (warp == 0) blu_pivot_row(W, k, 0, Dinv, lane, bad);
    __syncthreads();
    for (int dd = 0; dd + 1 < k; ++dd) {
        const int x = k - dd - 1;  // trailing columns dd + 1 .. k - 1
        const double *U = W + dd * k;
        if (warp == 0) {
            double *wr = W + (dd + 1) * k;
            const double lid = wr[dd];
            for (int c = dd + 1 + lane; c < k; c += 32) wr[c] = wr[c] - lid * U[c];
            __syncwarp();
            blu_pivot_row(W, k, dd + 1, Dinv, lane, bad);
        } else {
            const uint32_t mg = bdiv_magic(x);
            for (int e = tid - 32; e < (x - 1) * x; e += kBThreads - 32) {
                const int q = bdiv(e, x, mg);
                double *wr = W + (dd + 2 + q) * k;
                const int c = dd + 1 + (e - q * x);
                wr[c] = wr[c] - wr[dd] * U[c];
            }
        }
        __syncthreads();
    }
    for (int e = tid; e < kk; e += blockDim.x) {
        const int i = e / k, jj = e - i * k;
        d.F[e] = W[e];
        FT[e] = W[jj * k + i];
    }
    if (bad) atomicOr(d.status, kStatusBreakdown);
}

// WHICH 0: beta = QtAQ_prev^{-1} QtAS (k columns); WHICH 1: alpha = QtAQ^{-1} QtR
// (m columns).  A warp solves one column by column sweeps (lane l holds rows
// l and l + 32): forward, y_i = z_i / L_ii through the reciprocal, then
// z_j -= L_ji y_i for j > i; backward with U's unit diagonal, z_j -= U_ji x_i
// for j < i (src/DLSsolvers.c:156-207).  The transposed factor in shared
// memory makes each step's reads of L_ji / U_ji contiguous over the lanes;
// the chain is 2k broadcasts and FMAs.
constexpr int kBLuWarps = 8;

template <int WHICH>
__global__ void __launch_bounds__(32 * kBLuWarps) bk_lu_solve(const BBatch *__restrict__ b) {
    extern __shared__ __align__(16) double bl_smem[];
    const int r = blockIdx.x;
    if (r >= b->nr) return;
    const BDesc &d = b->d[r];
    if (!(d.flags & kBActive) || (WHICH == 0 && d.it == 0)) return;
    const int k = d.k, kk = k * k;
    const int nrhs = WHICH == 0 ? k : d.m;
    const int c0 = blockIdx.y * kBLuWarps;
    if (c0 >= nrhs) return;
    double *Dinv = bl_smem, *FT = bl_smem + k;
    {
        const double *src = d.F + kk;  // 1 / L_ii, then the transposed factors
        for (int i = threadIdx.x; i < k + kk; i += blockDim.x) bl_smem[i] = src[i];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, c = c0 + (threadIdx.x >> 5);
    if (c >= nrhs) return;  // no block-wide barrier follows
    const double *RHS = WHICH == 0 ? d.QtAS : d.QtR;
    double *Y = WHICH == 0 ? d.beta : d.alpha;
    constexpr int TT = kBMaxK / 32;
    double z[TT];
#pragma unroll
    for (int t = 0; t < TT; ++t) {
        const int jj = lane + 32 * t;
        z[t] = jj < k ? RHS[(size_t)jj * nrhs + c] : 0.0;
    }
#pragma unroll
    for (int t = 0; t < TT; ++t) {
        for (int ii = 0; ii < 32; ++ii) {
            const int i = 32 * t + ii;
            if (i >= k) break;
            const double yi = __shfl_sync(0xffffffffu, z[t], ii) * Dinv[i];
            if (lane == ii) z[t] = yi;
            const double *col = FT + (size_t)i * k;
#pragma unroll
            for (int tt = t; tt < TT; ++tt) {
                const int jj = lane + 32 * tt;
                if (jj > i && jj < k) z[tt] = fma(-col[jj], yi, z[tt]);
            }
        }
    }
#pragma unroll
    for (int t = TT - 1; t >= 0; --t) {
        for (int ii = 31; ii >= 0; --ii) {
            const int i = 32 * t + ii;
            if (i >= k) continue;
            const double xi = __shfl_sync(0xffffffffu, z[t], ii);
            const double *col = FT + (size_t)i * k;
#pragma unroll
            for (int tt = 0; tt <= t; ++tt) {
                const int jj = lane + 32 * tt;
                if (jj < i) z[tt] = fma(-col[jj], xi, z[tt]);
            }
        }
    }
#pragma unroll
    for (int t = 0; t < TT; ++t) {
        const int jj = lane + 32 * t;
        if (jj < k) Y[(size_t)jj * nrhs + c] = z[t];
    }
}

// ------------------------------------------------------------ updates
// Q = S - Q_old beta, in place over S (requests past their first iteration).
// Q_old's rows go through shared memory bxsub rows at a time; beta (zero
// padded to a power-of-two number of 4-column groups G) stays in shared
// memory for the request.  A thread owns column group cg = tid mod G of two
// rows rpp apart (rpp = kBThreads / G): per 4 coefficients one 16-byte piece
// of each row and four of beta feed 32 FMAs.
template <typename T>
__global__ void __launch_bounds__(kBThreads, 3) bk_qupdate(const BBatch *__restrict__ b) {
    extern __shared__ __align__(16) unsigned char bq_smem[];
    constexpr int RS = bxsub<T>();
    T *Bs = reinterpret_cast<T *>(bq_smem);  // k4 x 4G
    T *Qs = Bs + kBMaxK * kBMaxK;              // RS x pk
    const int nr = b->nr, total = b->total_tiles;
    const int tid = threadIdx.x;
    int cur = -1;
    for (int t = blockIdx.x; t < total; t += gridDim.x) {
        const int r = bfind(b->tile_start, nr, t);
        const BDesc &d = b->d[r];
        if (!(d.flags & kBActive) || d.it == 0) continue;
        const int k = d.k, k4 = (k + 3) & ~3, pk = bpitch<T>(k);
        const int lgG = blog2_ceil(k4 >> 2), G = 1 << lgG, kq = 4 * G;
        if (r != cur) {
            __syncthreads();
            for (int i = tid; i < k4 * kq; i += kBThreads) {
                const int jj = i >> (lgG + 2), c = i & (kq - 1);
                Bs[i] = (jj < k && c < k) ? (T)d.beta[jj * k + c] : (T)0.0;
            }
            bzero_pad(Qs, pk, RS, k);
            cur = r;
        }
        const int64_t row0 = (int64_t)(t - b->tile_start[r]) * kBRows;
        const int rows = (int)min((int64_t)kBRows, d.n - row0);
        T *S = (T *)d.S;
        const T *Q = (const T *)d.Qold;
        const uint32_t mgk = bdiv_magic(k);
        const int cg = tid & (G - 1), rpp = kBThreads >> lgG;
        const T *bcol = Bs + 4 * cg;
        for (int s0 = 0; s0 < rows; s0 += RS) {
            const int sr = min(RS, rows - s0);
            __syncthreads();
            bstage(Qs, pk, Q + (row0 + s0) * k, sr, k, mgk);
            bstage_wait();
            __syncthreads();
            for (int lr = tid >> lgG; lr < sr; lr += 2 * rpp) {
                const bool two = lr + rpp < sr;
                const T *qa = Qs + lr * pk, *qb = two ? qa + rpp * pk : qa;
                // S's values first: their loads overlap the products
                T *sa = S + (row0 + s0 + lr) * k + 4 * cg, *sb = sa + (size_t)rpp * k;
                T s0v[4], s1v[4];
#pragma unroll
                for (int v = 0; v < 4; ++v) {
                    const bool in = 4 * cg + v < k;
                    s0v[v] = in ? sa[v] : (T)0.0;
                    s1v[v] = in && two ? sb[v] : (T)0.0;
                }
                T acc0[4] = {(T)0.0, (T)0.0, (T)0.0, (T)0.0};
                T acc1[4] = {(T)0.0, (T)0.0, (T)0.0, (T)0.0};
                for (int jj = 0; jj < k4; jj += 4) {
                    T va[4], vb[4];
                    ld4(qa + jj, va);
                    ld4(qb + jj, vb);
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        T bv[4];
                        ld4(bcol + (jj + u) * kq, bv);
#pragma unroll
                        for (int v = 0; v < 4; ++v) {
                            acc0[v] = fma(va[u], bv[v], acc0[v]);
                            acc1[v] = fma(vb[u], bv[v], acc1[v]);
                        }
                    }
                }
#pragma unroll
                for (int v = 0; v < 4; ++v)
                    if (4 * cg + v < k) sa[v] = s0v[v] - acc0[v];
                if (two)
#pragma unroll
                    for (int v = 0; v < 4; ++v)
                        if (4 * cg + v < k) sb[v] = s1v[v] - acc1[v];
            }
        }
    }
}

// X += Q alpha; R -= AQ alpha (products summed in the class's precision, the
// sums added to X and R in FP64); the next T_0 = R into Q_old; per-tile
// squared column norms of R into npart.  Q and AQ rows go through shared
// memory bxsub rows at a time; alpha (zero padded to a power-of-two number of
// 4-column groups G) stays in shared memory for the request.  A thread owns
// one row x columns 4 cg .. 4 cg + 3 (cg = tid mod G): per 4 coefficients a
// 16-byte piece of its Q row and of its AQ row and four of alpha feed 32 FMAs.
template <typename T>
__global__ void __launch_bounds__(kBThreads, 3) bk_xrupdate(const BBatch *__restrict__ b) {
    extern __shared__ __align__(16) unsigned char bx_smem[];
    __shared__ double Ws[kBThreads / 32][32];
    constexpr int RS = bxsub<T>();
    T *As = reinterpret_cast<T *>(bx_smem);  // k4 x 4G
    T *Qs = As + kBMaxK * kBMaxM;              // RS x pk
    T *AQs = Qs + RS * kBPitchK;               // RS x pk
    const int nr = b->nr, total = b->total_tiles;
    const int tid = threadIdx.x;
    int cur = -1;
    for (int t = blockIdx.x; t < total; t += gridDim.x) {
        const int r = bfind(b->tile_start, nr, t);
        const BDesc &d = b->d[r];
        if (!(d.flags & kBActive)) continue;
        const int k = d.k, m = d.m, k4 = (k + 3) & ~3, pk = bpitch<T>(k);
        const int lgG = blog2_ceil((m + 3) >> 2), G = 1 << lgG, mq = 4 * G;
        if (r != cur) {
            __syncthreads();
            for (int i = tid; i < k4 * mq; i += kBThreads) {
                const int jj = i >> (lgG + 2), c = i & (mq - 1);
                As[i] = (jj < k && c < m) ? (T)d.alpha[jj * m + c] : (T)0.0;
            }
            bzero_pad(Qs, pk, RS, k);
            bzero_pad(AQs, pk, RS, k);
            cur = r;
        }
        const int lt = t - b->tile_start[r];
        const int64_t row0 = (int64_t)lt * kBRows;
        const int rows = (int)min((int64_t)kBRows, d.n - row0);
        const T *Q = (const T *)d.S, *AQ = (const T *)d.AQ;
        T *T0 = (T *)d.Qold;
        double *X = d.X, *R = d.R;
        float *R32 = d.R32;
        const uint32_t mgk = bdiv_magic(k);
        const int cg = tid & (G - 1), c0 = 4 * cg;
        const T *acol = As + c0;
        double nsq[4] = {0.0, 0.0, 0.0, 0.0};
        for (int s0 = 0; s0 < rows; s0 += RS) {
            const int sr = min(RS, rows - s0);
            __syncthreads();
            bstage(Qs, pk, Q + (row0 + s0) * k, sr, k, mgk);
            bstage(AQs, pk, AQ + (row0 + s0) * k, sr, k, mgk);
            bstage_wait();
            __syncthreads();
            for (int lr = tid >> lgG; lr < sr; lr += kBThreads >> lgG) {
                const T *qp = Qs + lr * pk, *ap = AQs + lr * pk;
                const int64_t row = row0 + s0 + lr;
                // X's and R's values first: their loads overlap the products
                double xv[4], rv[4];
#pragma unroll
                for (int v = 0; v < 4; ++v) {
                    const bool in = c0 + v < m;
                    xv[v] = in ? X[row * m + c0 + v] : 0.0;
                    rv[v] = in ? R[row * m + c0 + v] : 0.0;
                }
                T xq[4] = {(T)0.0, (T)0.0, (T)0.0, (T)0.0};
                T ra[4] = {(T)0.0, (T)0.0, (T)0.0, (T)0.0};
                for (int jj = 0; jj < k4; jj += 4) {
                    T q[4], aq[4];
                    ld4(qp + jj, q);
                    ld4(ap + jj, aq);
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        T al[4];
                        ld4(acol + (jj + u) * mq, al);
#pragma unroll
                        for (int v = 0; v < 4; ++v) {
                            xq[v] = fma(q[u], al[v], xq[v]);
                            ra[v] = fma(aq[u], al[v], ra[v]);
                        }
                    }
                }
#pragma unroll
                for (int v = 0; v < 4; ++v) {
                    const int c = c0 + v;
                    if (c >= m) break;
                    X[row * m + c] = xv[v] + (double)xq[v];
                    const double rn = rv[v] - (double)ra[v];
                    R[row * m + c] = rn;
                    T0[row * k + c] = (T)rn;
                    if (R32) R32[row * m + c] = (float)rn;
                    nsq[v] = fma(rn, rn, nsq[v]);
                }
            }
        }
        bcolsum_store(nsq, G, m, Ws, d.npart + (size_t)lt * m);
    }
}

// norms[c] = the sum of request r's tile partials (requests with `flag`):
// warp c of the block, lane l summing tiles l, l + 32, ... in order, then a
// fixed butterfly over the lanes
__global__ void __launch_bounds__(32 * kBMaxM) bk_norm_reduce(const BBatch *__restrict__ b,
                                                             int flag) {
    const int r = blockIdx.x;
    if (r >= b->nr) return;
    const BDesc &d = b->d[r];
    const int c = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (!(d.flags & flag) || c >= d.m) return;
    const int m = d.m, nt = d.ntile;
    const double *p = d.npart + c;
    double s = 0.0;
    int t = lane;
    for (; t + 96 < nt; t += 128) {
        double v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) v[u] = p[(size_t)(t + 32 * u) * m];
#pragma unroll
        for (int u = 0; u < 4; ++u) s += v[u];
    }
    for (; t < nt; t += 32) s += p[(size_t)t * m];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) d.norms[c] = s;
}

// ------------------------------------------------------------ launchers
static int bgrid(const BTune &tu, int kind) {
    const int per = tu.blocks_per_sm[kind] > 0 ? tu.blocks_per_sm[kind] : 2;
    return per * sm_count();
}

template <typename T>
int bl_basis_step(cudaStream_t st, const BBatch *b, int j, const BTune &tu) {
    bk_spmm<T, 0><<<bgrid(tu, kBKSpmm), kBThreads, 0, st>>>(b, j);
    return check_launch();
}

template <typename T>
int bl_aq(cudaStream_t st, const BBatch *b, const BTune &tu) {
    bk_spmm<T, 1><<<bgrid(tu, kBKSpmm), kBThreads, 0, st>>>(b, 0);
    return check_launch();
}

template <typename T>
int bl_gram(cudaStream_t st, const BBatch *b, int which, const BTune &tu) {
    const int smem = (int)((size_t)bgchunk<T>() * (2 * kBPitchK + kBPitchM) * sizeof(T));
    static_assert(kBThreads * 16 <= bgchunk<T>() * (2 * kBPitchK + kBPitchM),
                  "the group scratch fits the staging area");
    if (which == 0) {
        set_smem_attr(bk_gram<T, 0>, smem);
        bk_gram<T, 0><<<bgrid(tu, kBKGram), kBThreads, smem, st>>>(b);
    } else {
        set_smem_attr(bk_gram<T, 1>, smem);
        bk_gram<T, 1><<<bgrid(tu, kBKGram), kBThreads, smem, st>>>(b);
    }
    int rc = check_launch();
    if (rc) return rc;
    const dim3 rg(kBMax, (kBMaxK * (kBMaxK + kBMaxM) + 31) / 32);
    if (which == 0)
        bk_gram_reduce<0><<<rg, kBThreads, 0, st>>>(b);
    else
        bk_gram_reduce<1><<<rg, kBThreads, 0, st>>>(b);
    return check_launch();
}

int bl_lu_factor(cudaStream_t st, const BBatch *b) {
    bk_lu_factor<<<kBMax, kBThreads, 0, st>>>(b);
    return check_launch();
}

int bl_lu_solve(cudaStream_t st, const BBatch *b, int which) {
    const int smem = (int)(sizeof(double) * ((size_t)kBMaxK * kBMaxK + kBMaxK));
    const dim3 grid(kBMax, (kBMaxK + kBLuWarps - 1) / kBLuWarps);
    if (which == 0) {
        set_smem_attr(bk_lu_solve<0>, smem);
        bk_lu_solve<0><<<grid, 32 * kBLuWarps, smem, st>>>(b);
    } else {
        set_smem_attr(bk_lu_solve<1>, smem);
        bk_lu_solve<1><<<grid, 32 * kBLuWarps, smem, st>>>(b);
    }
    return check_launch();
}

template <typename T>
int bl_qupdate(cudaStream_t st, const BBatch *b, const BTune &tu) {
    const int smem = (int)(sizeof(T) * ((size_t)kBMaxK * kBMaxK + (size_t)bxsub<T>() * kBPitchK));
    set_smem_attr(bk_qupdate<T>, smem);
    bk_qupdate<T><<<bgrid(tu, kBKQupd), kBThreads, smem, st>>>(b);
    return check_launch();
}

template <typename T>
int bl_xrupdate(cudaStream_t st, const BBatch *b, const BTune &tu) {
    const int smem =
        (int)(sizeof(T) * ((size_t)kBMaxK * kBMaxM + (size_t)2 * bxsub<T>() * kBPitchK));
    set_smem_attr(bk_xrupdate<T>, smem);
    bk_xrupdate<T><<<bgrid(tu, kBKXr), kBThreads, smem, st>>>(b);
    int rc = check_launch();
    if (rc) return rc;
    bk_norm_reduce<<<kBMax, 32 * kBMaxM, 0, st>>>(b, kBActive);
    return check_launch();
}

template <typename T>
int bl_residual(cudaStream_t st, const BBatch *b, const BTune &tu) {
    bk_residual<T><<<bgrid(tu, kBKXr), kBThreads, 0, st>>>(b);
    int rc = check_launch();
    if (rc) return rc;
    bk_norm_reduce<<<kBMax, 32 * kBMaxM, 0, st>>>(b, kBResid);
    return check_launch();
}

#define CACG_BATCH_INST(T)                                                           \
    template int bl_basis_step<T>(cudaStream_t, const BBatch *, int, const BTune &); \
    template int bl_aq<T>(cudaStream_t, const BBatch *, const BTune &);               \
    template int bl_gram<T>(cudaStream_t, const BBatch *, int, const BTune &);        \
    template int bl_qupdate<T>(cudaStream_t, const BBatch *, const BTune &);          \
    template int bl_xrupdate<T>(cudaStream_t, const BBatch *, const BTune &);         \
    template int bl_residual<T>(cudaStream_t, const BBatch *, const BTune &);
CACG_BATCH_INST(double)
CACG_BATCH_INST(float)
#undef CACG_BATCH_INST

}  // namespace cacg
