// k_batch.cu -- the serving engine's batched kernels (no reference
// counterpart: sclc/cacg solves one system per process, src/main.c:22-221).
//
// One launch per phase covers every admitted request of a precision class.
// Blocks stride over the class's tile table (batch.h): a row tile is kBRows
// consecutive rows of one request, a Gram chunk bchunk<T>() rows.  The work of
// a tile depends only on its own request's data, and every sum runs in a fixed
// order inside the tile (SpMM: the CSR row order; Gram: a fixed row-group
// split inside a chunk, then chunks in order; norms: rows in order inside a
// tile, then tiles in order), so results do not depend on the grid size or on
// which other requests share the launch.
//
// The operations are the reference iteration's (src/bcbcgKernel.c:172-526):
//   basis step j  T_j = 2a A T_{j-1} + 2b T_{j-1} - T_{j-2}   (src/common.c:182-249)
//   Gram          C = L^T [R1 | R2]                            (src/BLAS3.c:699-758)
//   LU            Crout, unit-diagonal U, no pivoting           (src/DLSsolvers.c:106-208)
//   Q update      Q = S - Q_old beta                            (src/BLAS3.c:794-825, 579-612)
//   X/R update    X += Q alpha, R -= AQ alpha, ||R(:,c)||^2     (src/bcbcgKernel.c:376-447)
//   residual      R = B - A X                                   (src/bcbcgKernel.c:136-154)
// FP64 class: every operand FP64.  FP32 class (the mixed mode): A, the basis,
// Q and AQ in FP32; the SpMMs, the Q update, the Gram sums inside a chunk and
// the X/R products in FP32; chunk partials, LU, X and R in FP64; residuals in
// FP64.  GB300's FP64 pipe runs at about 1/58 of the FP32 rate, so the FP32
// class keeps FP64 to the small dense work and the additions into X and R.
//
// No kernel here waits on another block or on an asynchronous copy.
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

// MODE 0: basis step j, Y = T_j (width m).  MODE 1: AQ = A Q (width k).
template <typename T, int MODE>
__global__ void __launch_bounds__(kBThreads) bk_spmm(const BBatch *__restrict__ b, int j) {
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
        const int32_t *rp = d.rp, *ci = d.ci;
        const int nout = rows * w;
        for (int e = threadIdx.x; e < nout; e += blockDim.x) {
            const int lr = e / w, c = e - lr * w;
            const int64_t row = row0 + lr;
            const int p1 = rp[row + 1];
            T acc = (T)0.0;
            for (int p = rp[row]; p < p1; ++p) acc = fma(val[p], X[(int64_t)ci[p] * k + c], acc);
            T y = ca * acc;
            if (MODE == 0) {
                y = fma(cb, X[row * k + c], y);
                if (Z2) y = fma(cc, Z2[row * k + c], y);
            }
            Y[row * k + c] = y;
        }
    }
}

// R = B - A X (FP64) for requests flagged kBResid; T_0 = R into S (and R32);
// per-tile squared column norms into npart.
template <typename T>
__global__ void __launch_bounds__(kBThreads) bk_residual(const BBatch *__restrict__ b) {
    const int nr = b->nr, total = b->total_tiles;
    for (int t = blockIdx.x; t < total; t += gridDim.x) {
        const int r = bfind(b->tile_start, nr, t);
        const BDesc &d = b->d[r];
        if (!(d.flags & kBResid)) continue;
        const int k = d.k, m = d.m;
        const int lt = t - b->tile_start[r];
        const int64_t row0 = (int64_t)lt * kBRows;
        const int rows = (int)min((int64_t)kBRows, d.n - row0);
        const int32_t *rp = d.rp, *ci = d.ci;
        const double *val = d.val, *X = d.X, *B = d.B;
        double *R = d.R;
        T *S = (T *)d.S;
        float *R32 = d.R32;
        for (int e = threadIdx.x; e < rows * m; e += blockDim.x) {
            const int lr = e / m, c = e - lr * m;
            const int64_t row = row0 + lr;
            const int p1 = rp[row + 1];
            double acc = 0.0;
            for (int p = rp[row]; p < p1; ++p) acc = fma(val[p], X[(int64_t)ci[p] * m + c], acc);
            const double rv = B[row * m + c] - acc;
            R[row * m + c] = rv;
            S[row * k + c] = (T)rv;
            if (R32) R32[row * m + c] = (float)rv;
        }
        __syncthreads();  // this tile's R, written by the block, is visible to it
        if ((int)threadIdx.x < m) {
            double sq = 0.0;
            for (int lr = 0; lr < rows; ++lr) {
                const double v = R[(row0 + lr) * m + threadIdx.x];
                sq = fma(v, v, sq);
            }
            d.npart[(size_t)lt * m + threadIdx.x] = sq;
        }
        __syncthreads();
    }
}

// WHICH 0: QtAS = AQ^T S (requests past their first iteration).
// WHICH 1: [QtAQ | QtR] = Q^T [AQ | R] (Q is the S buffer after the update).
// A block takes one chunk (bchunk<T>() rows): it copies the chunk's rows of
// both operands into shared memory with coalesced loads (one sync), then
// threads own 4 x 4 tiles of the (<= 64) x (<= 96) product; when the product
// has few tiles, G row groups (rows i = g mod G) run side by side and their
// sums are added in group order.  The chunk sums in the operands' precision
// (FP64 class: FP64; FP32 class: FP32 over 128 rows, the accuracy class of
// the single-request solver's tensor-core Gram, which sums 256-row groups in
// FP32); the chunk partials are summed in FP64, chunk by chunk.
constexpr int kBGT = 4;  // thread tile edge
// group sums: G x ka x kb <= (G x tiles) x 16 <= kBThreads x 16 entries
constexpr int kBGScratch = kBThreads * kBGT * kBGT;

__device__ __forceinline__ int bk_gram_groups(int ntiles) {
    int G = 1;
    while (G < 8 && ntiles * G * 2 <= kBThreads) G *= 2;
    return G;
}

template <typename T, int WHICH>
__global__ void __launch_bounds__(kBThreads) bk_gram(const BBatch *__restrict__ b) {
    extern __shared__ __align__(16) unsigned char bg_smem[];
    constexpr int CH = bchunk<T>();
    T *Ls = reinterpret_cast<T *>(bg_smem);     // CH x ka
    T *Rs = Ls + (size_t)CH * kBMaxK;             // CH x kb
    T *Sc = Rs + (size_t)CH * (kBMaxK + kBMaxM);  // G x ka x kb <= kBGScratch
    const int nr = b->nr, total = b->total_chunks;
    const int tid = threadIdx.x;
    for (int t = blockIdx.x; t < total; t += gridDim.x) {
        const int r = bfind(b->chunk_start, nr, t);
        const BDesc &d = b->d[r];
        if (!(d.flags & kBActive)) continue;
        if (WHICH == 0 && d.it == 0) continue;
        const int k = d.k, m = d.m;
        const int lc = t - b->chunk_start[r];
        const int64_t row0 = (int64_t)lc * CH;
        const int rows = (int)min((int64_t)CH, d.n - row0);
        const int ka = k, kb1 = k, kb2 = WHICH ? m : 0, kb = kb1 + kb2;
        const T *L = (const T *)(WHICH == 0 ? d.AQ : d.S);
        const T *R1 = (const T *)(WHICH == 0 ? d.S : d.AQ);
        const T *R2 = nullptr;
        if (WHICH == 1) R2 = std::is_same<T, float>::value ? (const T *)(const void *)d.R32
                                                             : (const T *)(const void *)d.R;
        __syncthreads();  // the previous chunk's readers are done with Ls, Rs, Sc
        {
            const T *Lc = L + row0 * k, *R1c = R1 + row0 * k;
            for (int idx = tid; idx < rows * k; idx += kBThreads) {
                const int i = idx / k, c = idx - i * k;
                Ls[i * ka + c] = Lc[idx];
                Rs[i * kb + c] = R1c[idx];
            }
            if (WHICH == 1) {
                const T *R2c = R2 + row0 * m;
                for (int idx = tid; idx < rows * m; idx += kBThreads) {
                    const int i = idx / m, c = idx - i * m;
                    Rs[i * kb + kb1 + c] = R2c[idx];
                }
            }
        }
        __syncthreads();
        const int nta = (ka + kBGT - 1) / kBGT, ntb = (kb + kBGT - 1) / kBGT;
        const int ntiles = nta * ntb;
        const int G = bk_gram_groups(ntiles);
        double *gp = d.gpart + (size_t)lc * ka * kb;
        // thread w: row group w / ntiles, tile w % ntiles (G = 1: tiles w, w + 256, ...)
        const int nwork = G == 1 ? ntiles : ntiles * G;
        for (int w = tid; w < nwork; w += kBThreads) {
            const int grp = w / ntiles, tile = w - grp * ntiles;
            const int a0 = (tile / ntb) * kBGT, b0 = (tile % ntb) * kBGT;
            T acc[kBGT][kBGT];
#pragma unroll
            for (int u = 0; u < kBGT; ++u)
#pragma unroll
                for (int v = 0; v < kBGT; ++v) acc[u][v] = (T)0.0;
            for (int i = grp; i < rows; i += G) {
                T lv[kBGT], rv[kBGT];
#pragma unroll
                for (int u = 0; u < kBGT; ++u) lv[u] = a0 + u < ka ? Ls[i * ka + a0 + u] : (T)0.0;
#pragma unroll
                for (int v = 0; v < kBGT; ++v) rv[v] = b0 + v < kb ? Rs[i * kb + b0 + v] : (T)0.0;
#pragma unroll
                for (int u = 0; u < kBGT; ++u)
#pragma unroll
                    for (int v = 0; v < kBGT; ++v) acc[u][v] = fma(lv[u], rv[v], acc[u][v]);
            }
            // G > 1: each group's sums go to the scratch area after Rs
#pragma unroll
            for (int u = 0; u < kBGT; ++u)
#pragma unroll
                for (int v = 0; v < kBGT; ++v)
                    if (a0 + u < ka && b0 + v < kb) {
                        if (G == 1)
                            gp[(a0 + u) * kb + b0 + v] = (double)acc[u][v];
                        else
                            Sc[(size_t)grp * ka * kb + (a0 + u) * kb + b0 + v] = acc[u][v];
                    }
        }
        if (G > 1) {
            __syncthreads();
            for (int e = tid; e < ka * kb; e += kBThreads) {
                T sum = Sc[e];
                for (int g = 1; g < G; ++g) sum += Sc[(size_t)g * ka * kb + e];
                gp[e] = (double)sum;
            }
        }
    }
}

// request r's chunk partials, summed in chunk order; grid (kBMax, entries / 256)
template <int WHICH>
__global__ void __launch_bounds__(kBThreads) bk_gram_reduce(const BBatch *__restrict__ b) {
    const int r = blockIdx.x;
    if (r >= b->nr) return;
    const BDesc &d = b->d[r];
    if (!(d.flags & kBActive) || (WHICH == 0 && d.it == 0)) return;
    const int k = d.k, m = d.m, kb = k + (WHICH ? m : 0), tot = k * kb;
    const int e = blockIdx.y * blockDim.x + threadIdx.x;
    if (e >= tot) return;
    const double *p = d.gpart + e;
    const int nch = d.nchunk;
    double s = 0.0;
    int c = 0;
    for (; c + 4 <= nch; c += 4) {
        const double v0 = p[(size_t)c * tot], v1 = p[(size_t)(c + 1) * tot],
                     v2 = p[(size_t)(c + 2) * tot], v3 = p[(size_t)(c + 3) * tot];
        s += v0;
        s += v1;
        s += v2;
        s += v3;
    }
    for (; c < nch; ++c) s += p[(size_t)c * tot];
    const int a = e / kb, bb = e - a * kb;
    if (WHICH == 0)
        d.QtAS[a * k + bb] = s;
    else if (bb < k)
        d.QtAQ[a * k + bb] = s;
    else
        d.QtR[a * m + (bb - k)] = s;
}

// Crout factor of QtAQ, unit-diagonal U, no pivoting (src/DLSsolvers.c:125-145):
// F = the factors (k x k) then the reciprocals of L's diagonal (k).
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
    double *Dinv = d.F + kk;
    int bad = 0;
    for (int dd = 0; dd < k; ++dd) {
        if (warp == 0) {
            double inv = 0.0;
            if (lane == 0) {
                const double piv = W[dd * k + dd];
                if (piv == 0.0 || !isfinite(piv)) bad = 1;
                inv = 1.0 / piv;
                Dinv[dd] = inv;
            }
            inv = __shfl_sync(0xffffffffu, inv, 0);
            for (int c = dd + 1 + lane; c < k; c += 32) W[dd * k + c] *= inv;
        }
        __syncthreads();
        for (int i = dd + 1 + warp; i < k; i += kBThreads / 32) {
            const double lid = W[i * k + dd];
            for (int c = dd + 1 + lane; c < k; c += 32) W[i * k + c] = W[i * k + c] - lid * W[dd * k + c];
        }
        __syncthreads();
    }
    for (int i = tid; i < kk; i += blockDim.x) d.F[i] = W[i];
    if (tid == 0 && bad) atomicOr(d.status, kStatusBreakdown);
}

// WHICH 0: beta = QtAQ_prev^{-1} QtAS (k columns); WHICH 1: alpha = QtAQ^{-1} QtR
// (m columns).  The solves are FP64 work of k^2 FMAs per column, and GB300's
// FP64 pipe does about two FMAs per clock per SM, so a request's columns are
// spread over blocks (grid y, kBLuCols columns each).  A block holds the
// factor and its columns (column-major) in shared memory; a warp sweeps one
// column: for each row the lanes take strided parts of the dot product with
// the solved entries and a butterfly of shuffles adds them (a fixed order),
// then lane 0 finishes the entry -- forward substitution through the
// reciprocals of L's diagonal, back substitution with U's unit diagonal
// (src/DLSsolvers.c:156-207).
constexpr int kBLuCols = 4;

__device__ __forceinline__ double bwarp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <int WHICH>
__global__ void __launch_bounds__(32 * kBLuCols) bk_lu_solve(const BBatch *__restrict__ b) {
    extern __shared__ __align__(16) double bl_smem[];
    const int r = blockIdx.x;
    if (r >= b->nr) return;
    const BDesc &d = b->d[r];
    if (!(d.flags & kBActive) || (WHICH == 0 && d.it == 0)) return;
    const int k = d.k, kk = k * k;
    const int nrhs = WHICH == 0 ? k : d.m;
    const int c0 = blockIdx.y * kBLuCols;
    if (c0 >= nrhs) return;
    const int nc = min(kBLuCols, nrhs - c0);
    const double *RHS = WHICH == 0 ? d.QtAS : d.QtR;
    double *Y = WHICH == 0 ? d.beta : d.alpha;
    double *Fs = bl_smem, *Yt = bl_smem + kk + k;  // Yt: nc columns of k
    for (int i = threadIdx.x; i < kk + k; i += blockDim.x) Fs[i] = d.F[i];
    for (int i = threadIdx.x; i < k * nc; i += blockDim.x) {
        const int cl = i / k, row = i - cl * k;
        Yt[i] = RHS[row * nrhs + c0 + cl];
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp < nc) {
        double *y = Yt + warp * k;
        for (int i = 0; i < k; ++i) {
            double part = 0.0;
            for (int jj = lane; jj < i; jj += 32) part = fma(Fs[i * k + jj], y[jj], part);
            const double dot = bwarp_sum(part);
            if (lane == 0) y[i] = (y[i] - dot) * Fs[kk + i];
            __syncwarp();
        }
        for (int i = k - 1; i >= 0; --i) {
            double part = 0.0;
            for (int jj = i + 1 + lane; jj < k; jj += 32) part = fma(Fs[i * k + jj], y[jj], part);
            const double dot = bwarp_sum(part);
            if (lane == 0) y[i] = y[i] - dot;
            __syncwarp();
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < k * nc; i += blockDim.x) {
        const int cl = i / k, row = i - cl * k;
        Y[row * nrhs + c0 + cl] = Yt[i];
    }
}

// Q = S - Q_old beta, in place over S (requests past their first iteration).
// A row tile goes through shared memory kBSub rows at a time (coalesced
// copies of Q_old's rows); beta sits in shared memory for the request.
constexpr int kBSub = 32;

template <typename T>
__global__ void __launch_bounds__(kBThreads) bk_qupdate(const BBatch *__restrict__ b) {
    __shared__ T Bs[kBMaxK * kBMaxK];
    __shared__ T Qs[kBSub * kBMaxK];
    const int nr = b->nr, total = b->total_tiles;
    int cur = -1;
    for (int t = blockIdx.x; t < total; t += gridDim.x) {
        const int r = bfind(b->tile_start, nr, t);
        const BDesc &d = b->d[r];
        if (!(d.flags & kBActive) || d.it == 0) continue;
        const int k = d.k;
        if (r != cur) {
            __syncthreads();
            for (int i = threadIdx.x; i < k * k; i += blockDim.x) Bs[i] = (T)d.beta[i];
            cur = r;
        }
        const int64_t row0 = (int64_t)(t - b->tile_start[r]) * kBRows;
        const int rows = (int)min((int64_t)kBRows, d.n - row0);
        T *S = (T *)d.S;
        const T *Q = (const T *)d.Qold;
        for (int s0 = 0; s0 < rows; s0 += kBSub) {
            const int sr = min(kBSub, rows - s0);
            __syncthreads();
            const T *Qc = Q + (row0 + s0) * k;
            for (int idx = threadIdx.x; idx < sr * k; idx += blockDim.x) Qs[idx] = Qc[idx];
            __syncthreads();
            T *Sc = S + (row0 + s0) * k;
            for (int e = threadIdx.x; e < sr * k; e += blockDim.x) {
                const int lr = e / k, c = e - lr * k;
                T acc = (T)0.0;
                for (int jj = 0; jj < k; ++jj) acc = fma(Qs[lr * k + jj], Bs[jj * k + c], acc);
                Sc[e] = Sc[e] - acc;
            }
        }
    }
}

// X += Q alpha; R -= AQ alpha (products summed in the class's precision, the
// sums added to X and R in FP64); the next T_0 = R into Q_old; per-tile
// squared column norms of R into npart.  Q and AQ rows go through shared
// memory kBSub rows at a time.
template <typename T>
__global__ void __launch_bounds__(kBThreads) bk_xrupdate(const BBatch *__restrict__ b) {
    __shared__ T As[kBMaxK * kBMaxM];
    __shared__ T Qs[kBSub * kBMaxK];
    __shared__ T AQs[kBSub * kBMaxK];
    const int nr = b->nr, total = b->total_tiles;
    int cur = -1;
    for (int t = blockIdx.x; t < total; t += gridDim.x) {
        const int r = bfind(b->tile_start, nr, t);
        const BDesc &d = b->d[r];
        if (!(d.flags & kBActive)) continue;
        const int k = d.k, m = d.m;
        if (r != cur) {
            __syncthreads();
            for (int i = threadIdx.x; i < k * m; i += blockDim.x) As[i] = (T)d.alpha[i];
            cur = r;
        }
        const int lt = t - b->tile_start[r];
        const int64_t row0 = (int64_t)lt * kBRows;
        const int rows = (int)min((int64_t)kBRows, d.n - row0);
        const T *Q = (const T *)d.S, *AQ = (const T *)d.AQ;
        T *T0 = (T *)d.Qold;
        double *X = d.X, *R = d.R;
        float *R32 = d.R32;
        for (int s0 = 0; s0 < rows; s0 += kBSub) {
            const int sr = min(kBSub, rows - s0);
            __syncthreads();
            const T *Qc = Q + (row0 + s0) * k, *AQc = AQ + (row0 + s0) * k;
            for (int idx = threadIdx.x; idx < sr * k; idx += blockDim.x) {
                Qs[idx] = Qc[idx];
                AQs[idx] = AQc[idx];
            }
            __syncthreads();
            for (int e = threadIdx.x; e < sr * m; e += blockDim.x) {
                const int lr = e / m, c = e - lr * m;
                const int64_t row = row0 + s0 + lr;
                T xq = (T)0.0, ra = (T)0.0;
                for (int jj = 0; jj < k; ++jj) {
                    const T a = As[jj * m + c];
                    xq = fma(Qs[lr * k + jj], a, xq);
                    ra = fma(AQs[lr * k + jj], a, ra);
                }
                X[row * m + c] += (double)xq;
                const double rn = R[row * m + c] - (double)ra;
                R[row * m + c] = rn;
                T0[row * k + c] = (T)rn;
                if (R32) R32[row * m + c] = (float)rn;
            }
        }
        __syncthreads();  // this tile's R, written by the block, is visible to it
        if ((int)threadIdx.x < m) {
            double sq = 0.0;
            for (int lr = 0; lr < rows; ++lr) {
                const double v = R[(row0 + lr) * m + threadIdx.x];
                sq = fma(v, v, sq);
            }
            d.npart[(size_t)lt * m + threadIdx.x] = sq;
        }
    }
}

// norms[c] = sum of request r's tile partials in tile order (requests with `flag`)
__global__ void bk_norm_reduce(const BBatch *__restrict__ b, int flag) {
    const int r = blockIdx.x;
    if (r >= b->nr) return;
    const BDesc &d = b->d[r];
    if (!(d.flags & flag) || (int)threadIdx.x >= d.m) return;
    double s = 0.0;
    for (int t = 0; t < d.ntile; ++t) s += d.npart[(size_t)t * d.m + threadIdx.x];
    d.norms[threadIdx.x] = s;
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
    const int smem =
        (int)(((size_t)bchunk<T>() * (kBMaxK + kBMaxK + kBMaxM) + kBGScratch) * sizeof(T));
    if (which == 0) {
        set_smem_attr(bk_gram<T, 0>, smem);
        bk_gram<T, 0><<<bgrid(tu, kBKGram), kBThreads, smem, st>>>(b);
    } else {
        set_smem_attr(bk_gram<T, 1>, smem);
        bk_gram<T, 1><<<bgrid(tu, kBKGram), kBThreads, smem, st>>>(b);
    }
    int rc = check_launch();
    if (rc) return rc;
    const dim3 rg(kBMax, (kBMaxK * (kBMaxK + kBMaxM) + kBThreads - 1) / kBThreads);
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
    const int smem = (int)(sizeof(double) * ((size_t)kBMaxK * kBMaxK + kBMaxK + (size_t)kBLuCols * kBMaxK));
    const dim3 grid(kBMax, kBMaxK / kBLuCols);
    if (which == 0)
        bk_lu_solve<0><<<grid, 32 * kBLuCols, smem, st>>>(b);
    else
        bk_lu_solve<1><<<grid, 32 * kBLuCols, smem, st>>>(b);
    return check_launch();
}

template <typename T>
int bl_qupdate(cudaStream_t st, const BBatch *b, const BTune &tu) {
    bk_qupdate<T><<<bgrid(tu, kBKQupd), kBThreads, 0, st>>>(b);
    return check_launch();
}

template <typename T>
int bl_xrupdate(cudaStream_t st, const BBatch *b, const BTune &tu) {
    bk_xrupdate<T><<<bgrid(tu, kBKXr), kBThreads, 0, st>>>(b);
    int rc = check_launch();
    if (rc) return rc;
    bk_norm_reduce<<<kBMax, kBMaxM, 0, st>>>(b, kBActive);
    return check_launch();
}

template <typename T>
int bl_residual(cudaStream_t st, const BBatch *b, const BTune &tu) {
    bk_residual<T><<<bgrid(tu, kBKXr), kBThreads, 0, st>>>(b);
    int rc = check_launch();
    if (rc) return rc;
    bk_norm_reduce<<<kBMax, kBMaxM, 0, st>>>(b, kBResid);
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
