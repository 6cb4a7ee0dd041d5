// k_dia.cu -- diagonal (DIA) view of CSR matrices whose nonzeros lie on a few
// diagonals, and the SpMM with the Chebyshev recurrence fused in over it.
//
// Reference operations replaced (sclc/cacg): the same products as k_spmm.cu
// (spmm_csr_v1 src/BLAS3.c:20-155, spmm_csr_info_data_sep_BCBCG
// src/BLAS3.c:913-976, and the basis axpbys src/BLAS3.c:828-847, 978-994);
// the reference has only CSR.
//
// Why: on stencil matrices every nonzero of a CSR row is one gather of a
// whole X row; on GB300 the L1 data pipe, not HBM, then bounds the SpMM
// (one L1 wavefront per gathered row piece).  Rows i and i+1 of a stencil
// touch X rows shifted by one, so over the diagonals, X rows are reusable in
// registers: a thread owns R = 8 consecutive rows x one 16-byte column chunk
// and walks groups of adjacent diagonals (offsets o, o+1, ..., at most
// kDiaGroupMax) with a register window of R + G - 1 X rows, loading each X row
// once per group instead of once per nonzero (27-point stencil: 11.25 row
// loads per output row instead of 27).  The value stream also shrinks: no
// column indices (FP32 values only in the mixed mode).
//
// Exactness: for every row the FMAs run over the diagonals in increasing
// offset = increasing column order, the order of the CSR kernel on sorted
// rows; a diagonal a row does not have contributes fma(0, x, acc) == acc for
// finite x.  So DIA and CSR results agree bit for bit.
//
// The view is built when the matrix is created: a device pass collects the
// exact set of offsets (hash tables in shared, then global memory); with at
// most kDiaMax of them and <= 1.5x padding a second pass checks every row
// (sorted, no duplicates) and scatters the values; anything else keeps the
// matrix CSR-only.
#include <algorithm>
#include <set>
#include <type_traits>
#include <vector>

#include "cacg_internal.cuh"
#include "cacg_solver.h"
#include "ff_util.cuh"

namespace cacg {

constexpr int kDiaR = 8;          // rows per thread (register window)
constexpr int kDiaThreads = 256;

// -------------------------------------------------------------- build
__global__ void dia_fill_kernel(int64_t n, int64_t npad, const int32_t *__restrict__ rp,
                                const int32_t *__restrict__ ci, const double *__restrict__ val,
                                DiaDesc desc, double *__restrict__ v64, float *__restrict__ v32,
                                int *__restrict__ bad) {
    for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < n;
         row += (int64_t)gridDim.x * blockDim.x) {
        const int b = rp[row], e = rp[row + 1];
        int d = 0;
        int64_t prev = -1;
        for (int p = b; p < e; ++p) {
            const int64_t c = ci[p];
            if (c <= prev || c < 0 || c >= n) {
                atomicOr(bad, 1);  // unsorted, duplicate or out of range
                return;
            }
            prev = c;
            const int64_t off = c - row;
            while (d < desc.ndiag && desc.off[d] < off) ++d;  // offsets sorted, columns sorted
            if (d == desc.ndiag || desc.off[d] != off) {
                atomicOr(bad, 2);  // offset outside the candidate set
                return;
            }
            v64[(size_t)d * npad + row] = val[p];
            if (v32) {  // FP32 view: hi, then lo = val - hi (float-float residuals)
                const float hi = (float)val[p];
                v32[(size_t)d * npad + row] = hi;
                v32[(size_t)desc.ndiag * npad + (size_t)d * npad + row] =
                    (float)(val[p] - (double)hi);
            }
        }
    }
}

// Exact set of diagonal offsets (col - row): each block hashes its rows'
// offsets into a shared-memory table (linear probing, bounded), then merges
// its distinct keys into a global table; *full is set when a table overflows.
constexpr int kOffTab = 128;
constexpr unsigned long long kOffEmpty = 0ull;
constexpr unsigned long long kOffBias = 1ull << 62;  // key = offset + bias, never 0

__device__ __forceinline__ bool off_insert(unsigned long long *tab, unsigned long long key) {
    unsigned h = (unsigned)((key * 0x9E3779B97F4A7C15ull) >> 57) & (kOffTab - 1);
    for (int probe = 0; probe < kOffTab; ++probe) {
        const unsigned long long v = *(volatile unsigned long long *)&tab[h];
        if (v == key) return true;
        if (v == kOffEmpty) {
            const unsigned long long prev = atomicCAS(&tab[h], kOffEmpty, key);
            if (prev == kOffEmpty || prev == key) return true;
        }
        h = (h + 1) & (kOffTab - 1);
    }
    return false;
}

__global__ void dia_offsets_kernel(int64_t n, const int32_t *__restrict__ rp,
                                   const int32_t *__restrict__ ci, unsigned long long *gtab,
                                   int *full) {
    __shared__ unsigned long long tab[kOffTab];
    for (int i = threadIdx.x; i < kOffTab; i += blockDim.x) tab[i] = kOffEmpty;
    __syncthreads();
    bool ok = true;
    for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < n && ok;
         row += (int64_t)gridDim.x * blockDim.x) {
        const int b = rp[row], e = rp[row + 1];
        for (int p = b; p < e && ok; ++p)
            ok = off_insert(tab, (unsigned long long)((int64_t)ci[p] - row) + kOffBias);
    }
    if (!ok) atomicOr(full, 1);
    __syncthreads();
    for (int i = threadIdx.x; i < kOffTab; i += blockDim.x) {
        const unsigned long long k = tab[i];
        if (k != kOffEmpty && !off_insert(gtab, k)) atomicOr(full, 1);
    }
}

int DevMatrix::build_dia(const cacg_csr *A, bool want_f32, cudaStream_t st) {
    dia_ndiag = 0;
    const int64_t n = A->n;
    if (n < 1 || A->nnz < 1) return CACG_OK;
    // a view needs at most kDiaMax diagonals with modest padding: n * nd <= 1.5 nnz
    if ((double)n > 1.5 * (double)A->nnz + 64.0) return CACG_OK;
    std::set<int64_t> offs;
    {
        unsigned long long *gtab = nullptr;
        CACG_CUDA_TRY(cudaMallocAsync((void **)&gtab, kOffTab * 8 + 16, st));
        int *gfull = reinterpret_cast<int *>(gtab + kOffTab);
        CACG_CUDA_TRY(cudaMemsetAsync(gtab, 0, kOffTab * 8 + 16, st));
        const int blocks = (int)std::min<int64_t>((n + 255) / 256, (int64_t)sm_count() * 8);
        dia_offsets_kernel<<<blocks, 256, 0, st>>>(n, rp, ci, gtab, gfull);
        int rc = check_launch();
        unsigned long long h[kOffTab + 2];
        if (rc == CACG_OK &&
            (cudaMemcpyAsync(h, gtab, kOffTab * 8 + 16, cudaMemcpyDeviceToHost, st) !=
                 cudaSuccess ||
             cudaStreamSynchronize(st) != cudaSuccess))
            rc = CACG_ERR_CUDA;
        cudaFreeAsync(gtab, st);
        if (rc != CACG_OK) return rc;
        if (*reinterpret_cast<int *>(&h[kOffTab])) return CACG_OK;  // more than 128 offsets
        for (int i = 0; i < kOffTab; ++i)
            if (h[i] != kOffEmpty) offs.insert((int64_t)(h[i] - kOffBias));
        if ((int)offs.size() > kDiaMax) return CACG_OK;
    }
    const int nd = (int)offs.size();
    if (nd == 0) return CACG_OK;
    // keep the view only when padding is modest
    if ((double)nd * (double)n > 1.5 * (double)A->nnz + 64.0) return CACG_OK;
    DiaDesc desc{};
    desc.ndiag = nd;
    int i = 0;
    for (int64_t o : offs) desc.off[i++] = o;
    // groups of adjacent offsets, at most kDiaGroupMax each
    desc.ngroups = 0;
    for (int d = 0; d < nd;) {
        int g = 1;
        while (d + g < nd && g < kDiaGroupMax && desc.off[d + g] == desc.off[d] + g) ++g;
        desc.gstart[desc.ngroups++] = d;
        d += g;
    }
    desc.gstart[desc.ngroups] = nd;
    const int64_t npad = (n + kDiaR - 1) / kDiaR * kDiaR + kDiaR;
    const size_t b64 = (size_t)nd * npad * 8, b32 = want_f32 ? (size_t)2 * nd * npad * 4 : 0;
    double *v64 = nullptr;
    float *v32 = nullptr;
    int *bad = nullptr;
    if (cudaMallocAsync((void **)&v64, b64, st) != cudaSuccess) {
        cudaGetLastError();
        return CACG_OK;  // no room for the view: CSR only
    }
    if (want_f32 && cudaMallocAsync((void **)&v32, b32, st) != cudaSuccess) {
        cudaGetLastError();
        cudaFreeAsync(v64, st);
        return CACG_OK;
    }
    CACG_CUDA_TRY(cudaMallocAsync((void **)&bad, sizeof(int), st));
    CACG_CUDA_TRY(cudaMemsetAsync(v64, 0, b64, st));
    if (v32) CACG_CUDA_TRY(cudaMemsetAsync(v32, 0, b32, st));
    CACG_CUDA_TRY(cudaMemsetAsync(bad, 0, sizeof(int), st));
    const int blocks = (int)std::min<int64_t>((n + 255) / 256, (int64_t)sm_count() * 16);
    dia_fill_kernel<<<blocks, 256, 0, st>>>(n, npad, rp, ci, val, desc, v64, v32, bad);
    int rc = check_launch();
    int hbad = 1;
    if (rc == CACG_OK) {
        if (cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            rc = CACG_ERR_CUDA;
    }
    cudaFreeAsync(bad, st);
    if (rc != CACG_OK || hbad) {
        cudaFreeAsync(v64, st);
        if (v32) cudaFreeAsync(v32, st);
        return rc;
    }
    dia = desc;
    dia_npad = npad;
    dia64 = v64;
    dia32 = v32;
    dia32lo = v32 ? v32 + (size_t)nd * npad : nullptr;
    dia_ndiag = nd;
    owned_bytes += b64 + b32;
    return CACG_OK;
}

// -------------------------------------------------------------- float-float
__global__ void ff_split_kernel(int64_t count, const double *__restrict__ x,
                                float *__restrict__ hi, float *__restrict__ lo) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
         i += (int64_t)gridDim.x * blockDim.x) {
        float h, l;
        ff_split_bits(x[i], h, l);
        hi[i] = h;
        lo[i] = l;
    }
}

int launch_ff_split(cudaStream_t st, int64_t count, const double *x, float *hi, float *lo) {
    if (count <= 0) return CACG_OK;
    const int blocks = (int)std::min<int64_t>((count + 255) / 256, (int64_t)sm_count() * 16);
    ff_split_kernel<<<blocks, 256, 0, st>>>(count, x, hi, lo);
    return check_launch();
}

// x = hi + lo in FP64 (the float-float state back to FP64: exact widenings,
// one rounding)
__global__ void ff_join_kernel(int64_t count, const float *__restrict__ hi,
                               const float *__restrict__ lo, double *__restrict__ x) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
         i += (int64_t)gridDim.x * blockDim.x)
        x[i] = ff_widen(hi[i]) + ff_widen(lo[i]);
}

int launch_ff_join(cudaStream_t st, int64_t count, const float *hi, const float *lo, double *x) {
    if (count <= 0) return CACG_OK;
    const int blocks = (int)std::min<int64_t>((count + 255) / 256, (int64_t)sm_count() * 16);
    ff_join_kernel<<<blocks, 256, 0, st>>>(count, hi, lo, x);
    return check_launch();
}

// FP32 hi/lo view from the FP64 view (matrices created without FP32 values)
__global__ void dia_hilo_kernel(int64_t count, const double *__restrict__ v64,
                                float *__restrict__ hi, float *__restrict__ lo) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
         i += (int64_t)gridDim.x * blockDim.x) {
        const float h = (float)v64[i];
        hi[i] = h;
        lo[i] = (float)(v64[i] - (double)h);
    }
}

int launch_dia_hilo(cudaStream_t st, int64_t count, const double *v64, float *hi, float *lo) {
    const int blocks = (int)std::min<int64_t>((count + 255) / 256, (int64_t)sm_count() * 16);
    dia_hilo_kernel<<<blocks, 256, 0, st>>>(count, v64, hi, lo);
    return check_launch();
}

// -------------------------------------------------------------- SpMM
// Y = ca * A X + cb * Z1 + cc * Z2 over the DIA view.  Thread = (run of R
// consecutive rows, column chunk of CW values); chunks of a row are adjacent
// lanes.  A CTA owns blocks of BR = runs_per_block * R rows; the values of
// all diagonals for its next block stream into shared memory (cp.async, two
// buffers) while it computes the current one, so the per-group wait is only
// for the X window (L2-resident neighbourhood).  R == 1 is the plain per-row
// variant (coalesced along rows, values straight from global memory).
__device__ __forceinline__ void dia_cp16(void *smem, const void *g, int bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(
                     (unsigned)__cvta_generic_to_shared(smem)),
                 "l"(g), "r"(bytes));
}

template <typename T, int R, int CW>
__global__ void __launch_bounds__(kDiaThreads, R <= 4 ? 3 : 2)
    dia_spmm_kernel(int64_t n, int64_t npad, DiaDesc desc, const T *__restrict__ vals, int cpr,
                    int runs_per_block, const T *__restrict__ X, int64_t ldx, T *__restrict__ Y,
                    int64_t ldy, const T *__restrict__ Z1, int64_t ldz1,
                    const T *__restrict__ Z2, int64_t ldz2, T ca, T cb, T cc) {
    constexpr int W = R + kDiaGroupMax - 1;  // register window rows
    constexpr int VN = 16 / (int)sizeof(T);
    extern __shared__ __align__(16) unsigned char dia_smem[];
    T *vs = reinterpret_cast<T *>(dia_smem);  // [2][ndiag][BR] when R > 1
    const int lr = threadIdx.x / cpr, c = threadIdx.x % cpr;
    const bool active = lr < runs_per_block;
    const int BR = runs_per_block * R;
    const int64_t nblk = (n + BR - 1) / BR;
    const int nd = desc.ndiag;

    auto stage = [&](int64_t blk, int buf) {
        if constexpr (R > 1) {
            if (blk < nblk) {
                T *dst = vs + (size_t)buf * nd * BR;
                const int per = BR / VN;  // 16-byte chunks per diagonal
                // (d, q) walks idx = tid, tid + blockDim, ... without a division per chunk
                const int dstep = blockDim.x / per, qstep = blockDim.x % per;
                int d = threadIdx.x / per, q = threadIdx.x % per;
                for (; d < nd; d += dstep, q += qstep) {
                    if (q >= per) {
                        q -= per;
                        ++d;
                        if (d >= nd) break;
                    }
                    const int64_t e0 = blk * BR + (int64_t)q * VN;
                    const int64_t left = npad - e0;
                    const int by = left >= VN ? 16 : (left > 0 ? (int)left * (int)sizeof(T) : 0);
                    dia_cp16(dst + (size_t)d * BR + q * VN,
                             by ? (const void *)(vals + (size_t)d * npad + e0) : vals, by);
                }
            }
            asm volatile("cp.async.commit_group;\n" ::);
        }
    };

    int buf = 0;
    stage(blockIdx.x, 0);
    for (int64_t blk = blockIdx.x; blk < nblk; blk += gridDim.x, buf ^= 1) {
        if constexpr (R > 1) {
            stage(blk + gridDim.x, buf ^ 1);
            asm volatile("cp.async.wait_group 1;\n" ::: "memory");
            __syncthreads();
        }
        if (active) {
            const int64_t r0 = blk * BR + (int64_t)lr * R;
            T acc[R][CW];
#pragma unroll
            for (int i = 0; i < R; ++i)
#pragma unroll
                for (int q = 0; q < CW; ++q) acc[i][q] = T(0);
            for (int g = 0; g < desc.ngroups; ++g) {
                const int d0 = desc.gstart[g], G = desc.gstart[g + 1] - d0;
                const int64_t o = desc.off[d0];
                T win[W][CW];
                const int64_t x0 = r0 + o;
                if (x0 >= 0 && x0 + W <= n) {
                    // window inside the matrix: one base pointer, constant steps
                    const T *xp = X + x0 * ldx + (int64_t)c * CW;
#pragma unroll
                    for (int t = 0; t < W; ++t) {
                        if (t < R + G - 1) {
                            if constexpr (CW == 1)
                                win[t][0] = __ldg(xp + t * ldx);
                            else
                                vload(win[t], xp + t * ldx);
                        }
                    }
                } else {
#pragma unroll
                    for (int t = 0; t < W; ++t) {
                        if (t < R + G - 1) {
                            int64_t xr = x0 + t;
                            xr = xr < 0 ? 0 : (xr >= n ? n - 1 : xr);  // value is 0 there
                            if constexpr (CW == 1)
                                win[t][0] = __ldg(X + xr * ldx + c);
                            else
                                vload(win[t], X + xr * ldx + (int64_t)c * CW);
                        }
                    }
                }
#pragma unroll
                for (int j = 0; j < kDiaGroupMax; ++j) {
                    if (j < G) {
                        T vv[R];
                        if constexpr (R == 1) {
                            vv[0] = __ldg(vals + (size_t)(d0 + j) * npad + r0);
                        } else {
                            const T *vp = vs + ((size_t)buf * nd + d0 + j) * BR + lr * R;
#pragma unroll
                            for (int i = 0; i < R; i += VN) {
                                T tmp[VN];
                                vload_plain(tmp, vp + i);
#pragma unroll
                                for (int u = 0; u < VN; ++u) vv[i + u] = tmp[u];
                            }
                        }
#pragma unroll
                        for (int i = 0; i < R; ++i)
#pragma unroll
                            for (int q = 0; q < CW; ++q)
                                acc[i][q] = fma(vv[i], win[i + j][q], acc[i][q]);
                    }
                }
            }
#pragma unroll
            for (int i = 0; i < R; ++i) {
                const int64_t row = r0 + i;
                if (row >= n) break;
                T y[CW];
#pragma unroll
                for (int q = 0; q < CW; ++q) y[q] = ca * acc[i][q];
                const int64_t col = (int64_t)c * CW;
                if (Z1) {
                    T z[CW];
                    if constexpr (CW == 1) z[0] = Z1[row * ldz1 + col]; else vload(z, Z1 + row * ldz1 + col);
#pragma unroll
                    for (int q = 0; q < CW; ++q) y[q] = fma(cb, z[q], y[q]);
                }
                if (Z2) {
                    T z[CW];
                    if constexpr (CW == 1) z[0] = Z2[row * ldz2 + col]; else vload(z, Z2 + row * ldz2 + col);
#pragma unroll
                    for (int q = 0; q < CW; ++q) y[q] = fma(cc, z[q], y[q]);
                }
                if constexpr (CW == 1) Y[row * ldy + col] = y[0]; else vstore(Y + row * ldy + col, y);
            }
        }
        if constexpr (R > 1) __syncthreads();  // buffer `buf` is refilled two blocks on
    }
    if constexpr (R > 1) asm volatile("cp.async.wait_all;\n" ::: "memory");
}

template <typename T, int R, int CW>
static int launch_dia_kernel(cudaStream_t st, const DevMatrix *A, const T *vals, int w,
                             const T *X, int64_t ldx, T *Y, int64_t ldy, const T *Z1,
                             int64_t ldz1, const T *Z2, int64_t ldz2, T ca, T cb, T cc) {
    const int cpr = w / CW;
    if (cpr > kDiaThreads) return CACG_ERR_UNSUPPORTED;
    // at most 512 rows per block keeps the staged values of narrow blocks small
    const int runs_per_block = std::min(kDiaThreads / cpr, std::max(1, 512 / R));
    const int BR = runs_per_block * R;
    const size_t smem = R > 1 ? 2 * (size_t)A->dia_ndiag * BR * sizeof(T) : 0;
    if (smem > 200 * 1024) return CACG_ERR_UNSUPPORTED;
    set_smem_attr(dia_spmm_kernel<T, R, CW>, 200 * 1024);
    const int64_t nblk = (A->n + BR - 1) / BR;
    int per_sm = 2;
    if (smem > 0) per_sm = std::max(1, std::min(R <= 4 ? 4 : 2, (int)(220 * 1024 / smem)));
    int64_t blocks = std::min<int64_t>(nblk, (int64_t)sm_count() * (R > 1 ? per_sm : 16));
    dia_spmm_kernel<T, R, CW><<<(unsigned)blocks, kDiaThreads, smem, st>>>(
        A->n, A->dia_npad, A->dia, vals, cpr, runs_per_block, X, ldx, Y, ldy, Z1, ldz1, Z2, ldz2,
        ca, cb, cc);
    return check_launch();
}

// R = B - A X in float-float arithmetic over the DIA view (mixed mode's
// residual replacement), with the residual post-pass fused in:
// S0 = R32 = (float)R, per-block partial ||R(:,c)||^2.  A = hi + lo (FP32
// views), X = Xh + Xl (ff_split_bits); each term a x is p + e + t with
// p = ah xh, e its exact FMA error, t = ah xl + al xh; the row sum is kept
// as (sh, sl) with TwoSum (about 2^-44 relative); B - sum is formed in
// float-float and widened to FP64 with one FP64 add.  Same thread layout as
// dia_spmm_kernel (R rows x 4 columns per thread, hi and lo values of the
// next row block staged in shared memory); m % 4 == 0.
__device__ __forceinline__ void ff_mac(float &sh, float &sl, float ah, float al, float xh,
                                       float xl) {
    const float p = ah * xh;
    const float e = fmaf(ah, xh, -p);
    const float t = fmaf(ah, xl, fmaf(al, xh, e));
    const float s = sh + p;
    const float bp = s - sh;
    const float err = (sh - (s - bp)) + (p - bp);
    sh = s;
    sl += err + t;
}

template <int R>
__global__ void __launch_bounds__(kDiaThreads, 2)
    dia_resid_ff_kernel(int64_t n, int64_t npad, DiaDesc desc, const float *__restrict__ vals,
                        int cpr, int runs_per_block, const float *__restrict__ Xh,
                        const float *__restrict__ Xl, int m, const double *__restrict__ B,
                        double *__restrict__ Rout, float *__restrict__ S0, int64_t lds,
                        float *__restrict__ R32, double *__restrict__ part) {
    constexpr int CW = 4;
    constexpr int W = R + kDiaGroupMax - 1;
    extern __shared__ __align__(16) unsigned char dia_smem[];
    float *vs = reinterpret_cast<float *>(dia_smem);  // [2][2 nd][BR]: hi rows, then lo rows
    const int lr = threadIdx.x / cpr, c = threadIdx.x % cpr;
    const bool active = lr < runs_per_block;
    const int BR = runs_per_block * R;
    const int64_t nblk = (n + BR - 1) / BR;
    const int nd = desc.ndiag, nd2 = 2 * nd;  // vals: hi view, then lo view (nd * npad apart)

    auto stage = [&](int64_t blk, int buf) {
        if (blk < nblk) {
            float *dst = vs + (size_t)buf * nd2 * BR;
            const int per = BR / 4;
            const int dstep = blockDim.x / per, qstep = blockDim.x % per;
            int d = threadIdx.x / per, q = threadIdx.x % per;
            for (; d < nd2; d += dstep, q += qstep) {
                if (q >= per) {
                    q -= per;
                    ++d;
                    if (d >= nd2) break;
                }
                const int64_t e0 = blk * BR + (int64_t)q * 4;
                const int64_t left = npad - e0;
                const int by = left >= 4 ? 16 : (left > 0 ? (int)left * 4 : 0);
                dia_cp16(dst + (size_t)d * BR + q * 4,
                         by ? (const void *)(vals + (size_t)d * npad + e0) : vals, by);
            }
        }
        asm volatile("cp.async.commit_group;\n" ::);
    };

    double sq[CW] = {0.0, 0.0, 0.0, 0.0};
    int buf = 0;
    stage(blockIdx.x, 0);
    for (int64_t blk = blockIdx.x; blk < nblk; blk += gridDim.x, buf ^= 1) {
        stage(blk + gridDim.x, buf ^ 1);
        asm volatile("cp.async.wait_group 1;\n" ::: "memory");
        __syncthreads();
        if (active) {
            const int64_t r0 = blk * BR + (int64_t)lr * R;
            float ah_[R][CW], al_[R][CW];
#pragma unroll
            for (int i = 0; i < R; ++i)
#pragma unroll
                for (int q = 0; q < CW; ++q) ah_[i][q] = al_[i][q] = 0.f;
            for (int g = 0; g < desc.ngroups; ++g) {
                const int d0 = desc.gstart[g], G = desc.gstart[g + 1] - d0;
                const int64_t x0 = r0 + desc.off[d0];
                float wh[W][CW], wl[W][CW];
#pragma unroll
                for (int t = 0; t < W; ++t) {
                    if (t < R + G - 1) {
                        int64_t xr = x0 + t;
                        xr = xr < 0 ? 0 : (xr >= n ? n - 1 : xr);  // value is 0 there
                        vload(wh[t], Xh + xr * m + (int64_t)c * CW);
                        vload(wl[t], Xl + xr * m + (int64_t)c * CW);
                    }
                }
#pragma unroll
                for (int j = 0; j < kDiaGroupMax; ++j) {
                    if (j < G) {
                        float vh[R], vl[R];
                        const float *ph = vs + ((size_t)buf * nd2 + d0 + j) * BR + lr * R;
                        const float *pl = ph + (size_t)nd * BR;
#pragma unroll
                        for (int i = 0; i < R; i += 4) {
                            float t4[4];
                            vload_plain(t4, ph + i);
#pragma unroll
                            for (int u = 0; u < 4; ++u) vh[i + u] = t4[u];
                            vload_plain(t4, pl + i);
#pragma unroll
                            for (int u = 0; u < 4; ++u) vl[i + u] = t4[u];
                        }
#pragma unroll
                        for (int i = 0; i < R; ++i)
#pragma unroll
                            for (int q = 0; q < CW; ++q)
                                ff_mac(ah_[i][q], al_[i][q], vh[i], vl[i], wh[i + j][q],
                                       wl[i + j][q]);
                    }
                }
            }
#pragma unroll
            for (int i = 0; i < R; ++i) {
                const int64_t row = r0 + i;
                if (row >= n) break;
                const int64_t col = (int64_t)c * CW;
                const double2 b01 = *reinterpret_cast<const double2 *>(B + row * m + col);
                const double2 b23 = *reinterpret_cast<const double2 *>(B + row * m + col + 2);
                const double bv[CW] = {b01.x, b01.y, b23.x, b23.y};
                double rd[CW];
                float rf[CW];
#pragma unroll
                for (int q = 0; q < CW; ++q) {
                    float bh, bl;
                    ff_split_bits(bv[q], bh, bl);
                    // (bh + bl) - (sh + sl) in float-float
                    const float sh = ah_[i][q], sl = al_[i][q];
                    const float s = bh - sh;
                    const float bp = s - bh;
                    const float err = (bh - (s - bp)) + (-sh - bp);
                    const float lo = err + (bl - sl);
                    rd[q] = ff_widen(s) + ff_widen(lo);
                    rf[q] = s + lo;
                    const double w = ff_widen(rf[q]);
                    sq[q] = fma(w, w, sq[q]);
                }
                *reinterpret_cast<double2 *>(Rout + row * m + col) = make_double2(rd[0], rd[1]);
                *reinterpret_cast<double2 *>(Rout + row * m + col + 2) = make_double2(rd[2], rd[3]);
                if (S0) vstore(S0 + row * lds + col, rf);
                if (R32) vstore(R32 + row * m + col, rf);
            }
        }
        __syncthreads();  // buffer `buf` is refilled two blocks on
    }
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    // per-block column partials in fixed order (runs ascending); staging reused
    if (part) {
        __syncthreads();
        double *red = reinterpret_cast<double *>(dia_smem);  // runs_per_block x m
        if (active)
#pragma unroll
            for (int q = 0; q < CW; ++q) red[(size_t)lr * m + c * CW + q] = sq[q];
        __syncthreads();
        for (int col = threadIdx.x; col < m; col += blockDim.x) {
            double t = 0.0;
            for (int r = 0; r < runs_per_block; ++r) t += red[(size_t)r * m + col];
            part[(size_t)blockIdx.x * m + col] = t;
        }
    }
}

// The same float-float residual for m = 16 with the row stride fixed at
// compile time (window rows at immediate offsets, no clamping inside the
// matrix) and the float-float products and sums on packed FP32 pairs
// (two columns per instruction: mul/fma/add/sub .rn.f32x2).  Every pair lane
// computes exactly what ff_mac computes for its column -- the product is
// formed as -p = (-a) x so that e = fma(a, x, -p) needs no negation -- so the
// FP64 R, S0, R32 and norms are bit-identical to dia_resid_ff_kernel's.  With
// Rff the kernel writes R as a normalised float-float pair instead (the
// mixed solve's float-float state) and sums the norms in float-float.
__device__ __forceinline__ unsigned long long ff_pack(float lo, float hi) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void ff_unpack(unsigned long long v, float &lo, float &hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
// (sh, sl) += a x over two columns: a = ah + al (broadcast A, NA = -A, AL),
// x = xh + xl (pairs)
__device__ __forceinline__ void ff_mac2(unsigned long long &sh, unsigned long long &sl,
                                        unsigned long long A, unsigned long long NA,
                                        unsigned long long AL, unsigned long long xh,
                                        unsigned long long xl) {
    asm("{\n"
        ".reg .b64 np, e, t, s, bp, t1, t2, t3, er, u;\n"
        "mul.rn.f32x2 np, %3, %5;\n"      // -p
        "fma.rn.f32x2 e, %2, %5, np;\n"   // e = a xh - p (exact)
        "fma.rn.f32x2 t, %4, %5, e;\n"    // al xh + e
        "fma.rn.f32x2 t, %2, %6, t;\n"    // ah xl + (al xh + e)
        "sub.rn.f32x2 s, %0, np;\n"       // s = sh + p
        "sub.rn.f32x2 bp, s, %0;\n"       // bp = s - sh
        "sub.rn.f32x2 t1, s, bp;\n"
        "sub.rn.f32x2 t2, %0, t1;\n"      // sh - (s - bp)
        "add.rn.f32x2 t3, np, bp;\n"      // -(p - bp)
        "sub.rn.f32x2 er, t2, t3;\n"      // (sh - (s - bp)) + (p - bp)
        "add.rn.f32x2 u, er, t;\n"
        "add.rn.f32x2 %1, %1, u;\n"
        "mov.b64 %0, s;\n"
        "}\n"
        : "+l"(sh), "+l"(sl)
        : "l"(A), "l"(NA), "l"(AL), "l"(xh), "l"(xl));
}

constexpr int kRf16R = 4;          // rows per thread
constexpr int kRf16Runs = 64;      // runs per block (256 threads, 4 per row)

__global__ void __launch_bounds__(kDiaThreads, 2)
    dia_resid_ff16_kernel(int64_t n, int64_t npad, const __grid_constant__ DiaDesc desc,
                          const float *__restrict__ vals, const float *__restrict__ Xh,
                          const float *__restrict__ Xl, const double *__restrict__ B,
                          double *__restrict__ Rout, float *__restrict__ Rff,
                          float *__restrict__ S0, int64_t lds, float *__restrict__ R32,
                          double *__restrict__ part) {
    // Rff (n x 16 high parts, then n x 16 low parts): R as a normalised
    // float-float pair instead of FP64 Rout, norms in float-float
    constexpr int M = 16, R = kRf16R, BR = kRf16Runs * R;
    constexpr int W = R + kDiaGroupMax - 1;
    extern __shared__ __align__(16) unsigned char dia_smem[];
    float *vs = reinterpret_cast<float *>(dia_smem);  // [2][2 nd][BR]: hi rows, then lo rows
    __shared__ int64_t g_off[kDiaMax];                 // group offset x M
    __shared__ int g_d0[kDiaMax], g_size[kDiaMax];
    const int nd = desc.ndiag, nd2 = 2 * nd, ng = desc.ngroups;
    for (int g = threadIdx.x; g < ng; g += blockDim.x) {
        g_off[g] = desc.off[desc.gstart[g]] * M;
        g_d0[g] = desc.gstart[g];
        g_size[g] = desc.gstart[g + 1] - desc.gstart[g];
    }
    const int lr = threadIdx.x >> 2, c = threadIdx.x & 3;
    const int64_t nblk = (n + BR - 1) / BR;
    const int64_t omin = desc.off[0], omax = desc.off[nd - 1];

    auto stage = [&](int64_t blk, int buf) {
        if (blk < nblk) {
            float *dst = vs + (size_t)buf * nd2 * BR;
            constexpr int per = BR / 4;
            for (int idx = threadIdx.x; idx < nd2 * per; idx += kDiaThreads) {
                const int d = idx / per, q = idx - d * per;
                const int64_t e0 = blk * BR + (int64_t)q * 4;
                const int64_t left = npad - e0;
                const int by = left >= 4 ? 16 : (left > 0 ? (int)left * 4 : 0);
                dia_cp16(dst + (size_t)d * BR + q * 4,
                         by ? (const void *)(vals + (size_t)d * npad + e0) : vals, by);
            }
        }
        asm volatile("cp.async.commit_group;\n" ::);
    };

    double sq[4] = {0.0, 0.0, 0.0, 0.0};
    float fq_hi[4] = {0.f, 0.f, 0.f, 0.f}, fq_lo[4] = {0.f, 0.f, 0.f, 0.f};
    int buf = 0;
    stage(blockIdx.x, 0);
    for (int64_t blk = blockIdx.x; blk < nblk; blk += gridDim.x, buf ^= 1) {
        stage(blk + gridDim.x, buf ^ 1);
        asm volatile("cp.async.wait_group 1;\n" ::: "memory");
        __syncthreads();
        const int64_t r0 = blk * BR + (int64_t)lr * R;
        const bool inside = blk * BR + omin >= 0 && blk * BR + BR - 1 + omax < n;
        unsigned long long sh[R][2], sl[R][2];
#pragma unroll
        for (int i = 0; i < R; ++i) sh[i][0] = sh[i][1] = sl[i][0] = sl[i][1] = 0ull;
        for (int g = 0; g < ng; ++g) {
            const int G = g_size[g];
            ulonglong2 wh[W], wl[W];
            if (inside) {
                const int64_t e = r0 * M + g_off[g] + 4 * c;
                const ulonglong2 *ph = reinterpret_cast<const ulonglong2 *>(Xh + e);
                const ulonglong2 *pl = reinterpret_cast<const ulonglong2 *>(Xl + e);
#pragma unroll
                for (int t = 0; t < W; ++t)
                    if (t < R + G - 1) {
                        wh[t] = __ldg(ph + t * (M / 4));
                        wl[t] = __ldg(pl + t * (M / 4));
                    }
            } else {
                const int64_t x0 = r0 + g_off[g] / M;
#pragma unroll
                for (int t = 0; t < W; ++t)
                    if (t < R + G - 1) {
                        int64_t xr = x0 + t;
                        xr = xr < 0 ? 0 : (xr >= n ? n - 1 : xr);  // value is 0 there
                        wh[t] = __ldg(reinterpret_cast<const ulonglong2 *>(Xh + xr * M + 4 * c));
                        wl[t] = __ldg(reinterpret_cast<const ulonglong2 *>(Xl + xr * M + 4 * c));
                    }
            }
            const float *vg = vs + ((size_t)buf * nd2 + g_d0[g]) * BR + lr * R;
#pragma unroll
            for (int j = 0; j < kDiaGroupMax; ++j) {
                if (j < G) {
                    const float4 vh = *reinterpret_cast<const float4 *>(vg + j * BR);
                    const float4 vl = *reinterpret_cast<const float4 *>(vg + (size_t)nd * BR + j * BR);
                    const float ah[R] = {vh.x, vh.y, vh.z, vh.w}, al[R] = {vl.x, vl.y, vl.z, vl.w};
#pragma unroll
                    for (int i = 0; i < R; ++i) {
                        const unsigned long long A = ff_pack(ah[i], ah[i]);
                        const unsigned long long NA = ff_pack(-ah[i], -ah[i]);
                        const unsigned long long AL = ff_pack(al[i], al[i]);
                        ff_mac2(sh[i][0], sl[i][0], A, NA, AL, wh[i + j].x, wl[i + j].x);
                        ff_mac2(sh[i][1], sl[i][1], A, NA, AL, wh[i + j].y, wl[i + j].y);
                    }
                }
            }
        }
#pragma unroll
        for (int i = 0; i < R; ++i) {
            const int64_t row = r0 + i;
            if (row >= n) break;
            const int64_t col = 4 * c;
            const double2 b01 = *reinterpret_cast<const double2 *>(B + row * M + col);
            const double2 b23 = *reinterpret_cast<const double2 *>(B + row * M + col + 2);
            const double bv[4] = {b01.x, b01.y, b23.x, b23.y};
            float shv[4], slv[4];
            ff_unpack(sh[i][0], shv[0], shv[1]);
            ff_unpack(sh[i][1], shv[2], shv[3]);
            ff_unpack(sl[i][0], slv[0], slv[1]);
            ff_unpack(sl[i][1], slv[2], slv[3]);
            double rd[4];
            float rf[4], rl[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                float bh, bl;
                ff_split_bits(bv[q], bh, bl);
                const float s = bh - shv[q];
                const float bp = s - bh;
                const float err = (bh - (s - bp)) + (-shv[q] - bp);
                const float lo = err + (bl - slv[q]);
                rf[q] = s + lo;
                if (Rff) {  // normalised pair (TwoSum: s may have cancelled)
                    const float tp = rf[q] - s;
                    rl[q] = (s - (rf[q] - tp)) + (lo - tp);
                    ff_add_square(rf[q], rl[q], fq_hi[q], fq_lo[q]);
                } else {
                    rd[q] = ff_widen(s) + ff_widen(lo);
                    const double w = ff_widen(rf[q]);
                    sq[q] = fma(w, w, sq[q]);
                }
            }
            if (Rff) {
                vstore(Rff + row * M + col, rf);
                vstore(Rff + (n + row) * M + col, rl);
            } else {
                *reinterpret_cast<double2 *>(Rout + row * M + col) = make_double2(rd[0], rd[1]);
                *reinterpret_cast<double2 *>(Rout + row * M + col + 2) =
                    make_double2(rd[2], rd[3]);
            }
            if (S0) vstore(S0 + row * lds + col, rf);
            if (R32) vstore(R32 + row * M + col, rf);
        }
        __syncthreads();  // buffer `buf` is refilled two blocks on
    }
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    if (part) {
        __syncthreads();
        double *red = reinterpret_cast<double *>(dia_smem);  // runs x 16
#pragma unroll
        for (int q = 0; q < 4; ++q)
            red[(size_t)lr * M + c * 4 + q] =
                Rff ? ff_widen(fq_hi[q]) + ff_widen(fq_lo[q]) : sq[q];
        __syncthreads();
        if (threadIdx.x < M) {
            double t = 0.0;
            for (int r = 0; r < kRf16Runs; ++r) t += red[(size_t)r * M + threadIdx.x];
            part[(size_t)blockIdx.x * M + threadIdx.x] = t;
        }
    }
}

// Float-float residual (see above); CACG_ERR_UNSUPPORTED when the matrix has
// no FP32 hi/lo view or m is not a multiple of 4.  Xh, Xl: n x m scratch.
int launch_dia_residual_ff(cudaStream_t st, const DevMatrix *A, int m, const double *X,
                           const double *B, double *R, float *Xh, float *Xl, float *S0,
                           int64_t lds, float *R32, double *norms, double *ws,
                           int64_t ws_doubles, float *Rff) {
    if (!A || A->dia_ndiag <= 0 || !A->dia32 || !A->dia32lo || m % 4 != 0 || m <= 0)
        return CACG_ERR_UNSUPPORTED;
    if ((X && !aligned16(X)) || !aligned16(B) || (!R && !Rff) || (R && !aligned16(R)) ||
        (Rff && (m != 16 || !aligned16(Rff))) || !aligned16(Xh) || !aligned16(Xl) ||
        (S0 && (lds % 4 || !aligned16(S0))) || (R32 && !aligned16(R32)))
        return CACG_ERR_UNSUPPORTED;
    constexpr int RR = kDiaR / 2;
    const int cpr = m / 4;
    if (cpr > kDiaThreads) return CACG_ERR_UNSUPPORTED;
    const int runs_per_block = std::min(kDiaThreads / cpr, std::max(1, 512 / RR));
    const int BR = runs_per_block * RR;
    const size_t smem = std::max((size_t)2 * 2 * A->dia_ndiag * BR * 4,
                                 (size_t)runs_per_block * m * 8);
    if (smem > 200 * 1024) return CACG_ERR_UNSUPPORTED;
    const int64_t nblk = (A->n + BR - 1) / BR;
    const int per_sm = std::max(1, std::min(2, (int)(220 * 1024 / smem)));
    const int64_t blocks = std::min<int64_t>(nblk, (int64_t)sm_count() * per_sm);
    if (norms && (int64_t)blocks * m > ws_doubles) return CACG_ERR_UNSUPPORTED;
    const bool k16 = m == 16 && A->dia.ngroups <= kDiaMax && runs_per_block == kRf16Runs &&
                     BR == kRf16Runs * kRf16R;
    if (Rff && !k16) return CACG_ERR_UNSUPPORTED;
    // X == NULL: Xh, Xl already hold X
    int rc = X ? launch_ff_split(st, A->n * (int64_t)m, X, Xh, Xl) : CACG_OK;
    if (rc != CACG_OK) return rc;
    set_smem_attr(dia_resid_ff_kernel<RR>, 200 * 1024);
    set_smem_attr(dia_resid_ff16_kernel, 200 * 1024);
    if (k16) {
        dia_resid_ff16_kernel<<<(unsigned)blocks, kDiaThreads, smem, st>>>(
            A->n, A->dia_npad, A->dia, A->dia32, Xh, Xl, B, Rff ? nullptr : R, Rff, S0, lds, R32,
            norms ? ws : nullptr);
        rc = check_launch();
        if (rc != CACG_OK || !norms) return rc;
        return launch_colsum(st, ws, (int)blocks, m, norms);
    }
    dia_resid_ff_kernel<RR><<<(unsigned)blocks, kDiaThreads, smem, st>>>(
        A->n, A->dia_npad, A->dia, A->dia32, cpr, runs_per_block, Xh, Xl, m, B, R, S0, lds, R32,
        norms ? ws : nullptr);
    rc = check_launch();
    if (rc != CACG_OK || !norms) return rc;
    return launch_colsum(st, ws, (int)blocks, m, norms);
}

template <typename T>
int launch_dia_spmm(cudaStream_t st, const DevMatrix *A, int w, const T *X, int64_t ldx, T *Y,
                    int64_t ldy, const T *Z1, int64_t ldz1, const T *Z2, int64_t ldz2,
                    double ca_, double cb_, double cc_) {
    if (!A || A->dia_ndiag <= 0 || w <= 0) return CACG_ERR_UNSUPPORTED;
    const T *vals = std::is_same<T, float>::value ? (const T *)(const void *)A->dia32
                                                  : (const T *)(const void *)A->dia64;
    if (!vals) return CACG_ERR_UNSUPPORTED;
    if (A->n <= 0) return CACG_OK;
    const T ca = T(ca_), cb = T(cb_), cc = T(cc_);
    constexpr int VN = Vec16<T>::N;
    const bool vec = w % VN == 0 && ldx % VN == 0 && ldy % VN == 0 && aligned16(X) &&
                     aligned16(Y) && (!Z1 || (ldz1 % VN == 0 && aligned16(Z1))) &&
                     (!Z2 || (ldz2 % VN == 0 && aligned16(Z2)));
    // narrow blocks (<= 8 chunks a row): 4 rows a thread and more CTAs per SM
    // hide the L2 latency of the X window; wide blocks: 8 rows a thread
    // amortise the window over more FMAs
    if (vec && w / VN <= 8)
        return launch_dia_kernel<T, kDiaR / 2, VN>(st, A, vals, w, X, ldx, Y, ldy, Z1, ldz1, Z2,
                                                   ldz2, ca, cb, cc);
    if (vec)
        return launch_dia_kernel<T, kDiaR, VN>(st, A, vals, w, X, ldx, Y, ldy, Z1, ldz1, Z2,
                                               ldz2, ca, cb, cc);
    // unaligned blocks (a column slice of width m % 4 != 0, e.g. a basis
    // step T_j inside the n x k basis): scalar columns, still 4 rows a thread
    // with the values staged (the same FMAs in the same order as R = 1)
    return launch_dia_kernel<T, kDiaR / 2, 1>(st, A, vals, w, X, ldx, Y, ldy, Z1, ldz1, Z2, ldz2,
                                              ca, cb, cc);
}

template int launch_dia_spmm<float>(cudaStream_t, const DevMatrix *, int, const float *, int64_t,
                                    float *, int64_t, const float *, int64_t, const float *,
                                    int64_t, double, double, double);
template int launch_dia_spmm<double>(cudaStream_t, const DevMatrix *, int, const double *,
                                     int64_t, double *, int64_t, const double *, int64_t,
                                     const double *, int64_t, double, double, double);

}  // namespace cacg
