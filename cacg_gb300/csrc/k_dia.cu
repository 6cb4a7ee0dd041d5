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
            if (v32) v32[(size_t)d * npad + row] = (float)val[p];
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
    const size_t b64 = (size_t)nd * npad * 8, b32 = want_f32 ? (size_t)nd * npad * 4 : 0;
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
    dia_ndiag = nd;
    owned_bytes += b64 + b32;
    return CACG_OK;
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
    static const bool attr = [] {
        cudaFuncSetAttribute(dia_spmm_kernel<T, R, CW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             200 * 1024);
        return true;
    }();
    (void)attr;
    const int64_t nblk = (A->n + BR - 1) / BR;
    int per_sm = 2;
    if (smem > 0) per_sm = std::max(1, std::min(R <= 4 ? 4 : 2, (int)(220 * 1024 / smem)));
    int64_t blocks = std::min<int64_t>(nblk, (int64_t)sm_count() * (R > 1 ? per_sm : 16));
    dia_spmm_kernel<T, R, CW><<<(unsigned)blocks, kDiaThreads, smem, st>>>(
        A->n, A->dia_npad, A->dia, vals, cpr, runs_per_block, X, ldx, Y, ldy, Z1, ldz1, Z2, ldz2,
        ca, cb, cc);
    return check_launch();
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
    return launch_dia_kernel<T, 1, 1>(st, A, vals, w, X, ldx, Y, ldy, Z1, ldz1, Z2, ldz2, ca, cb,
                                      cc);
}

template int launch_dia_spmm<float>(cudaStream_t, const DevMatrix *, int, const float *, int64_t,
                                    float *, int64_t, const float *, int64_t, const float *,
                                    int64_t, double, double, double);
template int launch_dia_spmm<double>(cudaStream_t, const DevMatrix *, int, const double *,
                                     int64_t, double *, int64_t, const double *, int64_t,
                                     const double *, int64_t, double, double, double);

}  // namespace cacg
