// k_spmm.cu -- CSR SpMM with the Chebyshev three-term recurrence fused into
// its epilogue (the matrix-power kernel of the CA solver).
//
// Reference operations replaced (sclc/cacg):
//   spmm_csr_v1 / spmm_csr_v2          src/BLAS3.c:20-232   Y = A X
//   spmm_csr_info_data_sep_{CBCG,BCBCG} src/BLAS3.c:851-976 A T_{j-1}
//   dense_mat_mat_add_TP_targetDisp    src/BLAS3.c:828-847  T_1 = a A R + b R
//   dense_array_mat_mat_mat_add_TP_disp src/BLAS3.c:978-994 T_j = 2a A T_{j-1}
//                                                            + 2b T_{j-1} - T_{j-2}
// On one GPU the MPI_Allgatherv before each SpMM (src/BLAS3.c:48-50) is the
// resident operand itself, so it disappears.
//
// Design (GB300): HBM-bound.  Each row of A is streamed once per basis step
// for all block columns: a team of TEAM lanes owns one row, each lane owns
// up to 4 chunks of CH contiguous columns (CH * sizeof(T) = 16 bytes, so the
// gather of X[col, :] is a set of 128-bit loads of the row-major block).
// The recurrence's axpby runs in registers before the single store, so a
// basis step reads A once, T_{j-1} (gathered, L2-resident neighbourhood) and
// T_{j-2} once, and writes T_j once.  For one column (CBCG) a team of lanes
// splits the nonzeros of a row and reduces with warp shuffles.
#include <algorithm>

#include "cacg_internal.cuh"

namespace cacg {

constexpr int kSpmmThreads = 256;
constexpr int kMaxNch = 4;
constexpr int kGroup = 8;  // nonzeros fetched together per lane

template <typename T, int CH>
__device__ __forceinline__ void load_chunk(T (&d)[CH], const T *p) {
    if constexpr (CH == 1) {
        d[0] = __ldg(p);
    } else {
        vload(d, p);
    }
}

template <typename T, int CH>
__device__ __forceinline__ void load_chunk_plain(T (&d)[CH], const T *p) {
    if constexpr (CH == 1) {
        d[0] = *p;
    } else {
        vload(d, p);
    }
}

template <typename T, int CH>
__device__ __forceinline__ void store_chunk(T *p, const T (&d)[CH]) {
    if constexpr (CH == 1) {
        *p = d[0];
    } else {
        vstore(p, d);
    }
}

// One team of TEAM lanes per row; lane lt owns chunks lt, lt+TEAM, ... (nch of them)
// of this column block (blockIdx.y).
template <typename T, int CH, int TEAM, int NCH>
__global__ void __launch_bounds__(kSpmmThreads)
    spmm_rows_kernel(int64_t n, const int32_t *__restrict__ rp, const int32_t *__restrict__ ci,
                     const T *__restrict__ val, int w, const T *__restrict__ X,
                     int64_t ldx, T *__restrict__ Y, int64_t ldy, const T *__restrict__ Z1,
                     int64_t ldz1, const T *__restrict__ Z2, int64_t ldz2, T ca, T cb, T cc,
                     Slices ysl) {
    const int lt = threadIdx.x % TEAM;
    const int64_t team0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / TEAM;
    const int64_t nteams = ((int64_t)gridDim.x * blockDim.x) / TEAM;
    const int colbase = blockIdx.y * (TEAM * NCH * CH);
    for (int64_t row = team0; row < n; row += nteams) {
        T acc[NCH][CH];
#pragma unroll
        for (int j = 0; j < NCH; ++j)
#pragma unroll
            for (int q = 0; q < CH; ++q) acc[j][q] = T(0);
        const int b = __ldg(rp + row), e = __ldg(rp + row + 1);
        int p = b;
        // groups of kGroup nonzeros: all index/value loads first, then all
        // gathers, so each lane keeps kGroup independent loads in flight
        for (; p + kGroup <= e; p += kGroup) {
            int cg[kGroup];
            T ag[kGroup];
#pragma unroll
            for (int u = 0; u < kGroup; ++u) {
                cg[u] = __ldg(ci + p + u);
                ag[u] = __ldg(val + p + u);
            }
#pragma unroll
            for (int j = 0; j < NCH; ++j) {
                const int col = (lt + j * TEAM) * CH;
                if (colbase + col < w) {
                    T x[kGroup][CH];
#pragma unroll
                    for (int u = 0; u < kGroup; ++u)
                        load_chunk<T, CH>(x[u], X + (int64_t)cg[u] * ldx + colbase + col);
#pragma unroll
                    for (int u = 0; u < kGroup; ++u)
#pragma unroll
                        for (int q = 0; q < CH; ++q) acc[j][q] = fma(ag[u], x[u][q], acc[j][q]);
                }
            }
        }
        for (; p < e; ++p) {
            const int c = __ldg(ci + p);
            const T a = __ldg(val + p);
            const T *xr = X + (int64_t)c * ldx + colbase;
#pragma unroll
            for (int j = 0; j < NCH; ++j) {
                const int col = (lt + j * TEAM) * CH;
                if (colbase + col < w) {
                    T x[CH];
                    load_chunk<T, CH>(x, xr + col);
#pragma unroll
                    for (int q = 0; q < CH; ++q) acc[j][q] = fma(a, x[q], acc[j][q]);
                }
            }
        }
#pragma unroll
        for (int j = 0; j < NCH; ++j) {
            const int col = colbase + (lt + j * TEAM) * CH;
            if (col < w) {
                T y[CH];
#pragma unroll
                for (int q = 0; q < CH; ++q) y[q] = ca * acc[j][q];
                if (Z1) {
                    T z[CH];
                    load_chunk_plain<T, CH>(z, Z1 + row * ldz1 + col);
#pragma unroll
                    for (int q = 0; q < CH; ++q) y[q] = fma(cb, z[q], y[q]);
                }
                if (Z2) {
                    T z[CH];
                    load_chunk_plain<T, CH>(z, Z2 + row * ldz2 + col);
#pragma unroll
                    for (int q = 0; q < CH; ++q) y[q] = fma(cc, z[q], y[q]);
                }
                store_chunk<T, CH>(Y + row * ldy + col, y);
                if constexpr (sizeof(T) == 4) {
                    if (ysl.p) {
                        if constexpr (CH == 4)
                            store_slices4(ysl, row * ldy + col, y);
                        else
#pragma unroll
                            for (int q = 0; q < CH; ++q) store_slices1(ysl, row * ldy + col + q, y[q]);
                    }
                }
            }
        }
    }
}

// Warp-staged variant: warp w owns blocks of RPW = 32 / TEAM consecutive
// rows (one row per team).  The column indices and values of a block are
// copied into this warp's shared-memory buffer with 16-byte cp.async one block
// ahead, and the block's row pointers are loaded two blocks ahead, so a row's
// dependent chain is only the X gathers (mostly L1/L2 hits) instead of row
// pointer -> index/value -> gather round trips to HBM.  A block with more
// than `cap` staged entries is processed straight from global memory.
// Requires 2 <= TEAM (RPW + 1 row pointers fit in the warp's lanes) and
// 16-byte aligned ci / val.
template <typename T, int CH, int NCH>
__device__ __forceinline__ void ws_row(int64_t row, int lt, int TEAMv, int colbase, int w,
                                       const int32_t *cis, const T *vs, int cnt,
                                       const T *__restrict__ X, int64_t ldx, T (&acc)[NCH][CH]) {
    int p = 0;
    for (; p + kGroup <= cnt; p += kGroup) {
        int cg[kGroup];
        T ag[kGroup];
#pragma unroll
        for (int u = 0; u < kGroup; ++u) {
            cg[u] = cis[p + u];
            ag[u] = vs[p + u];
        }
#pragma unroll
        for (int j = 0; j < NCH; ++j) {
            const int col = (lt + j * TEAMv) * CH;
            if (colbase + col < w) {
                T x[kGroup][CH];
#pragma unroll
                for (int u = 0; u < kGroup; ++u)
                    load_chunk<T, CH>(x[u], X + (int64_t)cg[u] * ldx + colbase + col);
#pragma unroll
                for (int u = 0; u < kGroup; ++u)
#pragma unroll
                    for (int q = 0; q < CH; ++q) acc[j][q] = fma(ag[u], x[u][q], acc[j][q]);
            }
        }
    }
    for (; p < cnt; ++p) {
        const int c = cis[p];
        const T a = vs[p];
#pragma unroll
        for (int j = 0; j < NCH; ++j) {
            const int col = (lt + j * TEAMv) * CH;
            if (colbase + col < w) {
                T x[CH];
                load_chunk<T, CH>(x, X + (int64_t)c * ldx + colbase + col);
#pragma unroll
                for (int q = 0; q < CH; ++q) acc[j][q] = fma(a, x[q], acc[j][q]);
            }
        }
    }
}

__device__ __forceinline__ void ws_cp16(void *smem, const void *g, int bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(
                     (unsigned)__cvta_generic_to_shared(smem)),
                 "l"(g), "r"(bytes));
}

template <typename T, int CH, int TEAM, int NCH>
__global__ void __launch_bounds__(kSpmmThreads)
    spmm_ws_kernel(int64_t n, const int32_t *__restrict__ rp, const int32_t *__restrict__ ci,
                   const T *__restrict__ val, int cap, int w, const T *__restrict__ X,
                   int64_t ldx, T *__restrict__ Y, int64_t ldy, const T *__restrict__ Z1,
                   int64_t ldz1, const T *__restrict__ Z2, int64_t ldz2, T ca, T cb, T cc,
                   Slices ysl) {
    static_assert(TEAM >= 2 && TEAM <= 32, "RPW + 1 row pointers must fit in a warp");
    constexpr int RPW = 32 / TEAM;
    constexpr int VPC = 16 / (int)sizeof(T);  // values per 16-byte chunk
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    // this warp: ci[2][cap], val[2][cap]
    int32_t *ci_s = reinterpret_cast<int32_t *>(smem_raw + (size_t)wib * 2 * cap * (4 + sizeof(T)));
    T *val_s = reinterpret_cast<T *>(ci_s + 2 * cap);
    const int lt = lane % TEAM, team = lane / TEAM;
    const int colbase = blockIdx.y * (TEAM * NCH * CH);
    const int64_t nblk = (n + RPW - 1) / RPW;
    const int64_t wg = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int nnz = __ldg(rp + n);

    auto load_rp = [&](int64_t blk) -> int {  // lane l <= RPW: rp[blk * RPW + l] (clamped)
        if (blk >= nblk || lane > RPW) return 0;
        int64_t r = blk * RPW + lane;
        return __ldg(rp + (r < n ? r : n));
    };
    auto stage = [&](int rpv, int64_t blk, int buf) {
        if (blk < nblk) {
            const int s = __shfl_sync(0xffffffffu, rpv, 0) & ~3;
            const int e = (__shfl_sync(0xffffffffu, rpv, RPW) + 3) & ~3;
            if (e - s <= cap) {
                for (int c = lane; c < (e - s) / 4; c += 32) {
                    const int g0 = s + 4 * c;
                    const int by = max(0, min(16, (nnz - g0) * 4));
                    ws_cp16(ci_s + buf * cap + 4 * c, by ? (const void *)(ci + g0) : ci, by);
                }
                for (int c = lane; c < (e - s) / VPC; c += 32) {
                    const int g0 = s + VPC * c;
                    const int by = max(0, min(16, (nnz - g0) * (int)sizeof(T)));
                    ws_cp16(val_s + buf * cap + VPC * c, by ? (const void *)(val + g0) : val, by);
                }
            }
        }
        asm volatile("cp.async.commit_group;\n" ::);
    };

    int64_t blk = wg;
    int rp_cur = load_rp(blk);
    stage(rp_cur, blk, 0);
    int rp_next = load_rp(blk + nw);
    int buf = 0;
    for (; blk < nblk; blk += nw, buf ^= 1) {
        stage(rp_next, blk + nw, buf ^ 1);
        const int rp_after = load_rp(blk + 2 * nw);
        asm volatile("cp.async.wait_group 1;\n" ::: "memory");
        __syncwarp();
        const int s = __shfl_sync(0xffffffffu, rp_cur, 0) & ~3;
        const int e = (__shfl_sync(0xffffffffu, rp_cur, RPW) + 3) & ~3;
        const bool staged = e - s <= cap;
        const int rb = __shfl_sync(0xffffffffu, rp_cur, team);
        const int re = __shfl_sync(0xffffffffu, rp_cur, team + 1);
        const int64_t row = blk * RPW + team;
        if (row < n) {
            T acc[NCH][CH];
#pragma unroll
            for (int j = 0; j < NCH; ++j)
#pragma unroll
                for (int q = 0; q < CH; ++q) acc[j][q] = T(0);
            if (staged)
                ws_row<T, CH, NCH>(row, lt, TEAM, colbase, w, ci_s + buf * cap + (rb - s),
                                   val_s + buf * cap + (rb - s), re - rb, X, ldx, acc);
            else
                ws_row<T, CH, NCH>(row, lt, TEAM, colbase, w, ci + rb, val + rb, re - rb, X, ldx,
                                   acc);
#pragma unroll
            for (int j = 0; j < NCH; ++j) {
                const int col = colbase + (lt + j * TEAM) * CH;
                if (col < w) {
                    T y[CH];
#pragma unroll
                    for (int q = 0; q < CH; ++q) y[q] = ca * acc[j][q];
                    if (Z1) {
                        T z[CH];
                        load_chunk_plain<T, CH>(z, Z1 + row * ldz1 + col);
#pragma unroll
                        for (int q = 0; q < CH; ++q) y[q] = fma(cb, z[q], y[q]);
                    }
                    if (Z2) {
                        T z[CH];
                        load_chunk_plain<T, CH>(z, Z2 + row * ldz2 + col);
#pragma unroll
                        for (int q = 0; q < CH; ++q) y[q] = fma(cc, z[q], y[q]);
                    }
                    store_chunk<T, CH>(Y + row * ldy + col, y);
                    if constexpr (sizeof(T) == 4) {
                        if (ysl.p) {
                            if constexpr (CH == 4)
                                store_slices4(ysl, row * ldy + col, y);
                            else
#pragma unroll
                                for (int q = 0; q < CH; ++q)
                                    store_slices1(ysl, row * ldy + col + q, y[q]);
                        }
                    }
                }
            }
        }
        __syncwarp();  // every lane is done with this buffer before it is refilled
        rp_cur = rp_next;
        rp_next = rp_after;
    }
    asm volatile("cp.async.wait_all;\n" ::: "memory");
}

// Single column: TEAM lanes split the nonzeros of a row, shuffle-reduce.
template <typename T, int TEAM>
__global__ void __launch_bounds__(kSpmmThreads)
    spmv_kernel(int64_t n, const int32_t *__restrict__ rp, const int32_t *__restrict__ ci,
                const T *__restrict__ val, const T *__restrict__ X, int64_t ldx,
                T *__restrict__ Y, int64_t ldy, const T *__restrict__ Z1, int64_t ldz1,
                const T *__restrict__ Z2, int64_t ldz2, T ca, T cb, T cc) {
    constexpr int RPW = 32 / TEAM;  // rows per warp step
    const int lane = threadIdx.x & 31;
    const int lt = lane % TEAM;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r0 = warp * RPW; r0 < n; r0 += nwarps * RPW) {
        const int64_t row = r0 + lane / TEAM;
        T acc = T(0);
        if (row < n) {
            const int b = __ldg(rp + row), e = __ldg(rp + row + 1);
#pragma unroll 4
            for (int p = b + lt; p < e; p += TEAM)
                acc = fma(__ldg(val + p), __ldg(X + (int64_t)__ldg(ci + p) * ldx), acc);
        }
#pragma unroll
        for (int off = TEAM / 2; off > 0; off >>= 1)
            acc += __shfl_xor_sync(0xffffffffu, acc, off, TEAM);
        if (row < n && lt == 0) {
            T y = ca * acc;
            if (Z1) y = fma(cb, Z1[row * ldz1], y);
            if (Z2) y = fma(cc, Z2[row * ldz2], y);
            Y[row * ldy] = y;
        }
    }
}

static int grid_for(int64_t units, int threads_per_unit_den) {
    // units of work -> blocks, capped at a few waves of resident blocks
    int64_t blocks = (units + threads_per_unit_den - 1) / threads_per_unit_den;
    int64_t cap = (int64_t)sm_count() * 8;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    return (int)blocks;
}

template <typename T, int CH, int TEAM, int NCH>
static int launch_rows(cudaStream_t st, int64_t n, const int32_t *rp, const int32_t *ci,
                       const T *val, int w, int ycols, const T *X, int64_t ldx, T *Y,
                       int64_t ldy, const T *Z1, int64_t ldz1, const T *Z2, int64_t ldz2, T ca,
                       T cb, T cc, Slices ysl, double avg_nnz) {
    const int rows_per_block = kSpmmThreads / TEAM;
    if constexpr (TEAM >= 2) {
        if (aligned16(ci) && aligned16(val) && avg_nnz > 0) {
            // staged entries per warp buffer: RPW rows at 1.5x the mean row
            // length (multiple of 4), plus alignment slack at both ends
            constexpr int RPW = 32 / TEAM;
            int per_row = ((int)(1.5 * avg_nnz) + 3) & ~3;
            if (per_row < 8) per_row = 8;
            int cap = RPW * per_row + 8;
            const int warps = kSpmmThreads / 32;
            const size_t max_smem = 96 * 1024;  // keep >= 2 blocks per SM
            while (cap > 16 && (size_t)warps * 2 * cap * (4 + sizeof(T)) > max_smem) cap -= 4;
            const size_t smem = (size_t)warps * 2 * cap * (4 + sizeof(T));
            set_smem_attr(spmm_ws_kernel<T, CH, TEAM, NCH>, 96 * 1024);
            const int64_t nblk = (n + RPW - 1) / RPW;
            dim3 grid(grid_for(nblk, warps), ycols);
            spmm_ws_kernel<T, CH, TEAM, NCH><<<grid, kSpmmThreads, smem, st>>>(
                n, rp, ci, val, cap, w, X, ldx, Y, ldy, Z1, ldz1, Z2, ldz2, ca, cb, cc, ysl);
            return check_launch();
        }
    }
    dim3 grid(grid_for(n, rows_per_block), ycols);
    spmm_rows_kernel<T, CH, TEAM, NCH><<<grid, kSpmmThreads, 0, st>>>(
        n, rp, ci, val, w, X, ldx, Y, ldy, Z1, ldz1, Z2, ldz2, ca, cb, cc, ysl);
    return check_launch();
}

template <typename T, int CH, int NCH>
static int dispatch_team(int team, cudaStream_t st, int64_t n, const int32_t *rp,
                         const int32_t *ci, const T *val, int w, int ycols, const T *X,
                         int64_t ldx, T *Y, int64_t ldy, const T *Z1, int64_t ldz1, const T *Z2,
                         int64_t ldz2, T ca, T cb, T cc, Slices ysl, double avg_nnz) {
#define CACG_TEAM_CASE(TM)                                                                \
    case TM:                                                                              \
        return launch_rows<T, CH, TM, NCH>(st, n, rp, ci, val, w, ycols, X, ldx, Y, ldy, Z1, \
                                           ldz1, Z2, ldz2, ca, cb, cc, ysl, avg_nnz);
    switch (team) {
        CACG_TEAM_CASE(1)
        CACG_TEAM_CASE(2)
        CACG_TEAM_CASE(4)
        CACG_TEAM_CASE(8)
        CACG_TEAM_CASE(16)
        CACG_TEAM_CASE(32)
    }
#undef CACG_TEAM_CASE
    return CACG_ERR_ARG;
}

template <typename T, int CH>
static int dispatch_nch(int nch, int team, cudaStream_t st, int64_t n, const int32_t *rp,
                        const int32_t *ci, const T *val, int w, int ycols, const T *X,
                        int64_t ldx, T *Y, int64_t ldy, const T *Z1, int64_t ldz1, const T *Z2,
                        int64_t ldz2, T ca, T cb, T cc, Slices ysl, double avg_nnz) {
    switch (nch) {
    case 1:
        return dispatch_team<T, CH, 1>(team, st, n, rp, ci, val, w, ycols, X, ldx, Y, ldy, Z1,
                                       ldz1, Z2, ldz2, ca, cb, cc, ysl, avg_nnz);
    case 2:
        return dispatch_team<T, CH, 2>(team, st, n, rp, ci, val, w, ycols, X, ldx, Y, ldy, Z1,
                                       ldz1, Z2, ldz2, ca, cb, cc, ysl, avg_nnz);
    case 3:
        return dispatch_team<T, CH, 3>(team, st, n, rp, ci, val, w, ycols, X, ldx, Y, ldy, Z1,
                                       ldz1, Z2, ldz2, ca, cb, cc, ysl, avg_nnz);
    default:
        return dispatch_team<T, CH, 4>(team, st, n, rp, ci, val, w, ycols, X, ldx, Y, ldy, Z1,
                                       ldz1, Z2, ldz2, ca, cb, cc, ysl, avg_nnz);
    }
}

template <typename T>
int launch_spmm(cudaStream_t st, int64_t n, const int32_t *rp, const int32_t *ci,
                const T *val, int w, const T *X, int64_t ldx, T *Y, int64_t ldy,
                const T *Z1, int64_t ldz1, const T *Z2, int64_t ldz2, double ca_,
                double cb_, double cc_, double avg_nnz) {
    return launch_spmm_sl<T>(st, n, rp, ci, val, w, X, ldx, Y, ldy, Z1, ldz1, Z2, ldz2, ca_, cb_,
                             cc_, avg_nnz, Slices());
}

template <typename T>
int launch_spmm_sl(cudaStream_t st, int64_t n, const int32_t *rp, const int32_t *ci,
                   const T *val, int w, const T *X, int64_t ldx, T *Y, int64_t ldy,
                   const T *Z1, int64_t ldz1, const T *Z2, int64_t ldz2, double ca_,
                   double cb_, double cc_, double avg_nnz, Slices ysl) {
    if (n <= 0) return CACG_OK;
    if (ysl.p && (sizeof(T) != 4 || w == 1)) return CACG_ERR_ARG;
    if (w <= 0 || !rp || !ci || !val || !X || !Y) return CACG_ERR_ARG;
    const T ca = T(ca_), cb = T(cb_), cc = T(cc_);
    if (w == 1) {
        int team = avg_nnz <= 6 ? 4 : (avg_nnz <= 12 ? 8 : (avg_nnz <= 24 ? 16 : 32));
        int blocks = grid_for(n * team, kSpmmThreads);
#define CACG_SPMV_CASE(TM)                                                              \
    case TM:                                                                            \
        spmv_kernel<T, TM><<<blocks, kSpmmThreads, 0, st>>>(n, rp, ci, val, X, ldx, Y, ldy, \
                                                            Z1, ldz1, Z2, ldz2, ca, cb, cc); \
        return check_launch();
        switch (team) {
            CACG_SPMV_CASE(4)
            CACG_SPMV_CASE(8)
            CACG_SPMV_CASE(16)
            CACG_SPMV_CASE(32)
        }
#undef CACG_SPMV_CASE
        return CACG_ERR_ARG;
    }
    constexpr int VN = Vec16<T>::N;
    bool vec = (w % VN == 0) && (ldx % VN == 0) && (ldy % VN == 0) && aligned16(X) &&
               aligned16(Y) && (!Z1 || ((ldz1 % VN == 0) && aligned16(Z1))) &&
               (!Z2 || ((ldz2 % VN == 0) && aligned16(Z2)));
    const int ch = vec ? VN : 1;
    const int chunks = w / ch;
    // choose (team, nch) covering the chunks with the least idle lanes;
    // ties go to the larger team (more lanes share one row's index stream).
    int best_team = 32, best_nch = kMaxNch, best_waste = 1 << 30;
    for (int team = 1; team <= 32; team *= 2) {
        for (int nch = 1; nch <= kMaxNch; ++nch) {
            int cover = team * nch;
            int passes = (chunks + cover - 1) / cover;
            int waste = passes * cover - chunks + (passes - 1) * 4;
            if (waste < best_waste || (waste == best_waste && team > best_team)) {
                best_waste = waste;
                best_team = team;
                best_nch = nch;
            }
        }
    }
    const int ycols = (chunks + best_team * best_nch - 1) / (best_team * best_nch);
    // with several column passes each pass covers team*kMaxNch chunks
    int nch = ycols > 1 ? kMaxNch : best_nch;
    int yc = ycols > 1 ? (chunks + best_team * kMaxNch - 1) / (best_team * kMaxNch) : 1;
    if (vec)
        return dispatch_nch<T, VN>(nch, best_team, st, n, rp, ci, val, w, yc, X, ldx, Y, ldy, Z1,
                                   ldz1, Z2, ldz2, ca, cb, cc, ysl, avg_nnz);
    return dispatch_nch<T, 1>(nch, best_team, st, n, rp, ci, val, w, yc, X, ldx, Y, ldy, Z1,
                              ldz1, Z2, ldz2, ca, cb, cc, ysl, avg_nnz);
}

template int launch_spmm_sl<float>(cudaStream_t, int64_t, const int32_t *, const int32_t *,
                                   const float *, int, const float *, int64_t, float *, int64_t,
                                   const float *, int64_t, const float *, int64_t, double, double,
                                   double, double, Slices);
template int launch_spmm<double>(cudaStream_t, int64_t, const int32_t *, const int32_t *,
                                 const double *, int, const double *, int64_t, double *,
                                 int64_t, const double *, int64_t, const double *, int64_t,
                                 double, double, double, double);
template int launch_spmm<float>(cudaStream_t, int64_t, const int32_t *, const int32_t *,
                                const float *, int, const float *, int64_t, float *, int64_t,
                                const float *, int64_t, const float *, int64_t, double,
                                double, double, double);

}  // namespace cacg

using namespace cacg;

extern "C" int cacg_k_spmm(int32_t vtype, int64_t n, const int32_t *row_ptr,
                           const int32_t *col_idx, const void *val, int32_t w, const void *X,
                           int64_t ldx, void *Y, int64_t ldy, const void *Z1, int64_t ldz1,
                           const void *Z2, int64_t ldz2, double ca, double cb, double cc,
                           void *stream) {
    cudaStream_t st = (cudaStream_t)stream;
    double avg = 8.0;
    if (vtype == CACG_VAL_F64)
        return launch_spmm<double>(st, n, row_ptr, col_idx, (const double *)val, w,
                                   (const double *)X, ldx, (double *)Y, ldy,
                                   (const double *)Z1, ldz1, (const double *)Z2, ldz2, ca, cb,
                                   cc, avg);
    if (vtype == CACG_VAL_F32)
        return launch_spmm<float>(st, n, row_ptr, col_idx, (const float *)val, w,
                                  (const float *)X, ldx, (float *)Y, ldy, (const float *)Z1,
                                  ldz1, (const float *)Z2, ldz2, ca, cb, cc, avg);
    return CACG_ERR_ARG;
}

// Basis: S[:, 0:m] = R (if R given), then T_1 .. T_{s-1} (src/common.c:182-256).
extern "C" int cacg_k_basis(int32_t vtype, int64_t n, const int32_t *row_ptr,
                            const int32_t *col_idx, const void *val, const void *R, int32_t m,
                            int32_t s, double alpha, double beta, void *S, int64_t lds,
                            void *stream) {
    cudaStream_t st = (cudaStream_t)stream;
    if (s < 1 || m < 1 || lds < (int64_t)s * m) return CACG_ERR_ARG;
    const size_t es = vtype == CACG_VAL_F64 ? 8 : 4;
    if (R) {
        cudaError_t e = cudaMemcpy2DAsync(S, lds * es, R, m * es, m * es, n,
                                          cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) return CACG_ERR_CUDA;
    }
    for (int j = 1; j < s; ++j) {
        char *Sb = (char *)S;
        const void *Tm1 = Sb + (size_t)(j - 1) * m * es;
        const void *Tm2 = j >= 2 ? Sb + (size_t)(j - 2) * m * es : nullptr;
        void *Tj = Sb + (size_t)j * m * es;
        double ca = j == 1 ? alpha : 2.0 * alpha, cb = j == 1 ? beta : 2.0 * beta;
        int rc = cacg_k_spmm(vtype, n, row_ptr, col_idx, val, m, Tm1, lds, Tj, lds, Tm1, lds,
                             Tm2, lds, ca, cb, -1.0, stream);
        if (rc != CACG_OK) return rc;
    }
    return CACG_OK;
}
