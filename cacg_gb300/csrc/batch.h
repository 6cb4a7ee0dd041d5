// batch.h -- descriptors of the serving engine's batched launches.
//
// The engine advances every admitted request by one outer iteration per
// step; each phase of the iteration is ONE launch over all requests of a
// precision class.  A launch walks a tile table: request r owns the tiles
// [tile_start[r], tile_start[r+1]) (row tiles of kBRows rows, or Gram pieces
// of bpiece rows); blocks stride over the table, so the grid size is free
// (the autotuner picks it) and never changes a result.  Every reduction is
// partitioned by the request's own shape only (row tiles, Gram pieces, fixed
// summation order), so a request's iterates are bit-identical whether it ran
// alone or with others.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace cacg {

constexpr int kBMax = 64;       // requests per precision class in one step
constexpr int kBMaxK = 64;      // basis width k = s * m
constexpr int kBMaxM = 32;      // right-hand sides
constexpr int kBMaxS = 16;      // basis length s
constexpr int kBRows = 128;     // rows per row tile (SpMM, updates, norms)
constexpr int kBThreads = 256;

// Gram split-K: a block takes one piece of a request (bpiece rows), staged
// through shared memory bgchunk rows at a time; the piece's sums stay in
// registers (FP32 class: FP32 over the piece's 256 rows) and are written as
// one FP64 partial.
template <typename T>
__host__ __device__ constexpr int bgchunk() {
    return sizeof(T) == 4 ? 64 : 32;
}
template <typename T>
__host__ __device__ constexpr int bpiece() {
    return 4 * bgchunk<T>();
}
inline int bpiece_rows(bool f32) { return f32 ? bpiece<float>() : bpiece<double>(); }

// request flags
constexpr int kBActive = 1;     // takes part in this step's iteration
constexpr int kBResid = 2;      // takes part in a residual launch

struct BDesc {
    const int32_t *rp, *ci;
    const double *val;  // FP64 CSR values (residuals, FP64 class)
    const float *val32;  // FP32 copy (FP32 class)
    const double *B;
    double *X, *R;
    float *R32;         // FP32 class: R as the Gram's right operand
    void *S;            // basis of this step; Q after the update
    void *Qold;         // Q of the previous step; receives the next T_0
    void *AQ;
    double *QtAS, *QtAQ, *QtR, *alpha, *beta;
    double *F;          // LU: the factors (k x k), 1 / L_ii (k), the factors transposed (k x k)
    double *norms;      // m: squared column norms (recurrence or residual)
    double *gpart;      // Gram partials: npiece x k x (k + m)
    double *npart;      // norm partials: ntile x m
    int *status;
    int64_t n;
    int m, s, k, it;
    int flags, ntile, npiece, pad;
    double sa, sb;      // Chebyshev map: 2 / (lmax - lmin), -(lmax + lmin) / (lmax - lmin)
};

struct BBatch {
    int nr;
    int total_tiles, total_pieces, pad;
    int tile_start[kBMax + 1];
    int piece_start[kBMax + 1];
    BDesc d[kBMax];
};

// kernel kinds the autotuner sizes (blocks per SM)
enum BKind { kBKSpmm = 0, kBKGram, kBKQupd, kBKXr, kBKNumKinds };

struct BTune {
    int blocks_per_sm[kBKNumKinds];
};

// launches (k_batch.cu); T is double (FP64 class) or float (FP32 class).
// `b` is the device copy of the class's BBatch.
template <typename T>
int bl_basis_step(cudaStream_t st, const BBatch *b, int j, const BTune &tu);
template <typename T>
int bl_aq(cudaStream_t st, const BBatch *b, const BTune &tu);
template <typename T>
int bl_gram(cudaStream_t st, const BBatch *b, int which, const BTune &tu);
int bl_lu_factor(cudaStream_t st, const BBatch *b);
int bl_lu_solve(cudaStream_t st, const BBatch *b, int which);
template <typename T>
int bl_qupdate(cudaStream_t st, const BBatch *b, const BTune &tu);
template <typename T>
int bl_xrupdate(cudaStream_t st, const BBatch *b, const BTune &tu);
template <typename T>
int bl_residual(cudaStream_t st, const BBatch *b, const BTune &tu);

}  // namespace cacg
