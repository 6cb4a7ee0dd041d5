// cacg_internal.cuh -- shared device/host helpers of libcacg.so (sm_103a).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

#include "cacg.h"

namespace cacg {

// ---------------------------------------------------------------- status
extern std::atomic<int64_t> g_launches;

// device-side status bits (one int per solve, read by the host between steps)
enum : int {
    kStatusBreakdown = 1,  // zero / non-finite pivot in the small LU
    kStatusNonFinite = 2,  // NaN/Inf in a residual norm
    kStatusTimeout = 4,    // a bounded device-side wait ran out
};

#define CACG_CUDA_TRY(expr)                                                  \
    do {                                                                     \
        cudaError_t _e = (expr);                                             \
        if (_e != cudaSuccess) {                                             \
            cacg::record_cuda_error(_e, #expr, __FILE__, __LINE__);          \
            return _e == cudaErrorMemoryAllocation ? CACG_ERR_OOM : CACG_ERR_CUDA; \
        }                                                                    \
    } while (0)

void record_cuda_error(cudaError_t e, const char *what, const char *file, int line);
const char *last_cuda_error_text();

inline int check_launch() {
    g_launches.fetch_add(1, std::memory_order_relaxed);
    cudaError_t e = cudaPeekAtLastError();
    if (e != cudaSuccess) {
        record_cuda_error(e, "kernel launch", __FILE__, __LINE__);
        return CACG_ERR_CUDA;
    }
    return CACG_OK;
}

int sm_count();              // multiprocessors of the current device
size_t max_smem_optin();     // opt-in shared memory per block (bytes)

// Opt-in dynamic shared memory of a kernel, set on the current device the
// first time that device launches it (the attribute belongs to the device's
// context: a process that drives several devices sets it on each).
void set_smem_attr_fn(const void *fn, int bytes);
template <typename K>
inline void set_smem_attr(K *fn, int bytes) {
    set_smem_attr_fn(reinterpret_cast<const void *>(fn), bytes);
}

// ------------------------------------------------------- vector traits
template <typename T> struct Vec16;
template <> struct Vec16<double> {
    using type = double2;
    static constexpr int N = 2;
};
template <> struct Vec16<float> {
    using type = float4;
    static constexpr int N = 4;
};

__device__ __forceinline__ void vload(double (&d)[2], const double *p) {
    double2 v = __ldg(reinterpret_cast<const double2 *>(p));
    d[0] = v.x; d[1] = v.y;
}
__device__ __forceinline__ void vload(float (&d)[4], const float *p) {
    float4 v = __ldg(reinterpret_cast<const float4 *>(p));
    d[0] = v.x; d[1] = v.y; d[2] = v.z; d[3] = v.w;
}
// generic-pointer vector loads (shared or global memory)
__device__ __forceinline__ void vload_plain(double (&d)[2], const double *p) {
    double2 v = *reinterpret_cast<const double2 *>(p);
    d[0] = v.x; d[1] = v.y;
}
__device__ __forceinline__ void vload_plain(float (&d)[4], const float *p) {
    float4 v = *reinterpret_cast<const float4 *>(p);
    d[0] = v.x; d[1] = v.y; d[2] = v.z; d[3] = v.w;
}
__device__ __forceinline__ void vstore(double *p, const double (&d)[2]) {
    *reinterpret_cast<double2 *>(p) = make_double2(d[0], d[1]);
}
__device__ __forceinline__ void vstore(float *p, const float (&d)[4]) {
    *reinterpret_cast<float4 *>(p) = make_float4(d[0], d[1], d[2], d[3]);
}

// a0 += v x0, a1 += v x1 as one packed FP32 FMA (fma.rn.f32x2, sm_100 and
// later): two independent round-to-nearest FMAs, bit-identical to fmaf
__device__ __forceinline__ void fma2_bcast(float &a0, float &a1, float v, float x0, float x1) {
    asm("{\n"
        ".reg .b64 va, xa, ac;\n"
        "mov.b64 va, {%2, %2};\n"
        "mov.b64 xa, {%3, %4};\n"
        "mov.b64 ac, {%0, %1};\n"
        "fma.rn.f32x2 ac, va, xa, ac;\n"
        "mov.b64 {%0, %1}, ac;\n"
        "}\n"
        : "+f"(a0), "+f"(a1)
        : "f"(v), "f"(x0), "f"(x1));
}

inline bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

// ------------------------------------------------------ bf16 slice planes
// An FP32 block may carry three bf16 "slice planes" (same shape and row
// stride, planes `plane` elements apart) with x == s1 + s2 + s3 exactly up to
// FP32's 24 bits: s1 = bf16(x), s2 = bf16(x - s1), s3 = bf16(x - s1 - s2).
// Producers write them next to the FP32 value; the tensor-core Gram reads them.
struct Slices {
    __nv_bfloat16 *p = nullptr;  // plane 0; planes 1, 2 at +plane, +2*plane
    int64_t plane = 0;
};

__device__ __forceinline__ void split3_bits(float x, unsigned short &h, unsigned short &m,
                                            unsigned short &l) {
    __nv_bfloat16 bh = __float2bfloat16_rn(x);
    float r1 = x - __bfloat162float(bh);
    __nv_bfloat16 bm = __float2bfloat16_rn(r1);
    float r2 = r1 - __bfloat162float(bm);
    __nv_bfloat16 bl = __float2bfloat16_rn(r2);
    h = __bfloat16_as_ushort(bh);
    m = __bfloat16_as_ushort(bm);
    l = __bfloat16_as_ushort(bl);
}

// slices of one value at element offset `off`
__device__ __forceinline__ void store_slices1(const Slices &S, int64_t off, float x) {
    unsigned short h, m, l;
    split3_bits(x, h, m, l);
    unsigned short *b = reinterpret_cast<unsigned short *>(S.p);
    b[off] = h;
    b[S.plane + off] = m;
    b[2 * S.plane + off] = l;
}

// slices of four consecutive values at an 8-byte-aligned element offset
__device__ __forceinline__ void store_slices4(const Slices &S, int64_t off, const float (&x)[4]) {
    unsigned short h[4], m[4], l[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) split3_bits(x[q], h[q], m[q], l[q]);
    unsigned short *b = reinterpret_cast<unsigned short *>(S.p);
    *reinterpret_cast<uint2 *>(b + off) =
        make_uint2(h[0] | ((unsigned)h[1] << 16), h[2] | ((unsigned)h[3] << 16));
    *reinterpret_cast<uint2 *>(b + S.plane + off) =
        make_uint2(m[0] | ((unsigned)m[1] << 16), m[2] | ((unsigned)m[3] << 16));
    *reinterpret_cast<uint2 *>(b + 2 * S.plane + off) =
        make_uint2(l[0] | ((unsigned)l[1] << 16), l[2] | ((unsigned)l[3] << 16));
}

// ------------------------------------------------- launcher declarations
// All launchers return CACG_OK or CACG_ERR_*; they are asynchronous.

// Y = ca*(A X) + cb*Z1 + cc*Z2, width w (T = double / float); for float Y may
// also get its bf16 slice planes (Ysl.p != nullptr).
template <typename T>
int launch_spmm_sl(cudaStream_t st, int64_t n, const int32_t *rp, const int32_t *ci,
                   const T *val, int w, const T *X, int64_t ldx, T *Y, int64_t ldy,
                   const T *Z1, int64_t ldz1, const T *Z2, int64_t ldz2, double ca, double cb,
                   double cc, double avg_nnz, Slices Ysl);
template <typename T>
int launch_spmm(cudaStream_t st, int64_t n, const int32_t *rp, const int32_t *ci,
                const T *val, int w, const T *X, int64_t ldx, T *Y, int64_t ldy,
                const T *Z1, int64_t ldz1, const T *Z2, int64_t ldz2, double ca,
                double cb, double cc, double avg_nnz);

// Residual in FP64 with optional cast copies:  R = B - A X ;  R32 = (float)R ;
// S0 = (T)R ; norms[c] = ||R(:,c)||^2 (partials in ws, finished by a 2nd pass).
int launch_residual(cudaStream_t st, int64_t n, const int32_t *rp, const int32_t *ci,
                    const double *val, int m, const double *X, const double *B,
                    double *R, void *S0, int s0_is_f32, int64_t lds, double *norms,
                    double *ws, double avg_nnz);
// Second half of launch_residual, for an R = B - A X formed elsewhere.
int launch_residual_post(cudaStream_t st, int64_t n, int m, double *R, void *S0, int s0_is_f32,
                         int64_t lds, double *norms, double *ws);
// Residual for the mixed mode: also R32 = (float)R and the slice planes of S0, R32.
int launch_residual_sl(cudaStream_t st, int64_t n, const int32_t *rp, const int32_t *ci,
                       const double *val, int m, const double *X, const double *B, double *R,
                       float *S0, int64_t lds, float *R32, double *norms, double *ws,
                       double avg_nnz, Slices S0sl, Slices R32sl);

// Gram: C (ka x (kb1+kb2)) = L^T [R1 | R2] (FP64 accumulation).  symmetric:
// L^T R1 is symmetric (R1 = A L with A symmetric); the FP64 CUDA-core Gram then
// computes its upper triangle only (one output tile) and mirrors it.
template <typename T>
int launch_gram(cudaStream_t st, int variant, int64_t n, const T *L, int64_t ldl, int ka,
                const T *R1, int64_t ldr1, int kb1, const T *R2, int64_t ldr2, int kb2,
                double *C1, int ldc1, double *C2, int ldc2, double *ws, size_t ws_bytes,
                bool symmetric = false);
size_t gram_workspace_bytes(int64_t n, int ka, int kb);

// dst = src for an n x w FP32 block (rows of lds / ldd values)
int launch_copy_rows_f32(cudaStream_t st, int64_t n, int w, const float *src, int64_t lds,
                         float *dst, int64_t ldd);

// Tensor-core Gram of FP32 blocks (three bf16 slices per value, six slice
// products, FP32 accumulation over 256-row groups, FP64 across groups).
int launch_gram_tc(cudaStream_t st, int64_t n, const float *L, int64_t ldl, int ka,
                   const float *R1, int64_t ldr1, int kb1, const float *R2, int64_t ldr2, int kb2,
                   double *C1, int ldc1, double *C2, int ldc2, double *ws, size_t ws_bytes);
size_t gram_tc_workspace_bytes(int64_t n, int ka, int kb);
// Tensor-core Gram reading precomputed slice planes (L, R1, R2 slices; the
// row strides ldl, ldr1, ldr2 and ka, kb1, kb2 multiples of 8).
int launch_gram_tcs(cudaStream_t st, int64_t n, Slices L, int64_t ldl, int ka, Slices R1,
                    int64_t ldr1, int kb1, Slices R2, int64_t ldr2, int kb2, double *C1,
                    int ldc1, double *C2, int ldc2, double *ws, size_t ws_bytes);
size_t gram_tcs_workspace_bytes(int64_t n, int ka, int kb);
// tcgen05 Gram of FP32 blocks (bf16 slices converted in the kernel, TMEM
// accumulators); *status gets kStatusTimeout if a bounded wait expires.
int launch_gram_tc5(cudaStream_t st, int64_t n, const float *L, int64_t ldl, int ka,
                    const float *R1, int64_t ldr1, int kb1, const float *R2, int64_t ldr2,
                    int kb2, double *C1, int ldc1, double *C2, int ldc2, double *ws,
                    size_t ws_bytes, int *status);
size_t gram_tc5_workspace_bytes(int64_t n, int ka, int kb);
bool gram_tc5_supported(int ka, int kb);
// Q_out = S - Q_in beta on tcgen05 (FP32 Q, S; FP64 beta), k % 16 == 0, k <= 96;
// TMA-fed unless allow_tma is false (then the cp.async-fed kernel, same results)
int launch_qupdate_tc5(cudaStream_t st, int64_t n, int k, float *Qout, int64_t ldo,
                       const float *Qin, int64_t ldq, const float *S, int64_t lds,
                       const double *beta, int *status, bool allow_tma = true);
bool tsm_q_tc5_supported(int k);
// X += Q alpha, R -= AQ alpha, S0 = R32 = (float)R, norms: tcgen05, m <= 16, k <= 256
int launch_xrupdate_tc5(cudaStream_t st, int64_t n, int k, int m, const float *Q,
                        const float *AQ, int64_t ldq, const double *alpha, double *X, double *R,
                        float *S0, int64_t lds, float *R32, double *norms, double *ws,
                        int *status);
bool tsm_xr_tc5_supported(int k, int m);
// norms[c] = sum over G partial rows of part[g * m + c] (fixed order)
int launch_colsum(cudaStream_t st, const double *part, int G, int m, double *norms);
int launch_split_planes(cudaStream_t st, int64_t n, int w, const float *X, int64_t ld,
                        Slices out);
bool gram_tcs_supported(int ka, int kb1, int kb2, int64_t ldl, int64_t ldr1, int64_t ldr2);

// Q_out = S - Q_in * beta  (Q_out may alias S; never Q_in).
template <typename T>
int launch_qupdate(cudaStream_t st, int64_t n, int k, T *Qout, int64_t ldo,
                   const T *Qin, int64_t ldq, const T *S, int64_t lds, const double *beta);
// Same, also writing Qout's slice planes (float, direct-load shapes only).
int launch_qupdate_sl(cudaStream_t st, int64_t n, int k, float *Qout, int64_t ldo,
                      const float *Qin, int64_t ldq, const float *S, int64_t lds,
                      const double *beta, Slices Qsl);

// X += Q alpha; R -= AQ alpha; S0 = (T)R; R32 = (float)R; norms.
template <typename T>
int launch_xrupdate(cudaStream_t st, int64_t n, int k, int m, const T *Q, const T *AQ,
                    int64_t ldq, const double *alpha, double *X, double *R, T *S0,
                    int64_t lds, float *R32, double *norms, double *ws);
size_t norm_workspace_doubles(int64_t n, int m);
// FP32 X/R update writing the slice planes of the next T_0 (S0) and of R32.
int launch_xrupdate_sl(cudaStream_t st, int64_t n, int k, int m, const float *Q,
                       const float *AQ, int64_t ldq, const double *alpha, double *X, double *R,
                       float *S0, int64_t lds, float *R32, double *norms, double *ws,
                       Slices S0sl, Slices R32sl);
// Same update with the k-term products accumulated in T (FP32 FMAs for float).
// X/R update for m = 16, k a multiple of 16, FP32 Q and AQ (k_xr16.cu):
// coalesced split-k rows, reduce-scatter over four lanes, FP64 only in the
// additions into X and R.  CACG_ERR_UNSUPPORTED for other shapes.
int launch_xrupdate_m16(cudaStream_t st, int64_t n, int k, const float *Q, const float *AQ,
                        int64_t ldq, const double *alpha, double *X, double *R, float *S0,
                        int64_t lds, float *R32, double *norms, double *ws);
// the same with Q and AQ fed by TMA (k % 4 == 0, k <= 128, 16-byte aligned
// operands and row strides); *status gets kStatusTimeout if a bounded wait expires
int launch_xrupdate_m16_tma(cudaStream_t st, int64_t n, int k, const float *Q, const float *AQ,
                            int64_t ldq, const double *alpha, double *X, double *R, float *S0,
                            int64_t lds, float *R32, double *norms, double *ws, int *status);
// the same on the float-float state: X and R as FP32 pairs (n x 16 high
// parts, then n x 16 low parts); no FP64 instruction
int launch_xrupdate_m16_ff(cudaStream_t st, int64_t n, int k, const float *Q, const float *AQ,
                           int64_t ldq, const double *alpha, float *Xff, float *Rff, float *S0,
                           int64_t lds, float *R32, double *norms, double *ws, int *status);

template <typename T>
int launch_xrupdate_fast(cudaStream_t st, int64_t n, int k, int m, const T *Q, const T *AQ,
                         int64_t ldq, const double *alpha, double *X, double *R, T *S0,
                         int64_t lds, float *R32, double *norms, double *ws);

// Small LU (Crout, U unit diagonal, no pivoting); F holds 2 k*k + k doubles
// (the factor, its reciprocal pivots, and the factor transposed for the solves).
int launch_lu_factor(cudaStream_t st, int k, const double *M, double *F, int *status);
int launch_lu_solve(cudaStream_t st, int k, const double *F, int r, const double *RHS,
                    double *Y);

int launch_gerschgorin(cudaStream_t st, int64_t n, const int32_t *rp, const int32_t *ci,
                       const double *val, double *out, double *ws);

// norms[c] = ||R(:,c)||^2 of an n x m FP64 block (two-pass, fixed order).
int launch_colnorm(cudaStream_t st, int64_t n, int m, const double *R, double *norms,
                   double *ws);

int launch_cast_f64_f32(cudaStream_t st, int64_t count, const double *in, float *out);
int launch_cast_strided(cudaStream_t st, int64_t n, int w, const double *in, int64_t ldi,
                        void *out, int out_is_f32, int64_t ldo);

// Lanczos helpers (FP64): dot products with fixed-order reduction.
int launch_dot(cudaStream_t st, int64_t n, const double *a, const double *b, double *out,
               double *ws);
int launch_axpby(cudaStream_t st, int64_t n, double a, const double *x, double b,
                 double *y);

}  // namespace cacg
