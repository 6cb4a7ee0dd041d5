// tc5_util.cuh -- inline-PTX helpers shared by the tcgen05 kernels
// (k_gram_tc5.cu, k_tsm_tc5.cu): shared-memory UMMA descriptors, MMA issue
// and commit, bounded mbarrier waits, TMEM loads, cp.async, and the exact
// three-way bf16 split of FP32 values.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

namespace cacg {

constexpr long long kT5SpinLimit = 1ll << 22;  // bounded mbarrier polls

__device__ __forceinline__ unsigned t5_smem_u32(const void *p) {
    return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ unsigned t5_bits(__nv_bfloat162 v) {
    return *reinterpret_cast<unsigned *>(&v);
}

__device__ __forceinline__ void t5_cp16(void *smem, const void *g, int bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(t5_smem_u32(smem)), "l"(g),
                 "r"(bytes));
}
__device__ __forceinline__ void t5_cp4(void *smem, const void *g, int bytes) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(t5_smem_u32(smem)), "l"(g),
                 "r"(bytes));
}
__device__ __forceinline__ void t5_cp_commit() { asm volatile("cp.async.commit_group;\n" ::); }

// UMMA shared-memory descriptor, K-major operand without swizzle: 8 x 16-byte
// core matrices, LBO = 128 B between K-adjacent core matrices, SBO = `sbo`
// bytes between 8-row groups; version bits 46-47 = 1.
__device__ __forceinline__ uint64_t t5_desc(unsigned saddr, unsigned sbo) {
    const uint64_t lbo = 128;
    return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

// Same with an explicit LBO (MN-major operands: LBO = bytes between 8-row K
// groups, SBO = bytes between 8-column MN groups).
__device__ __forceinline__ uint64_t t5_desc_lbo(unsigned saddr, unsigned lbo, unsigned sbo) {
    return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: D FP32, A and B bf16, both K-major,
// M x N tile.
__host__ __device__ constexpr unsigned t5_idesc(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(N >> 3) << 17) |
           ((unsigned)(M >> 4) << 24);
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

__device__ __forceinline__ void t5_mbar_arrive(uint64_t *bar) {
    asm volatile(
        "{\n"
        ".reg .b64 st;\n"
        "mbarrier.arrive.shared::cta.b64 st, [%0];\n"
        "}\n" ::"r"(t5_smem_u32(bar))
        : "memory");
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
        : "r"(t5_smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// bounded wait; false on expiry
__device__ __forceinline__ bool t5_mbar_wait(uint64_t *bar, unsigned parity) {
    for (long long i = 0; i < kT5SpinLimit; ++i)
        if (t5_mbar_try(bar, parity)) return true;
    return false;
}

// bounded wait that also gives up once *abort is set by another warp; the
// pipeline waits of the tcgen05 Gram pass their limit at run time (a test
// shortens it to exercise the expiry path), every drain wait keeps the full one
__device__ __forceinline__ bool t5_mbar_wait_or_abort(uint64_t *bar, unsigned parity,
                                                      const volatile int *abort,
                                                      long long limit = kT5SpinLimit) {
    for (long long i = 0; i < limit; ++i) {
        if (t5_mbar_try(bar, parity)) return true;
        if ((i & 63) == 63 && *abort) return false;
    }
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

__device__ __forceinline__ void t5_ld4(unsigned taddr, float (&v)[4]) {
    unsigned r[4];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int q = 0; q < 4; ++q) v[q] = __uint_as_float(r[q]);
}

// the same load without the wait: several can be in flight before one
// t5_wait_ld(); the registers are valid only after it
__device__ __forceinline__ void t5_ld4_nowait(unsigned taddr, unsigned (&r)[4]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(taddr));
}
__device__ __forceinline__ void t5_wait_ld() {
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
}

__device__ __forceinline__ void t5_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
}
__device__ __forceinline__ void t5_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
}
__device__ __forceinline__ void t5_fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

// Named barrier over the first `count` threads of the block (id >= 1), with
// an OR reduction of `pred` (uniform result for the participating threads).
__device__ __forceinline__ int t5_bar_or(int id, int count, int pred) {
    int out;
    asm volatile(
        "{\n"
        ".reg .pred p, q;\n"
        "setp.ne.s32 p, %1, 0;\n"
        "bar.red.or.pred q, %2, %3, p;\n"
        "selp.s32 %0, 1, 0, q;\n"
        "}\n"
        : "=r"(out)
        : "r"(pred), "r"(id), "r"(count)
        : "memory");
    return out;
}

// x0, x1 -> three bf16x2 words (high, middle, low slices; round-to-nearest
// at each split, so x = h + m + l up to the last slice's rounding).
// The two residual subtractions run as packed FP32 pairs (sub.rn.f32x2); the
// widening of a bf16 pair is exact bit placement, so the words equal those of
// the scalar sequence.
__device__ __forceinline__ void t5_split2(float x0, float x1, unsigned &hw, unsigned &mw,
                                          unsigned &lw) {
    asm("{\n"
        ".reg .b32 wl, wh;\n"
        ".reg .b64 v, w, r;\n"
        ".reg .f32 ra, rb;\n"
        "cvt.rn.bf16x2.f32 %0, %4, %3;\n"   // x1 -> high half, x0 -> low half
        "shl.b32 wl, %0, 16;\n"
        "and.b32 wh, %0, 0xFFFF0000;\n"
        "mov.b64 v, {%3, %4};\n"
        "mov.b64 w, {wl, wh};\n"
        "sub.rn.f32x2 r, v, w;\n"
        "mov.b64 {ra, rb}, r;\n"
        "cvt.rn.bf16x2.f32 %1, rb, ra;\n"
        "shl.b32 wl, %1, 16;\n"
        "and.b32 wh, %1, 0xFFFF0000;\n"
        "mov.b64 w, {wl, wh};\n"
        "sub.rn.f32x2 r, r, w;\n"
        "mov.b64 {ra, rb}, r;\n"
        "cvt.rn.bf16x2.f32 %2, rb, ra;\n"
        "}\n"
        : "=r"(hw), "=r"(mw), "=r"(lw)
        : "f"(x0), "f"(x1));
}

// (hi, lo) += v on two lanes at once: TwoSum (Knuth) as packed FP32 pairs,
// per lane s = hi + v; bp = s - hi; lo += (hi - (s - bp)) + (v - bp); hi = s,
// each operation rounded to nearest as in the scalar sequence, so the pairs
// equal the scalar results bit for bit (7 packed instructions for 2 values).
__device__ __forceinline__ void t5_twosum2(float &h0, float &h1, float &l0, float &l1, float v0,
                                           float v1) {
    asm("{\n"
        ".reg .b64 h, v, l, s, bp, t, e1, e2;\n"
        "mov.b64 h, {%0, %1};\n"
        "mov.b64 l, {%2, %3};\n"
        "mov.b64 v, {%4, %5};\n"
        "add.rn.f32x2 s, h, v;\n"
        "sub.rn.f32x2 bp, s, h;\n"
        "sub.rn.f32x2 t, s, bp;\n"
        "sub.rn.f32x2 e1, h, t;\n"
        "sub.rn.f32x2 e2, v, bp;\n"
        "add.rn.f32x2 e1, e1, e2;\n"
        "add.rn.f32x2 l, l, e1;\n"
        "mov.b64 {%0, %1}, s;\n"
        "mov.b64 {%2, %3}, l;\n"
        "}\n"
        : "+f"(h0), "+f"(h1), "+f"(l0), "+f"(l1)
        : "f"(v0), "f"(v1));
}

}  // namespace cacg
