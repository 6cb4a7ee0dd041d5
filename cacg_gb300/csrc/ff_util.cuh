// ff_util.cuh -- float-float helpers that keep FP64 values off GB300's FP64
// pipe (1/64 of the FP32 rate): exact splits and conversions by bit
// operations, used by the residual replacement (k_dia.cu) and the X/R update
// (k_xr16.cu).
#pragma once

#include <cuda_runtime.h>

namespace cacg {

// x = hi + lo with FP32 hi, lo, using integer operations only (GB300's FP64
// pipe runs at 1/64 of the FP32 rate): hi = x truncated to 24 significant
// bits, lo = the next 29 bits rounded to FP32 (about 48 bits in all).
// Values outside the normal FP32 exponent range give (float)x, 0.
__device__ __forceinline__ void ff_split_bits(double x, float &hi, float &lo) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7FF);
    const unsigned long long sgn = b >> 63;
    if (e < 1023 - 126 + 24 || e > 1023 + 127) {  // tiny, huge, inf, NaN, zero
        hi = (float)x;
        lo = 0.f;
        return;
    }
    const unsigned long long mant = b & ((1ull << 52) - 1);
    hi = __uint_as_float((unsigned)((sgn << 31) | ((unsigned long long)(e - 1023 + 127) << 23) |
                                    (mant >> 29)));
    const unsigned rem = (unsigned)(mant & ((1u << 29) - 1));
    // rem * 2^(e - 1075): the scale is a normal FP32 power of two in this range
    const int se = e - 1075 + 127;
    const float scale = se >= 1 ? __uint_as_float((unsigned)se << 23) : 0.f;
    // (float)rem, rounded to nearest, without an integer conversion (which
    // runs on the slow conversion pipe here): each 16-bit half is exact as
    // (2^23 + half) - 2^23, the high half times 2^16 stays exact, and the one
    // addition rounds like the conversion would
    const float rh = __fsub_rn(__uint_as_float(0x4B000000u | (rem >> 16)), 8388608.f);
    const float rl = __fsub_rn(__uint_as_float(0x4B000000u | (rem & 0xFFFFu)), 8388608.f);
    const float l = __fadd_rn(__fmul_rn(rh, 65536.f), rl) * scale;
    lo = sgn ? -l : l;
}

// exact FP32 -> FP64 by bits for normal values (others through the cast)
__device__ __forceinline__ double ff_widen(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xFF;
    if (e == 0 || e == 0xFF) return (double)f;
    const unsigned long long b = ((unsigned long long)(u >> 31) << 63) |
                                 ((unsigned long long)(e - 127 + 1023) << 52) |
                                 ((unsigned long long)(u & 0x7FFFFF) << 29);
    return __longlong_as_double((long long)b);
}

// (float)x, round to nearest even, for x in the normal FP32 range by bit
// operations; zero, underflow, overflow, infinities and NaN take the cast.
__device__ __forceinline__ float ff_narrow(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7FF) - 896;
    if (e <= 0 || e >= 255) return (float)x;
    const unsigned long long mant = b & 0xFFFFFFFFFFFFFull;
    const unsigned top = (unsigned)(mant >> 29);
    const unsigned long long rem = mant & 0x1FFFFFFFull, half = 0x10000000ull;
    const unsigned up = (rem > half || (rem == half && (top & 1u))) ? 1u : 0u;
    // a mantissa carry moves into the exponent (up to infinity), as rounding does
    return __uint_as_float((((unsigned)e << 23) + top + up) | ((unsigned)(b >> 32) & 0x80000000u));
}

// (hi, lo) += x * x for x = xh + xl (float-float, about 2^-44 relative):
// xh^2 exactly as p + e (FMA), the cross term 2 xh xl in FP32, xl^2 dropped;
// TwoSum folds p into hi.
__device__ __forceinline__ void ff_add_square(float xh, float xl, float &hi, float &lo) {
    const float p = xh * xh;
    const float e = fmaf(xh, xh, -p);
    const float s = hi + p;
    const float bp = s - hi;
    lo += ((hi - (s - bp)) + (p - bp)) + (e + 2.f * xh * xl);
    hi = s;
}

}  // namespace cacg
