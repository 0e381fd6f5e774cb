// Double-float arithmetic on the float32 pipes.
//
// GB300 issues float64 arithmetic at about 2 operations per clock per SM (and
// float64 <-> float32 conversions no faster) against 128 float32/int32 lanes.
// Reductions and projections that would spend one or two float64 operations
// per loaded element run here on pairs of float32 values (hi, lo) instead:
// float64 operands are split into hi + lo with integer operations only,
// products are formed to about 2^-45.5 relative (hi*hi with its FMA rounding
// error, plus the two cross terms; the dropped lo*lo is at most 2^-46 of the
// product) and sums are error-free (TwoSum, Knuth, The Art of Computer
// Programming vol. 2, 4.2.2); a sum is folded into float64 once, at the end.
#pragma once

#include <cuda_runtime.h>

namespace tdscha {

// x = hi + lo, hi = x truncated to 24 significant bits, lo the remaining 29
// mantissa bits rounded to 24 (so |x - hi - lo| <= 2^-48 |x|).  Built from the
// bit pattern: the float32 exponent is the float64 one rebiased by 896, lo is
// the integer of the low 29 mantissa bits scaled by 2^(exponent - 52).
// |x| < 2^-126 (zero included) gives hi = lo = 0, |x| < 2^-74 gives lo = 0
// (an error below 2^-97 on the unit-norm vectors, their coefficients and the
// symmetry matrix entries split here).  Finite |x| < 2^128 is assumed: every
// value split here is normalised or far below that bound, and a NaN in a new
// Lanczos vector propagates through its float64 update regardless.
__device__ __forceinline__ float2 split_f64(double x) {
    const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
    const unsigned hw = (unsigned)(bits >> 32), lw = (unsigned)bits;
    const unsigned e = (hw >> 20) & 0x7ffu;
    // (hw << 3 | lw >> 29) keeps the low 9 exponent bits and the top 23
    // mantissa bits; subtracting 896 << 23 (0xC0000000 modulo 2^32) rebiases
    // the exponent
    const unsigned hb = ((__funnelshift_l(lw, hw, 3) - 0xC0000000u) & 0x7fffffffu) | (hw & 0x80000000u);
    const float scale = __uint_as_float((hb & 0xff800000u) - (52u << 23));
    const float lo = __uint2float_rn(lw & 0x1fffffffu) * scale;
    float2 r;
    r.x = e > 896u ? __uint_as_float(hb) : 0.0f;
    r.y = e > 948u ? lo : 0.0f;
    return r;
}

// s + v into (s, c) by TwoSum: s the rounded sum, its rounding error added to c
__device__ __forceinline__ void df_two_sum_acc(float &s, float &c, float v) {
    const float t = s + v;
    const float z = t - s;
    c += (s - (t - z)) + (v - z);
    s = t;
}

// (s, c) += a * b for double-float a, b: the product to about 2^-45.5
// relative (a.lo * b.lo dropped), its hi part added to s by TwoSum, every
// rounding error collected in c.
__device__ __forceinline__ void df_fma_acc(float &s, float &c, float2 a, float2 b) {
    const float p = a.x * b.x;
    float e = fmaf(a.x, b.x, -p);
    e = fmaf(a.x, b.y, e);
    e = fmaf(a.y, b.x, e);
    df_two_sum_acc(s, c, p);
    c += e;
}

// (s, c) as a normalised pair (hi, lo), |lo| <= ulp(hi) / 2 (FastTwoSum)
__device__ __forceinline__ float2 df_norm(float s, float c) {
    const float h = s + c;
    return make_float2(h, c - (h - s));
}

// a + b for double-float a, b
__device__ __forceinline__ float2 df_add(float2 a, float2 b) {
    float s = a.x, c = a.y + b.y;
    df_two_sum_acc(s, c, b.x);
    return df_norm(s, c);
}

// a * b for double-float a, b (a.lo * b.lo dropped), normalised
__device__ __forceinline__ float2 df_mul(float2 a, float2 b) {
    const float p = a.x * b.x;
    float e = fmaf(a.x, b.x, -p);
    e = fmaf(a.x, b.y, e);
    e = fmaf(a.y, b.x, e);
    return df_norm(p, e);
}

__device__ __forceinline__ double df_to_double(float2 a) { return (double)a.x + (double)a.y; }

}  // namespace tdscha
