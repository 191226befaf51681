// Float-float ("double-float") arithmetic for the mixed-form block solve.
//
// A value is an unevaluated sum hi + lo of two FP32 numbers with |lo| <=
// ulp(hi) / 2, about 48 significant bits.  On GB300 an FP64 warp
// instruction occupies a sub-partition's FP64 pipe for about 64 cycles and
// has about 60 cycles of dependent latency, while FP32 instructions issue
// every cycle with a few cycles of latency, so a float-float operation of
// 7-24 FP32 instructions is both cheaper in issue slots and far shorter on a
// dependent chain than one FP64 operation.
//
// Algorithms (published; restated here):
//   two_sum        Knuth, TAOCP vol. 2, 4.2.2, Theorem B (error-free sum)
//   quick_two_sum  Dekker 1971 (error-free sum when |a| >= |b|)
//   two_prod       error-free product with a fused multiply-add
//   add            the accurate double-word sum of Hida, Li and Bailey
//                  ("Library for double-double and quad-double arithmetic",
//                  2007): both words summed error-free, two renormalisations
//   mul            product with the cross terms folded into the error word
//   rcp            one Newton step y + y (1 - a y) from the FP32 reciprocal
// Every FP32 operation is written with an explicit rounding intrinsic so
// that the compiler cannot contract or reorder the error-free
// transformations.
#pragma once

#include <cstdint>

namespace khs {
namespace ff {

struct FF {
    float hi, lo;
};

__device__ __forceinline__ FF make(float hi, float lo = 0.0f) { FF r; r.hi = hi; r.lo = lo; return r; }

__device__ __forceinline__ FF two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float v = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, v)), __fsub_rn(b, v));
    return make(s, e);
}

__device__ __forceinline__ FF quick_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    return make(s, __fsub_rn(b, __fsub_rn(s, a)));
}

__device__ __forceinline__ FF add(FF a, FF b)
{
    FF s = two_sum(a.hi, b.hi);
    const FF t = two_sum(a.lo, b.lo);
    s.lo = __fadd_rn(s.lo, t.hi);
    s = quick_two_sum(s.hi, s.lo);
    s.lo = __fadd_rn(s.lo, t.lo);
    return quick_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ FF neg(FF a) { return make(-a.hi, -a.lo); }
__device__ __forceinline__ FF sub(FF a, FF b) { return add(a, neg(b)); }

__device__ __forceinline__ FF mul(FF a, FF b)
{
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return quick_two_sum(p, e);
}

// acc + a * b with the product kept as an unnormalised pair (the accurate
// sum below is exact in its first step for any pair).
__device__ __forceinline__ FF fma(FF acc, FF a, FF b)
{
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return add(acc, make(p, e));
}

// acc - a * b
__device__ __forceinline__ FF fms(FF acc, FF a, FF b) { return fma(acc, neg(a), b); }

__device__ __forceinline__ FF rcp(FF a)
{
    const float y = __frcp_rn(a.hi);
    const FF r = sub(make(1.0f), mul(a, make(y)));  // 1 - a y, small
    return add(make(y), make(__fmul_rn(y, r.hi), 0.0f));
}

// Splits an FP64 value into float-float with integer operations only (no
// FP64 instruction): hi keeps the leading 24 significant bits (truncated),
// lo the next 24 (rounded).  Zero, FP64 subnormals and magnitudes below the
// FP32 normal range (< 2^-126) become zero; the low word is dropped below
// 2^-74.  Infinities, NaNs and magnitudes of 2^128 or more set `bad`.
__device__ __forceinline__ FF split(double x, bool &bad)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned top = unsigned(b >> 32);
    const unsigned sign = top & 0x80000000u;
    const int biased = int((top >> 20) & 0x7ffu);
    if (biased == 0x7ff) { bad = true; return make(0.0f); }
    const int e = biased - 1023;
    if (biased == 0 || e < -126) return make(0.0f);
    if (e > 127) { bad = true; return make(0.0f); }
    const unsigned long long m = b & 0x000fffffffffffffull;
    const float hi = __uint_as_float(sign | (unsigned(e + 127) << 23) | unsigned(m >> 29));
    float lo = 0.0f;
    if (e >= -74) {
        const float scale = __uint_as_float(unsigned(e + 75) << 23);  // 2^(e - 52)
        lo = __fmul_rn(__uint2float_rn(unsigned(m & 0x1fffffffull)), scale);
        if (sign) lo = -lo;
    }
    return make(hi, lo);
}

// hi + lo rounded to FP64 (two conversions and one FP64 add).
__device__ __forceinline__ double to_double(FF a) { return double(a.hi) + double(a.lo); }

// |a| ordered like the sign-cleared bit pattern of its high word.
__device__ __forceinline__ unsigned abs_bits(FF a) { return __float_as_uint(a.hi) & 0x7fffffffu; }

__device__ __forceinline__ FF shfl(FF a, int src)
{
    return make(__shfl_sync(0xffffffffu, a.hi, src), __shfl_sync(0xffffffffu, a.lo, src));
}

}  // namespace ff
}  // namespace khs
