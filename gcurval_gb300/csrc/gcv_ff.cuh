// Float-float ("double-float") arithmetic on the FP32 pipes.
//
// A value is an unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)/2,
// about 48 significant bits.  The building blocks are the published
// error-free transformations: Knuth's TwoSum, Dekker's Fast2Sum, and the
// FMA-based exact product (TwoProd).  Every operation below is a handful of
// FP32 instructions; on GB300 an FP32 instruction costs 1/75 of an FP64 one,
// so a float-float polynomial evaluation is several times cheaper than the
// same evaluation in FP64 while keeping ~1e-14 relative accuracy.
//
// Nothing here may be compiled with fast-math (it relies on IEEE rounding and
// on the compiler not reassociating additions; the files are built without
// --use_fast_math and multiply-adds are written as explicit fmaf).
#pragma once

#include <cuda_runtime.h>

namespace gcv {

struct ff {
    float hi, lo;
};

// Dekker Fast2Sum (|a| >= |b|)
__device__ __forceinline__ ff fast_two_sum(float a, float b);

// double -> float-float from the bit pattern (integer and FP32 operations
// only: on GB300 every FP64-pipe instruction, conversions included, costs as
// much issue time as dozens of FP32 ones).  hi = the leading 24 significand
// bits, lo = the remaining 29 bits scaled by 2^(e-52) (rounded to 24 bits),
// then renormalised.  Outside 2^-100 <= |x| < 2^127 (and for 0, NaN, Inf) the
// FP64 conversions are used.
__device__ __forceinline__ ff ff_from_double(double x)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned top = (unsigned)(b >> 32);
    const int e = (int)((top >> 20) & 0x7FFu) - 1023;
    if (e < -100 || e > 126) {
        const float h = __double2float_rn(x);
        return ff{h, __double2float_rn(x - (double)h)};
    }
    const unsigned sign = top & 0x80000000u;
    const unsigned long long m = b & 0xFFFFFFFFFFFFFull;  // 52 significand bits
    const float hi = __uint_as_float(sign | ((unsigned)(e + 127) << 23) | (unsigned)(m >> 29));
    const int sc = e - 52, s1 = sc / 2, s2 = sc - s1;   // two factors inside the float range
    float lo = __uint2float_rn((unsigned)(m & 0x1FFFFFFFull));
    lo = lo * __int_as_float((s1 + 127) << 23) * __int_as_float((s2 + 127) << 23);
    return fast_two_sum(hi, sign ? -lo : lo);
}

__device__ __forceinline__ double ff_to_double(ff a) { return (double)a.hi + (double)a.lo; }

// double -> float by truncation of the significand, from the bit pattern
// (integer operations only), for scale factors that need a few digits;
// outside the normal float range (and for 0, NaN, Inf) the FP64 conversion
__device__ __forceinline__ float f32_of_f64_trunc(double x)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned top = (unsigned)(b >> 32);
    const int e = (int)((top >> 20) & 0x7FFu) - 1023 + 127;
    if (e <= 0 || e >= 255) return __double2float_rn(x);
    return __uint_as_float((top & 0x80000000u) | ((unsigned)e << 23) | (unsigned)((b >> 29) & 0x7FFFFFull));
}

// Knuth TwoSum: s + e == a + b exactly
__device__ __forceinline__ ff two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return ff{s, e};
}

// Dekker Fast2Sum (|a| >= |b|)
__device__ __forceinline__ ff fast_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    return ff{s, __fsub_rn(b, __fsub_rn(s, a))};
}

// a + b, "sloppy" variant: error relative to |a| + |b|
__device__ __forceinline__ ff ff_add(ff a, ff b)
{
    const ff s = two_sum(a.hi, b.hi);
    return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}

__device__ __forceinline__ ff ff_add_f(ff a, float b)
{
    const ff s = two_sum(a.hi, b);
    return fast_two_sum(s.hi, __fadd_rn(s.lo, a.lo));
}

__device__ __forceinline__ ff ff_neg(ff a) { return ff{-a.hi, -a.lo}; }

// a * b with the exact product of the high parts
__device__ __forceinline__ ff ff_mul(ff a, ff b)
{
    const float p = __fmul_rn(a.hi, b.hi);
    const float e = fmaf(a.hi, b.hi, -p);
    return fast_two_sum(p, fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e)));
}

__device__ __forceinline__ ff ff_mul_f(ff a, float b)
{
    const float p = __fmul_rn(a.hi, b);
    const float e = fmaf(a.hi, b, -p);
    return fast_two_sum(p, fmaf(a.lo, b, e));
}

// exact scaling by a power of two
__device__ __forceinline__ ff ff_scale(ff a, float pow2) { return ff{a.hi * pow2, a.lo * pow2}; }

// a * b + c in one pass: the exact product of the high parts (p + e) and the
// cross terms enter the sloppy sum with c without first renormalising the
// product, 15 FP32 instructions instead of ff_add(ff_mul(a, b), c)'s 18,
// with the same error bound relative to |a b| + |c| (the unnormalised tail t
// is below 2^-22 |p| and is rounded once more, into the low-order sum).
__device__ __forceinline__ ff ff_fma(ff a, ff b, ff c)
{
    const float p = __fmul_rn(a.hi, b.hi);
    const float t = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, fmaf(a.hi, b.hi, -p)));
    const ff s = two_sum(p, c.hi);
    return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(t, c.lo)));
}

// 1 / b: y = rcp(b.hi), then one Newton step y + y (1 - b y) with the
// residual 1 - b y formed by FMAs (b.lo enters there)
__device__ __forceinline__ ff ff_recip(ff b)
{
    const float y = __frcp_rn(b.hi);
    const float e = fmaf(-b.lo, y, fmaf(-b.hi, y, 1.0f));
    return fast_two_sum(y, __fmul_rn(y, e));
}

// sqrt: s = a * rsqrt(a) (a few ulp), then one Newton correction
// s + (a - s^2) / (2 s) with the residual a - s^2 formed exactly by an FMA.
__device__ __forceinline__ ff ff_sqrt(ff a)
{
    if (!(a.hi > 0.0f)) return ff{a.hi == 0.0f ? 0.0f : __fsqrt_rn(a.hi), 0.0f};
    const float y = rsqrtf(a.hi);
    const float s = __fmul_rn(a.hi, y);
    const float r = __fadd_rn(fmaf(-s, s, a.hi), a.lo);
    return fast_two_sum(s, __fmul_rn(r, 0.5f * y));
}

}  // namespace gcv
