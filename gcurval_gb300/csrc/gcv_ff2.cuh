// Two float-float numbers at once on the packed FP32 instructions of sm_100+
// (FFMA2 / FADD2 / FMUL2: one instruction rounds two independent FP32
// operations, each exactly as its scalar counterpart would).
//
// An ff2 holds two float-float values in the lanes of two float2 registers:
// hi = (a.hi, b.hi), lo = (a.lo, b.lo).  Every operation below is the
// operation of gcv_ff.cuh applied lane by lane, with the same sequence of
// roundings, so a packed evaluation gives bit for bit the results of the two
// scalar evaluations it replaces, in about half the issued instructions.
#pragma once

#include <cuda_runtime.h>

#include "gcv_ff.cuh"

namespace gcv {

struct ff2 {
    float2 hi, lo;
};

__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __fadd2_rn(a, neg2(b)); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

__device__ __forceinline__ ff2 pack(ff a, ff b) { return ff2{make_float2(a.hi, b.hi), make_float2(a.lo, b.lo)}; }
__device__ __forceinline__ ff2 splat(ff a) { return pack(a, a); }
__device__ __forceinline__ ff lane0(ff2 a) { return ff{a.hi.x, a.lo.x}; }
__device__ __forceinline__ ff lane1(ff2 a) { return ff{a.hi.y, a.lo.y}; }

// Knuth TwoSum, lane by lane
__device__ __forceinline__ ff2 two_sum2(float2 a, float2 b)
{
    const float2 s = add2(a, b);
    const float2 bb = sub2(s, a);
    const float2 e = add2(sub2(a, sub2(s, bb)), sub2(b, bb));
    return ff2{s, e};
}

// Dekker Fast2Sum (|a| >= |b| in each lane)
__device__ __forceinline__ ff2 fast_two_sum2(float2 a, float2 b)
{
    const float2 s = add2(a, b);
    return ff2{s, sub2(b, sub2(s, a))};
}

// ff_add, lane by lane
__device__ __forceinline__ ff2 ff2_add(ff2 a, ff2 b)
{
    const ff2 s = two_sum2(a.hi, b.hi);
    return fast_two_sum2(s.hi, add2(s.lo, add2(a.lo, b.lo)));
}

__device__ __forceinline__ ff2 ff2_neg(ff2 a) { return ff2{neg2(a.hi), neg2(a.lo)}; }

// ff_mul, lane by lane
__device__ __forceinline__ ff2 ff2_mul(ff2 a, ff2 b)
{
    const float2 p = mul2(a.hi, b.hi);
    const float2 e = fma2(a.hi, b.hi, neg2(p));
    return fast_two_sum2(p, fma2(a.hi, b.lo, fma2(a.lo, b.hi, e)));
}

// ff_fma, lane by lane: a * b + c
__device__ __forceinline__ ff2 ff2_fma(ff2 a, ff2 b, ff2 c)
{
    const float2 p = mul2(a.hi, b.hi);
    const float2 t = fma2(a.hi, b.lo, fma2(a.lo, b.hi, fma2(a.hi, b.hi, neg2(p))));
    const ff2 s = two_sum2(p, c.hi);
    return fast_two_sum2(s.hi, add2(s.lo, add2(t, c.lo)));
}

// ff_sqrt, lane by lane (0 for a zero lane, NaN for a negative one)
__device__ __forceinline__ ff2 ff2_sqrt(ff2 a)
{
    const float2 y = make_float2(rsqrtf(a.hi.x), rsqrtf(a.hi.y));
    const float2 s = mul2(a.hi, y);
    const float2 r = add2(fma2(neg2(s), s, a.hi), a.lo);
    ff2 q = fast_two_sum2(s, mul2(r, make_float2(0.5f * y.x, 0.5f * y.y)));
    if (!(a.hi.x > 0.0f)) {
        q.hi.x = a.hi.x == 0.0f ? 0.0f : __fsqrt_rn(a.hi.x);
        q.lo.x = 0.0f;
    }
    if (!(a.hi.y > 0.0f)) {
        q.hi.y = a.hi.y == 0.0f ? 0.0f : __fsqrt_rn(a.hi.y);
        q.lo.y = 0.0f;
    }
    return q;
}

// exact scaling of both lanes by the same power of two
__device__ __forceinline__ ff2 ff2_scale(ff2 a, float pow2)
{
    const float2 s = make_float2(pow2, pow2);
    return ff2{mul2(a.hi, s), mul2(a.lo, s)};
}

}  // namespace gcv
