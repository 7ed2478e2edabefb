// dfloat.cuh -- float-pair ("double-float") arithmetic for the per-pair time of
// flight.  A value is hi + lo with |lo| <= ulp(hi)/2, giving about 48 bits of
// significand from FP32 FMA instructions (error-free transformations of Knuth
// and Dekker, as summarised in Hida, Li & Bailey, "Library for double-double and
// quad-double arithmetic", 2007).  GB300's FP64 rate is a small fraction of its
// FP32 rate, so the projection kernels use these instead of native double.
#pragma once
#include <cuda_runtime.h>

namespace bcsim_gb300 {

struct df { float hi, lo; };

__device__ __forceinline__ df df_make(float h, float l) { df r; r.hi = h; r.lo = l; return r; }

// |a| >= |b| or a == 0
__device__ __forceinline__ df fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float e = __fsub_rn(b, __fsub_rn(s, a));
    return df_make(s, e);
}

__device__ __forceinline__ df two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return df_make(s, e);
}

__device__ __forceinline__ df two_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    const float e = __fmaf_rn(a, b, -p);
    return df_make(p, e);
}

__device__ __forceinline__ df df_add(df a, df b) {
    df s = two_sum(a.hi, b.hi);
    df t = two_sum(a.lo, b.lo);
    s.lo = __fadd_rn(s.lo, t.hi);
    s = fast_two_sum(s.hi, s.lo);
    s.lo = __fadd_rn(s.lo, t.lo);
    return fast_two_sum(s.hi, s.lo);
}

// a (pair) * b (float)
__device__ __forceinline__ df df_mul_f(df a, float b) {
    df p = two_prod(a.hi, b);
    p.lo = __fmaf_rn(a.lo, b, p.lo);
    return fast_two_sum(p.hi, p.lo);
}

// a * b, both pairs
__device__ __forceinline__ df df_mul(df a, df b) {
    df p = two_prod(a.hi, b.hi);
    p.lo = __fmaf_rn(a.hi, b.lo, p.lo);
    p.lo = __fmaf_rn(a.lo, b.hi, p.lo);
    return fast_two_sum(p.hi, p.lo);
}

// a^2 for a pair
__device__ __forceinline__ df df_sqr(df a) {
    df p = two_prod(a.hi, a.hi);
    p.lo = __fmaf_rn(2.0f * a.hi, a.lo, p.lo);
    return fast_two_sum(p.hi, p.lo);
}

// sqrt of a non-negative pair: one Newton step on the FP32 square root.
__device__ __forceinline__ df df_sqrt(df a) {
    if (a.hi <= 0.0f) return df_make(0.0f, 0.0f);
    const float s = __fsqrt_rn(a.hi);
    const df s2 = two_prod(s, s);
    // residual (a - s^2), exact to pair precision
    const float r = __fadd_rn(__fadd_rn(__fsub_rn(a.hi, s2.hi), -s2.lo), a.lo);
    const float corr = __fdiv_rn(r, 2.0f * s);
    return fast_two_sum(s, corr);
}

// a - b for two floats, exact as a pair
__device__ __forceinline__ df df_diff_f(float a, float b) { return two_sum(a, -b); }

}  // namespace bcsim_gb300
