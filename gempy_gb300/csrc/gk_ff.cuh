// Float-float ("double-single") arithmetic on the FP32 pipe: a value is the
// unevaluated sum hi + lo of two floats, giving a ~48-bit significand.  The
// error-free transformations are the classical ones (Knuth TwoSum, Dekker
// Fast2Sum, FMA-based TwoProd; e.g. Muller et al., Handbook of
// Floating-Point Arithmetic, ch. 4-5).  Only adds, multiplies and fmaf are
// used; the compiler must not reassociate (no fast-math), and contracting
// a*b+c into fmaf only makes the low words more accurate.
#pragma once

#include <cuda_runtime.h>

namespace gk {

struct ff {
    float h, l;
};

__device__ __forceinline__ ff two_sum(float a, float b) {
    float s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}

__device__ __forceinline__ ff fast_two_sum(float a, float b) {  // |a| >= |b| or a == 0
    float s = __fadd_rn(a, b);
    float e = __fsub_rn(b, __fsub_rn(s, a));
    return {s, e};
}

__device__ __forceinline__ ff two_prod(float a, float b) {
    float p = __fmul_rn(a, b);
    float e = __fmaf_rn(a, b, -p);
    return {p, e};
}

__device__ __forceinline__ ff ff_add(ff a, ff b) {
    ff s = two_sum(a.h, b.h);
    float e = s.l + (a.l + b.l);
    return fast_two_sum(s.h, e);
}

__device__ __forceinline__ ff ff_add_f(ff a, float c) {
    ff s = two_sum(a.h, c);
    float e = s.l + a.l;
    return fast_two_sum(s.h, e);
}

__device__ __forceinline__ ff ff_mul(ff a, ff b) {
    ff p = two_prod(a.h, b.h);
    float e = __fmaf_rn(a.h, b.l, __fmaf_rn(a.l, b.h, p.l));
    return fast_two_sum(p.h, e);
}

__device__ __forceinline__ ff ff_mul_f(ff a, float c) {
    ff p = two_prod(a.h, c);
    float e = __fmaf_rn(a.l, c, p.l);
    return fast_two_sum(p.h, e);
}

// c + x * t, the Horner step: the product is left unnormalized, the add
// renormalizes.
__device__ __forceinline__ ff ff_horner(ff x, ff t, float c) {
    ff p = two_prod(x.h, t.h);
    float e = __fmaf_rn(x.h, t.l, __fmaf_rn(x.l, t.h, p.l));
    ff s = two_sum(p.h, c);
    return fast_two_sum(s.h, s.l + e);
}

// sqrt of a non-negative float-float: one Newton correction of rsqrt-based
// sqrt (the 2-ulp start squares to ~2^-44 relative error).
__device__ __forceinline__ ff ff_sqrt(ff a) {
    if (a.h <= 0.f) return {0.f, 0.f};
    float y = rsqrtf(a.h);
    float s = a.h * y;
    float e = __fmaf_rn(-s, s, a.h) + a.l;
    return fast_two_sum(s, e * 0.5f * y);
}

__device__ __forceinline__ double ff_to_double(ff a) { return (double)a.h + (double)a.l; }

__device__ __forceinline__ ff ff_from_double(double x) {
    float h = (float)x;
    return {h, (float)(x - (double)h)};
}

}  // namespace gk
