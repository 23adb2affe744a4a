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

// ---------------------------------------------------------------------------
// Float-float evaluation points.  Coordinates u = x / range are split as
// u = hi + lo with hi a multiple of the quantum q; for |hi| <= 2^23 q every
// difference of two hi values is an exactly representable float.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double ff_quantum(const unsigned int* maxbits) {
    float m = __uint_as_float(*maxbits);
    if (!(m > 1e-30f)) m = 1.f;
    int e = (int)ceil(log2((double)m));
    return ldexp(1.0, e + 4 - 23);
}

__device__ __forceinline__ void ff_split(double u, double q, float& h, float& l) {
    double hi = rint(u / q) * q;
    h = (float)hi;
    l = (float)(u - hi);
}

struct PointFF {
    float h[3], l[3];
    bool exact;
};

__device__ __forceinline__ void ff_point(const double* xd, double inv_a, double q, PointFF& P) {
    const double lim = ldexp(q, 23);
    P.exact = true;
    for (int k = 0; k < 3; ++k) {
        double u = xd[k] * inv_a;
        double hi = rint(u / q) * q;
        P.h[k] = (float)hi;
        P.l[k] = (float)(u - hi);
        if (fabs(hi) > lim) P.exact = false;
    }
}

// r^2 + eps2 of d = x - p as float-float (eps2 is the distance regulariser
// in the scaled frame, kDistEps2 / range^2); d_k = dh_k + dl_k with dh_k exact
// when the split is exact, else recovered with a two-sum.
__device__ __forceinline__ ff ff_dist2(const PointFF& X, const float* ph, const float* pl, float* dh, float* dl,
                                       float eps2) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        if (X.exact) {
            dh[k] = X.h[k] - ph[k];
            dl[k] = X.l[k] - pl[k];
        } else {
            ff t = two_sum(X.h[k], -ph[k]);
            dh[k] = t.h;
            dl[k] = t.l + (X.l[k] - pl[k]);
        }
    }
    ff a0 = two_prod(dh[0], dh[0]), a1 = two_prod(dh[1], dh[1]), a2 = two_prod(dh[2], dh[2]);
    ff s1 = two_sum(a0.h, a1.h);
    ff s2 = two_sum(s1.h, a2.h);
    float low = s1.l + s2.l + a0.l + a1.l + a2.l + eps2;
    low = __fmaf_rn(dl[0], 2.f * dh[0] + dl[0], low);
    low = __fmaf_rn(dl[1], 2.f * dh[1] + dl[1], low);
    low = __fmaf_rn(dl[2], 2.f * dh[2] + dl[2], low);
    return fast_two_sum(s2.h, low);
}

}  // namespace gk
