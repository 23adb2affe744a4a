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

// a + b of two non-negative floats as an exact pair: Fast2Sum on the
// ordered operands (two comparisons instead of TwoSum's three extra adds)
__device__ __forceinline__ ff two_sum_nonneg(float a, float b) {
    const float hi = fmaxf(a, b), lo = fminf(a, b);
    return fast_two_sum(hi, lo);
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
// The result is left unnormalised (|lo| within a few ulps of hi): every user
// reads it through exact products and sums.
__device__ __forceinline__ ff ff_sqrt(ff a) {
    if (a.h <= 0.f) return {0.f, 0.f};
    float y = rsqrtf(a.h);
    float s = a.h * y;
    float e = __fmaf_rn(-s, s, a.h) + a.l;
    return {s, e * 0.5f * y};
}

// ff_sqrt for an argument known to be positive: r^2 + eps2 of the tile
// loops, whose distance regulariser eps2 is a positive normal float.
__device__ __forceinline__ ff ff_sqrt_pos(ff a) {
    float y = rsqrtf(a.h);
    float s = a.h * y;
    float e = __fmaf_rn(-s, s, a.h) + a.l;
    return {s, e * 0.5f * y};
}

__device__ __forceinline__ double ff_to_double(ff a) { return (double)a.h + (double)a.l; }

// ---------------------------------------------------------------------------
// Cubic covariance in float-float, as polynomials of s = r / a (0 <= s < 1):
//   C(s)         = 1 + s^2 (-7 + s (8.75 + s^2 (-3.5 + 0.75 s^2)))
//   a^2 C'(r)/r  = -14 + s (26.25 + s^2 (-17.5 + 5.25 s^2))
// In every Horner step c + x t of these two polynomials |x t| <= |c| holds on
// 0 <= s <= 1 (each inner polynomial is monotone on [0, 1]; the bounds are
// 0.75 <= 3.5, 3.5 <= 8.75, 6 <= 7, 1 - C(s) <= 1 and 5.25 <= 17.5,
// 17.5 <= 26.25, 14 <= 14), so Fast2Sum(c, x t) is exact and replaces TwoSum.
// ---------------------------------------------------------------------------
// The steps leave their result unnormalised (lo = exact Fast2Sum error plus
// the product's low-order terms, within a few ulps of hi); the next step
// reads both words through exact products.  The polynomial's variable (s^2,
// s) is normalised, so the dropped product of the two low words stays at the
// eps^2 level.
__device__ __forceinline__ ff ff_horner_dom(ff x, ff t, float c) {
    ff p = two_prod(x.h, t.h);
    float e = __fmaf_rn(x.h, t.l, __fmaf_rn(x.l, t.h, p.l));
    ff s = fast_two_sum(c, p.h);
    return {s.h, s.l + e};
}

// c + m x with |m x| <= |c| (the innermost step; m a float constant)
__device__ __forceinline__ ff ff_lin_dom(ff x, float m, float c) {
    ff p = two_prod(x.h, m);
    float e = __fmaf_rn(x.l, m, p.l);
    ff s = fast_two_sum(c, p.h);
    return {s.h, s.l + e};
}

// a * b left unnormalised (|lo| a few ulps of hi): for operands that are
// only read through exact products
__device__ __forceinline__ ff ff_mul_un(ff a, ff b) {
    const ff p = two_prod(a.h, b.h);
    return {p.h, __fmaf_rn(a.h, b.l, __fmaf_rn(a.l, b.h, p.l))};
}

__device__ __forceinline__ ff ff_cubic_C(ff s2, ff s) {
    ff c = ff_lin_dom(s2, 0.75f, -3.5f);
    c = ff_horner_dom(s2, c, 8.75f);
    c = ff_horner_dom(s, c, -7.f);
    return ff_horner_dom(s2, c, 1.f);
}

__device__ __forceinline__ ff ff_cubic_d1(ff s2, ff s) {
    ff k = ff_lin_dom(s2, 5.25f, -17.5f);
    k = ff_horner_dom(s2, k, 26.25f);
    return ff_horner_dom(s, k, -14.f);
}

// Accumulator of float-float products: the high word is a running sum kept
// exact by TwoSum, the low word collects the rounding errors in FP32 and is
// folded back into the high word every few terms (ff_acc_norm), so it stays
// within a few ulps of the high word's error and adds ~eps^2-level error.
struct ffacc {
    float h, l;
};

__device__ __forceinline__ void ff_acc_fma(ffacc& a, ff x, ff y) {
    ff p = two_prod(x.h, y.h);
    float e = __fmaf_rn(x.h, y.l, __fmaf_rn(x.l, y.h, p.l));
    ff s = two_sum(a.h, p.h);
    a.h = s.h;
    a.l += s.l + e;
}

__device__ __forceinline__ void ff_acc_norm(ffacc& a) {
    ff s = two_sum(a.h, a.l);
    a.h = s.h;
    a.l = s.l;
}

__device__ __forceinline__ double ff_acc_to_double(const ffacc& a) { return (double)a.h + (double)a.l; }

// w . h for float-float 3-vectors: exact products and a TwoSum chain on the
// high words, the low-order terms added in FP32.
__device__ __forceinline__ ff ff_dot3(ff wx, ff wy, ff wz, ff hx, ff hy, ff hz) {
    ff p0 = two_prod(wx.h, hx.h), p1 = two_prod(wy.h, hy.h), p2 = two_prod(wz.h, hz.h);
    float e = __fmaf_rn(wx.h, hx.l, __fmaf_rn(wx.l, hx.h, p0.l));
    e += __fmaf_rn(wy.h, hy.l, __fmaf_rn(wy.l, hy.h, p1.l));
    e += __fmaf_rn(wz.h, hz.l, __fmaf_rn(wz.l, hz.h, p2.l));
    ff s1 = two_sum(p0.h, p1.h);
    ff s2 = two_sum(s1.h, p2.h);
    return {s2.h, s1.l + s2.l + e};   // unnormalised, read through exact products
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
    double hi = rint(u * (1.0 / q)) * q;   // q is a power of two: u * (1/q) == u / q exactly
    h = (float)hi;
    l = (float)(u - hi);
}

struct PointFF {
    float h[3], l[3];
    bool exact;
};

__device__ __forceinline__ void ff_point(const double* xd, double inv_a, double q, PointFF& P) {
    const double lim = ldexp(q, 23), inv_q = 1.0 / q;   // q a power of two: exact inverse
    P.exact = true;
    for (int k = 0; k < 3; ++k) {
        double u = xd[k] * inv_a;
        double hi = rint(u * inv_q) * q;
        P.h[k] = (float)hi;
        P.l[k] = (float)(u - hi);
        if (fabs(hi) > lim) P.exact = false;
    }
}

// r^2 + eps2 of d = x - p as float-float (eps2 is the distance regulariser
// in the scaled frame, kDistEps2 / range^2); d_k = dh_k + dl_k with dh_k exact
// when the split is exact (EXACT: every point of the caller is), else
// recovered with a two-sum.  The result is normalised: it is the variable of
// the covariance polynomials, and an unnormalised variable's low word would
// enter every Horner step (emulated: 3e-12 instead of 1e-13 per term).
template <bool EXACT>
__device__ __forceinline__ ff ff_dist2(const PointFF& X, const float* ph, const float* pl, float* dh, float* dl,
                                       float eps2) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        if (EXACT) {
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

// One staged tile of float-float records against PPT points: orientation
// records (16 floats: x, y, z hi/lo, then w_x, w_y, w_z hi/lo) add
// C'/r(|x - x_o|) (w . (x_o - x)), surface-point records (8 floats: x, y, z
// hi/lo, alpha hi/lo) add alpha C(|x - p|); coordinates are scaled by 1/range.
// EXACT: every point's split is exact (the common case).  ALL_ACT: every
// point slot holds a point (all but a grid's last chunk), so the per-pair
// slot test is compiled out.  eps2 must be a positive normal float.
template <int PPT, bool EXACT, bool ALL_ACT = false>
__device__ __forceinline__ void ff_tile(const float* __restrict__ rec, bool orientation, int nr,
                                        const PointFF (&X)[PPT], const bool (&act)[PPT], float eps2,
                                        ffacc (&acc)[PPT]) {
    if (orientation) {
        for (int qr = 0; qr < nr; ++qr) {
            const float4* R4 = reinterpret_cast<const float4*>(rec + 16 * qr);
            const float4 a0 = R4[0], a1 = R4[1], a2 = R4[2];
            const float ph[3] = {a0.x, a0.z, a1.x}, pl[3] = {a0.y, a0.w, a1.y};
            const ff wx = {a1.z, a1.w}, wy = {a2.x, a2.y}, wz = {a2.z, a2.w};
#pragma unroll
            for (int p = 0; p < PPT; ++p) {
                if (!ALL_ACT && !act[p]) continue;  // a slot past the end of the point list
                float dh[3], dl[3];
                const ff r2 = ff_dist2<EXACT>(X[p], ph, pl, dh, dl, eps2);
                if (r2.h >= 1.f) continue;  // beyond the range: C'/r = 0
                const ff k = ff_cubic_d1(r2, ff_sqrt_pos(r2));
                // h = x_o - x = -(dh + dl)
                const ff wh = ff_dot3(wx, wy, wz, ff{-dh[0], -dl[0]}, ff{-dh[1], -dl[1]}, ff{-dh[2], -dl[2]});
                ff_acc_fma(acc[p], k, wh);
            }
            if ((qr & 7) == 7) {  // fold the low words back every 8 records
#pragma unroll
                for (int p = 0; p < PPT; ++p) ff_acc_norm(acc[p]);
            }
        }
    } else {
        for (int qr = 0; qr < nr; ++qr) {
            const float4* R4 = reinterpret_cast<const float4*>(rec + 8 * qr);
            const float4 a0 = R4[0], a1 = R4[1];
            const float ph[3] = {a0.x, a0.z, a1.x}, pl[3] = {a0.y, a0.w, a1.y};
            const ff W = {a1.z, a1.w};
#pragma unroll
            for (int p = 0; p < PPT; ++p) {
                if (!ALL_ACT && !act[p]) continue;
                float dh[3], dl[3];
                const ff r2 = ff_dist2<EXACT>(X[p], ph, pl, dh, dl, eps2);
                if (r2.h >= 1.f) continue;  // beyond the range: C = 0
                ff_acc_fma(acc[p], ff_cubic_C(r2, ff_sqrt_pos(r2)), W);
            }
            if ((qr & 7) == 7) {
#pragma unroll
                for (int p = 0; p < PPT; ++p) ff_acc_norm(acc[p]);
            }
        }
    }
}

// ff_tile for NP points of one grid column (equal x and y, exact splits,
// every slot filled): the x and y terms of r^2 -- their exact squares, the
// two-sum of their high words and the low-order terms -- and, for an
// orientation record, the x and y terms of w . h are formed once per record
// and shared; only the z terms are per point.
// CUT = false: the caller has shown that every pair lies within the range,
// so the per-pair range test is compiled out.  Then, without FOLD, the caller
// starts each accumulator of a surface-point tile at the tile's sum of
// weights (cta_weight_sum): C = 1 + s^2 k, so only W s^2 k is accumulated per
// pair.  With FOLD, the caller starts each accumulator at the tile's terms
// that are polynomials in x (cta_fold_sums, tile_fold): for surface-point records
// C = 1 - 7 s^2 + s^3 m(s), and only W s^3 m is accumulated per pair; for
// orientation records a^2 C'/r = -14 + s m(s), and only s m (w . h) is.
template <int NP, bool CUT = true, bool FOLD = false>
__device__ __forceinline__ void ff_tile_col(const float* __restrict__ rec, bool orientation, int nr,
                                            const PointFF (&X)[NP], float eps2, ffacc (&acc)[NP]) {
    for (int qr = 0; qr < nr; ++qr) {
        const float* R = rec + (orientation ? 16 : 8) * qr;
        const float4 a0 = reinterpret_cast<const float4*>(R)[0];
        const float4 a1 = reinterpret_cast<const float4*>(R)[1];
        const float dh0 = X[0].h[0] - a0.x, dl0 = X[0].l[0] - a0.y;
        const float dh1 = X[0].h[1] - a0.z, dl1 = X[0].l[1] - a0.w;
        const ff b0 = two_prod(dh0, dh0), b1 = two_prod(dh1, dh1);
        const ff sxy = two_sum_nonneg(b0.h, b1.h);
        float lxy = sxy.l + b0.l + b1.l + eps2;
        lxy = __fmaf_rn(dl0, 2.f * dh0 + dl0, lxy);
        lxy = __fmaf_rn(dl1, 2.f * dh1 + dl1, lxy);
        if (orientation) {
            const float4 a2 = reinterpret_cast<const float4*>(R)[2];
            const ff wx = {a1.z, a1.w}, wy = {a2.x, a2.y}, wz = {a2.z, a2.w};
            // w . h with h = x_o - x = -(dh + dl): the x and y products once
            const ff q0 = two_prod(wx.h, -dh0), q1 = two_prod(wy.h, -dh1);
            float exy = __fmaf_rn(wx.h, -dl0, __fmaf_rn(wx.l, -dh0, q0.l));
            exy += __fmaf_rn(wy.h, -dl1, __fmaf_rn(wy.l, -dh1, q1.l));
            const ff sw = two_sum(q0.h, q1.h);
            exy += sw.l;
#pragma unroll
            for (int p = 0; p < NP; ++p) {
                const float dh2 = X[p].h[2] - a1.x, dl2 = X[p].l[2] - a1.y;
                const ff b2 = two_prod(dh2, dh2);
                const ff s2 = two_sum_nonneg(sxy.h, b2.h);
                float low = lxy + s2.l + b2.l;
                low = __fmaf_rn(dl2, 2.f * dh2 + dl2, low);
                const ff r2 = fast_two_sum(s2.h, low);
                ff k;
                if (CUT || !FOLD) {
                    if (CUT && r2.h >= 1.f) continue;  // beyond the range: C'/r = 0
                    k = ff_cubic_d1(r2, ff_sqrt_pos(r2));
                } else {
                    // every pair in range: a^2 C'/r = -14 + s m(s), and the caller
                    // added the tile's -14 sum_o w_o . (x_o - x), so only s m is used
                    k = ff_lin_dom(r2, 5.25f, -17.5f);
                    k = ff_horner_dom(r2, k, 26.25f);
                    k = ff_mul_un(ff_sqrt_pos(r2), k);
                }
                const ff q2 = two_prod(wz.h, -dh2);
                const float e2 = __fmaf_rn(wz.h, -dl2, __fmaf_rn(wz.l, -dh2, q2.l));
                const ff sz = two_sum(sw.h, q2.h);
                ff_acc_fma(acc[p], k, ff{sz.h, exy + sz.l + e2});   // unnormalised, read through exact products
            }
        } else {
            const ff W = {a1.z, a1.w};
#pragma unroll
            for (int p = 0; p < NP; ++p) {
                const float dh2 = X[p].h[2] - a1.x, dl2 = X[p].l[2] - a1.y;
                const ff b2 = two_prod(dh2, dh2);
                const ff s2 = two_sum_nonneg(sxy.h, b2.h);
                float low = lxy + s2.l + b2.l;
                low = __fmaf_rn(dl2, 2.f * dh2 + dl2, low);
                const ff r2 = fast_two_sum(s2.h, low);
                if (CUT) {
                    if (r2.h >= 1.f) continue;  // beyond the range: C = 0
                    ff_acc_fma(acc[p], ff_cubic_C(r2, ff_sqrt_pos(r2)), W);
                } else if (!FOLD) {
                    // every pair in range: C = 1 + s^2 k, and the caller started the
                    // accumulators at the tile's sum of weights, so only W s^2 k is added
                    const ff s = ff_sqrt_pos(r2);
                    ff k = ff_lin_dom(r2, 0.75f, -3.5f);
                    k = ff_horner_dom(r2, k, 8.75f);
                    k = ff_horner_dom(s, k, -7.f);
                    ff_acc_fma(acc[p], ff_mul_un(r2, k), W);
                } else {
                    // every pair in range: C = 1 - 7 s^2 + s^3 m(s), and the caller
                    // added the tile's sum of W (1 - 7 s^2) (a quadratic in x), so
                    // only W s^3 m is added
                    ff m = ff_lin_dom(r2, 0.75f, -3.5f);
                    m = ff_horner_dom(r2, m, 8.75f);
                    ff_acc_fma(acc[p], ff_mul_un(r2, ff_mul_un(ff_sqrt_pos(r2), m)), W);
                }
            }
        }
        if ((qr & 7) == 7) {  // fold the low words back every 8 records
#pragma unroll
            for (int p = 0; p < NP; ++p) ff_acc_norm(acc[p]);
        }
    }
}

// Bounding box of a set of points over the CTA: v = {min x, y, z, max x, y,
// z} per thread in, the CTA's box out (every thread).  sh holds 6 floats per
// warp.
__device__ __forceinline__ void cta_bbox(float (&v)[6], float* sh) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int c = 0; c < 6; ++c)
        for (int o = 16; o > 0; o >>= 1) {
            const float t = __shfl_xor_sync(0xffffffffu, v[c], o);
            v[c] = c < 3 ? fminf(v[c], t) : fmaxf(v[c], t);
        }
    if (lane == 0)
        for (int c = 0; c < 6; ++c) sh[6 * wid + c] = v[c];
    __syncthreads();
    for (int c = 0; c < 6; ++c) {
        float r = sh[c];
        for (int w = 1; w < nw; ++w) r = c < 3 ? fminf(r, sh[6 * w + c]) : fmaxf(r, sh[6 * w + c]);
        v[c] = r;
    }
    __syncthreads();
}

// The sums behind the constant and r^2 terms of an in-range tile, in
// float-float on the FP32 pipe, reduced over the CTA in a fixed order (every
// thread gets them), with record positions p taken relative to the centre o
// of the CTA's points (which keeps the terms of |x - p|^2 small).  Surface-
// point records: f = {sum W, sum W (p - o) (3), sum W |p - o|^2}; orientation
// records: f = {sum w . (x_o - o), sum w (3), 0}.  sh holds 10 floats per warp.
__device__ __forceinline__ void cta_fold_sums(const float* __restrict__ rec, int nr, bool orientation,
                                              const float (&o)[3], ff (&f)[5], float* sh) {
#pragma unroll
    for (int c = 0; c < 5; ++c) f[c] = {0.f, 0.f};
    for (int r = threadIdx.x; r < nr; r += blockDim.x) {
        const float* R = rec + (orientation ? 16 : 8) * r;
        const ff px = ff_add_f(ff{R[0], R[1]}, -o[0]), py = ff_add_f(ff{R[2], R[3]}, -o[1]),
                 pz = ff_add_f(ff{R[4], R[5]}, -o[2]);
        if (orientation) {
            const ff wx = {R[6], R[7]}, wy = {R[8], R[9]}, wz = {R[10], R[11]};
            f[0] = ff_add(f[0], ff_dot3(wx, wy, wz, px, py, pz));
            f[1] = ff_add(f[1], wx);
            f[2] = ff_add(f[2], wy);
            f[3] = ff_add(f[3], wz);
        } else {
            const ff w = {R[6], R[7]};
            f[0] = ff_add(f[0], w);
            f[1] = ff_add(f[1], ff_mul(w, px));
            f[2] = ff_add(f[2], ff_mul(w, py));
            f[3] = ff_add(f[3], ff_mul(w, pz));
            f[4] = ff_add(f[4], ff_mul(w, ff_dot3(px, py, pz, px, py, pz)));
        }
    }
#pragma unroll
    for (int c = 0; c < 5; ++c)
        for (int o = 16; o > 0; o >>= 1)
            f[c] = ff_add(f[c], ff{__shfl_xor_sync(0xffffffffu, f[c].h, o), __shfl_xor_sync(0xffffffffu, f[c].l, o)});
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (lane == 0)
        for (int c = 0; c < 5; ++c) {
            sh[10 * wid + 2 * c] = f[c].h;
            sh[10 * wid + 2 * c + 1] = f[c].l;
        }
    __syncthreads();
    for (int c = 0; c < 5; ++c) {
        ff t = {sh[2 * c], sh[2 * c + 1]};
        for (int w = 1; w < nw; ++w) t = ff_add(t, ff{sh[10 * w + 2 * c], sh[10 * w + 2 * c + 1]});
        f[c] = t;
    }
    __syncthreads();
}

// The folded terms of an in-range tile at point x (scaled, float-float; f
// and o from cta_fold_sums): surface points sum W (1 - 7 (|x - p|^2 + eps2)),
// orientations -14 sum w . (x_o - x).  The start value of the point's
// accumulator.
__device__ __forceinline__ ff tile_fold(const ff (&f)[5], bool orientation, const PointFF& X, const float (&o)[3],
                                        float eps2) {
    const ff x = ff_add_f(ff{X.h[0], X.l[0]}, -o[0]), y = ff_add_f(ff{X.h[1], X.l[1]}, -o[1]),
             z = ff_add_f(ff{X.h[2], X.l[2]}, -o[2]);
    const ff xf = ff_dot3(x, y, z, f[1], f[2], f[3]);
    if (orientation) return ff_mul_f(ff_add(f[0], ff{-xf.h, -xf.l}), -14.f);
    const ff xx = ff_add_f(ff_dot3(x, y, z, x, y, z), eps2);
    const ff r2 = ff_add(ff_add(ff_mul(f[0], xx), ff{-2.f * xf.h, -2.f * xf.l}), f[4]);
    return ff_add(f[0], ff_mul_f(r2, -7.f));
}

// Sum of the weights of a tile's nr surface-point records (float-float,
// reduced over the CTA; every thread gets the sum).  sh holds 2 floats per
// warp.
__device__ __forceinline__ ff cta_weight_sum(const float* __restrict__ rec, int nr, float* sh) {
    ff s = {0.f, 0.f};
    for (int r = threadIdx.x; r < nr; r += blockDim.x) s = ff_add(s, ff{rec[8 * r + 6], rec[8 * r + 7]});
    for (int o = 16; o > 0; o >>= 1) {
        const ff t = {__shfl_xor_sync(0xffffffffu, s.h, o), __shfl_xor_sync(0xffffffffu, s.l, o)};
        s = ff_add(s, t);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (lane == 0) {
        sh[2 * wid] = s.h;
        sh[2 * wid + 1] = s.l;
    }
    __syncthreads();
    ff t = {sh[0], sh[1]};
    for (int w = 1; w < nw; ++w) t = ff_add(t, ff{sh[2 * w], sh[2 * w + 1]});
    __syncthreads();
    return t;
}

__device__ __forceinline__ ff ff_from_double(double x) {
    float h = (float)x;
    return {h, (float)(x - (double)h)};
}

}  // namespace gk
