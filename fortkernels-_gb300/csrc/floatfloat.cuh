// Float-float arithmetic (pairs of FP32 values, ~2^-44 relative) for the
// parts of the FP32-class forms that need more than FP32: GB300's FP64 pipe
// runs at 1/64 of the FP32 rate, so these run on the FP32 pipe instead.
// Products use the FMA-exact product error, sums TwoSum.
#pragma once

#include "sigma_internal.cuh"

namespace sigma {

// x = hi + lo: hi is x truncated to 24 significant bits (exact in FP32), lo
// the remaining 29 bits rounded to FP32 (|x - hi - lo| <= 2^-48 |x|), for
// 2^-74 <= |x| < 2^128.  Integer operations only (hi assembled from the bits,
// lo one 32-bit integer conversion scaled by a power of two): a conversion
// from a 64-bit operand runs on GB300's FP64 pipe, at 1/64 of the FP32 rate,
// and so would a slow path the compiler evaluates predicated off for every
// value.  Outside that range: 2^-126 <= |x| < 2^-74 keeps hi with lo = 0
// (error below 2^-23 |x|, far below any value that matters next to the FP32
// forms' range); smaller magnitudes give a signed zero; |x| >= 2^128 gives
// an infinite hi (NaN for a NaN), so such inputs show up as non-finite
// outputs of the FP32 forms instead of wrong finite values.
__device__ __forceinline__ void split_exact(double x, float& hi, float& lo) {
  const unsigned int whi = (unsigned int)__double2hiint(x), wlo = (unsigned int)__double2loint(x);
  const unsigned int sign = whi & 0x80000000u;
  const unsigned int ex = (whi >> 20) & 0x7FFu;
  if (ex - 949u <= 201u) {  // 949 <= ex <= 1150: hi and lo normal FP32 values
    // (whi << 3 | wlo >> 29) holds the exponent's low 8 bits and the leading
    // 23 fraction bits; ex - 896 = (ex mod 256) + 128 modulo 256 in this range
    const unsigned int f = __funnelshift_l(wlo, whi, 3);
    hi = __uint_as_float(((f + 0x40000000u) & 0x7FFFFFFFu) | sign);
    const float l = __uint2float_rn(wlo & 0x1FFFFFFFu) * __uint_as_float((ex - 948u) << 23);  // x 2^(ex - 1075)
    lo = __uint_as_float(__float_as_uint(l) ^ sign);
    return;
  }
  unsigned int hb;
  if (ex > 1150u) {
    hb = sign | 0x7F800000u | ((ex == 2047u && ((whi & 0xFFFFFu) | wlo)) ? 0x400000u : 0u);
  } else if (ex >= 897u) {
    hb = sign | ((ex - 896u) << 23) | ((whi & 0xFFFFFu) << 3) | (wlo >> 29);
  } else {
    hb = sign;
  }
  hi = __uint_as_float(hb);
  lo = 0.f;
}

// x = hi + lo with hi = x rounded to the nearest FP32 value (ties to even,
// as cvt.rn.f32.f64) and lo = x - hi rounded to FP32, on the integer pipe,
// for 2^-74 <= |x| < 2^128 (|x| at or above FLT_MAX + 1/2 ulp gives an
// infinite hi, as the conversion does).  |lo| <= 2^-24 |x| and lo takes
// either sign, so the lo parts that float-float products drop (lo * lo) and
// the splits' own errors average out over long sums; the truncated split's
// lo always carries x's sign, and those dropped parts then add up in one
// direction (a bias of ~2^-46 per term in an FP64-class sum).  Outside the
// range as split_exact.
__device__ __forceinline__ void split_round(double x, float& hi, float& lo) {
  const unsigned int whi = (unsigned int)__double2hiint(x), wlo = (unsigned int)__double2loint(x);
  const unsigned int sign = whi & 0x80000000u;
  const unsigned int ex = (whi >> 20) & 0x7FFu;
  if (ex - 949u <= 201u) {
    // round up when the dropped 29 bits exceed half an ulp, or equal it with
    // an odd kept mantissa; the carry may run into the exponent field
    const unsigned int rest = wlo & 0x1FFFFFFFu;
    const unsigned int up = rest > 0x10000000u || (rest == 0x10000000u && ((wlo >> 29) & 1u));
    const unsigned int f = __funnelshift_l(wlo, whi, 3) + up;
    hi = __uint_as_float(((f + 0x40000000u) & 0x7FFFFFFFu) | sign);
    const int m = (int)rest - (int)(up << 29);  // x - hi in units of 2^(ex - 1075), |m| <= 2^28
    const float l = __int2float_rn(m) * __uint_as_float((ex - 948u) << 23);
    lo = __uint_as_float(__float_as_uint(l) ^ sign);
    return;
  }
  split_exact(x, hi, lo);
}

struct FF {
  float hi, lo;
};
__device__ __forceinline__ FF ff_of(double x) {
  FF r;
  split_exact(x, r.hi, r.lo);
  return r;
}
// The rounded split, for the FP64 forms' float-float terms.
__device__ __forceinline__ FF ff_of_rn(double x) {
  FF r;
  split_round(x, r.hi, r.lo);
  return r;
}
__device__ __forceinline__ FF ff_norm(float s, float e) {
  const float h = s + e;
  return FF{h, e - (h - s)};
}
__device__ __forceinline__ FF ff_add(FF x, FF y) {
  float s, e;
  two_sum_f(x.hi, y.hi, s, e);
  return ff_norm(s, e + (x.lo + y.lo));
}
__device__ __forceinline__ FF ff_neg(FF x) { return FF{-x.hi, -x.lo}; }
__device__ __forceinline__ FF ff_mul(FF x, FF y) {
  const float p = x.hi * y.hi;
  float e = fmaf(x.hi, y.hi, -p);
  e = fmaf(x.hi, y.lo, fmaf(x.lo, y.hi, e));
  return ff_norm(p, e);
}
// 1/x for x > 0: FP32 reciprocal, one float-float correction
__device__ __forceinline__ FF ff_rcp(FF x) {
  const float r0 = rcp_f32(x.hi);
  const float e = fmaf(-x.hi, r0, 1.0f) - x.lo * r0;
  return ff_norm(r0, r0 * e);
}
__device__ __forceinline__ float ff_round(FF x) { return x.hi + x.lo; }
// x y rounded once to FP32: the cross terms in one FMA, the final FMA exact
// before its rounding, so the result is within 1/2 ulp + 2^-47 |xy| of xy
__device__ __forceinline__ float ff_mul_round(FF x, FF y) {
  return fmaf(x.hi, y.hi, fmaf(x.hi, y.lo, x.lo * y.hi));
}
// x > y for non-negative float-float values, with `near` set when they are
// within 2^-30 (relative) of each other
__device__ __forceinline__ bool ff_gt(FF x, FF y, bool& near) {
  const float d = (x.hi - y.hi) + (x.lo - y.lo);
  near = fabsf(d) <= 9.3132257e-10f * fmaxf(x.hi, y.hi);  // 2^-30
  return d > 0.f;
}

// x > y for non-negative normalised float-float values, taken on the hi
// parts when they differ by more than 2^-21 of the larger (|lo| <= 2^-24
// |hi| and one rounding of the difference cannot flip the sign then), else
// with the full compare; `near` as ff_gt.  Same result as ff_gt, without a
// branch.
__device__ __forceinline__ bool ff_gt_fast(FF x, FF y, bool& near) {
  const float d = x.hi - y.hi, m = fmaxf(x.hi, y.hi);
  const bool clear = fabsf(d) > 4.76837158e-07f * m;  // 2^-21
  const float full = d + (x.lo - y.lo);
  near = !clear && fabsf(full) <= 9.3132257e-10f * m;  // 2^-30
  return clear ? d > 0.f : full > 0.f;
}

// x > 0.25 for a non-negative normalised float-float x, with `near` set
// within 2^-30 of 0.25 (relative): ff_gt_fast(x, {0.25, 0}, near) in four
// instructions.  x.hi - 0.25 is exact where x.hi is within a factor of two
// of 0.25 (Sterbenz); elsewhere it and the sum keep the sign of x - 0.25.
__device__ __forceinline__ bool ff_gt_quarter(FF x, bool& near) {
  const float full = (x.hi - 0.25f) + x.lo;
  near = fabsf(full) <= 2.3283064e-10f;  // 2^-32 = 2^-30 x 0.25
  return full > 0.f;
}

// x - y as an unnormalised pair (TwoSum of the hi parts plus the lo
// parts): exact to ~2^-46 of the operands, for a product or square next.
__device__ __forceinline__ FF ff_sub_raw(FF x, FF y) {
  float s, e;
  two_sum_f(x.hi, -y.hi, s, e);
  return FF{s, e + (x.lo - y.lo)};
}
// c^2 + b2 (b2 normalised), normalised: the square's exact error by FMA.
__device__ __forceinline__ FF ff_sq_add(FF c, FF b2) {
  const float p = c.hi * c.hi;
  const float e = fmaf(2.f * c.hi, c.lo, fmaf(c.hi, c.hi, -p));
  float s, t;
  two_sum_f(p, b2.hi, s, t);
  return ff_norm(s, t + (e + b2.lo));
}
// Unnormalised float-float results (hi, lo) for operands that feed only
// further products, TwoSums or one final rounding: the pair's value is the
// same as the normalised one's, its lo may exceed half an ulp of hi.
// x y: the exact product of the hi parts (FMA) plus the cross terms.
__device__ __forceinline__ FF ff_mul_raw(FF x, FF y) {
  const float p = x.hi * y.hi;
  return FF{p, fmaf(x.hi, y.lo, fmaf(x.lo, y.hi, fmaf(x.hi, y.hi, -p)))};
}
// a g - b h: the hi products' difference by TwoSum, their exact errors and
// the cross terms in lo (lo * lo terms dropped, ~2^-46 of the products).
__device__ __forceinline__ FF ff_dot2_raw(FF a, FF g, FF b, FF h) {
  const float p1 = a.hi * g.hi, p2 = b.hi * h.hi;
  const float e1 = fmaf(a.hi, g.hi, -p1), e2 = fmaf(b.hi, h.hi, -p2);
  const float t = fmaf(a.hi, g.lo, fmaf(a.lo, g.hi, e1)) - fmaf(b.hi, h.lo, fmaf(b.lo, h.hi, e2));
  float s, es;
  two_sum_f(p1, -p2, s, es);
  return FF{s, es + t};
}
// 1 / x for x > 0 (x normalised): FP32 reciprocal and one float-float
// correction, unnormalised.
__device__ __forceinline__ FF ff_rcp_raw(FF x) {
  const float r0 = rcp_f32(x.hi);
  return FF{r0, r0 * (fmaf(-x.hi, r0, 1.0f) - x.lo * r0)};
}

// Paired FP32 (f32x2) helpers: halves of a float4, and ff_add of two
// independent float-float accumulators (hi.x, lo.x) += x.x, (hi.y, lo.y) +=
// x.y with the same roundings as ff_add, one paired instruction per step
// (differences as fma(a, -1, b) = b - a, exact up to the one rounding).
__device__ __forceinline__ float2 f4_lo(float4 v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 f4_hi(float4 v) { return make_float2(v.z, v.w); }
__device__ __forceinline__ void ff_add2(float2& hi, float2& lo, float2 x, float2 m1) {
  const float2 s = __fadd2_rn(hi, x);
  const float2 bv = __ffma2_rn(hi, m1, s);  // s - hi
  const float2 av = __ffma2_rn(bv, m1, s);  // s - bv
  const float2 e = __fadd2_rn(__fadd2_rn(__ffma2_rn(av, m1, hi), __ffma2_rn(bv, m1, x)), lo);
  hi = __fadd2_rn(s, e);
  lo = __ffma2_rn(__ffma2_rn(s, m1, hi), m1, e);  // e - (hi - s)
}

// An FP32 value as a double, on the integer pipe (exponent rebiased,
// mantissa shifted): exact for normal values and zero; FP32 subnormals (below
// 1.2e-38) give zero.  cvt.f64.f32 would take the FP64 pipe, GB300's
// scarcest.
__device__ __forceinline__ double f32_widen(float f) {
  const unsigned u = __float_as_uint(f), mag = u & 0x7FFFFFFFu;
  const unsigned hi = (u & 0x80000000u) | (mag >= 0x00800000u ? (mag >> 3) + 0x38000000u : 0u);
  return __hiloint2double((int)hi, mag >= 0x00800000u ? (int)(mag << 29) : 0);
}
// A float-float value as the nearest double: both halves widened exactly,
// one FP64 addition.
__device__ __forceinline__ double ff_widen(FF x) { return f32_widen(x.hi) + f32_widen(x.lo); }

// The range in which the FP64 forms take float-float factors: a complex
// input that is zero (or an FP64 subnormal, which the split flushes) or has
// its larger component in [2^-20, 2^20), and a frequency with |wx| in
// [2^-20, 2^20).  Inside it every float-float intermediate of a factor
// keeps both FP32 halves normal and finite; elements outside it take the
// FP64 expressions.  Biased exponents compared on the integer pipe.
__device__ __forceinline__ int f64_exp(double x) { return (__double2hiint(x) >> 20) & 0x7FF; }
__device__ __forceinline__ bool ff_range(double x, double y) {
  const int e = max(f64_exp(x), f64_exp(y));
  return e == 0 || (unsigned)(e - (1023 - 20)) < 40u;
}
__device__ __forceinline__ bool ff_freq_range(double wx) {
  return (unsigned)(f64_exp(wx) - (1023 - 20)) < 40u;
}

// The pole-guard decisions of the FP64 path (guard_w / guard_thr /
// guard_thr2), for the float-float kernels' rare values near a threshold.
// Out of line so that those kernels branch to them instead of running their
// FP64 instructions predicated off for every value.
static __device__ __noinline__ bool keep_fp64(double wx, double a, double b) {
  const double b2 = guard_b2(b);
  return keep_nonneg(guard_w(wx, a, b2), guard_thr(a, b2));
}
// second occupied-band branch: 0 < |wdiff|^2 < |wtilde|^2 / to1
static __device__ __noinline__ bool second_fp64(double wx, double a, double b) {
  const double b2 = guard_b2(b);
  const double w = guard_w(wx, a, b2);
  return gt_nonneg(w, 0.0) && gt_nonneg(guard_thr2(a, b2), w);
}

}  // namespace sigma
