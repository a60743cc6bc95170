// Float-float arithmetic (pairs of FP32 values, ~2^-44 relative) for the
// parts of the FP32-class forms that need more than FP32: GB300's FP64 pipe
// runs at 1/64 of the FP32 rate, so these run on the FP32 pipe instead.
// Products use the FMA-exact product error, sums TwoSum.
#pragma once

#include "sigma_internal.cuh"

namespace sigma {

// x = hi + lo: hi is x truncated to 24 significant bits (exact in FP32), lo
// the remaining 29 bits rounded to FP32 (|x - hi - lo| <= 2^-48 |x|).  For
// exponents where both are normal FP32 values, hi is assembled from the
// bits and lo is one 32-bit integer conversion scaled by a power of two: no
// conversion from a 64-bit operand (with those, an FP32 kernel kept GB300's
// FP64 pipe half busy).
__device__ __forceinline__ void split_exact(double x, float& hi, float& lo) {
  const unsigned int whi = (unsigned int)__double2hiint(x), wlo = (unsigned int)__double2loint(x);
  const int ex = (int)((whi >> 20) & 0x7FFu);
  if (ex >= 949 && ex <= 1150) {  // 2^-74 <= |x| < 2^128
    hi = __uint_as_float((whi & 0x80000000u) | ((unsigned int)(ex - 896) << 23) |
                         ((whi & 0xFFFFFu) << 3) | (wlo >> 29));
    const float m = __uint2float_rn(wlo & 0x1FFFFFFFu);    // < 2^29
    const float scale = __uint_as_float((unsigned int)(ex - 948) << 23);  // 2^(ex - 1075)
    lo = (whi >> 31) ? -(m * scale) : m * scale;
    return;
  }
  const long long bits = __double_as_longlong(x);
  constexpr long long kLow = (1LL << 29) - 1;
  hi = __double2float_rn(__longlong_as_double(bits & ~kLow));
  const int e = (int)((bits >> 52) & 0x7FF);
  const float m = __ll2float_rn(bits & kLow);  // low 29 mantissa bits, < 2^29
  const float scale = e > 948 ? __int_as_float((e - 948) << 23) : 0.f;  // 2^(e - 1075)
  lo = (bits < 0) ? -(m * scale) : m * scale;
}

struct FF {
  float hi, lo;
};
__device__ __forceinline__ FF ff_of(double x) {
  FF r;
  split_exact(x, r.hi, r.lo);
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

}  // namespace sigma
