// Double-FP32 ("float-float") arithmetic for the mixed form of the analytic
// surfaces: a value is hi + lo with |lo| <= ulp(hi)/2, about 44 significant
// bits carried by FP32 operations only -- no FP64 instruction, which on this
// GPU issues at 1/64 of the FP32 rate.  Sums use Knuth's error-free TwoSum,
// products the FMA split (TwoProd); division and square root take one
// correction step of the FP32 estimate; exp reduces by n ln 2 (ln 2 as a
// float pair) and sums the Taylor series of degree 11 on |r| <= ln2/2
// (truncation < 1e-14 relative).  Used where FP32 rounding would be
// amplified by cancellation (the LEPS stretch terms of CH4 + H, the bend
// angles' differences from their references).
#pragma once
#include <cuda_runtime.h>

namespace cr {

struct ff {
  float hi, lo;
};

__host__ __device__ constexpr ff ff_const(double d) {
  return ff{(float)d, (float)(d - (double)(float)d)};
}

__device__ __forceinline__ ff ff_quick(float s, float e) {
  const float h = s + e;
  return ff{h, e - (h - s)};
}
__device__ __forceinline__ ff ff_two_sum(float a, float b) {
  const float s = a + b, bb = s - a;
  return ff{s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ ff ff_from(float a) { return ff{a, 0.f}; }
__device__ __forceinline__ ff operator-(ff a) { return ff{-a.hi, -a.lo}; }
__device__ __forceinline__ ff operator+(ff a, ff b) {
  const ff s = ff_two_sum(a.hi, b.hi);
  return ff_quick(s.hi, s.lo + (a.lo + b.lo));
}
__device__ __forceinline__ ff operator-(ff a, ff b) { return a + (-b); }
__device__ __forceinline__ ff operator+(ff a, float b) {
  const ff s = ff_two_sum(a.hi, b);
  return ff_quick(s.hi, s.lo + a.lo);
}
__device__ __forceinline__ ff operator-(ff a, float b) { return a + (-b); }
__device__ __forceinline__ ff operator*(ff a, ff b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
  return ff_quick(p, e);
}
__device__ __forceinline__ ff operator*(ff a, float b) {
  const float p = a.hi * b;
  float e = fmaf(a.hi, b, -p);
  e = fmaf(a.lo, b, e);
  return ff_quick(p, e);
}
__device__ __forceinline__ ff operator/(ff a, ff b) {
  const float q1 = a.hi / b.hi;
  const ff r = a - b * q1;
  return ff_quick(q1, r.hi / b.hi);
}
__device__ __forceinline__ ff& operator+=(ff& a, ff b) { return a = a + b; }
__device__ __forceinline__ ff& operator-=(ff& a, ff b) { return a = a - b; }
__device__ __forceinline__ ff& operator+=(ff& a, float b) { return a = a + b; }

__device__ __forceinline__ ff ff_sqrt(ff a) {
  if (!(a.hi > 0.f)) return ff{0.f, 0.f};
  const float s = sqrtf(a.hi);
  const float p = s * s, pe = fmaf(s, s, -p);   // s^2 exactly as p + pe
  const float r = ((a.hi - p) - pe) + a.lo;
  return ff_quick(s, r / (2.f * s));
}

__device__ __forceinline__ ff ff_recip(ff a) { return ff_from(1.f) / a; }

__device__ inline ff ff_exp(ff x) {
  constexpr ff kLn2 = ff_const(0.6931471805599453094);
  const float n = rintf(x.hi * 1.44269504f);
  const ff r = x - kLn2 * n;               // |r| <= ln2/2 (to a few ulp)
  // Taylor series of exp(r) to degree 11 by Horner, coefficients 1/k!
  constexpr ff c[12] = {ff_const(1.0), ff_const(1.0), ff_const(1.0 / 2), ff_const(1.0 / 6), ff_const(1.0 / 24),
                        ff_const(1.0 / 120), ff_const(1.0 / 720), ff_const(1.0 / 5040), ff_const(1.0 / 40320),
                        ff_const(1.0 / 362880), ff_const(1.0 / 3628800), ff_const(1.0 / 39916800)};
  ff p = c[11];
#pragma unroll
  for (int k = 10; k >= 0; --k) p = p * r + c[k];
  const int ni = (int)n;
  return ff{ldexpf(p.hi, ni), ldexpf(p.lo, ni)};
}

__device__ __forceinline__ float ff_float(ff a) { return a.hi + a.lo; }

}  // namespace cr
