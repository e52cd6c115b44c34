// Forward-mode dual numbers x + eps dx (eps^2 = 0) for directional
// derivatives of the FP64 force-field code: evaluating a term with dual
// coordinates x + eps w gives its energy, gradient and, in the eps parts, the
// directional derivative of the energy and the Hessian-vector product H w.
// Comparisons and branches act on the value part.  Derivative rules are the
// textbook ones (d sqrt(x) = dx / (2 sqrt x), d exp(x) = exp(x) dx, ...).
// The type and its functions live in their own namespace: unqualified calls
// with Dual arguments find them by argument-dependent lookup, while calls
// with plain doubles elsewhere keep resolving to the C math functions.
#pragma once
#include <cuda_runtime.h>

#include <cmath>

namespace cr {
namespace ad {

struct Dual {
  double v, d;
  Dual() = default;
  __host__ __device__ constexpr Dual(double x) : v(x), d(0.0) {}  // NOLINT: constants promote implicitly
  __host__ __device__ constexpr Dual(double x, double dx) : v(x), d(dx) {}
  __host__ __device__ inline Dual& operator+=(const Dual& o) {
    v += o.v;
    d += o.d;
    return *this;
  }
  __host__ __device__ inline Dual& operator-=(const Dual& o) {
    v -= o.v;
    d -= o.d;
    return *this;
  }
  __host__ __device__ inline Dual& operator*=(const Dual& o) {
    d = d * o.v + v * o.d;
    v *= o.v;
    return *this;
  }
  __host__ __device__ inline Dual& operator/=(const Dual& o) {
    const double r = 1.0 / o.v;
    v *= r;
    d = (d - v * o.d) * r;
    return *this;
  }
};

__host__ __device__ inline Dual operator-(const Dual& a) { return Dual(-a.v, -a.d); }
__host__ __device__ inline Dual operator+(const Dual& a, const Dual& b) { return Dual(a.v + b.v, a.d + b.d); }
__host__ __device__ inline Dual operator-(const Dual& a, const Dual& b) { return Dual(a.v - b.v, a.d - b.d); }
__host__ __device__ inline Dual operator*(const Dual& a, const Dual& b) { return Dual(a.v * b.v, a.d * b.v + a.v * b.d); }
__host__ __device__ inline Dual operator/(const Dual& a, const Dual& b) {
  const double r = 1.0 / b.v, q = a.v * r;
  return Dual(q, (a.d - q * b.d) * r);
}
__host__ __device__ inline Dual operator+(const Dual& a, double b) { return Dual(a.v + b, a.d); }
__host__ __device__ inline Dual operator+(double a, const Dual& b) { return Dual(a + b.v, b.d); }
__host__ __device__ inline Dual operator-(const Dual& a, double b) { return Dual(a.v - b, a.d); }
__host__ __device__ inline Dual operator-(double a, const Dual& b) { return Dual(a - b.v, -b.d); }
__host__ __device__ inline Dual operator*(const Dual& a, double b) { return Dual(a.v * b, a.d * b); }
__host__ __device__ inline Dual operator*(double a, const Dual& b) { return Dual(a * b.v, a * b.d); }
__host__ __device__ inline Dual operator/(const Dual& a, double b) { return Dual(a.v / b, a.d / b); }
__host__ __device__ inline Dual operator/(double a, const Dual& b) {
  const double q = a / b.v;
  return Dual(q, -q * b.d / b.v);
}

#define CR_DUAL_CMP(op)                                                                         \
  __host__ __device__ inline bool operator op(const Dual& a, const Dual& b) { return a.v op b.v; } \
  __host__ __device__ inline bool operator op(const Dual& a, double b) { return a.v op b; }        \
  __host__ __device__ inline bool operator op(double a, const Dual& b) { return a op b.v; }
CR_DUAL_CMP(<)
CR_DUAL_CMP(>)
CR_DUAL_CMP(<=)
CR_DUAL_CMP(>=)
CR_DUAL_CMP(==)
CR_DUAL_CMP(!=)
#undef CR_DUAL_CMP

// value part (identity for plain numbers)
__host__ __device__ inline double val(const Dual& a) { return a.v; }
__host__ __device__ inline double val(double a) { return a; }
__host__ __device__ inline float val(float a) { return a; }

__host__ __device__ inline Dual sqrt(const Dual& a) {
  const double s = ::sqrt(a.v);
  return Dual(s, s > 0.0 ? a.d / (2.0 * s) : 0.0);
}
__host__ __device__ inline Dual exp(const Dual& a) {
  const double e = ::exp(a.v);
  return Dual(e, e * a.d);
}
__host__ __device__ inline Dual log(const Dual& a) { return Dual(::log(a.v), a.d / a.v); }
__host__ __device__ inline Dual pow(const Dual& a, double p) {
  const double y = ::pow(a.v, p);
  return Dual(y, a.v != 0.0 ? p * y / a.v * a.d : 0.0);
}
__host__ __device__ inline Dual sin(const Dual& a) { return Dual(::sin(a.v), ::cos(a.v) * a.d); }
__host__ __device__ inline Dual cos(const Dual& a) { return Dual(::cos(a.v), -::sin(a.v) * a.d); }
__host__ __device__ inline Dual acos(const Dual& a) {
  const double s = ::sqrt(1.0 - a.v * a.v);
  return Dual(::acos(a.v), s > 0.0 ? -a.d / s : 0.0);
}
__host__ __device__ inline Dual asin(const Dual& a) {
  const double s = ::sqrt(1.0 - a.v * a.v);
  return Dual(::asin(a.v), s > 0.0 ? a.d / s : 0.0);
}
// d erf(x) = 2 / sqrt(pi) exp(-x^2) dx
__host__ __device__ inline Dual erf(const Dual& a) {
  return Dual(::erf(a.v), 1.1283791670955125739 * ::exp(-a.v * a.v) * a.d);
}
__host__ __device__ inline Dual erfc(const Dual& a) {
  return Dual(::erfc(a.v), -1.1283791670955125739 * ::exp(-a.v * a.v) * a.d);
}
__host__ __device__ inline Dual fabs(const Dual& a) { return a.v < 0.0 ? -a : a; }
__host__ __device__ inline Dual fmin(const Dual& a, const Dual& b) { return b.v < a.v ? b : a; }
__host__ __device__ inline Dual fmax(const Dual& a, const Dual& b) { return b.v > a.v ? b : a; }

}  // namespace ad
using ad::Dual;
}  // namespace cr
