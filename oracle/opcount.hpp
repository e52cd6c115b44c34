// ORACLE (test infrastructure only) -- op-counting scalar.
//
// Instantiating the oracle's PES and step templates on `OC` tallies the
// floating-point work of the reference formulas, one counter per operation
// class.  The tallies give the algorithmic FLOP count per bead-step that the
// roofline figures divide by; they never run on a product path.
#pragma once
#include <cmath>
#include <cstdint>

namespace orc {

struct OpTally {
  uint64_t add = 0, mul = 0, div = 0, sqrt = 0, exp = 0, log = 0, pow = 0;
  uint64_t sin = 0, cos = 0, acos = 0, erf = 0, cmp = 0, tanh = 0, cosh = 0;
  void reset() { *this = OpTally(); }
};

inline OpTally& tally() {
  static thread_local OpTally t;
  return t;
}

struct OC {
  double v;
  OC() : v(0.0) {}
  OC(double x) : v(x) {}  // constants are free
  OC& operator+=(const OC& o) { tally().add++; v += o.v; return *this; }
  OC& operator-=(const OC& o) { tally().add++; v -= o.v; return *this; }
  OC& operator*=(const OC& o) { tally().mul++; v *= o.v; return *this; }
  OC& operator/=(const OC& o) { tally().div++; v /= o.v; return *this; }
};

inline OC operator+(OC a, OC b) { tally().add++; return OC(a.v + b.v); }
inline OC operator-(OC a, OC b) { tally().add++; return OC(a.v - b.v); }
inline OC operator*(OC a, OC b) { tally().mul++; return OC(a.v * b.v); }
inline OC operator/(OC a, OC b) { tally().div++; return OC(a.v / b.v); }
inline OC operator-(OC a) { return OC(-a.v); }
inline bool operator<(OC a, OC b) { tally().cmp++; return a.v < b.v; }
inline bool operator>(OC a, OC b) { tally().cmp++; return a.v > b.v; }
inline bool operator<=(OC a, OC b) { tally().cmp++; return a.v <= b.v; }
inline bool operator>=(OC a, OC b) { tally().cmp++; return a.v >= b.v; }
inline bool operator==(OC a, OC b) { tally().cmp++; return a.v == b.v; }
inline bool operator!=(OC a, OC b) { tally().cmp++; return a.v != b.v; }

inline OC exp(OC a) { tally().exp++; return OC(std::exp(a.v)); }
inline OC log(OC a) { tally().log++; return OC(std::log(a.v)); }
inline OC sqrt(OC a) { tally().sqrt++; return OC(std::sqrt(a.v)); }
inline OC pow(OC a, OC b) { tally().pow++; return OC(std::pow(a.v, b.v)); }
inline OC sin(OC a) { tally().sin++; return OC(std::sin(a.v)); }
inline OC cos(OC a) { tally().cos++; return OC(std::cos(a.v)); }
inline OC acos(OC a) { tally().acos++; return OC(std::acos(a.v)); }
inline OC erf(OC a) { tally().erf++; return OC(std::erf(a.v)); }
inline OC tanh(OC a) { tally().tanh++; return OC(std::tanh(a.v)); }
inline OC cosh(OC a) { tally().cosh++; return OC(std::cosh(a.v)); }
inline OC fabs(OC a) { return OC(std::fabs(a.v)); }
inline OC asin(OC a) { tally().acos++; return OC(std::asin(a.v)); }    // counted with acos
inline OC erfc(OC a) { tally().erf++; return OC(std::erfc(a.v)); }     // counted with erf
inline OC fmin(OC a, OC b) { tally().cmp++; return OC(std::fmin(a.v, b.v)); }
inline OC fmax(OC a, OC b) { tally().cmp++; return OC(std::fmax(a.v, b.v)); }
inline double val(OC a) { return a.v; }
inline double val(double a) { return a; }

}  // namespace orc
