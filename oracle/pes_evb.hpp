// ORACLE (test infrastructure only) -- dE-EVB of two QMDFFs, CPU restatement.
//
// Restates the two-QMDFF branch of Caracal's gradient (src/gradient.f90:
// 361-386 and 1228-1304): E_i = ff_eg + ff_nonb (+ ff_hb) + E_zero_i of each
// force field on the same geometry, dE = E_1 - E_2, the coupling V12(dE) of
// the chosen basis ("const", "1g", "2g", "3g", "sp", "sd", "sd2", "sp2d"),
// and the lower root E = (E_1 + E_2 - sqrt(dE^2 + 4 V12^2)) / 2 with the
// gradient 0.5 (g_1 + g_2 - d/2 / root) as Caracal writes it per basis.
#pragma once
#include <cmath>
#include <vector>

#include "pes_qmdff.hpp"

namespace orc {
namespace evb {

enum Basis { CONST = 0, G1 = 1, G2 = 2, G3 = 3, SP = 4, SD = 5, SD2 = 6, SP2D = 7 };

struct Coupling {
  int basis = CONST;
  double a = 0, b = 0, c = 0, d = 0, e = 0, f = 0, g = 0, h = 0, m = 0, n = 0;  // offa..offh, offm, offn
};

template <class T>
inline void egrad(const qmdff::FF& f1, const qmdff::FF& f2, const Coupling& C, const T* x, T* V, T* g) {
  using std::exp;
  using std::sqrt;
  const int n3 = 3 * f1.n;
  std::vector<T> g1((size_t)n3), g2((size_t)n3);
  T e1, e2;
  qmdff::egrad<T>(f1, x, &e1, g1.data());  // e1 + E_zero1
  qmdff::egrad<T>(f2, x, &e2, g2.data());  // e2 + E_zero2
  const T ediff = e1 - e2;
  T offdiag;
  switch (C.basis) {
    case CONST: offdiag = C.a; break;
    case G1: offdiag = C.a * exp(-C.b * ediff * ediff); break;
    case G2:
      offdiag = C.a * exp(-C.b * ediff * ediff) + C.c * exp(-C.d * (ediff + C.m) * (ediff + C.m));
      break;
    case G3:
      offdiag = C.a * exp(-C.b * ediff * ediff) + C.c * exp(-C.d * (ediff + C.m) * (ediff + C.m)) +
                C.e * exp(-C.f * (ediff + C.n) * (ediff + C.n));
      break;
    case SP: offdiag = C.a * exp(-C.b * ediff * ediff) + C.c * ediff * exp(-C.d * ediff * ediff); break;
    case SD: offdiag = C.a * exp(-C.b * ediff * ediff) + C.c * ediff * ediff * exp(-C.d * ediff * ediff); break;
    case SD2:
      offdiag = C.a * exp(-C.b * ediff * ediff) + C.c * ediff * ediff * exp(-C.d * ediff * ediff) +
                C.e * ediff * ediff * exp(-C.f * ediff * ediff);
      break;
    default:  // SP2D
      offdiag = C.a * exp(-C.b * ediff * ediff) + C.c * ediff * exp(-C.d * ediff * ediff) +
                C.e * ediff * exp(-C.f * ediff * ediff) + ediff * ediff * C.g * exp(-C.h * ediff * ediff);
      break;
  }
  const T off4 = 4.0 * offdiag * offdiag;
  const T root2 = sqrt(ediff * ediff + off4);
  *V = 0.5 * (e1 + e2 - root2);
  for (int k = 0; k < n3; ++k) {
    const T dg = g1[(size_t)k] - g2[(size_t)k];
    T deldiscr;
    switch (C.basis) {
      case CONST: deldiscr = ediff * dg; break;
      case G1: deldiscr = ediff * dg * (1.0 - 2.0 * off4 * C.b); break;
      case G2:
        deldiscr = dg * (1.0 * ediff + 4.0 * offdiag *
                                           (-2.0 * C.a * C.b * ediff * exp(-C.b * ediff * ediff) -
                                            2.0 * C.c * C.d * (C.m + ediff) * exp(-C.d * (ediff + C.m) * (ediff + C.m))));
        break;
      case G3:
        deldiscr = dg * (1.0 * ediff + 4.0 * offdiag *
                                           (-2.0 * C.a * C.b * ediff * exp(-C.b * ediff * ediff) -
                                            2.0 * C.c * C.d * (C.m + ediff) * exp(-C.d * (ediff + C.m) * (ediff + C.m)) -
                                            2.0 * C.e * C.f * (C.n + ediff) * exp(-C.f * (ediff + C.n) * (ediff + C.n))));
        break;
      case SP:
        deldiscr = dg * (1.0 * ediff + 4.0 * offdiag *
                                           (-2.0 * C.a * C.b * ediff * exp(-C.b * ediff * ediff) +
                                            C.c * (1.0 - 2.0 * ediff * ediff * C.d) * exp(-C.d * ediff * ediff)));
        break;
      case SD:
        deldiscr = dg * (1.0 * ediff + 4.0 * offdiag *
                                           (-2.0 * C.a * C.b * ediff * exp(-C.b * ediff * ediff) +
                                            C.c * (2.0 * ediff - 2.0 * ediff * ediff * ediff * C.d) *
                                                exp(-C.d * ediff * ediff)));
        break;
      case SD2:
        deldiscr = dg * (1.0 * ediff + 4.0 * offdiag *
                                           (-2.0 * C.a * C.b * ediff * exp(-C.b * ediff * ediff) +
                                            C.c * (2.0 * ediff - 2.0 * ediff * ediff * ediff * C.d) *
                                                exp(-C.d * ediff * ediff) +
                                            C.e * (2.0 * ediff - 2.0 * ediff * ediff * ediff * C.f) *
                                                exp(-C.f * ediff * ediff)));
        break;
      default:  // SP2D
        deldiscr = dg * (1.0 * ediff + 4.0 * offdiag *
                                           (-2.0 * C.a * C.b * ediff * exp(-C.b * ediff * ediff) +
                                            C.c * (1.0 - 2.0 * ediff * ediff * C.d) * exp(-C.d * ediff * ediff) +
                                            C.e * (1.0 - 2.0 * ediff * ediff * C.f) * exp(-C.f * ediff * ediff) +
                                            C.g * (2.0 * ediff - 2.0 * ediff * ediff * ediff * C.h) *
                                                exp(-C.h * ediff * ediff)));
        break;
    }
    const T delsqrt = deldiscr / root2;
    g[k] = 0.5 * (g1[(size_t)k] + g2[(size_t)k] - delsqrt);
  }
}

}  // namespace evb
}  // namespace orc
