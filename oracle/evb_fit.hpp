// ORACLE (test infrastructure only) -- dE-EVB coupling fit, CPU restatement.
//
// Restates the residual of Caracal's EVB coupling fit, lm_de_func
// (src/lm_de_func.f90:35-181): for reference points i with QMDFF energies
// E1_i, E2_i and reference energies E_ref,i, dE = |E1 - E2| and
//   fvec_i = (E_ref,i - (E1 + E2 - sqrt(dE^2 + 4 V12(dE)^2)) / 2)^2
// with the coupling basis's parameters in x (1g: a b; 2g: a b c d m;
// 3g: a b c d e f m n; sd, sp: a b c d; sd2: a b c d e f; sp2d: a b c d e f g
// h; sp2d3: a .. l), and MINPACK's forward-difference Jacobian fdjac2
// (src/lm_good.f:795-840): h = sqrt(max(epsfcn, epsmch)) |x_j| (or the root
// itself for x_j = 0), fjac(i,j) = (fvec_i(x + h e_j) - fvec_i) / h.
#pragma once
#include <cfloat>
#include <cmath>
#include <vector>

namespace orc {
namespace evbfit {

// Caracal's basis names in the order of the C-ABI ids 1..8 (const has no fit).
enum Basis { G1 = 1, G2 = 2, G3 = 3, SP = 4, SD = 5, SD2 = 6, SP2D = 7, SP2D3 = 8 };

inline double coupling(int basis, const double* x, double dE) {
  using std::exp;
  const double d2 = dE * dE;
  switch (basis) {
    case G1: return x[0] * exp(-x[1] * d2);
    case G2: return x[0] * exp(-x[1] * d2) + x[2] * exp(-x[3] * (dE + x[4]) * (dE + x[4]));
    case G3:
      return x[0] * exp(-x[1] * d2) + x[2] * exp(-x[3] * (dE + x[6]) * (dE + x[6])) +
             x[4] * exp(-x[5] * (dE + x[7]) * (dE + x[7]));
    case SP: return x[0] * exp(-x[1] * d2) + x[2] * dE * exp(-x[3] * d2);
    case SD: return x[0] * exp(-x[1] * d2) + x[2] * d2 * exp(-x[3] * d2);
    case SD2: return x[0] * exp(-x[1] * d2) + x[2] * d2 * exp(-x[3] * d2) + x[4] * d2 * exp(-x[5] * d2);
    case SP2D:
      return x[0] * exp(-x[1] * d2) + x[2] * dE * exp(-x[3] * d2) + x[4] * dE * exp(-x[5] * d2) +
             x[6] * d2 * exp(-x[7] * d2);
    default:  // SP2D3
      return x[0] * exp(-x[1] * d2) + x[2] * dE * exp(-x[3] * d2) + x[4] * dE * exp(-x[5] * d2) +
             x[6] * d2 * exp(-x[7] * d2) + x[8] * d2 * exp(-x[9] * d2) + x[10] * d2 * exp(-x[11] * d2);
  }
}

inline void residual(int basis, const double* x, int m, const double* e1, const double* e2, const double* eref,
                     double* fvec) {
  for (int i = 0; i < m; ++i) {
    const double dE = std::fabs(e1[i] - e2[i]);
    const double v = coupling(basis, x, dE);
    const double r = eref[i] - 0.5 * (e1[i] + e2[i] - std::sqrt(dE * dE + 4.0 * v * v));
    fvec[i] = r * r;
  }
}

inline void fdjac2(int basis, std::vector<double> x, int m, const double* e1, const double* e2, const double* eref,
                   const double* fvec, double epsfcn, double* fjac) {
  const double epsmch = DBL_EPSILON;
  const double eps = std::sqrt(std::fmax(epsfcn, epsmch));
  std::vector<double> wa((size_t)m);
  for (size_t j = 0; j < x.size(); ++j) {
    const double temp = x[j];
    double h = eps * std::fabs(temp);
    if (h == 0.0) h = eps;
    x[j] = temp + h;
    residual(basis, x.data(), m, e1, e2, eref, wa.data());
    x[j] = temp;
    for (int i = 0; i < m; ++i) fjac[(size_t)j * m + i] = (wa[(size_t)i] - fvec[i]) / h;
  }
}

}  // namespace evbfit
}  // namespace orc
