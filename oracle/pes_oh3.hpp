// Oracle (test infrastructure only): CPU restatement of Caracal's ANA_OH3
// surface, src/egrad_oh3.f: the OH + H2 potential of G. C. Schatz and
// H. Elgersma, Chem. Phys. Lett. 73, 21 (1980).  Atoms O, H1, H2, H3 (bohr,
// hartree).  Distances R1 = O-H1, R2 = O-H2, R3 = O-H3, R4 = H1-H2,
// R5 = H1-H3, R6 = H2-H3 (egrad_oh3:60-105).  pot_oh3 (:260-360) sums
// Morse terms on R1, R4, R5, the LEPS three-body term V3POT on (R2, R3, R6),
// the water-like terms VH2O on (R1, R2, R4) and (R1, R3, R5), the Gaussian
// four-body term V4POT on (R2, R3, R4, R5), then
// -2 DE(2) + DE(3).  Constants: the BLOCK DATA PTPACM_oh3, with V4POT
// reading ALP, CLAM, ACON and VH2O reading CON through their COMMON layouts.
#pragma once
#include <cmath>

#include "opcount.hpp"

namespace orc {
namespace oh3 {

struct Con {
  double de[3] = {0.148201, 0.0275690, 0.151548};
  double beta[3] = {1.260580, 0.924180, 1.068620};
  double re[3] = {1.863300, 2.907700, 1.428600};
  double sato = 0.10;
  double gam[3] = {2.399700, 1.058350, 2.399700};
  double reoh = 1.808090, rehh = 2.861590;
  double con[7] = {-.0015920, 0.026963, 0.0014689, 0.080011, 0.085816, -0.063179, 0.101380};
  double alp[4] = {4.773, 7.14, 2.938, 5.28};
  double clam[4] = {0.10, 0.10, 0.20, 0.03};
  double acon[2] = {0.10, 0.009};
};

// D (1 - exp(-B (R - T)))^2 and its derivative (pot_oh3's statement functions)
template <class T>
inline T vmor(double d, double b, double t, T r) {
  using std::exp;
  const T u = T(1.0) - exp(-b * (r - t));
  return d * (u * u);
}
template <class T>
inline T dvmor(double d, double b, double t, T r) {
  using std::exp;
  return 2.0 * b * d * (T(1.0) - exp(-b * (r - t))) * exp(-b * (r - t));
}

// V3POT_oh3: LEPS of R(1..3) with DE/BETA/RE = (XDE1, XDE1, XDE3) etc.
template <class T>
inline T v3pot(const Con& c, const T (&r)[3], T (&dedr)[3]) {
  using std::exp;
  using std::sqrt;
  const double de[3] = {c.de[0], c.de[0], c.de[2]};
  const double be[3] = {c.beta[0], c.beta[0], c.beta[2]};
  const double re[3] = {c.re[0], c.re[0], c.re[2]};
  double zpo[3], op3z[3], top3z[3], zp3[3], tzp3[3], do4z[3], b[3];
  for (int i = 0; i < 3; ++i) {
    const double z = c.sato;
    zpo[i] = 1.0 + z;
    op3z[i] = 1.0 + 3.0 * z;
    top3z[i] = 2.0 * op3z[i];
    zp3[i] = z + 3.0;
    tzp3[i] = 2.0 * zp3[i];
    do4z[i] = de[i] / 4.0 / zpo[i];
    b[i] = be[i] * do4z[i] * 2.0;
  }
  T e = T(0.0), x[3], exch[3];
  for (int i = 0; i < 3; ++i) {
    x[i] = exp(-be[i] * (r[i] - re[i]));
    const T coul = do4z[i] * (zp3[i] * x[i] - top3z[i]) * x[i];
    exch[i] = do4z[i] * (op3z[i] * x[i] - tzp3[i]) * x[i];
    e = e + coul;
  }
  const T d01 = exch[0] - exch[1], d12 = exch[1] - exch[2], d20 = exch[2] - exch[0];
  const T rad = sqrt(d01 * d01 + d12 * d12 + d20 * d20);
  e = e - rad / std::sqrt(2.0);
  const T s = exch[0] + exch[1] + exch[2];
  for (int i = 0; i < 3; ++i)
    dedr[i] = b[i] * x[i] * ((3.0 * exch[i] - s) / std::sqrt(2.0) * (op3z[i] * x[i] - zp3[i]) / rad -
                             zp3[i] * x[i] + op3z[i]);
  return e;
}

// V4POT_oh3 (A = ALP, C = CLAM, COF = ACON)
template <class T>
inline T v4pot(const Con& c, const T (&r)[4], T (&dedr)[4]) {
  using std::exp;
  const double* A = c.alp;
  const double* C = c.clam;
  const double* cof = c.acon;
  auto sq = [](T x) { return x * x; };
  const T t1 = exp(-(C[0] * sq(r[0] - A[0])) - C[0] * sq(r[1] - A[0]) - C[2] * sq(r[2] - A[2]) -
                   C[2] * sq(r[3] - A[2])) * cof[0];
  const T t2 = exp(-(C[1] * sq(r[0] - A[1])) - C[1] * sq(r[1] - A[1]) - C[3] * sq(r[2] - A[3]) -
                   C[3] * sq(r[3] - A[3])) * cof[1];
  dedr[0] = -2.0 * (t1 * C[0] * (r[0] - A[0]) + t2 * C[1] * (r[0] - A[1]));
  dedr[1] = -2.0 * (t1 * C[0] * (r[1] - A[0]) + t2 * C[1] * (r[1] - A[1]));
  dedr[2] = -2.0 * (t1 * C[2] * (r[2] - A[2]) + t2 * C[3] * (r[2] - A[3]));
  dedr[3] = -2.0 * (t1 * C[2] * (r[3] - A[2]) + t2 * C[3] * (r[3] - A[3]));
  return t1 + t2;
}

// VH2O_oh3: Q1 Q2 Q3 P with Q = 1 - tanh(x) (2 / (1 + exp(2x)) for
// 15 <= x < 43, 0 beyond), x = gam s / 2, with s ordered (OH, HH, OH) so the
// derivatives come out in that order and are swapped back to the argument
// order on return (the reference's TEMP exchange).  Where Q = 0 the reference
// leaves DEDR(I) as the previous call left it in its COMMON block; here it
// is 0 (E is 0 there anyway; only at separations beyond ~36 bohr).
template <class T>
inline T vh2o(const Con& c, const T (&r)[3], T (&dedr)[3]) {
  using std::cosh;
  using std::exp;
  using std::tanh;
  const double* C = c.con;
  T s[3], q[3], dq[3];
  s[0] = r[0] - c.reoh;
  s[2] = r[1] - c.reoh;
  s[1] = r[2] - c.rehh;
  for (int i = 0; i < 3; ++i) {
    const T x = 0.5 * c.gam[i] * s[i];
    if (x < T(15.0)) {
      q[i] = T(1.0) - tanh(x);
    } else if (x < T(43.0)) {
      q[i] = 2.0 / (T(1.0) + exp(2.0 * x));
    } else {
      q[i] = T(0.0);
      dq[i] = T(0.0);
      continue;
    }
    const T ch = cosh(x);
    dq[i] = -0.5 * c.gam[i] / (ch * ch);
  }
  const T p = C[0] + C[1] * (s[0] + s[2]) + C[2] * s[1] + 0.5 * C[3] * (s[0] * s[0] + s[2] * s[2]) +
              0.5 * C[4] * s[1] * s[1] + C[5] * s[1] * (s[0] + s[2]) + C[6] * s[0] * s[2];
  const T e = q[0] * q[1] * q[2] * p;
  T dp[3];
  dp[0] = C[1] + C[3] * s[0] + C[5] * s[1] + C[6] * s[2];
  dp[1] = C[2] + C[4] * s[1] + C[5] * (s[0] + s[2]);
  dp[2] = C[1] + C[3] * s[2] + C[5] * s[1] + C[6] * s[0];
  for (int i = 0; i < 3; ++i) {
    dedr[i] = T(0.0);
    if (val(q[i]) == 0.0) continue;
    dedr[i] = e * (dq[i] / q[i] + (dp[i] / p));
  }
  const T tmp = dedr[1];
  dedr[1] = dedr[2];
  dedr[2] = tmp;
  return e;
}

// pot_oh3: energy and dV/dR(1..6)
template <class T>
inline T pot(const T (&R)[6], T (&dv)[6]) {
  const Con c;
  for (int i = 0; i < 6; ++i) dv[i] = T(0.0);
  T v = vmor(c.de[0], c.beta[0], c.re[0], R[0]) + vmor(c.de[1], c.beta[1], c.re[1], R[3]) +
        vmor(c.de[1], c.beta[1], c.re[1], R[4]);
  dv[0] = dv[0] + dvmor(c.de[0], c.beta[0], c.re[0], R[0]);
  dv[3] = dv[3] + dvmor(c.de[1], c.beta[1], c.re[1], R[3]);
  dv[4] = dv[4] + dvmor(c.de[1], c.beta[1], c.re[1], R[4]);
  {
    const T r3[3] = {R[1], R[2], R[5]};
    T d[3];
    v = v + v3pot(c, r3, d);
    dv[1] = dv[1] + d[0];
    dv[2] = dv[2] + d[1];
    dv[5] = dv[5] + d[2];
  }
  {
    const T r3[3] = {R[0], R[1], R[3]};
    T d[3];
    v = v + vh2o(c, r3, d);
    dv[0] = dv[0] + d[0];
    dv[1] = dv[1] + d[1];
    dv[3] = dv[3] + d[2];
  }
  {
    const T r3[3] = {R[0], R[2], R[4]};
    T d[3];
    v = v + vh2o(c, r3, d);
    dv[0] = dv[0] + d[0];
    dv[2] = dv[2] + d[1];
    dv[4] = dv[4] + d[2];
  }
  {
    const T r4[4] = {R[1], R[2], R[3], R[4]};
    T d[4];
    v = v + v4pot(c, r4, d);
    dv[1] = dv[1] + d[0];
    dv[2] = dv[2] + d[1];
    dv[3] = dv[3] + d[2];
    dv[4] = dv[4] + d[3];
  }
  return v - 2.0 * c.de[1] + c.de[2];
}

// egrad_oh3 for one bead: q(3, 4) -> V, dV/dq(3, 4)
template <class T>
inline void egrad_bead(const T* q, T* V, T* g) {
  using std::sqrt;
  static const int pr[6][2] = {{1, 0}, {2, 0}, {3, 0}, {2, 1}, {3, 1}, {3, 2}};  // (b, a): q_b - q_a
  T d[6][3], R[6], dv[6];
  for (int k = 0; k < 6; ++k) {
    for (int x = 0; x < 3; ++x) d[k][x] = q[3 * pr[k][0] + x] - q[3 * pr[k][1] + x];
    R[k] = sqrt(d[k][0] * d[k][0] + d[k][1] * d[k][1] + d[k][2] * d[k][2]);
  }
  *V = pot(R, dv);
  for (int x = 0; x < 12; ++x) g[x] = T(0.0);
  for (int k = 0; k < 6; ++k)
    for (int x = 0; x < 3; ++x) {
      const T t = dv[k] * d[k][x] / R[k];
      g[3 * pr[k][1] + x] = g[3 * pr[k][1] + x] - t;
      g[3 * pr[k][0] + x] = g[3 * pr[k][0] + x] + t;
    }
}

}  // namespace oh3
}  // namespace orc
