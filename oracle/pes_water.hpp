// Oracle (test infrastructure only): CPU restatement of Caracal's flexible
// SPC water box, src/egrad_water.f90:36-333, with the parameters of
// src/water_init.f90:74-103 and the minimum image of src/box_image.f90:36-63.
//
// Atoms come in molecules O, H, H.  Per molecule: two Morse OH stretches
// D_e (1 - exp(a dr))^2 (the reference's sign of the exponent), a harmonic
// HH stretch 0.5 k_theta dr_HH^2, the couplings k_rtheta dr_HH (dr_OH1 +
// dr_OH2) and k_rr dr_OH1 dr_OH2.  Between atoms of different molecules
// (i < j): point-charge Coulomb (or the Zahn form) and, where atom i is an
// oxygen, the LJ 12-6 term (src/egrad_water.f90:285 tests name(i) twice,
// so an O-H pair with the O first gets it too).  With periodic boundaries,
// every distance vector takes the minimum image and pairs at r >= coul_cut
// are skipped.  Parameter quirks kept: k_rr and epsilon_OO are REAL(4)
// literals (111.70765, 0.1554).
#pragma once
#include <cmath>
#include <vector>

#include "opcount.hpp"

namespace orc {
namespace water {

constexpr double kBohr = 0.52917721092;    // src/general.f90:256
constexpr double kHartree = 627.5094743;   // src/general.f90:257

struct Params {
  double r0, r0hh, de, a, ktheta, krtheta, krr, eh, eo, sigma, eps;
};

// src/water_init.f90:74-103 in atomic units
inline Params params() {
  Params p;
  p.r0 = 1.0 / kBohr;
  p.r0hh = 1.633 / kBohr;
  p.de = 101.9188 / kHartree;
  p.a = 2.567 * kBohr;
  p.ktheta = 328.645606 / kHartree * kBohr * kBohr;
  p.krtheta = -211.4672 / kHartree * kBohr * kBohr;
  p.krr = (double)111.70765f / kHartree * kBohr * kBohr;
  p.eh = 0.41;
  p.eo = -0.82;
  p.sigma = 3.166 / kBohr;
  p.eps = (double)0.1554f / kHartree;
  return p;
}

struct Box {
  int nwater = 0;
  int periodic = 0;
  double len[3] = {0, 0, 0};  // bohr
  double coul_cut = 0.0;      // bohr
  int zahn = 0;
  double zahn_a = 0.0, zahn_par = 0.0;
};

// src/box_image.f90: subtract the box length (sign of the component) while
// the component exceeds half the box length.
template <class T>
inline void box_image(const Box& b, T* d) {
  using std::fabs;
  for (int k = 0; k < 3; ++k) {
    const double L = b.len[k], L2 = 0.5 * b.len[k];
    while (fabs(d[k]) > T(L2)) d[k] = d[k] - T(std::copysign(L, val(d[k])));
  }
}

template <class T>
inline T egrad(const Box& b, const T* x, T* g) {
  using std::erfc;
  using std::exp;
  using std::sqrt;
  const Params P = params();
  const int n = 3 * b.nwater;
  T e = T(0);
  for (int i = 0; i < 3 * n; ++i) g[i] = T(0);
  for (int w = 0; w < b.nwater; ++w) {
    const int o = 3 * w, h1 = 3 * w + 1, h2 = 3 * w + 2;
    T oh1[3], oh2[3], hh[3];
    for (int k = 0; k < 3; ++k) {
      oh1[k] = x[3 * o + k] - x[3 * h1 + k];
      oh2[k] = x[3 * o + k] - x[3 * h2 + k];
      hh[k] = x[3 * h1 + k] - x[3 * h2 + k];
    }
    if (b.periodic) {
      box_image(b, oh1);
      box_image(b, oh2);
      box_image(b, hh);
    }
    const T r1 = sqrt(oh1[0] * oh1[0] + oh1[1] * oh1[1] + oh1[2] * oh1[2]);
    const T d1 = r1 - P.r0;
    const T r2 = sqrt(oh2[0] * oh2[0] + oh2[1] * oh2[1] + oh2[2] * oh2[2]);
    const T d2 = r2 - P.r0;
    const T rh = sqrt(hh[0] * hh[0] + hh[1] * hh[1] + hh[2] * hh[2]);
    const T dh = rh - P.r0hh;
    // Morse OH stretches
    const T ex1 = exp(P.a * d1), ex2 = exp(P.a * d2);
    e = e + P.de * (T(1) - ex1) * (T(1) - ex1);
    e = e + P.de * (T(1) - ex2) * (T(1) - ex2);
    const T de1 = -2.0 * P.a * P.de * ex1 * (T(1) - ex1) / r1;
    for (int k = 0; k < 3; ++k) {
      const T ga = de1 * oh1[k];
      g[3 * h1 + k] = g[3 * h1 + k] - ga;
      g[3 * o + k] = g[3 * o + k] + ga;
    }
    const T de2 = -2.0 * P.a * P.de * ex2 * (T(1) - ex2) / r2;
    for (int k = 0; k < 3; ++k) {
      const T ga = de2 * oh2[k];
      g[3 * h2 + k] = g[3 * h2 + k] - ga;
      g[3 * o + k] = g[3 * o + k] + ga;
    }
    // harmonic HH stretch
    e = e + 0.5 * P.ktheta * dh * dh;
    for (int k = 0; k < 3; ++k) {
      const T ga = P.ktheta * hh[k] * dh / rh;
      g[3 * h1 + k] = g[3 * h1 + k] + ga;
      g[3 * h2 + k] = g[3 * h2 + k] - ga;
    }
    // bond-angle coupling
    e = e + P.krtheta * dh * (d1 + d2);
    for (int k = 0; k < 3; ++k) {
      const T ga = dh / r1 * oh1[k] * P.krtheta;
      const T gb = dh / r2 * oh2[k] * P.krtheta;
      const T gh = P.krtheta * 1.0 * (d1 + d2) / rh * hh[k];
      g[3 * h1 + k] = g[3 * h1 + k] + gh - ga;
      g[3 * h2 + k] = g[3 * h2 + k] - gh - gb;
      g[3 * o + k] = g[3 * o + k] + ga + gb;
    }
    // bond-bond coupling
    e = e + P.krr * d1 * d2;
    for (int k = 0; k < 3; ++k) {
      const T ga = P.krr * (d2 / r1 * oh1[k]);
      const T gb = P.krr * (d1 / r2 * oh2[k]);
      g[3 * h1 + k] = g[3 * h1 + k] - ga;
      g[3 * h2 + k] = g[3 * h2 + k] - gb;
      g[3 * o + k] = g[3 * o + k] + gb + ga;
    }
  }
  // intermolecular: Coulomb and LJ (atom i an oxygen)
  for (int i = 0; i < n; ++i) {
    const double qi = (i % 3 == 0) ? P.eo : P.eh;
    for (int j = i + 1; j < n; ++j) {
      if (i / 3 == j / 3) continue;
      const double qj = (j % 3 == 0) ? P.eo : P.eh;
      T d[3];
      for (int k = 0; k < 3; ++k) d[k] = x[3 * i + k] - x[3 * j + k];
      if (b.periodic) box_image(b, d);
      const T r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
      if (!(r < T(b.coul_cut) || !b.periodic)) continue;
      const T oner = T(1) / r;
      T e0;
      if (b.zahn) e0 = qi * qj * ((erfc(b.zahn_a * r) * oner) - b.zahn_par * (r - b.coul_cut));
      else e0 = qi * qj * oner;
      e = e + e0;
      for (int k = 0; k < 3; ++k) {
        const T gv = e0 * oner * oner * d[k];
        g[3 * i + k] = g[3 * i + k] - gv;
        g[3 * j + k] = g[3 * j + k] + gv;
      }
      if (i % 3 == 0) {
        const T sr = P.sigma * oner;
        const T sr2 = sr * sr;
        const T sigr6 = sr2 * sr2 * sr2;
        e = e + 4.0 * P.eps * (sigr6 * sigr6 - sigr6);
        for (int k = 0; k < 3; ++k) {
          const T gv = 24.0 * P.eps * oner * oner * d[k] * sigr6 * (2.0 * sigr6 - 1.0);
          g[3 * i + k] = g[3 * i + k] - gv;
          g[3 * j + k] = g[3 * j + k] + gv;
        }
      }
    }
  }
  return e;
}

}  // namespace water
}  // namespace orc
