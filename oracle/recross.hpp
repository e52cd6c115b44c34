// ORACLE (test infrastructure only) -- recrossing children of calc_rate.
//
// CPU restatement of the child part of Caracal's `recross`
// (src/recross.f90:540-614) with the BIMOLEC reaction coordinate of
// `calc_xi` in its recrossing mode (src/calc_xi.f90:63-279, mode 2) and
// `calc_com` (src/calc_com.f90:36-59):
//   xi  = xi_ideal * s1 + (1 - xi_ideal) * s0
//   s1  = (r_break - r_break_ref) - (r_form - r_form_ref)   (one bond each)
//   s0  = R_inf - |COM(reactant 2) - COM(reactant 1)|
// For each child: q = the parent ring polymer, p = Andersen draw (the pair
// partner gets -p), forces, xi and dxi at the centroid, vs = dxi . sum_k p_k /
// m / P, fs = sqrt(sum dxi^2 / m / (2 pi beta)), denominator += vs/fs if
// vs > 0; then child_evol NVE steps (no thermostat, no transrot: verlet with
// constrain = 2), numerator(t) += vs/fs whenever xi(centroid) > 0 after step t.
#pragma once
#include <cmath>
#include <vector>

#include "philox.hpp"
#include "rpmd.hpp"

namespace orc {

struct XiDef {
  int nreac1 = 0, reac1[8] = {0};  // 0-based atom indices
  int nreac2 = 0, reac2[8] = {0};
  int form[2] = {0, 0}, brk[2] = {0, 0};
  double form_ref = 0, break_ref = 0, r_inf = 0, xi_ideal = 1.0;
};

// xi (mode 2) and dxi(3,N) at coordinates c(3,N).
inline double calc_xi_mode2(const XiDef& x, int N, const double* c, const double* mass, double* dxi) {
  double Rf[3], Rb[3];
  for (int d = 0; d < 3; ++d) {
    Rf[d] = c[3 * x.form[0] + d] - c[3 * x.form[1] + d];
    Rb[d] = c[3 * x.brk[0] + d] - c[3 * x.brk[1] + d];
  }
  double form_act = std::sqrt(Rf[0] * Rf[0] + Rf[1] * Rf[1] + Rf[2] * Rf[2]);
  double break_act = std::sqrt(Rb[0] * Rb[0] + Rb[1] * Rb[1] + Rb[2] * Rb[2]);
  double s1 = 0.0;
  s1 = s1 + (break_act - x.break_ref) / 1.0;
  s1 = s1 - (form_act - x.form_ref) / 1.0;
  double com[2][3] = {{0, 0, 0}, {0, 0, 0}}, mreac[2] = {0, 0};
  for (int k = 0; k < x.nreac1; ++k) mreac[0] += mass[x.reac1[k]];
  for (int k = 0; k < x.nreac2; ++k) mreac[1] += mass[x.reac2[k]];
  for (int k = 0; k < x.nreac1; ++k)
    for (int d = 0; d < 3; ++d) com[0][d] = com[0][d] + mass[x.reac1[k]] * c[3 * x.reac1[k] + d] / mreac[0];
  for (int k = 0; k < x.nreac2; ++k)
    for (int d = 0; d < 3; ++d) com[1][d] = com[1][d] + mass[x.reac2[k]] * c[3 * x.reac2[k] + d] / mreac[1];
  double Red[3] = {com[1][0] - com[0][0], com[1][1] - com[0][1], com[1][2] - com[0][2]};
  double reds = std::sqrt(Red[0] * Red[0] + Red[1] * Red[1] + Red[2] * Red[2]);
  double s0 = 0.0;
  s0 = s0 + (x.r_inf - reds);
  s0 = s0 / 1.0;
  double xi = x.xi_ideal * s1 + (1.0 - x.xi_ideal) * s0;
  if (dxi) {
    std::vector<double> ds1(3 * N, 0.0), ds0(3 * N, 0.0);
    double ri = 1.0 / form_act;
    for (int d = 0; d < 3; ++d) {
      ds1[3 * x.form[0] + d] = ds1[3 * x.form[0] + d] - Rf[d] * ri / 1.0;
      ds1[3 * x.form[1] + d] = ds1[3 * x.form[1] + d] + Rf[d] * ri / 1.0;
    }
    ri = 1.0 / break_act;
    for (int d = 0; d < 3; ++d) {
      ds1[3 * x.brk[0] + d] = ds1[3 * x.brk[0] + d] + Rb[d] * ri / 1.0;
      ds1[3 * x.brk[1] + d] = ds1[3 * x.brk[1] + d] - Rb[d] * ri / 1.0;
    }
    ri = 1.0 / reds;
    for (int k = 0; k < x.nreac1; ++k) {
      int a = x.reac1[k];
      for (int d = 0; d < 3; ++d) ds0[3 * a + d] = ds0[3 * a + d] + Red[d] * ri * mass[a] / mreac[0] / 1.0;
    }
    for (int k = 0; k < x.nreac2; ++k) {
      int a = x.reac2[k];
      for (int d = 0; d < 3; ++d) ds0[3 * a + d] = ds0[3 * a + d] - Red[d] * ri * mass[a] / mreac[1] / 1.0;
    }
    for (int i = 0; i < 3 * N; ++i) dxi[i] = x.xi_ideal * ds1[i] + (1.0 - x.xi_ideal) * ds0[i];
  }
  return xi;
}

inline void centroid(int N, int P, const double* q, double* c) {
  for (int x = 0; x < 3 * N; ++x) {
    double s = 0.0;
    for (int k = 0; k < P; ++k) s = s + q[(size_t)k * 3 * N + x];
    c[x] = s / P;
  }
}

// One child trajectory t; side[s] = xi(centroid) > 0 after step s+1.
// Returns the flux weight vs/fs and whether vs > 0.
template <class EGrad>
inline double recross_child(const StepConfig& cf, const XiDef& xd, uint32_t traj_key, bool negate,
                            const double* q_parent, int nsteps, double* q, double* p, double* f,
                            unsigned char* side, bool* vs_positive, EGrad egrad) {
  const int N = cf.natoms, P = cf.nbeads, nc = 3 * N;
  for (int x = 0; x < nc * P; ++x) q[x] = q_parent[x];
  andersen(cf, traj_key, 0, TAG_CHILD_MOMENTA, p);
  if (negate)
    for (int x = 0; x < nc * P; ++x) p[x] = -p[x];
  std::vector<double> c(nc), dxi(nc);
  centroid(N, P, q, c.data());
  calc_xi_mode2(xd, N, c.data(), cf.mass, dxi.data());
  for (int k = 0; k < P; ++k) {
    double v;
    egrad(&q[(size_t)k * nc], &v, &f[(size_t)k * nc]);
  }
  double vs = 0.0;
  for (int l = 0; l < 3; ++l)
    for (int m = 0; m < N; ++m)
      for (int o = 0; o < P; ++o) vs = vs + dxi[3 * m + l] * p[(size_t)o * nc + 3 * m + l] / cf.mass[m];
  vs = vs / P;
  double fs = 0.0;
  for (int l = 0; l < 3; ++l)
    for (int m = 0; m < N; ++m) fs = fs + dxi[3 * m + l] * dxi[3 * m + l] / cf.mass[m];
  const double pi = 3.1415926535897932384;
  fs = std::sqrt(fs / (2.0 * pi * cf.beta));
  *vs_positive = vs > 0;
  StepConfig child = cf;
  child.thermostat = 0;
  child.transrot = 0;
  double e;
  for (int s = 1; s <= nsteps; ++s) {
    verlet_step(child, traj_key, s, q, p, f, &e, egrad);
    centroid(N, P, q, c.data());
    side[s - 1] = calc_xi_mode2(xd, N, c.data(), cf.mass, nullptr) > 0.0 ? 1 : 0;
  }
  return vs / fs;
}

}  // namespace orc
