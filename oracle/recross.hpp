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
// The parent trajectory (verlet with constrain = 1) is kept on the dividing
// surface by SHAKE on the centroid (constrain_q, src/constrain_q.f90:35-113)
// and RATTLE on the momenta (constrain_p, src/constrain_p.f90:36-76).
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

// constrain_q (src/constrain_q.f90:35-113): Newton iterations (at most 200)
// for the multiplier that moves the centroid c along dxi_act onto xi = 0,
// then every bead is shifted.  As in the reference, q moves by the
// coefficient of the last iteration's start and p by the updated multiplier.
// Returns false when the iterations do not converge (q, p unchanged).
inline bool constrain_q(const StepConfig& cf, const XiDef& xd, const double* c, const double* dxi_act, double* q,
                        double* p) {
  const int N = cf.natoms, P = cf.nbeads, nc = 3 * N;
  const double dt = cf.dt;
  double mult = 0.0, coeff = 0.0;
  std::vector<double> qt(nc), dxn(nc);
  const int maxiters = 200;
  for (int iter = 1; iter <= maxiters; ++iter) {
    coeff = mult * dt * dt / P;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < N; ++j) qt[3 * j + i] = c[3 * j + i] + coeff * dxi_act[3 * j + i] / cf.mass[j];
    const double sigma = calc_xi_mode2(xd, N, qt.data(), cf.mass, dxn.data());
    double dsigma = 0.0;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < N; ++j)
        dsigma = dsigma + dxn[3 * j + i] * dt * dt * dxi_act[3 * j + i] / (cf.mass[j] * P);
    const double dx = sigma / dsigma;
    mult = mult - dx;
    if (std::fabs(dx) < (double)1.0E-8f || std::fabs(sigma) < (double)1.0E-10f) break;
    if (iter == maxiters) return false;
  }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < N; ++j)
      for (int k = 0; k < P; ++k) {
        q[(size_t)k * nc + 3 * j + i] = q[(size_t)k * nc + 3 * j + i] + coeff / cf.mass[j] * dxi_act[3 * j + i];
        p[(size_t)k * nc + 3 * j + i] = p[(size_t)k * nc + 3 * j + i] + mult * dt / P * dxi_act[3 * j + i];
      }
  return true;
}

// constrain_p (src/constrain_p.f90:36-76): removes the momentum along dxi_act.
inline void constrain_p(const StepConfig& cf, const double* dxi_act, double* p) {
  const int N = cf.natoms, P = cf.nbeads, nc = 3 * N;
  double coeff1 = 0.0, coeff2 = 0.0;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < N; ++j)
      for (int k = 0; k < P; ++k) coeff1 = coeff1 + dxi_act[3 * j + i] * p[(size_t)k * nc + 3 * j + i] / cf.mass[j];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < N; ++j) coeff2 = coeff2 + dxi_act[3 * j + i] * dxi_act[3 * j + i] / cf.mass[j];
  const double lambdas = -coeff1 / coeff2 / P;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < N; ++j)
      for (int k = 0; k < P; ++k) p[(size_t)k * nc + 3 * j + i] = p[(size_t)k * nc + 3 * j + i] + lambdas * dxi_act[3 * j + i];
}

enum ParentStatus : int { TRAJ_SHAKE_FAILED = 4 };

// One step of the constrained parent (verlet with constrain = 1): thermostat
// as configured, no transrot; dxi_act carries dxi at the previous step's
// centroid taken before its SHAKE (src/verlet.f90:649, 746-757, 1043-1049,
// 1080-1082).  A failed SHAKE sets TRAJ_SHAKE_FAILED and, like the
// reference, gives the step the 1e5 energy penalty.
template <class EGrad>
inline int parent_step(const StepConfig& cf, const XiDef& xd, uint32_t traj, int istep, double* q, double* p,
                       double* f, double* epot, double* dxi_act, EGrad egrad, double* vnh = nullptr) {
  const int N = cf.natoms, P = cf.nbeads, n3 = 3 * N;
  const size_t nall = (size_t)n3 * P;
  if (cf.thermostat == 2) nhc_half(cf, vnh, p);
  if (cf.thermostat == 3) pile_half(cf, traj, (uint32_t)istep, TAG_PILE_A, p);
  for (size_t x = 0; x < nall; ++x) p[x] = p[x] - 0.5 * cf.dt * f[x];
  free_rp_step(cf, q, p);
  std::vector<double> c(n3);
  centroid(N, P, q, c.data());
  int status = TRAJ_OK;
  double e = 0.0;
  if (!constrain_q(cf, xd, c.data(), dxi_act, q, p)) {
    status |= TRAJ_SHAKE_FAILED;
    e = 100000.0;
  }
  for (int k = 0; k < P; ++k) {
    double v;
    egrad(&q[(size_t)k * n3], &v, &f[(size_t)k * n3]);
    e = e + v;
  }
  *epot = e;
  calc_xi_mode2(xd, N, c.data(), cf.mass, dxi_act);
  for (size_t x = 0; x < nall; ++x) p[x] = p[x] - 0.5 * cf.dt * f[x];
  constrain_p(cf, dxi_act, p);
  if (cf.thermostat == 2) nhc_half(cf, vnh, p);
  if (cf.thermostat == 1 && istep % cf.andersen_step == 0) andersen(cf, traj, (uint32_t)istep, TAG_ANDERSEN, p);
  if (cf.thermostat == 3) pile_half(cf, traj, (uint32_t)istep, TAG_PILE_B, p);
  for (size_t x = 0; x < nall; ++x)
    if (!std::isfinite(q[x])) status |= TRAJ_NONFINITE;
  return status;
}

// Umbrella sampling (calc_xi mode 1, src/calc_xi.f90:63-470; one forming and
// one breaking bond, two reactants): xi = s0 / (s0 - s1),
// dxi = (s0 ds1 - s1 ds0) / (s0 - s1)^2 and, if d2xi (3N x 3N, row-major over
// (atom, dim)) is given, the reference's explicit Hessian from the bond and
// centre-of-mass distance Hessians d2s1, d2s0.
inline double calc_xi_mode1(const XiDef& x, int N, const double* c, const double* mass, double* dxi,
                            double* d2xi) {
  const int n3 = 3 * N;
  double Rf[3], Rb[3];
  for (int d = 0; d < 3; ++d) {
    Rf[d] = c[3 * x.form[0] + d] - c[3 * x.form[1] + d];
    Rb[d] = c[3 * x.brk[0] + d] - c[3 * x.brk[1] + d];
  }
  const double rf = std::sqrt(Rf[0] * Rf[0] + Rf[1] * Rf[1] + Rf[2] * Rf[2]);
  const double rb = std::sqrt(Rb[0] * Rb[0] + Rb[1] * Rb[1] + Rb[2] * Rb[2]);
  double s1 = 0.0;
  s1 = s1 + (rb - x.break_ref) / 1.0;
  s1 = s1 - (rf - x.form_ref) / 1.0;
  const int* rs[2] = {x.reac1, x.reac2};
  const int nr[2] = {x.nreac1, x.nreac2};
  double com[2][3] = {{0, 0, 0}, {0, 0, 0}}, mr[2] = {0, 0};
  for (int r = 0; r < 2; ++r)
    for (int k = 0; k < nr[r]; ++k) mr[r] += mass[rs[r][k]];
  for (int r = 0; r < 2; ++r)
    for (int k = 0; k < nr[r]; ++k)
      for (int d = 0; d < 3; ++d) com[r][d] = com[r][d] + mass[rs[r][k]] * c[3 * rs[r][k] + d] / mr[r];
  const double Red[3] = {com[1][0] - com[0][0], com[1][1] - com[0][1], com[1][2] - com[0][2]};
  const double reds = std::sqrt(Red[0] * Red[0] + Red[1] * Red[1] + Red[2] * Red[2]);
  double s0 = 0.0;
  s0 = s0 + (x.r_inf - reds);
  s0 = s0 / 1.0;
  const double xi = s0 / (s0 - s1);
  std::vector<double> ds1(n3, 0.0), ds0(n3, 0.0);
  double ri = 1.0 / rf;
  for (int d = 0; d < 3; ++d) {
    ds1[3 * x.form[0] + d] = ds1[3 * x.form[0] + d] - Rf[d] * ri / 1.0;
    ds1[3 * x.form[1] + d] = ds1[3 * x.form[1] + d] + Rf[d] * ri / 1.0;
  }
  ri = 1.0 / rb;
  for (int d = 0; d < 3; ++d) {
    ds1[3 * x.brk[0] + d] = ds1[3 * x.brk[0] + d] + Rb[d] * ri / 1.0;
    ds1[3 * x.brk[1] + d] = ds1[3 * x.brk[1] + d] - Rb[d] * ri / 1.0;
  }
  ri = 1.0 / reds;
  for (int r = 0; r < 2; ++r) {
    const double sg = r == 0 ? 1.0 : -1.0;
    for (int k = 0; k < nr[r]; ++k) {
      const int a = rs[r][k];
      for (int d = 0; d < 3; ++d) ds0[3 * a + d] = ds0[3 * a + d] + sg * Red[d] * ri * mass[a] / mr[r] / 1.0;
    }
  }
  const double D = s0 - s1;
  if (dxi)
    for (int i = 0; i < n3; ++i) dxi[i] = (s0 * ds1[i] - s1 * ds0[i]) / (D * D);
  if (d2xi) {
    // second derivatives of the bond lengths and the COM distance: for a
    // vector R of length r, d2 r / dR_a dR_b = (delta_ab r^2 - R_a R_b) / r^3
    std::vector<double> d2s1((size_t)n3 * n3, 0.0), d2s0((size_t)n3 * n3, 0.0);
    auto blk = [](const double* R, double r, double sgn, double h[3][3]) {
      const double r3 = 1.0 / (r * r * r);
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) h[a][b] = sgn * ((a == b ? r * r : 0.0) - R[a] * R[b]) * r3;
    };
    auto add2 = [&](std::vector<double>& H, int i, int j, double h[3][3], double w) {
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) H[(size_t)(3 * i + a) * n3 + 3 * j + b] += w * h[a][b];
    };
    double hf[3][3], hb[3][3], hr[3][3];
    blk(Rf, rf, -1.0, hf);  // s1 contains -r_form
    blk(Rb, rb, 1.0, hb);
    blk(Red, reds, -1.0, hr);  // s0 contains -|Red|
    const int fa = x.form[0], fb = x.form[1], ba = x.brk[0], bb = x.brk[1];
    add2(d2s1, fa, fa, hf, 1.0);
    add2(d2s1, fa, fb, hf, -1.0);
    add2(d2s1, fb, fa, hf, -1.0);
    add2(d2s1, fb, fb, hf, 1.0);
    add2(d2s1, ba, ba, hb, 1.0);
    add2(d2s1, ba, bb, hb, -1.0);
    add2(d2s1, bb, ba, hb, -1.0);
    add2(d2s1, bb, bb, hb, 1.0);
    for (int r1 = 0; r1 < 2; ++r1)
      for (int k = 0; k < nr[r1]; ++k)
        for (int r2 = 0; r2 < 2; ++r2)
          for (int l = 0; l < nr[r2]; ++l) {
            const int a1 = rs[r1][k], a2 = rs[r2][l];
            const double mf = mass[a1] / mr[r1] * mass[a2] / mr[r2];
            add2(d2s0, a1, a2, hr, (r1 == r2 ? 1.0 : -1.0) * mf);
          }
    for (int i = 0; i < n3; ++i)
      for (int j = 0; j < n3; ++j)
        d2xi[(size_t)i * n3 + j] =
            ((s0 * d2s1[(size_t)i * n3 + j] + ds0[j] * ds1[i] - ds1[j] * ds0[i] - s1 * d2s0[(size_t)i * n3 + j]) * D -
             2.0 * (s0 * ds1[i] - s1 * ds0[i]) * (ds0[j] - ds1[j])) /
            (D * D * D);
  }
  return xi;
}

// Umbrella bias of one ring polymer (umbrella mode 0, src/umbrella.f90:100-176):
// at the centroid, every bead's gradient gets k (xi - xi0) dxi plus the
// gradient of -(1/beta) log fs, fs^2 = sum dxi^2 / m / (2 pi beta):
// (-1/beta) / (2 pi beta fs^2) * sum_j d2xi(j, i) dxi(j) / m(j).  Returns xi.
inline double umbrella_bias(const StepConfig& cf, const XiDef& xd, double xi0, double kforce, const double* q,
                            double* f) {
  const int N = cf.natoms, P = cf.nbeads, n3 = 3 * N;
  std::vector<double> c(n3), dxi(n3), d2xi((size_t)n3 * n3);
  centroid(N, P, q, c.data());
  const double xi = calc_xi_mode1(xd, N, c.data(), cf.mass, dxi.data(), d2xi.data());
  const double delta = xi - xi0;
  for (int k = 0; k < P; ++k)
    for (int i = 0; i < n3; ++i) f[(size_t)k * n3 + i] = f[(size_t)k * n3 + i] + kforce * delta * dxi[i];
  const double pi = 3.1415926535897932384;
  double fs2 = 0.0;
  for (int l = 0; l < 3; ++l)
    for (int m = 0; m < N; ++m) fs2 = fs2 + dxi[3 * m + l] * dxi[3 * m + l] / cf.mass[m];
  const double coeff1 = 2.0 * pi * cf.beta;
  fs2 = fs2 / coeff1;
  const double coeff2 = -1.0 / cf.beta;
  for (int l = 0; l < 3; ++l)
    for (int m = 0; m < N; ++m) {
      double dh = 0.0;
      for (int l2 = 0; l2 < 3; ++l2)
        for (int m2 = 0; m2 < N; ++m2)
          dh = dh + d2xi[(size_t)(3 * m2 + l2) * n3 + 3 * m + l] * dxi[3 * m2 + l2] / cf.mass[m2];
      dh = dh * coeff2 / (coeff1 * fs2);
      for (int k = 0; k < P; ++k) f[(size_t)k * n3 + 3 * m + l] = f[(size_t)k * n3 + 3 * m + l] + dh;
    }
  return xi;
}

}  // namespace orc
