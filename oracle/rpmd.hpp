// ORACLE (test infrastructure only) -- one RPMD velocity-Verlet step.
//
// CPU restatement of Caracal's `verlet` (src/verlet.f90:65-1308) for the
// gas-phase, non-periodic configurations of the engine:
//   1/2 kick                       src/verlet.f90:216-218
//   free ring polymer (P>1)        src/verlet.f90:377-463 (rfft -> poly -> irfft)
//   plain drift (P=1)              src/verlet.f90:350-356
//   per-bead forces                src/verlet.f90:772-777
//   1/2 kick                       src/verlet.f90:1060-1062
//   Andersen every andersen_step   src/verlet.f90:1159-1165, src/andersen.f90:37-71
//   Nose-Hoover chain              src/verlet.f90:186-208 and 1085-1106, src/nhc.f90
//   kinetic energy / temperature   src/verlet.f90:1174-1188
//   NaN / Inf stop                 src/verlet.f90:1256-1275
//   transrot (constrain <= 0)      src/verlet.f90:1300-1306, src/transrot.f90:36-237
// plus the PILE thermostat (Ceriotti, Parrinello, Markland, Manolopoulos,
// J. Chem. Phys. 133, 124104 (2010)), which Caracal does not have; it sits
// where Caracal's Nose-Hoover half chains sit (src/verlet.f90:189-209 and
// 1090-1107).
//
// The "normal-mode" transform is Caracal's, not an orthogonal one: rfft and
// irfft (src/rfft.f90:36-62, src/irfft.f90:36-64) both keep sqrt(1/P) times
// the real part of FFTW's forward DFT, i.e. x_k <- sqrt(1/P) sum_j x_j
// cos(2 pi j k / P).  Here that DFT is a direct sum (FFTW itself is not in
// the reference tree; its result is the DFT to rounding).
//
// Memory layout: per trajectory q[(k*N + i)*3 + d] -- exactly Fortran's
// q_i(3, natoms, nbeads) column-major flattening.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "philox.hpp"

namespace orc {

struct StepConfig {
  int natoms = 0;
  int nbeads = 1;
  double dt = 0.0;        // a.u.
  double beta = 0.0;      // 1/(k_B T), a.u.; +inf allowed only for nbeads == 1
  int thermostat = 0;     // 0 none, 1 Andersen, 2 Nose-Hoover chain, 3 PILE
  int andersen_step = 70;
  double pile_tau0 = 0.0; // a.u. (centroid friction 1/tau0)
  double nose_q = 0.0;    // a.u. (NOSE_Q time steps x dt, src/dynamic.f90:578)
  int transrot = 1;       // 1: remove COM translation/rotation (constrain <= 0)
  uint32_t seed = 0;
  const double* mass = nullptr;  // natoms, a.u.
  int nm_mode = 0;        // 0: Caracal's cosine transform; 1: orthonormal real normal modes
};

constexpr double kPi = 3.1415926535897932384626433832795029;
constexpr double kBoltzmannAu = 0.316679e-5;   // src/dynamic.f90:79
constexpr double kBohrAngstrom = 0.52917721092; // src/general.f90:256
constexpr double kElectronMassAmu = 5.485799095e-4; // src/general.f90:252

// fs -> a.u.; the divisor is the REAL(4) literal 2.41888428E-2 (src/dynamic.f90:589)
inline double dt_fs_to_au(double dt_fs) { return dt_fs / (double)2.41888428E-2f; }

// Caracal's rfft/irfft: x <- sqrt(1/P) Re(DFT_forward(x)).
inline void caracal_cos_transform(double* x, int P) {
  std::vector<double> y(P, 0.0);
  const double factor = std::sqrt(1.0 / P);
  for (int k = 0; k < P; ++k) {
    double s = 0.0;
    for (int j = 0; j < P; ++j) {
      int m = (int)(((long long)j * k) % P);
      s += x[j] * std::cos(2.0 * kPi * m / P);
    }
    y[k] = factor * s;
  }
  for (int k = 0; k < P; ++k) x[k] = y[k];
}

// Orthonormal real normal modes (the RPMD transform Caracal's rfft/irfft are
// meant to be; not the reference's code path -- an engine option for runs
// that compare with results of a correct transform): forward y = O x with
// O[0][j] = 1/sqrt(P), O[k][j] = sqrt(2/P) cos(2 pi j k/P) for 0 < k < P/2,
// O[P/2][j] = (-1)^j/sqrt(P), O[k][j] = sqrt(2/P) sin(2 pi j k/P) for k > P/2;
// inverse x = O^T y.  Mode k and P - k share the frequency of poly.
inline double nm_matrix(int P, int k, int j) {
  const long long m = ((long long)j * k) % P;
  const double a = 2.0 * kPi * (double)m / P;
  if (k == 0) return std::sqrt(1.0 / P);
  if (2 * k == P) return (j % 2 ? -1.0 : 1.0) * std::sqrt(1.0 / P);
  if (2 * k < P) return std::sqrt(2.0 / P) * std::cos(a);
  return std::sqrt(2.0 / P) * std::sin(a);
}
inline void nm_forward(double* x, int P) {
  std::vector<double> y(P, 0.0);
  for (int k = 0; k < P; ++k) {
    double s = 0.0;
    for (int j = 0; j < P; ++j) s += nm_matrix(P, k, j) * x[j];
    y[k] = s;
  }
  for (int k = 0; k < P; ++k) x[k] = y[k];
}
inline void nm_inverse(double* x, int P) {
  std::vector<double> y(P, 0.0);
  for (int j = 0; j < P; ++j) {
    double s = 0.0;
    for (int k = 0; k < P; ++k) s += nm_matrix(P, k, j) * x[k];
    y[j] = s;
  }
  for (int j = 0; j < P; ++j) x[j] = y[j];
}

// poly(1:4,k) of src/verlet.f90:405-429 for one atom of mass m.
inline void free_rp_poly(int P, double beta, double dt, double m, double* poly /*4*P*/) {
  poly[0] = 1.0;
  poly[1] = 0.0;
  poly[2] = dt / m;
  poly[3] = 1.0;
  if (P > 1) {
    double beta_n = beta / P;
    double twown = 2.0 / beta_n;
    double pi_n = kPi / P;
    for (int k = 1; k <= P / 2; ++k) {
      double wk = twown * std::sin(k * pi_n);
      double wt = wk * dt;
      double wm = wk * m;
      double c = std::cos(wt), s = std::sin(wt);
      poly[4 * k + 0] = c;
      poly[4 * k + 1] = -wm * s;
      poly[4 * k + 2] = s / wm;
      poly[4 * k + 3] = c;
    }
    for (int k = 1; k <= (P - 1) / 2; ++k)
      for (int c = 0; c < 4; ++c) poly[4 * (P - k) + c] = poly[4 * k + c];
  }
}

// Free ring-polymer propagation of one trajectory (src/verlet.f90:344-463).
inline void free_rp_step(const StepConfig& cf, double* q, double* p) {
  const int N = cf.natoms, P = cf.nbeads;
  if (P == 1) {
    for (int d = 0; d < 3; ++d)
      for (int i = 0; i < N; ++i) q[3 * i + d] = q[3 * i + d] + p[3 * i + d] * cf.dt / cf.mass[i];
    return;
  }
  std::vector<double> vp(P), vq(P), poly(4 * P);
  for (int i = 0; i < N; ++i) {
    free_rp_poly(P, cf.beta, cf.dt, cf.mass[i], poly.data());
    for (int d = 0; d < 3; ++d) {
      // q enters relative to its bead-0 value: a constant vector is the
      // centroid mode, which poly keeps in q and leaves out of p
      // (poly(2,0) = 0, poly(4,0) = 1), so the map is unchanged while the
      // transforms round on bead spreads instead of absolute positions
      // (otherwise ~1e-12 of |p| for heavy atoms at P = 64, dt = 0.5 fs)
      const double shift = q[(0 * N + i) * 3 + d];
      for (int k = 0; k < P; ++k) {
        vp[k] = p[(k * N + i) * 3 + d];
        vq[k] = q[(k * N + i) * 3 + d] - shift;
      }
      if (cf.nm_mode == 1) {
        nm_forward(vp.data(), P);
        nm_forward(vq.data(), P);
      } else {
        caracal_cos_transform(vp.data(), P);
        caracal_cos_transform(vq.data(), P);
      }
      for (int k = 0; k < P; ++k) {
        double pn = vp[k] * poly[4 * k + 0] + vq[k] * poly[4 * k + 1];
        vq[k] = vp[k] * poly[4 * k + 2] + vq[k] * poly[4 * k + 3];
        vp[k] = pn;
      }
      if (cf.nm_mode == 1) {
        nm_inverse(vp.data(), P);
        nm_inverse(vq.data(), P);
      } else {
        caracal_cos_transform(vp.data(), P);
        caracal_cos_transform(vq.data(), P);
      }
      for (int k = 0; k < P; ++k) {
        p[(k * N + i) * 3 + d] = vp[k];
        q[(k * N + i) * 3 + d] = vq[k] + shift;
      }
    }
  }
}

// Andersen full resample (src/andersen.f90:37-71): p = N(0,1) * sqrt(m P / beta).
inline void andersen(const StepConfig& cf, uint32_t traj, uint32_t step, uint32_t tag, double* p) {
  const int N = cf.natoms, P = cf.nbeads;
  double beta_n = cf.beta / P;
  std::vector<double> z(3 * N);
  for (int k = 0; k < P; ++k) {
    normals_bead(cf.seed, traj, (uint32_t)k, step, tag, 3 * N, z.data());
    for (int i = 0; i < N; ++i) {
      double dp = std::sqrt(cf.mass[i] / beta_n);
      for (int d = 0; d < 3; ++d) p[(k * N + i) * 3 + d] = z[3 * i + d] * dp;
    }
  }
}

// Orthonormal real normal-mode matrix O (rows = modes) used by PILE.
inline void pile_modes(int P, std::vector<double>& O, std::vector<double>& freq_index) {
  O.assign((size_t)P * P, 0.0);
  freq_index.assign(P, 0.0);
  for (int k = 0; k < P; ++k) {
    for (int j = 0; j < P; ++j) {
      int m = (int)(((long long)j * k) % P);
      double ang = 2.0 * kPi * m / P;
      double v;
      if (k == 0) v = std::sqrt(1.0 / P);
      else if (2 * k < P) v = std::sqrt(2.0 / P) * std::cos(ang);
      else if (2 * k == P) v = (j % 2 == 0 ? 1.0 : -1.0) * std::sqrt(1.0 / P);
      else v = std::sqrt(2.0 / P) * std::sin(ang);
      O[(size_t)k * P + j] = v;
    }
    freq_index[k] = (2 * k <= P) ? k : P - k;
  }
}

// PILE-L half step (Ceriotti et al. 2010, eqs. 27-28 with lambda = 1/2):
// modes p~ = O p; p~_k <- c1_k p~_k + sqrt(m P/beta) c2_k xi_k, xi = O eta with
// eta the per-bead Gaussian stream; p = O^T p~.
inline void pile_half(const StepConfig& cf, uint32_t traj, uint32_t step, uint32_t tag, double* p) {
  const int N = cf.natoms, P = cf.nbeads;
  std::vector<double> O, fk;
  pile_modes(P, O, fk);
  std::vector<double> c1(P), c2(P);
  double twown = 2.0 * P / cf.beta;
  for (int k = 0; k < P; ++k) {
    double gamma = (k == 0) ? 1.0 / cf.pile_tau0 : 2.0 * twown * std::sin(fk[k] * kPi / P);
    c1[k] = std::exp(-0.5 * cf.dt * gamma);
    c2[k] = std::sqrt(1.0 - c1[k] * c1[k]);
  }
  std::vector<double> eta((size_t)P * 3 * N);
  for (int k = 0; k < P; ++k)
    normals_bead(cf.seed, traj, (uint32_t)k, step, tag, 3 * N, &eta[(size_t)k * 3 * N]);
  std::vector<double> pm(P), xm(P);
  for (int i = 0; i < N; ++i) {
    double s = std::sqrt(cf.mass[i] * P / cf.beta);
    for (int d = 0; d < 3; ++d) {
      for (int k = 0; k < P; ++k) {
        double a = 0.0, b = 0.0;
        for (int j = 0; j < P; ++j) {
          a += O[(size_t)k * P + j] * p[(j * N + i) * 3 + d];
          b += O[(size_t)k * P + j] * eta[(size_t)j * 3 * N + 3 * i + d];
        }
        pm[k] = c1[k] * a + s * c2[k] * b;
      }
      for (int j = 0; j < P; ++j) {
        double a = 0.0;
        for (int k = 0; k < P; ++k) a += O[(size_t)k * P + j] * pm[k];
        p[(j * N + i) * 3 + d] = a;
      }
    }
  }
}

// Gauss-Jordan inverse with full pivoting (src/invert.f90:38-124); returns 0
// on success, 1 for a singular matrix (Caracal calls fatal there).
inline int invert3(double a[3][3]) {
  const int n = 3;
  int ipiv[3] = {0, 0, 0}, indxr[3], indxc[3];
  for (int i = 0; i < n; ++i) {
    double big = 0.0;
    int irow = 0, icol = 0;
    for (int j = 0; j < n; ++j) {
      if (ipiv[j] != 1) {
        for (int k = 0; k < n; ++k) {
          if (ipiv[k] == 0) {
            if (std::fabs(a[j][k]) >= big) {
              big = std::fabs(a[j][k]);
              irow = j;
              icol = k;
            }
          } else if (ipiv[k] > 1) {
            return 1;
          }
        }
      }
    }
    ipiv[icol] += 1;
    if (irow != icol)
      for (int j = 0; j < n; ++j) std::swap(a[irow][j], a[icol][j]);
    indxr[i] = irow;
    indxc[i] = icol;
    if (a[icol][icol] == 0.0) return 1;
    double pivot = a[icol][icol];
    a[icol][icol] = 1.0;
    for (int j = 0; j < n; ++j) a[icol][j] = a[icol][j] / pivot;
    for (int j = 0; j < n; ++j) {
      if (j != icol) {
        double t = a[j][icol];
        a[j][icol] = 0.0;
        for (int k = 0; k < n; ++k) a[j][k] = a[j][k] - a[icol][k] * t;
      }
    }
  }
  for (int i = n - 1; i >= 0; --i)
    if (indxr[i] != indxc[i])
      for (int k = 0; k < n; ++k) std::swap(a[k][indxr[i]], a[k][indxc[i]]);
  return 0;
}

// transrot (src/transrot.f90:36-237), including its quirk: the accumulated
// total mass already sums over beads and is multiplied by nbeads once more,
// so both the removed COM velocity and the rotation centre carry 1/P.
inline int transrot(const StepConfig& cf, const double* q, double* p) {
  const int N = cf.natoms, P = cf.nbeads;
  std::vector<double> vel((size_t)3 * N * P);
  for (int k = 0; k < P; ++k)
    for (int i = 0; i < N; ++i)
      for (int d = 0; d < 3; ++d) vel[(k * N + i) * 3 + d] = p[(k * N + i) * 3 + d] / cf.mass[i];
  double totmass = 0.0, vtot[3] = {0, 0, 0};
  for (int i = 0; i < N; ++i) {
    double w = cf.mass[i];
    for (int k = 0; k < P; ++k) {
      totmass = totmass + w;
      for (int d = 0; d < 3; ++d) vtot[d] = vtot[d] + vel[(k * N + i) * 3 + d] * w;
    }
  }
  totmass = totmass * P;
  for (int d = 0; d < 3; ++d) vtot[d] = vtot[d] / totmass;
  double xt = 0, yt = 0, zt = 0;
  for (int i = 0; i < N; ++i) {
    double w = cf.mass[i];
    for (int k = 0; k < P; ++k) {
      xt = xt + q[(k * N + i) * 3 + 0] * w;
      yt = yt + q[(k * N + i) * 3 + 1] * w;
      zt = zt + q[(k * N + i) * 3 + 2] * w;
    }
  }
  xt = xt / totmass;
  yt = yt / totmass;
  zt = zt / totmass;
  double mang[3] = {0, 0, 0};
  for (int i = 0; i < N; ++i) {
    double w = cf.mass[i];
    for (int k = 0; k < P; ++k) {
      const double* qq = &q[(k * N + i) * 3];
      const double* vv = &vel[(k * N + i) * 3];
      mang[0] = mang[0] + (qq[1] * vv[2] - qq[2] * vv[1]) * w;
      mang[1] = mang[1] + (qq[2] * vv[0] - qq[0] * vv[2]) * w;
      mang[2] = mang[2] + (qq[0] * vv[1] - qq[1] * vv[0]) * w;
    }
  }
  mang[0] = mang[0] - (yt * vtot[2] - zt * vtot[1]) * totmass;
  mang[1] = mang[1] - (zt * vtot[0] - xt * vtot[2]) * totmass;
  mang[2] = mang[2] - (xt * vtot[1] - yt * vtot[0]) * totmass;
  double xx = 0, xy = 0, xz = 0, yy = 0, yz = 0, zz = 0;
  for (int i = 0; i < N; ++i) {
    double w = cf.mass[i];
    for (int k = 0; k < P; ++k) {
      double xd = q[(k * N + i) * 3 + 0] - xt;
      double yd = q[(k * N + i) * 3 + 1] - yt;
      double zd = q[(k * N + i) * 3 + 2] - zt;
      xx = xx + xd * xd * w;
      xy = xy + xd * yd * w;
      xz = xz + xd * zd * w;
      yy = yy + yd * yd * w;
      yz = yz + yd * zd * w;
      zz = zz + zd * zd * w;
    }
  }
  double t[3][3] = {{yy + zz, -xy, -xz}, {-xy, xx + zz, -yz}, {-xz, -yz, xx + yy}};
  if (N <= 2) {
    t[0][0] += 0.000001;
    t[1][1] += 0.000001;
    t[2][2] += 0.000001;
  }
  if (invert3(t)) return 1;
  double vang[3];
  for (int a = 0; a < 3; ++a) {
    vang[a] = 0.0;
    for (int b = 0; b < 3; ++b) vang[a] = vang[a] + t[a][b] * mang[b];
  }
  for (int k = 0; k < P; ++k)
    for (int i = 0; i < N; ++i) {
      double* vv = &vel[(k * N + i) * 3];
      for (int d = 0; d < 3; ++d) vv[d] = vv[d] - vtot[d];
    }
  for (int i = 0; i < N; ++i)
    for (int k = 0; k < P; ++k) {
      double xd = q[(k * N + i) * 3 + 0] - xt;
      double yd = q[(k * N + i) * 3 + 1] - yt;
      double zd = q[(k * N + i) * 3 + 2] - zt;
      double* vv = &vel[(k * N + i) * 3];
      vv[0] = vv[0] - vang[1] * zd + vang[2] * yd;
      vv[1] = vv[1] - vang[2] * xd + vang[0] * zd;
      vv[2] = vv[2] - vang[0] * yd + vang[1] * xd;
    }
  for (int k = 0; k < P; ++k)
    for (int i = 0; i < N; ++i)
      for (int d = 0; d < 3; ++d) p[(k * N + i) * 3 + d] = vel[(k * N + i) * 3 + d] * cf.mass[i];
  return 0;
}

inline double kinetic_energy(const StepConfig& cf, const double* p) {
  double e = 0.0;
  for (int i = 0; i < cf.natoms; ++i)
    for (int k = 0; k < cf.nbeads; ++k) {
      const double* pp = &p[(k * cf.natoms + i) * 3];
      e = e + (pp[0] * pp[0] + pp[1] * pp[1] + pp[2] * pp[2]) / (2.0 * cf.mass[i]);
    }
  return e;
}

// Nose-Hoover chain (src/nhc.f90:35-171): 4 links, nc = 5 Suzuki-Yoshida
// passes of ns = 3 weights, one global scale of every momentum.  The chain
// masses come from mdinit (src/mdinit.f90:128-147): Q = k_B T nose_q^2 with
// k_B = 0.316679D-5, Q_1 = 3N Q.  nhc's own kT is 1.380649E-23/4.3597447E-18
// * kelvin, a REAL(4) quotient, kelvin = 1/(beta k_B).  vnh[4] is the chain
// velocity state of one trajectory (zero at mdinit).
inline void nhc_half(const StepConfig& cf, double* vnh, double* p) {
  const int N = cf.natoms, P = cf.nbeads;
  const double kelvin = 1.0 / (cf.beta * kBoltzmannAu);
  const double ekt_md = kBoltzmannAu * kelvin;
  const double qterm = ekt_md * cf.nose_q * cf.nose_q;
  const int nfree = 3 * N;
  double qnh[4] = {(double)nfree * qterm, qterm, qterm, qterm};
  double gnh[4] = {0.0, 0.0, 0.0, 0.0};
  const double ekt = (double)(1.380649E-23f / 4.3597447E-18f) * kelvin;
  const int nc = 5, ns = 3;
  const double dtc = cf.dt / (double)nc;
  double w[3];
  w[0] = 1.0 / (2.0 - std::pow(2.0, 1.0 / 3.0));
  w[1] = 1.0 - 2.0 * w[0];
  w[2] = w[0];
  double scale = 1.0;
  double eksum = 0.0;
  for (int i = 0; i < N; ++i)
    for (int k = 0; k < P; ++k) {
      const double* pp = &p[(k * N + i) * 3];
      eksum = eksum + (pp[0] * pp[0] + pp[1] * pp[1] + pp[2] * pp[2]) / (2.0 * cf.mass[i]) / P / P;
    }
  for (int ic = 0; ic < nc; ++ic)
    for (int j = 0; j < ns; ++j) {
      const double dts = w[j] * dtc;
      const double dt2 = 0.5 * dts, dt4 = 0.25 * dts, dt8 = 0.125 * dts;
      double ex;
      gnh[3] = (qnh[2] * vnh[2] * vnh[2] - ekt) / qnh[3];
      vnh[3] = vnh[3] + gnh[3] * dt4;
      gnh[2] = (qnh[1] * vnh[1] * vnh[1] - ekt) / qnh[2];
      ex = std::exp(-vnh[3] * dt8);
      vnh[2] = ex * (vnh[2] * ex + gnh[2] * dt4);
      gnh[1] = (qnh[0] * vnh[0] * vnh[0] - ekt) / qnh[1];
      ex = std::exp(-vnh[2] * dt8);
      vnh[1] = ex * (vnh[1] * ex + gnh[1] * dt4);
      gnh[0] = (2.0 * eksum - (double)nfree * ekt) / qnh[0];
      ex = std::exp(-vnh[1] * dt8);
      vnh[0] = ex * (vnh[0] * ex + gnh[0] * dt4);
      ex = std::exp(-vnh[0] * dt2);
      scale = scale * ex;
      eksum = eksum * ex * ex;
      gnh[0] = (2.0 * eksum - (double)nfree * ekt) / qnh[0];
      ex = std::exp(-vnh[1] * dt8);
      vnh[0] = ex * (vnh[0] * ex + gnh[0] * dt4);
      gnh[1] = (qnh[0] * vnh[0] * vnh[0] - ekt) / qnh[1];
      ex = std::exp(-vnh[2] * dt8);
      vnh[1] = ex * (vnh[1] * ex + gnh[1] * dt4);
      gnh[2] = (qnh[1] * vnh[1] * vnh[1] - ekt) / qnh[2];
      ex = std::exp(-vnh[3] * dt8);
      vnh[2] = ex * (vnh[2] * ex + gnh[2] * dt4);
      gnh[3] = (qnh[2] * vnh[2] * vnh[2] - ekt) / qnh[3];
      vnh[3] = vnh[3] + gnh[3] * dt4;
    }
  for (int x = 0; x < 3 * N * P; ++x) p[x] = scale * p[x];
}

// Trajectory status bits (shared meaning with the engine).
enum TrajStatus : int { TRAJ_OK = 0, TRAJ_NONFINITE = 1, TRAJ_SINGULAR_INERTIA = 2 };

// One verlet step of one trajectory.  `egrad(q_bead, &V, g_bead)` evaluates a
// bead; f holds dV/dq of the previous step on entry and of this step on exit.
struct NoBias {
  void operator()(const double*, double*) const {}
};

template <class EGrad>
inline int verlet_step(const StepConfig& cf, uint32_t traj, int istep, double* q, double* p,
                       double* f, double* epot, EGrad egrad, double* vnh = nullptr) {
  return verlet_step(cf, traj, istep, q, p, f, epot, egrad, vnh, NoBias());
}

// The same step with a bias added to the bead gradients after the forces
// (umbrella sampling: src/verlet.f90:1043-1046, umbrella mode 0).
template <class EGrad, class Bias>
inline int verlet_step(const StepConfig& cf, uint32_t traj, int istep, double* q, double* p,
                       double* f, double* epot, EGrad egrad, double* vnh, Bias bias) {
  const int N = cf.natoms, P = cf.nbeads, n3 = 3 * N;
  const size_t nall = (size_t)n3 * P;
  if (cf.thermostat == 2) nhc_half(cf, vnh, p);  // src/verlet.f90:186-208
  if (cf.thermostat == 3) pile_half(cf, traj, (uint32_t)istep, TAG_PILE_A, p);
  for (size_t x = 0; x < nall; ++x) p[x] = p[x] - 0.5 * cf.dt * f[x];
  free_rp_step(cf, q, p);
  double e = 0.0;
  for (int k = 0; k < P; ++k) {
    double v;
    egrad(&q[(size_t)k * n3], &v, &f[(size_t)k * n3]);
    e = e + v;
  }
  *epot = e;
  bias(q, f);
  for (size_t x = 0; x < nall; ++x) p[x] = p[x] - 0.5 * cf.dt * f[x];
  if (cf.thermostat == 2) nhc_half(cf, vnh, p);  // src/verlet.f90:1085-1106
  if (cf.thermostat == 1 && istep % cf.andersen_step == 0)
    andersen(cf, traj, (uint32_t)istep, TAG_ANDERSEN, p);
  if (cf.thermostat == 3) pile_half(cf, traj, (uint32_t)istep, TAG_PILE_B, p);
  int status = TRAJ_OK;
  for (size_t x = 0; x < nall; ++x)
    if (!std::isfinite(q[x])) status |= TRAJ_NONFINITE;
  if (cf.transrot && transrot(cf, q, p)) status |= TRAJ_SINGULAR_INERTIA;
  return status;
}

// NpT with the Berendsen barostat (src/verlet.f90, barostat 1): the box
// (3 edges, bohr) scales with the coordinates after each step.
struct NptConfig {
  double pressure = 0.0;  // target, a.u. (PRES / prescon, src/dynamic.f90:1331-1335)
  double compress = 0.0;  // mdinit: 0.000046 prescon / 1000 (src/mdinit.f90:155-158)
  double taupres = 0.0;   // mdinit: 2.0
};

// One NpT step: verlet_step's order with the virial trace reset at the start
// (src/verlet.f90:164-167) and accumulated by `egrad` into *vir over the
// beads; NHC is not applied (under the Berendsen barostat the reference
// calls neither nhc nor nhc_npt, src/verlet.f90:189-208, 1088-1106); after the
// second half kick the pressure from the virial alone (the kinetic stress
// tensor is accumulated by multiplication from zero and stays zero,
// src/verlet.f90:1111-1132) and the Berendsen scaling of box and coordinates
// (src/verlet.f90:1138-1151), then Andersen, the NaN check and transrot.
template <class EGrad>
inline int verlet_step_npt(const StepConfig& cf, const NptConfig& np, uint32_t traj, int istep, double* q,
                           double* p, double* f, double* epot, EGrad egrad, double* box, double* press,
                           double* vir) {
  const int N = cf.natoms, P = cf.nbeads, n3 = 3 * N;
  const size_t nall = (size_t)n3 * P;
  const double volbox = box[0] * box[1] * box[2];
  *vir = 0.0;
  if (cf.thermostat == 3) pile_half(cf, traj, (uint32_t)istep, TAG_PILE_A, p);
  for (size_t x = 0; x < nall; ++x) p[x] = p[x] - 0.5 * cf.dt * f[x];
  free_rp_step(cf, q, p);
  double e = 0.0;
  for (int k = 0; k < P; ++k) {
    double v;
    egrad(&q[(size_t)k * n3], &v, &f[(size_t)k * n3]);
    e = e + v;
  }
  *epot = e;
  for (size_t x = 0; x < nall; ++x) p[x] = p[x] - 0.5 * cf.dt * f[x];
  const double factor = 1.0 / volbox;
  *press = (factor * (0.0 - *vir)) / 3.0;
  const double scale = std::pow(1.0 + (cf.dt * np.compress / np.taupres) * (*press - np.pressure), 1.0 / 3.0);
  for (int k = 0; k < 3; ++k) box[k] = box[k] * scale;
  for (size_t x = 0; x < nall; ++x) q[x] = q[x] * scale;
  if (cf.thermostat == 1 && istep % cf.andersen_step == 0)
    andersen(cf, traj, (uint32_t)istep, TAG_ANDERSEN, p);
  if (cf.thermostat == 3) pile_half(cf, traj, (uint32_t)istep, TAG_PILE_B, p);
  int status = TRAJ_OK;
  for (size_t x = 0; x < nall; ++x)
    if (!std::isfinite(q[x])) status |= TRAJ_NONFINITE;
  if (cf.transrot && transrot(cf, q, p)) status |= TRAJ_SINGULAR_INERTIA;
  return status;
}

}  // namespace orc
