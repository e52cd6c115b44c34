// Caracal's ANA_BRH2 surface (src/egrad_brh2.f, the BrH2 DIM-3C surface of
// POTLIB: D. C. Clary, Chem. Phys. 71, 117 (1982); I. Last and M. Baer) on
// the device, one thread per bead.  Atoms H, Br, H; R(1) = r(1,2),
// R(2) = r(1,3), R(3) = r(2,3) (egrad_brh2 :33-78); POT_brh2 (:160-420):
// the 4x4 diatomics-in-molecules Hamiltonian of the H2 and HBr curves
// (VHX :421-447), its lowest root with the Hellmann-Feynman derivatives
// u^T dH/dR u (EISPACK RSP in the reference; cyclic Jacobi rotations here,
// unrolled over the 4x4 matrix in registers, at most 50 sweeps), and the
// three-centre term; constants of BLOCK DATA PTPARM (:448-465) after
// initialize_brh2.  The surface is a few hundred FP64 operations per bead
// and its eigenvector projections cancel, so both precision forms evaluate
// it in FP64.
#pragma once
#include <cuda_runtime.h>

namespace cr {
namespace brh2 {

struct K {
  static constexpr double eps = 1.0e-6, one = 1.0;
  static constexpr double rhh = 1.4016, ahh = 1.0291, dhh = 0.17447, bhh = 0.018;
  static constexpr double xih = 1.0, xix = 1.6, g0 = 0.22, alfw = 1.0;
  static constexpr double rhx = 2.673, ahx = 0.957, dhx = 0.1439, bhx = 0.012;
  static constexpr double etahh = 0.393764, eta3s = 0.322, eta1p = 0.20286, eta3p = 0.1771;
};

struct Setup {
  double xib, denom, g, rt34, rt38, c3;
};
__device__ inline Setup setup() {
  Setup s;
  s.xib = 0.5 * (K::xih + K::xix);
  const double t = s.xib * K::rhx;
  s.c3 = 1.0 / 3.0;
  s.denom = 2.0 * K::rhx * (1.0 + t * (1.0 + s.c3 * t)) * exp(-t);
  s.g = K::g0 / K::rhx;
  s.rt34 = 0.25 * sqrt(3.0);
  s.rt38 = 0.5 * s.rt34;
  return s;
}

// VHX: the HBr singlet-sigma curve and the scaled anti-Morse forms.
__device__ inline void vhx(double r, double* v, double* dv) {
  const double rdif = r - K::rhx, rdif2 = rdif * rdif;
  const double ex1 = exp(-K::ahx * rdif), ex2 = exp(-K::bhx * rdif2 * rdif);
  double t1 = K::dhx * ex1 * ex2;
  const double v1s = t1 * (ex1 - 2.0), v1 = t1 * (ex1 + 2.0);
  t1 = 2.0 * K::ahx * t1;
  const double t2 = 3.0 * K::bhx * rdif2;
  const double dv1s = t1 * (1.0 - ex1) - t2 * v1s, dv1 = -t1 * (1.0 + ex1) - t2 * v1;
  v[0] = v1s;               // V1S
  v[1] = K::eta3s * v1;     // V3S
  v[2] = K::eta1p * v1;     // V1P
  v[3] = K::eta3p * v1;     // V3P
  dv[0] = dv1s;
  dv[1] = K::eta3s * dv1;
  dv[2] = K::eta1p * dv1;
  dv[3] = K::eta3p * dv1;
}

// Lowest eigenvalue and its unit eigenvector of the symmetric 4x4 matrix a
// (packed row-wise lower triangle, as RSP takes it) by cyclic Jacobi
// rotations (at most 50 sweeps).
__device__ inline double lowest_root(const double* hp, double* u) {
  double a[4][4], v[4][4];
  int idx = 0;
  for (int l = 0; l < 4; ++l)
    for (int k = 0; k <= l; ++k) {
      a[l][k] = a[k][l] = hp[idx++];
    }
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) v[i][j] = (i == j) ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 50; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) {
        tot += a[i][j] * a[i][j];
        if (i != j) off += a[i][j] * a[i][j];
      }
    if (off <= 1e-32 * tot) break;
#pragma unroll
    for (int p = 0; p < 3; ++p)
#pragma unroll
      for (int q = p + 1; q < 4; ++q) {
        if (a[p][q] == 0.0) continue;
        const double theta = (a[q][q] - a[p][p]) / (2.0 * a[p][q]);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
#pragma unroll
        for (int k = 0; k < 4; ++k) {  // columns p, q
          const double akp = a[k][p], akq = a[k][q];
          a[k][p] = c * akp - s * akq;
          a[k][q] = s * akp + c * akq;
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {  // rows p, q
          const double apk = a[p][k], aqk = a[q][k];
          a[p][k] = c * apk - s * aqk;
          a[q][k] = s * apk + c * aqk;
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const double vkp = v[k][p], vkq = v[k][q];
          v[k][p] = c * vkp - s * vkq;
          v[k][q] = s * vkp + c * vkq;
        }
      }
  }
  int m = 0;
  for (int i = 1; i < 4; ++i)
    if (a[i][i] < a[m][m]) m = i;
  for (int k = 0; k < 4; ++k) u[k] = v[k][m];
  return a[m][m];
}

// POT_brh2: R(3) -> energy and dE/dR(3).
__device__ inline double pot(const double* R, double* dedr) {
  const Setup S = setup();
  double r1 = R[0], r2 = R[2], r3 = R[1];
  if (r1 > r2 + r3) r1 = r2 + r3;
  if (r2 > r1 + r3) r2 = r1 + r3;
  if (r3 > r1 + r2) r3 = r1 + r2;
  const double r1s = r1 * r1, r2s = r2 * r2, r3s = r3 * r3;
  const double r12 = r1 * r2, r13 = r1 * r3, r23 = r2 * r3;
  const double t3 = (r1s + r2s - r3s) * 0.5, t2 = (r1s + r3s - r2s) * 0.5, t1 = (r2s + r3s - r1s) * 0.5;
  double csa = t2 / r13;
  if (fabs(csa) > K::one) csa = copysign(K::one, csa);
  const double csa2 = csa * csa, sna2 = 1.0 - csa2;
  const bool lcol = sna2 < K::eps;
  const double sna = sqrt(sna2);
  double t22 = 2.0 * csa, t11 = 0.0;
  if (!lcol) t11 = 2.0 * (sna2 - csa2) / sna;
  const double sn2a = t22 * sna;
  double t = t3 / (r1 * r13);
  const double dcsa21 = t22 * t, dsn2a1 = t11 * t;
  t = -r2 / r13;
  const double dcsa22 = t22 * t, dsn2a2 = t11 * t;
  t = t1 / (r13 * r3);
  const double dcsa23 = t22 * t, dsn2a3 = t11 * t;
  double csb = t1 / r23;
  if (fabs(csb) > K::one) csb = copysign(K::one, csb);
  const double csb2 = csb * csb, snb2 = 1.0 - csb2, snb = sqrt(snb2);
  t11 = 0.0;
  if (!lcol) t11 = 2.0 * (snb2 - csb2) / snb;
  t22 = 2.0 * csb;
  const double sn2b = t22 * snb;
  t = -r1 / r23;
  const double dcsb21 = t22 * t, dsn2b1 = t11 * t;
  t = t3 / (r2 * r23);
  const double dcsb22 = t22 * t, dsn2b2 = t11 * t;
  t = t2 / (r23 * r3);
  const double dcsb23 = t22 * t, dsn2b3 = t11 * t;
  t = t3 / r12;
  const double csg2 = t * t;
  t = 2.0 * t;
  const double dcsg21 = t * t2 / (r1 * r12), dcsg22 = t * t1 / (r12 * r2), dcsg23 = -t * r3 / r12;

  // H2 curves
  double rdif = r3 - K::rhh;
  double ex1 = exp(-K::ahh * rdif);
  const double rdif2 = rdif * rdif;
  const double ex2 = exp(-K::bhh * rdif * rdif2);
  double u1 = K::dhh * ex1 * ex2;
  const double v1hh = u1 * (ex1 - 2.0), v3hh = K::etahh * u1 * (ex1 + 2.0);
  u1 = 2.0 * K::ahh * u1;
  const double u2 = 3.0 * K::bhh * rdif2;
  const double dv1hh = u1 * (1.0 - ex1) - u2 * v1hh, dv3hh = -u1 * K::etahh * (1.0 + ex1) - u2 * v3hh;
  // HBr curves at R1 and R2: V1S, V3S, V1P, V3P
  double a[4], da[4], b[4], db[4];
  vhx(r1, a, da);
  vhx(r2, b, db);
  const double s11 = a[0] + 3.0 * a[1], s12 = b[0] + 3.0 * b[1], s21 = 3.0 * a[0] + a[1], s22 = 3.0 * b[0] + b[1];
  const double s31 = a[0] - a[1], s32 = b[0] - b[1];
  const double p11 = a[2] + 3.0 * a[3], p12 = b[2] + 3.0 * b[3], p21 = 3.0 * a[2] + a[3], p22 = 3.0 * b[2] + b[3];
  const double p31 = a[2] - a[3], p32 = b[2] - b[3];
  const double ds11 = da[0] + 3.0 * da[1], ds12 = db[0] + 3.0 * db[1], ds21 = 3.0 * da[0] + da[1],
               ds22 = 3.0 * db[0] + db[1], ds31 = da[0] - da[1], ds32 = db[0] - db[1];
  const double dp11 = da[2] + 3.0 * da[3], dp12 = db[2] + 3.0 * db[3], dp21 = 3.0 * da[2] + da[3],
               dp22 = 3.0 * db[2] + db[3], dp31 = da[2] - da[3], dp32 = db[2] - db[3];

  // the Hamiltonian, packed (1-based H(1..10) in h[0..9])
  double h[10];
  h[0] = v1hh + 0.25 * (s11 * csa2 + p11 * sna2 + s12 * csb2 + p12 * snb2);
  h[2] = v1hh + 0.25 * (s11 * sna2 + p11 * csa2 + s12 * snb2 + p12 * csb2);
  h[5] = v3hh + 0.25 * (s21 * csa2 + p21 * sna2 + s22 * csb2 + p22 * snb2);
  h[9] = v3hh + 0.25 * (s21 * sna2 + p21 * csa2 + s22 * snb2 + p22 * csb2);
  const double w11 = s11 - p11, w12 = s12 - p12;
  h[1] = 0.0;
  if (!lcol) h[1] = 0.125 * (w11 * sn2a - w12 * sn2b);
  h[3] = S.rt34 * (s31 * csa2 + p31 * sna2 - s32 * csb2 - p32 * snb2);
  const double w31 = s31 - p31, w32 = s32 - p32;
  h[4] = 0.0;
  if (!lcol) h[4] = S.rt38 * (w31 * sn2a + w32 * sn2b);
  h[6] = h[4];
  h[7] = S.rt34 * (s31 * sna2 + p31 * csa2 - s32 * snb2 - p32 * csb2);
  const double w21 = s21 - p21, w22 = s22 - p22;
  h[8] = 0.0;
  if (!lcol) h[8] = 0.125 * (w21 * sn2a - w22 * sn2b);

  // its derivatives with respect to R1, R2, R3
  double d1[10], d2[10], d3[10];
  t = w11 * dcsa21 + w12 * dcsb21;
  d1[0] = 0.25 * (ds11 * csa2 + dp11 * sna2 + t);
  d1[1] = 0.125 * ((ds11 - dp11) * sn2a + w11 * dsn2a1 - w12 * dsn2b1);
  d1[2] = 0.25 * (ds11 * sna2 + dp11 * csa2 - t);
  t = w11 * dcsa22 + w12 * dcsb22;
  d2[0] = 0.25 * (ds12 * csb2 + dp12 * snb2 + t);
  d2[1] = 0.125 * (-(ds12 - dp12) * sn2b + w11 * dsn2a2 - w12 * dsn2b2);
  d2[2] = 0.25 * (ds12 * snb2 + dp12 * csb2 - t);
  t = 0.25 * (w11 * dcsa23 + w12 * dcsb23);
  d3[0] = dv1hh + t;
  d3[1] = 0.125 * (w11 * dsn2a3 - w12 * dsn2b3);
  d3[2] = dv1hh - t;
  t = w21 * dcsa21 + w22 * dcsb21;
  d1[5] = 0.25 * (ds21 * csa2 + dp21 * sna2 + t);
  d1[8] = 0.125 * ((ds21 - dp21) * sn2a + w21 * dsn2a1 - w22 * dsn2b1);
  d1[9] = 0.25 * (ds21 * sna2 + dp21 * csa2 - t);
  t = w21 * dcsa22 + w22 * dcsb22;
  d2[5] = 0.25 * (ds22 * csb2 + dp22 * snb2 + t);
  d2[8] = 0.125 * ((dp22 - ds22) * sn2b + w21 * dsn2a2 - w22 * dsn2b2);
  d2[9] = 0.25 * (ds22 * snb2 + dp22 * csb2 - t);
  t = 0.25 * (w21 * dcsa23 + w22 * dcsb23);
  d3[5] = dv3hh + t;
  d3[8] = 0.125 * (w21 * dsn2a3 - w22 * dsn2b3);
  d3[9] = dv3hh - t;
  t = w31 * dcsa21 - w32 * dcsb21;
  d1[3] = S.rt34 * (ds31 * csa2 + dp31 * sna2 + t);
  d1[4] = S.rt38 * ((ds31 - dp31) * sn2a + w31 * dsn2a1 + w32 * dsn2b1);
  d1[6] = d1[4];
  d1[7] = S.rt34 * (ds31 * sna2 + dp31 * csa2 - t);
  t = w31 * dcsa22 - w32 * dcsb22;
  d2[3] = S.rt34 * (-ds32 * csb2 - dp32 * snb2 + t);
  d2[4] = S.rt38 * ((ds32 - dp32) * sn2b + w31 * dsn2a2 + w32 * dsn2b2);
  d2[6] = d2[4];
  d2[7] = S.rt34 * (-ds32 * snb2 - dp32 * csb2 - t);
  t = w31 * dcsa23 - w32 * dcsb23;
  d3[3] = S.rt34 * t;
  d3[4] = S.rt38 * (w31 * dsn2a3 + w32 * dsn2b3);
  d3[6] = d3[4];
  d3[7] = -d3[3];

  double u[4];
  const double e1 = lowest_root(h, u);
  double g1 = 0.0, g2 = 0.0, g3 = 0.0;
  for (int l = 0; l < 4; ++l)
    for (int k = 0; k < 4; ++k) {
      const double w = u[l] * u[k];
      const int index = (l >= k) ? l * (l + 1) / 2 + k : k * (k + 1) / 2 + l;
      g1 += w * d1[index];
      g2 += w * d2[index];
      g3 += w * d3[index];
    }

  // three-centre term
  t = K::xih * r3;
  ex1 = exp(-t);
  const double shh = (1.0 + t * (1.0 + S.c3 * t)) * ex1, dshh = -K::xih * t * (1.0 + t) * S.c3 * ex1;
  t = S.xib * r1;
  ex1 = exp(-t);
  const double shx1 = r1 * (1.0 + t * (1.0 + S.c3 * t)) * ex1 / S.denom;
  const double dshx1 = (1.0 + t * (1.0 - S.c3 * t * t)) * ex1 / S.denom;
  t = S.xib * r2;
  ex1 = exp(-t);
  const double shx2 = r2 * (1.0 + t * (1.0 + S.c3 * t)) * ex1 / S.denom;
  const double dshx2 = (1.0 + t * (1.0 - S.c3 * t * t)) * ex1 / S.denom;
  rdif = r1 - r2;
  const double f1 = S.g * exp(-K::alfw * rdif * rdif);
  const double f2 = shh * (shx1 + shx2) + shx1 * shx2;
  const double energy = e1 + f2 * f1 * csg2 + K::dhh;
  const double f3 = 2.0 * K::alfw * rdif * csg2;
  dedr[0] = g1 + (dshx1 * (shh + shx2) * csg2 + f2 * (dcsg21 - f3)) * f1;
  dedr[2] = g2 + (dshx2 * (shh + shx1) * csg2 + f2 * (dcsg22 + f3)) * f1;
  dedr[1] = g3 + (dshh * (shx1 + shx2) * csg2 + f2 * dcsg23) * f1;
  return energy;
}

// egrad_brh2 for one bead: q(3,3) column-major in bohr -> V (Eh), g (Eh/bohr).
__device__ inline void egrad_bead(const double* q, double* V, double* g) {
  double ab[3], ac[3], bc[3];
  for (int d = 0; d < 3; ++d) {
    ab[d] = q[3 + d] - q[d];
    ac[d] = q[d] - q[6 + d];
    bc[d] = q[6 + d] - q[3 + d];
  }
  const double rab = sqrt(ab[0] * ab[0] + ab[1] * ab[1] + ab[2] * ab[2]);
  const double rac = sqrt(ac[0] * ac[0] + ac[1] * ac[1] + ac[2] * ac[2]);
  const double rbc = sqrt(bc[0] * bc[0] + bc[1] * bc[1] + bc[2] * bc[2]);
  const double R[3] = {rab, rac, rbc};
  double dvdr[3];
  *V = pot(R, dvdr);
  for (int d = 0; d < 3; ++d) {
    g[d] = dvdr[1] * ac[d] / rac - dvdr[0] * ab[d] / rab;
    g[3 + d] = dvdr[0] * ab[d] / rab - dvdr[2] * bc[d] / rbc;
    g[6 + d] = dvdr[2] * bc[d] / rbc - dvdr[1] * ac[d] / rac;
  }
}

}  // namespace brh2

struct PesBrH2 {
  static constexpr int N = 3;
  template <class F>
  __device__ static inline void egrad(const double (&q)[9], double& V, double (&g)[9]) {
    brh2::egrad_bead(q, &V, g);
  }
};

}  // namespace cr
