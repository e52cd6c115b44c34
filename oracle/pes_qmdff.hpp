// ORACLE (test infrastructure only) -- QMDFF energy and gradient, CPU restatement.
//
// Restates Caracal's QMDFF force field for one structure, non-periodic, one
// molecule (nmols = 1):
//   ff_eg   src/ff_eg.f90:41-629      bonds (generalised LJ, :87-163), angles
//           with abdamp damping (:167-299), torsions with erf-blended cosine
//           series (:303-440) and inversions (tors(6) = 2, :441-618);
//           helpers abdamp src/abdamp.f90:36-51, valijkl src/valijkl.f90:34,
//           dphidr src/dphidr.f90:34, omega src/omega.f90:35, domegadr
//           src/domegadr.f90:35, crprod, impsc, vlen
//   ff_nonb src/ff_nonb.f90:34-889    over the nci list: BJ-damped C6/C8
//           dispersion and exponential repulsion (r < 25 bohr) scaled by
//           eps2(nk) (:79-193), Coulomb eps1(nk) q q / r within coul_cut, or the
//           Zahn form q q (erfc(a r)/r - b (r - coul_cut)) (:337-416); the
//           dipole moment (:743-762) never reaches the outputs and is skipped
//   gradient src/gradient.f90:342-358 e = ff_eg + ff_nonb (+ ff_hb) + E_zero
// H/halogen-bond terms (ff_hb) are not restated yet (nhb must be 0).
// REAL(4) literals reproduced: abdamp's cutoff 3.0 * 3.5710642 (a float
// product), eps1(3) = 0.85 (src/setnonb.f90:164-190).
#pragma once
#include <cmath>
#include <vector>

namespace orc {
namespace qmdff {

struct FF {
  int n = 0;
  std::vector<int> at;          // element numbers (n)
  std::vector<double> q;        // charges (n)
  std::vector<double> rad;      // covalent radius of atom i in bohr (Caracal's rad(at(i)))
  int nbond = 0, nangl = 0, ntors = 0, nnci = 0;
  std::vector<int> bond;        // 2 per bond, 0-based
  std::vector<double> vbond;    // r0, k, a
  std::vector<int> angl;        // center j, i, k (Caracal's angl(1..3)), 0-based
  std::vector<double> vangl;    // theta0, k
  std::vector<int> tors;        // i, j, k, l (0-based), nt, type
  std::vector<double> vtors;    // 14 per torsion: phi0, V, (rn, phase*pi, V_n) x 4
  std::vector<int> nci;         // i, j (0-based), category nk (1..6)
  // per nci pair parameters: R0 (r094), C6, sr42, zab, alpha (r0ab)
  std::vector<double> pR0, pC6, pSr42, pZab, pAlpha;
  double eps1[7] = {0, 0, 0, 0, 0, 0, 0};
  double eps2[7] = {0, 0, 0, 0, 0, 0, 0};
  double coul_cut = 50.0;
  bool zahn = false;
  double zahn_a = 0.0, zahn_par = 0.0;
  double e_zero = 0.0;
};

inline double vlen(const double* a) {
  double tot = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
  return tot > 0.0 ? std::sqrt(tot) : 0.0;
}
inline void crprod(const double* a, const double* b, double* c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}
inline double impsc(const double* a, const double* b) {
  double rimp = a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
  double al = vlen(a), bl = vlen(b);
  return (al > 0.0 && bl > 0.0) ? rimp / (al * bl) : 0.0;
}
inline double vecnorm(double* r, bool normalise) {
  double sp = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
  double rn = std::sqrt(sp);
  if (normalise && std::fabs(rn) > 1e-14) {
    double o = 1.0 / rn;
    r[0] *= o;
    r[1] *= o;
    r[2] *= o;
  }
  return rn;
}

// abdamp (src/abdamp.f90:36-51); the cutoff prefactor is a REAL(4) product
inline void abdamp(double radi, double radj, double r2, double* damp, double* ddamp) {
  const double pre = (double)(3.0f * 3.5710642f);
  double s = radi + radj;
  double rcut = pre * (s * s);
  double rr = (r2 / rcut) * (r2 / rcut);
  *damp = 1.0 / (1.0 + rr);
  *ddamp = -2.0 * 2 * rr / (r2 * ((1.0 + rr) * (1.0 + rr)));
}

// torsion angle (valijkl)
inline double valijkl(const double* x, int i, int j, int k, int l) {
  double ra[3], rb[3], rc[3], na[3], nb[3];
  for (int c = 0; c < 3; ++c) {
    ra[c] = x[3 * j + c] - x[3 * i + c];
    rb[c] = x[3 * k + c] - x[3 * j + c];
    rc[c] = x[3 * l + c] - x[3 * k + c];
  }
  crprod(ra, rb, na);
  crprod(rb, rc, nb);
  vecnorm(na, true);
  vecnorm(nb, true);
  double s = na[0] * nb[0] + na[1] * nb[1] + na[2] * nb[2];
  if (std::fabs(std::fabs(s) - 1.0) < 1e-14) s = s >= 0 ? 1.0 : -1.0;
  return std::acos(s);
}

// d phi / d r (dphidr)
inline void dphidr(const double* x, int i, int j, int k, int l, double phi, double* di, double* dj,
                   double* dk, double* dl) {
  double cosphi = std::cos(phi), sinphi = std::sin(phi);
  double ra[3], rb[3], rc[3], rapb[3], rbpc[3], na[3], nb[3];
  for (int c = 0; c < 3; ++c) {
    ra[c] = x[3 * j + c] - x[3 * i + c];
    rb[c] = x[3 * k + c] - x[3 * j + c];
    rc[c] = x[3 * l + c] - x[3 * k + c];
    rapb[c] = ra[c] + rb[c];
    rbpc[c] = rb[c] + rc[c];
  }
  crprod(ra, rb, na);
  crprod(rb, rc, nb);
  double nan_ = vecnorm(na, false), nbn = vecnorm(nb, false);
  double nenner = nan_ * nbn * sinphi;
  if (std::fabs(nenner) < 1e-14) {
    for (int c = 0; c < 3; ++c) di[c] = dj[c] = dk[c] = dl[c] = 0.0;
    return;
  }
  double on = 1.0 / nenner;
  double rab[3], rba[3], rac[3], rbb[3], rbc[3], raa[3], rapba[3], rapbb[3], rbpca[3], rbpcb[3];
  crprod(na, rb, rab);
  crprod(nb, ra, rba);
  crprod(na, rc, rac);
  crprod(nb, rb, rbb);
  crprod(nb, rc, rbc);
  crprod(na, ra, raa);
  crprod(rapb, na, rapba);
  crprod(rapb, nb, rapbb);
  crprod(rbpc, na, rbpca);
  crprod(rbpc, nb, rbpcb);
  for (int c = 0; c < 3; ++c) {
    di[c] = on * (cosphi * nbn / nan_ * rab[c] - rbb[c]);
    dj[c] = on * (cosphi * (nbn / nan_ * rapba[c] + nan_ / nbn * rbc[c]) - (rac[c] + rapbb[c]));
    dk[c] = on * (cosphi * (nbn / nan_ * raa[c] + nan_ / nbn * rbpcb[c]) - (rba[c] + rbpca[c]));
    dl[c] = on * (cosphi * nan_ / nbn * rbb[c] - rab[c]);
  }
}

// out-of-plane angle (omega) and its gradient (domegadr)
inline double omega(const double* x, int i, int j, int k, int l) {
  double re[3], rd[3], rv[3], rn[3];
  for (int c = 0; c < 3; ++c) {
    re[c] = x[3 * i + c] - x[3 * j + c];
    rd[c] = x[3 * k + c] - x[3 * j + c];
    rv[c] = x[3 * l + c] - x[3 * i + c];
  }
  crprod(re, rd, rn);
  vecnorm(rn, true);
  vecnorm(rv, true);
  return std::asin(rn[0] * rv[0] + rn[1] * rv[1] + rn[2] * rv[2]);
}

inline void domegadr(const double* x, int i, int j, int k, int l, double om, double* di, double* dj,
                     double* dk, double* dl) {
  double sinom = std::sin(om);
  double rv[3], rd[3], re[3], rdme[3], rn[3];
  for (int c = 0; c < 3; ++c) {
    rv[c] = x[3 * l + c] - x[3 * i + c];
    rd[c] = x[3 * k + c] - x[3 * j + c];
    re[c] = x[3 * i + c] - x[3 * j + c];
    rdme[c] = rd[c] - re[c];
  }
  crprod(re, rd, rn);
  double rvn = vecnorm(rv, false), rnn = vecnorm(rn, false);
  double rve[3], rne[3], rdv[3], rdn[3], rvdme[3], rndme[3];
  crprod(rv, re, rve);
  crprod(rn, re, rne);
  crprod(rd, rv, rdv);
  crprod(rd, rn, rdn);
  crprod(rv, rdme, rvdme);
  crprod(rn, rdme, rndme);
  double nenner = rnn * rvn * std::cos(om);
  if (std::fabs(nenner) > 1e-14) {
    double on = 1.0 / nenner;
    for (int c = 0; c < 3; ++c) {
      di[c] = on * (rdv[c] - rn[c] - sinom * (rvn / rnn * rdn[c] - rnn / rvn * rv[c]));
      dj[c] = on * (rvdme[c] - sinom * rvn / rnn * rndme[c]);
      dk[c] = on * (rve[c] - sinom * rvn / rnn * rne[c]);
      dl[c] = on * (rn[c] - sinom * rnn / rvn * rv[c]);
    }
  } else {
    for (int c = 0; c < 3; ++c) di[c] = dj[c] = dk[c] = dl[c] = 0.0;
  }
}

// ff_eg: overwrites e and g(3,n)
inline void ff_eg(const FF& ff, const double* x, double* e_out, double* g) {
  const double pi = 3.1415926535897932384626433832795029;
  const double pi2 = 6.28318530717958623199592693708837;
  const double spi = 1.77245385090551599275151910313925;
  double e = 0.0;
  for (int a = 0; a < 3 * ff.n; ++a) g[a] = 0.0;
  for (int m = 0; m < ff.nbond; ++m) {
    int i = ff.bond[2 * m], j = ff.bond[2 * m + 1];
    double rb[3];
    for (int c = 0; c < 3; ++c) rb[c] = x[3 * i + c] - x[3 * j + c];
    double r2 = rb[0] * rb[0] + rb[1] * rb[1] + rb[2] * rb[2];
    double r = std::sqrt(r2);
    double rij = ff.vbond[3 * m], kij = ff.vbond[3 * m + 1], aai = ff.vbond[3 * m + 2];
    double aai2 = aai / 2;
    double pa = std::pow(rij / r, aai), pa2 = std::pow(rij / r, aai2);
    e = e + kij * (1. + pa - 2. * pa2);
    double fac = aai * kij * (-pa + pa2) / r2;
    for (int c = 0; c < 3; ++c) {
      g[3 * i + c] += fac * rb[c];
      g[3 * j + c] -= fac * rb[c];
    }
  }
  for (int m = 0; m < ff.nangl; ++m) {
    int j = ff.angl[3 * m], i = ff.angl[3 * m + 1], k = ff.angl[3 * m + 2];
    double c0 = ff.vangl[2 * m], kijk = ff.vangl[2 * m + 1];
    double vab[3], vcb[3], vp[3];
    for (int c = 0; c < 3; ++c) {
      vab[c] = x[3 * i + c] - x[3 * j + c];
      vcb[c] = x[3 * k + c] - x[3 * j + c];
    }
    double rab2 = vab[0] * vab[0] + vab[1] * vab[1] + vab[2] * vab[2];
    double rcb2 = vcb[0] * vcb[0] + vcb[1] * vcb[1] + vcb[2] * vcb[2];
    crprod(vcb, vab, vp);
    double rp = vlen(vp) + 1e-14;
    double cosa = impsc(vab, vcb);
    cosa = std::fmin(1.0, std::fmax(-1.0, cosa));
    double theta = std::acos(cosa);
    double dampij, damp2ij, dampjk, damp2jk;
    abdamp(ff.rad[i], ff.rad[j], rab2, &dampij, &damp2ij);
    abdamp(ff.rad[k], ff.rad[j], rcb2, &dampjk, &damp2jk);
    double damp = dampij * dampjk;
    double ea, deddt;
    if (pi - c0 < 1e-6) {
      double dt = theta - c0;
      ea = kijk * (dt * dt);
      deddt = 2.0 * kijk * dt;
    } else {
      double d = cosa - std::cos(c0);
      ea = kijk * (d * d);
      deddt = 2. * kijk * std::sin(theta) * (std::cos(c0) - cosa);
    }
    e = e + ea * damp;
    double deda[3], dedc[3];
    crprod(vab, vp, deda);
    double rmul1 = -deddt / (rab2 * rp);
    crprod(vcb, vp, dedc);
    double rmul2 = deddt / (rcb2 * rp);
    for (int c = 0; c < 3; ++c) {
      deda[c] *= rmul1;
      dedc[c] *= rmul2;
      double dedb = deda[c] + dedc[c];
      double t1 = ea * damp2ij * dampjk * vab[c];
      double t2 = ea * damp2jk * dampij * vcb[c];
      g[3 * i + c] += deda[c] * damp + t1;
      g[3 * j + c] += -dedb * damp - t1 - t2;
      g[3 * k + c] += dedc[c] * damp + t2;
    }
  }
  for (int m = 0; m < ff.ntors; ++m) {
    int i = ff.tors[6 * m], j = ff.tors[6 * m + 1], k = ff.tors[6 * m + 2], l = ff.tors[6 * m + 3];
    int nt = ff.tors[6 * m + 4], type = ff.tors[6 * m + 5];
    const double* vt = &ff.vtors[14 * m];
    double phi0 = vt[0];
    double vab[3], vcb[3], vdc[3], dda[3], ddb[3], ddc[3], ddd[3];
    double et, dij, damp, d2a, d2b, d2c;
    double dmp[3];
    if (type != 2) {
      for (int c = 0; c < 3; ++c) {
        vab[c] = x[3 * i + c] - x[3 * j + c];
        vcb[c] = x[3 * j + c] - x[3 * k + c];
        vdc[c] = x[3 * k + c] - x[3 * l + c];
      }
      double rij = vab[0] * vab[0] + vab[1] * vab[1] + vab[2] * vab[2];
      double rjk = vcb[0] * vcb[0] + vcb[1] * vcb[1] + vcb[2] * vcb[2];
      double rkl = vdc[0] * vdc[0] + vdc[1] * vdc[1] + vdc[2] * vdc[2];
      abdamp(ff.rad[i], ff.rad[j], rij, &dmp[0], &d2a);
      abdamp(ff.rad[k], ff.rad[j], rjk, &dmp[1], &d2b);
      abdamp(ff.rad[k], ff.rad[l], rkl, &dmp[2], &d2c);
      double dampij = dmp[0], dampjk = dmp[1], dampkl = dmp[2];
      damp = dampjk * dampij * dampkl;
      double phi = valijkl(x, i, j, k, l);
      dphidr(x, i, j, k, l, phi, dda, ddb, ddc, ddd);
      et = 0.0;
      dij = 0.0;
      int mm = 2;
      for (int it = 0; it < nt; ++it) {
        double rn = vt[mm];
        double dphi1 = phi - phi0, dphi2 = phi + phi0 - pi2;
        double c1 = rn * dphi1 + vt[mm + 1];
        double c2 = rn * dphi2 + vt[mm + 1];
        double x1cos = std::cos(c1), x2cos = std::cos(c2), x1sin = std::sin(c1), x2sin = std::sin(c2);
        double phipi = phi - pi;
        double ef = std::erf(phipi);
        double e1 = vt[mm + 2] * (1. + x1cos);
        double e2 = vt[mm + 2] * (1. + x2cos);
        et = et + 0.5 * (1. - ef) * e1 + (0.5 + 0.5 * ef) * e2;
        double expo = std::exp(-(phipi * phipi)) / spi;
        dij = dij - expo * e1 - 0.5 * (1. - ef) * vt[mm + 2] * x1sin * rn + expo * e2 -
              (0.5 + 0.5 * ef) * vt[mm + 2] * x2sin * rn;
        mm += 3;
      }
      et = et * vt[1];
      dij = dij * vt[1] * damp;
      for (int c = 0; c < 3; ++c) {
        double t1 = et * d2a * dampjk * dampkl * vab[c];
        double t2 = et * d2b * dampij * dampkl * vcb[c];
        double t3 = et * d2c * dampij * dampjk * vdc[c];
        g[3 * i + c] += dij * dda[c] + t1;
        g[3 * j + c] += dij * ddb[c] - t1 + t2;
        g[3 * k + c] += dij * ddc[c] + t3 - t2;
        g[3 * l + c] += dij * ddd[c] - t3;
      }
      e = e + et * damp;
    } else {
      for (int c = 0; c < 3; ++c) {
        vab[c] = x[3 * j + c] - x[3 * i + c];
        vcb[c] = x[3 * j + c] - x[3 * k + c];
        vdc[c] = x[3 * j + c] - x[3 * l + c];
      }
      double rij = vab[0] * vab[0] + vab[1] * vab[1] + vab[2] * vab[2];
      double rjk = vcb[0] * vcb[0] + vcb[1] * vcb[1] + vcb[2] * vcb[2];
      double rjl = vdc[0] * vdc[0] + vdc[1] * vdc[1] + vdc[2] * vdc[2];
      abdamp(ff.rad[i], ff.rad[j], rij, &dmp[0], &d2a);
      abdamp(ff.rad[k], ff.rad[j], rjk, &dmp[1], &d2b);
      abdamp(ff.rad[j], ff.rad[l], rjl, &dmp[2], &d2c);
      double dampij = dmp[0], dampjk = dmp[1], dampjl = dmp[2];
      damp = dampjk * dampij * dampjl;
      double phi = omega(x, i, j, k, l);
      domegadr(x, i, j, k, l, phi, dda, ddb, ddc, ddd);
      double rn = vt[2];
      if (rn > 1e-6) {
        double c1 = (phi - phi0) + pi;
        et = (1. + std::cos(c1)) * vt[1];
        dij = -std::sin(c1) * vt[1] * damp;
      } else {
        double d = std::cos(phi) - std::cos(phi0);
        et = vt[1] * (d * d);
        dij = 2. * vt[1] * std::sin(phi) * (std::cos(phi0) - std::cos(phi)) * damp;
      }
      for (int c = 0; c < 3; ++c) {
        double t1 = et * d2a * dampjk * dampjl * vab[c];
        double t2 = et * d2b * dampij * dampjl * vcb[c];
        double t3 = et * d2c * dampij * dampjk * vdc[c];
        g[3 * i + c] += dij * dda[c] - t1;
        g[3 * j + c] += dij * ddb[c] + t1 + t2 + t3;
        g[3 * k + c] += dij * ddc[c] - t2;
        g[3 * l + c] += dij * ddd[c] - t3;
      }
      e = e + et * damp;
    }
  }
  *e_out = e;
}

// ff_nonb (non-periodic, one molecule): accumulates into enb and g
inline void ff_nonb(const FF& ff, const double* x, double* enb, double* g) {
  double e = 0.0;
  for (int kp = 0; kp < ff.nnci; ++kp) {
    int i1 = ff.nci[3 * kp], i2 = ff.nci[3 * kp + 1], nk = ff.nci[3 * kp + 2];
    double vab[3];
    for (int c = 0; c < 3; ++c) vab[c] = x[3 * i1 + c] - x[3 * i2 + c];
    double r2 = vab[0] * vab[0] + vab[1] * vab[1] + vab[2] * vab[2];
    double r = std::sqrt(r2);
    double oner = 1.0 / r;
    double R0 = ff.pR0[kp], c6 = ff.pC6[kp];
    double r4 = r2 * r2, r6 = r4 * r2;
    double R02 = R0 * R0, r06 = R02 * R02 * R02;
    double t6 = r6 + r06;
    double t8 = r6 * r2 + r06 * R0 * R0;
    double c6t6 = c6 / t6, c6t8 = c6 / t8;
    double t27 = ff.pSr42[kp] * c6t8;
    double e0 = c6t6 + t27;
    e = e - e0 * ff.eps2[nk];
    double drij = ff.eps2[nk] * (c6t6 * 6.0 * r4 / t6 + 8.0 * t27 * r6 / t8);
    double ga[3] = {vab[0] * drij, vab[1] * drij, vab[2] * drij};
    if (r < 25) {
      double xz = ff.pZab[kp], alpha = ff.pAlpha[kp];
      double t = xz * std::exp(-alpha * r);
      double e1 = t * oner;
      e = e + e1 * ff.eps2[nk];
      double dr2 = ff.eps2[nk] * t * (alpha * r + 1.0) * oner / r2;
      for (int c = 0; c < 3; ++c) ga[c] = ga[c] - vab[c] * dr2;
    }
    for (int c = 0; c < 3; ++c) {
      g[3 * i1 + c] += ga[c];
      g[3 * i2 + c] -= ga[c];
    }
  }
  for (int kp = 0; kp < ff.nnci; ++kp) {
    int i1 = ff.nci[3 * kp], i2 = ff.nci[3 * kp + 1], nk = ff.nci[3 * kp + 2];
    double vab[3];
    for (int c = 0; c < 3; ++c) vab[c] = x[3 * i1 + c] - x[3 * i2 + c];
    double r2 = vab[0] * vab[0] + vab[1] * vab[1] + vab[2] * vab[2];
    double r = std::sqrt(r2);
    if (r > ff.coul_cut) continue;
    double oner = 1.0 / r;
    double e0;
    if (ff.zahn)
      e0 = ff.q[i1] * ff.q[i2] * ((std::erfc(ff.zahn_a * r) * oner) - ff.zahn_par * (r - ff.coul_cut));
    else
      e0 = ff.q[i1] * ff.q[i2] * oner * ff.eps1[nk] * 1.0;
    e = e + e0;
    double drij = e0 / r2;
    for (int c = 0; c < 3; ++c) {
      double ga = -vab[c] * drij;
      g[3 * i1 + c] += ga;
      g[3 * i2 + c] -= ga;
    }
  }
  *enb = *enb + e;
}

// gradient dispatch for one QMDFF (src/gradient.f90:342-358)
inline void egrad(const FF& ff, const double* x, double* V, double* g) {
  double e;
  ff_eg(ff, x, &e, g);
  ff_nonb(ff, x, &e, g);
  *V = e + ff.e_zero;
}

}  // namespace qmdff
}  // namespace orc
