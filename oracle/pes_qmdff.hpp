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
//   ff_hb   src/ff_hb.f90:36-93 (one molecule: the listed triples only)
//           eabhag src/eabhag.f90:35-220 (analytic H bond), eabxag
//           src/eabxag.f90:35-156 with eabx src/eabx.f90:34-111 (halogen
//           bond, central-difference gradient).  Quirk reproduced: eabxag
//           assigns the scalar difference quotient to the whole 3-vector in
//           each of its j loops, so every component of each atom's gradient
//           is the z derivative.
// REAL(4) literals reproduced: abdamp's cutoff 3.0 * 3.5710642 (a float
// product), eps1(3) = 0.85 (src/setnonb.f90:164-190).
#pragma once
#include <algorithm>
#include <cmath>
#include <type_traits>
#include <vector>

namespace orc {
namespace qmdff {

using std::acos;
using std::asin;
using std::cos;
using std::erf;
using std::erfc;
using std::exp;
using std::fabs;
using std::fmax;
using std::fmin;
using std::pow;
using std::sin;
using std::sqrt;

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
  int nhb = 0;
  std::vector<int> hb;          // A, B, H (0-based): H-bond if at(H) = 1, else halogen bond
  std::vector<double> vhb;      // 2 per triple: ca, cb (rdsolvff's hbpara * scalehb / scalexb)
  // per nci pair parameters: R0 (r094), C6, sr42, zab, alpha (r0ab)
  std::vector<double> pR0, pC6, pSr42, pZab, pAlpha;
  double eps1[7] = {0, 0, 0, 0, 0, 0, 0};
  double eps2[7] = {0, 0, 0, 0, 0, 0, 0};
  double coul_cut = 50.0;
  bool zahn = false;
  double zahn_a = 0.0, zahn_par = 0.0;
  double e_zero = 0.0;
  // periodic box (src/set_periodic.f90, pbc_mod): edges and halves (bohr),
  // dispersion/repulsion cutoff
  bool periodic = false;
  double len[3] = {0, 0, 0}, half[3] = {0, 0, 0};
  double vdw_cut = 0.0;
  // NpT: where set, the terms add their share of the virial trace here
  // (vir_ten of src/ff_eg.f90, ff_nonb.f90, eabhag.f90, eabxag.f90; the
  // pressure uses its diagonal only, src/verlet.f90:1123-1131)
  double* vir = nullptr;
};

// vir += a . b (FP64 evaluations only)
template <class T>
inline void vir_add(const FF& ff, const T* a, const T* b) {
  if constexpr (std::is_same<T, double>::value)
    if (ff.vir) *ff.vir += a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}
// a torsion's or inversion's vir_ten: vab.g_a + vcb.(g_c + g_d) + vdc.g_d
template <class T>
inline void vir_tors(const FF& ff, const T* vab, const T* vcb, const T* vdc, const T* ga, const T* gc, const T* gd) {
  if constexpr (std::is_same<T, double>::value)
    if (ff.vir) {
      const T gcd[3] = {gc[0] + gd[0], gc[1] + gd[1], gc[2] + gd[2]};
      vir_add(ff, vab, ga);
      vir_add(ff, vcb, gcd);
      vir_add(ff, vdc, gd);
    }
}

// box_image (src/box_image.f90:36-63): subtract the edge while a component
// exceeds half of it (bounded here at 64 subtractions).
template <class T>
inline void box_image(const FF& ff, T* v) {
  if (!ff.periodic) return;
  for (int k = 0; k < 3; ++k)
    for (int it = 0; it < 64 && (v[k] > T(ff.half[k]) || v[k] < T(-ff.half[k])); ++it)
      v[k] = v[k] - T(v[k] > T(0.0) ? ff.len[k] : -ff.len[k]);
}

// set_periodic (src/set_periodic.f90:67-113): box edges and the Coulomb and
// dispersion cutoffs from Angstrom; a Coulomb cutoff below 5 bohr becomes
// half the shortest edge minus 0.1 bohr, the Zahn form fixes it at 10 A and
// sets its parameters, and no cutoff may exceed half the shortest edge.
inline void set_periodic(FF& ff, const double box_ang[3], double coul_cut_ang, double vdw_cut_ang) {
  const double bohr = 0.52917721092;
  ff.periodic = true;
  for (int k = 0; k < 3; ++k) {
    ff.len[k] = box_ang[k] / bohr;
    ff.half[k] = ff.len[k] * 0.5;
  }
  const double hmin = std::min(ff.half[0], std::min(ff.half[1], ff.half[2]));
  ff.coul_cut = coul_cut_ang / bohr;
  ff.vdw_cut = vdw_cut_ang / bohr;
  if (ff.coul_cut < 5.0) ff.coul_cut = hmin - 0.1;
  if (ff.zahn) {
    const double spi = std::sqrt(3.14159265358979323846);
    ff.zahn_a = 0.2 * bohr;
    ff.coul_cut = 10.0 / bohr;
    const double acut = ff.zahn_a * ff.coul_cut;
    ff.zahn_par = std::erfc(acut) / (ff.coul_cut * ff.coul_cut) +
                  2 * ff.zahn_a / spi * std::exp(-acut * acut) / ff.coul_cut;
  }
  if (ff.coul_cut > hmin) ff.coul_cut = hmin - 0.1;
}

template <class T>
inline T vlen(const T* a) {
  T tot = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
  return tot > 0.0 ? sqrt(tot) : T(0.0);
}
template <class T>
inline void crprod(const T* a, const T* b, T* c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}
template <class T>
inline T impsc(const T* a, const T* b) {
  T rimp = a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
  T al = vlen(a), bl = vlen(b);
  return (al > 0.0 && bl > 0.0) ? rimp / (al * bl) : T(0.0);
}
template <class T>
inline T vecnorm(T* r, bool normalise) {
  T sp = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
  T rn = sqrt(sp);
  if (normalise && fabs(rn) > 1e-14) {
    T o = 1.0 / rn;
    r[0] *= o;
    r[1] *= o;
    r[2] *= o;
  }
  return rn;
}

// abdamp (src/abdamp.f90:36-51); the cutoff prefactor is a REAL(4) product
template <class T>
inline void abdamp(double radi, double radj, T r2, T* damp, T* ddamp) {
  const double pre = (double)(3.0f * 3.5710642f);
  const double s = radi + radj;
  const double rcut = pre * (s * s);
  T rr = (r2 / rcut) * (r2 / rcut);
  *damp = 1.0 / (1.0 + rr);
  *ddamp = -2.0 * 2 * rr / (r2 * ((1.0 + rr) * (1.0 + rr)));
}

// torsion angle (valijkl)
template <class T>
inline T valijkl(const T* x, int i, int j, int k, int l) {
  T ra[3], rb[3], rc[3], na[3], nb[3];
  for (int c = 0; c < 3; ++c) {
    ra[c] = x[3 * j + c] - x[3 * i + c];
    rb[c] = x[3 * k + c] - x[3 * j + c];
    rc[c] = x[3 * l + c] - x[3 * k + c];
  }
  crprod(ra, rb, na);
  crprod(rb, rc, nb);
  vecnorm(na, true);
  vecnorm(nb, true);
  T s = na[0] * nb[0] + na[1] * nb[1] + na[2] * nb[2];
  if (fabs(fabs(s) - 1.0) < 1e-14) s = s >= 0.0 ? T(1.0) : T(-1.0);
  return acos(s);
}

// d phi / d r (dphidr)
template <class T>
inline void dphidr(const T* x, int i, int j, int k, int l, T phi, T* di, T* dj, T* dk, T* dl) {
  T cosphi = cos(phi), sinphi = sin(phi);
  T ra[3], rb[3], rc[3], rapb[3], rbpc[3], na[3], nb[3];
  for (int c = 0; c < 3; ++c) {
    ra[c] = x[3 * j + c] - x[3 * i + c];
    rb[c] = x[3 * k + c] - x[3 * j + c];
    rc[c] = x[3 * l + c] - x[3 * k + c];
    rapb[c] = ra[c] + rb[c];
    rbpc[c] = rb[c] + rc[c];
  }
  crprod(ra, rb, na);
  crprod(rb, rc, nb);
  T nan_ = vecnorm(na, false), nbn = vecnorm(nb, false);
  T nenner = nan_ * nbn * sinphi;
  if (fabs(nenner) < 1e-14) {
    for (int c = 0; c < 3; ++c) di[c] = dj[c] = dk[c] = dl[c] = 0.0;
    return;
  }
  T on = 1.0 / nenner;
  T rab[3], rba[3], rac[3], rbb[3], rbc[3], raa[3], rapba[3], rapbb[3], rbpca[3], rbpcb[3];
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
template <class T>
inline T omega(const T* x, int i, int j, int k, int l) {
  T re[3], rd[3], rv[3], rn[3];
  for (int c = 0; c < 3; ++c) {
    re[c] = x[3 * i + c] - x[3 * j + c];
    rd[c] = x[3 * k + c] - x[3 * j + c];
    rv[c] = x[3 * l + c] - x[3 * i + c];
  }
  crprod(re, rd, rn);
  vecnorm(rn, true);
  vecnorm(rv, true);
  return asin(rn[0] * rv[0] + rn[1] * rv[1] + rn[2] * rv[2]);
}

template <class T>
inline void domegadr(const T* x, int i, int j, int k, int l, T om, T* di, T* dj, T* dk, T* dl) {
  T sinom = sin(om);
  T rv[3], rd[3], re[3], rdme[3], rn[3];
  for (int c = 0; c < 3; ++c) {
    rv[c] = x[3 * l + c] - x[3 * i + c];
    rd[c] = x[3 * k + c] - x[3 * j + c];
    re[c] = x[3 * i + c] - x[3 * j + c];
    rdme[c] = rd[c] - re[c];
  }
  crprod(re, rd, rn);
  T rvn = vecnorm(rv, false), rnn = vecnorm(rn, false);
  T rve[3], rne[3], rdv[3], rdn[3], rvdme[3], rndme[3];
  crprod(rv, re, rve);
  crprod(rn, re, rne);
  crprod(rd, rv, rdv);
  crprod(rd, rn, rdn);
  crprod(rv, rdme, rvdme);
  crprod(rn, rdme, rndme);
  T nenner = rnn * rvn * cos(om);
  if (fabs(nenner) > 1e-14) {
    T on = 1.0 / nenner;
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
template <class T>
inline void ff_eg(const FF& ff, const T* x, T* e_out, T* g) {
  const double pi = 3.1415926535897932384626433832795029;
  const double pi2 = 6.28318530717958623199592693708837;
  const double spi = 1.77245385090551599275151910313925;
  T e = 0.0;
  for (int a = 0; a < 3 * ff.n; ++a) g[a] = 0.0;
  for (int m = 0; m < ff.nbond; ++m) {
    int i = ff.bond[2 * m], j = ff.bond[2 * m + 1];
    T rb[3];
    for (int c = 0; c < 3; ++c) rb[c] = x[3 * i + c] - x[3 * j + c];
    box_image(ff, rb);
    T r2 = rb[0] * rb[0] + rb[1] * rb[1] + rb[2] * rb[2];
    T r = sqrt(r2);
    T rij = ff.vbond[3 * m], kij = ff.vbond[3 * m + 1], aai = ff.vbond[3 * m + 2];
    T aai2 = aai / 2;
    T pa = pow(rij / r, aai), pa2 = pow(rij / r, aai2);
    e = e + kij * (1. + pa - 2. * pa2);
    T fac = aai * kij * (-pa + pa2) / r2;
    T ga[3];
    for (int c = 0; c < 3; ++c) {
      ga[c] = fac * rb[c];
      g[3 * i + c] += ga[c];
      g[3 * j + c] -= ga[c];
    }
    vir_add(ff, rb, ga);  // src/ff_eg.f90:138-150
  }
  for (int m = 0; m < ff.nangl; ++m) {
    int j = ff.angl[3 * m], i = ff.angl[3 * m + 1], k = ff.angl[3 * m + 2];
    T c0 = ff.vangl[2 * m], kijk = ff.vangl[2 * m + 1];
    T vab[3], vcb[3], vp[3];
    for (int c = 0; c < 3; ++c) {
      vab[c] = x[3 * i + c] - x[3 * j + c];
      vcb[c] = x[3 * k + c] - x[3 * j + c];
    }
    box_image(ff, vab);
    box_image(ff, vcb);
    T rab2 = vab[0] * vab[0] + vab[1] * vab[1] + vab[2] * vab[2];
    T rcb2 = vcb[0] * vcb[0] + vcb[1] * vcb[1] + vcb[2] * vcb[2];
    crprod(vcb, vab, vp);
    T rp = vlen(vp) + 1e-14;
    T cosa = impsc(vab, vcb);
    cosa = fmin(1.0, fmax(-1.0, cosa));
    T theta = acos(cosa);
    T dampij, damp2ij, dampjk, damp2jk;
    abdamp(ff.rad[i], ff.rad[j], rab2, &dampij, &damp2ij);
    abdamp(ff.rad[k], ff.rad[j], rcb2, &dampjk, &damp2jk);
    T damp = dampij * dampjk;
    T ea, deddt;
    if (pi - c0 < 1e-6) {
      T dt = theta - c0;
      ea = kijk * (dt * dt);
      deddt = 2.0 * kijk * dt;
    } else {
      T d = cosa - cos(c0);
      ea = kijk * (d * d);
      deddt = 2. * kijk * sin(theta) * (cos(c0) - cosa);
    }
    e = e + ea * damp;
    T deda[3], dedc[3];
    crprod(vab, vp, deda);
    T rmul1 = -deddt / (rab2 * rp);
    crprod(vcb, vp, dedc);
    T rmul2 = deddt / (rcb2 * rp);
    T gla[3], glc[3];
    for (int c = 0; c < 3; ++c) {
      deda[c] *= rmul1;
      dedc[c] *= rmul2;
      T dedb = deda[c] + dedc[c];
      T t1 = ea * damp2ij * dampjk * vab[c];
      T t2 = ea * damp2jk * dampij * vcb[c];
      gla[c] = deda[c] * damp + t1;
      glc[c] = dedc[c] * damp + t2;
      g[3 * i + c] += gla[c];
      g[3 * j + c] += -dedb * damp - t1 - t2;
      g[3 * k + c] += glc[c];
    }
    vir_add(ff, vab, gla);  // src/ff_eg.f90:270-281
    vir_add(ff, vcb, glc);
  }
  for (int m = 0; m < ff.ntors; ++m) {
    int i = ff.tors[6 * m], j = ff.tors[6 * m + 1], k = ff.tors[6 * m + 2], l = ff.tors[6 * m + 3];
    int nt = ff.tors[6 * m + 4], type = ff.tors[6 * m + 5];
    const double* vt = &ff.vtors[14 * m];
    T phi0 = vt[0];
    T vab[3], vcb[3], vdc[3], dda[3], ddb[3], ddc[3], ddd[3];
    T et, dij, damp, d2a, d2b, d2c;
    T dmp[3];
    if (type != 2) {
      for (int c = 0; c < 3; ++c) {
        vab[c] = x[3 * i + c] - x[3 * j + c];
        vcb[c] = x[3 * j + c] - x[3 * k + c];
        vdc[c] = x[3 * k + c] - x[3 * l + c];
      }
      box_image(ff, vab);
      box_image(ff, vcb);
      box_image(ff, vdc);
      T rij = vab[0] * vab[0] + vab[1] * vab[1] + vab[2] * vab[2];
      T rjk = vcb[0] * vcb[0] + vcb[1] * vcb[1] + vcb[2] * vcb[2];
      T rkl = vdc[0] * vdc[0] + vdc[1] * vdc[1] + vdc[2] * vdc[2];
      abdamp(ff.rad[i], ff.rad[j], rij, &dmp[0], &d2a);
      abdamp(ff.rad[k], ff.rad[j], rjk, &dmp[1], &d2b);
      abdamp(ff.rad[k], ff.rad[l], rkl, &dmp[2], &d2c);
      T dampij = dmp[0], dampjk = dmp[1], dampkl = dmp[2];
      damp = dampjk * dampij * dampkl;
      T phi = valijkl(x, i, j, k, l);
      dphidr(x, i, j, k, l, phi, dda, ddb, ddc, ddd);
      et = 0.0;
      dij = 0.0;
      int mm = 2;
      for (int it = 0; it < nt; ++it) {
        T rn = vt[mm];
        T dphi1 = phi - phi0, dphi2 = phi + phi0 - pi2;
        T c1 = rn * dphi1 + vt[mm + 1];
        T c2 = rn * dphi2 + vt[mm + 1];
        T x1cos = cos(c1), x2cos = cos(c2), x1sin = sin(c1), x2sin = sin(c2);
        T phipi = phi - pi;
        T ef = erf(phipi);
        T e1 = vt[mm + 2] * (1. + x1cos);
        T e2 = vt[mm + 2] * (1. + x2cos);
        et = et + 0.5 * (1. - ef) * e1 + (0.5 + 0.5 * ef) * e2;
        T expo = exp(-(phipi * phipi)) / spi;
        dij = dij - expo * e1 - 0.5 * (1. - ef) * vt[mm + 2] * x1sin * rn + expo * e2 -
              (0.5 + 0.5 * ef) * vt[mm + 2] * x2sin * rn;
        mm += 3;
      }
      et = et * vt[1];
      dij = dij * vt[1] * damp;
      T gla[3], glc[3], gld[3];
      for (int c = 0; c < 3; ++c) {
        T t1 = et * d2a * dampjk * dampkl * vab[c];
        T t2 = et * d2b * dampij * dampkl * vcb[c];
        T t3 = et * d2c * dampij * dampjk * vdc[c];
        gla[c] = dij * dda[c] + t1;
        glc[c] = dij * ddc[c] + t3 - t2;
        gld[c] = dij * ddd[c] - t3;
        g[3 * i + c] += gla[c];
        g[3 * j + c] += dij * ddb[c] - t1 + t2;
        g[3 * k + c] += glc[c];
        g[3 * l + c] += gld[c];
      }
      vir_tors(ff, vab, vcb, vdc, gla, glc, gld);  // src/ff_eg.f90:420-440
      e = e + et * damp;
    } else {
      for (int c = 0; c < 3; ++c) {
        vab[c] = x[3 * j + c] - x[3 * i + c];
        vcb[c] = x[3 * j + c] - x[3 * k + c];
        vdc[c] = x[3 * j + c] - x[3 * l + c];
      }
      box_image(ff, vab);
      box_image(ff, vcb);
      box_image(ff, vdc);
      T rij = vab[0] * vab[0] + vab[1] * vab[1] + vab[2] * vab[2];
      T rjk = vcb[0] * vcb[0] + vcb[1] * vcb[1] + vcb[2] * vcb[2];
      T rjl = vdc[0] * vdc[0] + vdc[1] * vdc[1] + vdc[2] * vdc[2];
      abdamp(ff.rad[i], ff.rad[j], rij, &dmp[0], &d2a);
      abdamp(ff.rad[k], ff.rad[j], rjk, &dmp[1], &d2b);
      abdamp(ff.rad[j], ff.rad[l], rjl, &dmp[2], &d2c);
      T dampij = dmp[0], dampjk = dmp[1], dampjl = dmp[2];
      damp = dampjk * dampij * dampjl;
      T phi = omega(x, i, j, k, l);
      domegadr(x, i, j, k, l, phi, dda, ddb, ddc, ddd);
      T rn = vt[2];
      if (rn > 1e-6) {
        T c1 = (phi - phi0) + pi;
        et = (1. + cos(c1)) * vt[1];
        dij = -sin(c1) * vt[1] * damp;
      } else {
        T d = cos(phi) - cos(phi0);
        et = vt[1] * (d * d);
        dij = 2. * vt[1] * sin(phi) * (cos(phi0) - cos(phi)) * damp;
      }
      T gla[3], glc[3], gld[3];
      for (int c = 0; c < 3; ++c) {
        T t1 = et * d2a * dampjk * dampjl * vab[c];
        T t2 = et * d2b * dampij * dampjl * vcb[c];
        T t3 = et * d2c * dampij * dampjk * vdc[c];
        gla[c] = dij * dda[c] - t1;
        glc[c] = dij * ddc[c] - t2;
        gld[c] = dij * ddd[c] - t3;
        g[3 * i + c] += gla[c];
        g[3 * j + c] += dij * ddb[c] + t1 + t2 + t3;
        g[3 * k + c] += glc[c];
        g[3 * l + c] += gld[c];
      }
      // the torsions' formula with the inversion's vectors, which point at
      // the centre j (src/ff_eg.f90:583-603)
      vir_tors(ff, vab, vcb, vdc, gla, glc, gld);
      e = e + et * damp;
    }
  }
  *e_out = e;
}

// ff_nonb (non-periodic, one molecule): accumulates into enb and g
template <class T>
inline void ff_nonb(const FF& ff, const T* x, T* enb, T* g) {
  T e = 0.0;
  for (int kp = 0; kp < ff.nnci; ++kp) {
    int i1 = ff.nci[3 * kp], i2 = ff.nci[3 * kp + 1], nk = ff.nci[3 * kp + 2];
    T vab[3];
    for (int c = 0; c < 3; ++c) vab[c] = x[3 * i1 + c] - x[3 * i2 + c];
    box_image(ff, vab);
    T r2 = vab[0] * vab[0] + vab[1] * vab[1] + vab[2] * vab[2];
    T r = sqrt(r2);
    if (ff.periodic && r > T(ff.vdw_cut)) continue;
    T oner = 1.0 / r;
    T R0 = ff.pR0[kp], c6 = ff.pC6[kp];
    T r4 = r2 * r2, r6 = r4 * r2;
    T R02 = R0 * R0, r06 = R02 * R02 * R02;
    T t6 = r6 + r06;
    T t8 = r6 * r2 + r06 * R0 * R0;
    T c6t6 = c6 / t6, c6t8 = c6 / t8;
    T t27 = ff.pSr42[kp] * c6t8;
    T e0 = c6t6 + t27;
    e = e - e0 * ff.eps2[nk];
    T drij = ff.eps2[nk] * (c6t6 * 6.0 * r4 / t6 + 8.0 * t27 * r6 / t8);
    T ga[3] = {vab[0] * drij, vab[1] * drij, vab[2] * drij};
    if (r < 25) {
      T xz = ff.pZab[kp], alpha = ff.pAlpha[kp];
      T t = xz * exp(-alpha * r);
      T e1 = t * oner;
      e = e + e1 * ff.eps2[nk];
      T dr2 = ff.eps2[nk] * t * (alpha * r + 1.0) * oner / r2;
      for (int c = 0; c < 3; ++c) ga[c] = ga[c] - vab[c] * dr2;
    }
    for (int c = 0; c < 3; ++c) {
      g[3 * i1 + c] += ga[c];
      g[3 * i2 + c] -= ga[c];
    }
    vir_add(ff, vab, ga);  // src/ff_nonb.f90:180-190, 318-328
  }
  for (int kp = 0; kp < ff.nnci; ++kp) {
    int i1 = ff.nci[3 * kp], i2 = ff.nci[3 * kp + 1], nk = ff.nci[3 * kp + 2];
    T vab[3];
    for (int c = 0; c < 3; ++c) vab[c] = x[3 * i1 + c] - x[3 * i2 + c];
    box_image(ff, vab);
    T r2 = vab[0] * vab[0] + vab[1] * vab[1] + vab[2] * vab[2];
    T r = sqrt(r2);
    if (r > ff.coul_cut) continue;
    T oner = 1.0 / r;
    T e0;
    if (ff.zahn)
      e0 = ff.q[i1] * ff.q[i2] * ((erfc(ff.zahn_a * r) * oner) - ff.zahn_par * (r - ff.coul_cut));
    else
      e0 = ff.q[i1] * ff.q[i2] * oner * ff.eps1[nk] * 1.0;
    e = e + e0;
    T drij = e0 / r2;
    T ga[3];
    for (int c = 0; c < 3; ++c) {
      ga[c] = -vab[c] * drij;
      g[3 * i1 + c] += ga[c];
      g[3 * i2 + c] -= ga[c];
    }
    vir_add(ff, vab, ga);  // src/ff_nonb.f90:405-415, 495-505
  }
  *enb = *enb + e;
}

// eabhag (src/eabhag.f90:35-220): one hydrogen bond A...H-B, energy and
// analytic gradient accumulated into e, g; nothing if E > -1e-8.
template <class T>
inline void eabhag(const FF& ff, const T* x, int A, int B, int H, double ca, double cb, T* e, T* g) {
  const double longcut = 8.0, alp7 = 12.0, alp3 = 6.0;
  T drah[3], drbh[3], drab[3];
  for (int c = 0; c < 3; ++c) {
    drah[c] = x[3 * A + c] - x[3 * H + c];
    drbh[c] = x[3 * B + c] - x[3 * H + c];
    drab[c] = x[3 * A + c] - x[3 * B + c];
  }
  box_image(ff, drah);  // as src/eabhag.f90:60-62 (the A-H vector only)
  T rab2 = drab[0] * drab[0] + drab[1] * drab[1] + drab[2] * drab[2];
  T rab = sqrt(rab2);
  T rah2 = drah[0] * drah[0] + drah[1] * drah[1] + drah[2] * drah[2];
  T rah = sqrt(rah2);
  T rbh2 = drbh[0] * drbh[0] + drbh[1] * drbh[1] + drbh[2] * drbh[2];
  T rbh = sqrt(rbh2);
  T ratio = pow(rab / longcut, T(alp7));
  T rdampl = 1.0 / (1.0 + ratio);
  rdampl = rdampl / rab2 / rab;
  T cosabh, aprod;
  const bool far_a = rah2 > rbh2;
  if (far_a) {
    aprod = 1.0 / rbh / rab;
    cosabh = -(drbh[0] * drab[0] + drbh[1] * drab[1] + drbh[2] * drab[2]) * aprod;
  } else {
    aprod = 1.0 / rah / rab;
    cosabh = (drah[0] * drab[0] + drah[1] * drab[1] + drah[2] * drab[2]) * aprod;
  }
  T aterm = 0.5 * (cosabh + 1.0);
  T apref = pow(aterm, T(alp3 - 1));
  aterm = aterm * apref;
  apref = alp3 * 0.5 * apref;
  T rah4 = rah2 * rah2, rbh4 = rbh2 * rbh2;
  T denom = 1.0 / (rah4 + rbh4);
  T da = (ca * rah4 + cb * rbh4) * denom;
  T eabh = -da * rdampl * aterm;
  if (eabh > -1.0e-8) return;
  *e = *e + eabh;
  T ga[3], gb[3], gh[3], dg[3], dg2[3];
  T gi = 4.0 * (ca - cb) * rah2 * rbh4 * denom * denom;
  gi = -gi * rdampl * aterm;
  for (int c = 0; c < 3; ++c) ga[c] = gi * drah[c];
  gi = 4.0 * (cb - ca) * rbh2 * rah4 * denom * denom;
  gi = -gi * rdampl * aterm;
  for (int c = 0; c < 3; ++c) {
    gb[c] = gi * drbh[c];
    gh[c] = -ga[c] - gb[c];
  }
  gi = rdampl * rdampl * rab * (3.0 + (3.0 + alp7) * ratio);
  gi = gi * da * aterm;
  for (int c = 0; c < 3; ++c) {
    dg[c] = gi * drab[c];
    ga[c] = ga[c] + dg[c];
    gb[c] = gb[c] - dg[c];
  }
  gi = -da * rdampl * apref;
  if (far_a) {
    for (int c = 0; c < 3; ++c) {
      dg[c] = -aprod * drbh[c] - cosabh * drab[c] / rab2;
      dg2[c] = aprod * drab[c] + cosabh * drbh[c] / rbh2;
      dg[c] = gi * dg[c];
      dg2[c] = gi * dg2[c];
      ga[c] = ga[c] + dg[c];
      gh[c] = gh[c] + dg2[c];
      gb[c] = gb[c] - dg[c] - dg2[c];
    }
  } else {
    for (int c = 0; c < 3; ++c) {
      dg[c] = -aprod * drah[c] + cosabh * drab[c] / rab2;
      dg2[c] = -aprod * drab[c] + cosabh * drah[c] / rah2;
      dg[c] = gi * dg[c];
      dg2[c] = gi * dg2[c];
      gb[c] = gb[c] + dg[c];
      gh[c] = gh[c] + dg2[c];
      ga[c] = ga[c] - dg[c] - dg2[c];
    }
  }
  for (int c = 0; c < 3; ++c) {
    g[3 * A + c] += ga[c];
    g[3 * B + c] += gb[c];
    g[3 * H + c] += gh[c];
  }
  vir_add(ff, drah, ga);  // src/eabhag.f90:203-216
  vir_add(ff, drbh, gb);
}

// eabx (src/eabx.f90:34-111): halogen-bond energy of A...X-B (X = H arg).
template <class T>
inline T eabx(const T* x, int A, int B, int H, double ca) {
  const double longcut = 120.0, alp7 = 6.0, alp3 = 6.0;
  T rb[3];
  for (int c = 0; c < 3; ++c) rb[c] = x[3 * A + c] - x[3 * B + c];
  T rab2 = rb[0] * rb[0] + rb[1] * rb[1] + rb[2] * rb[2];
  T dampl = 1.0 / (1.0 + pow(rab2 / longcut, T(alp7)));
  for (int c = 0; c < 3; ++c) rb[c] = x[3 * A + c] - x[3 * H + c];
  T d2ik = rb[0] * rb[0] + rb[1] * rb[1] + rb[2] * rb[2];
  for (int c = 0; c < 3; ++c) rb[c] = x[3 * H + c] - x[3 * B + c];
  T d2jk = rb[0] * rb[0] + rb[1] * rb[1] + rb[2] * rb[2];
  T xy, term;
  if (d2ik > d2jk) {
    xy = sqrt(rab2 * d2jk);
    term = 0.5 * (rab2 + d2jk - d2ik) / xy;
  } else {
    xy = sqrt(rab2 * d2ik);
    term = 0.5 * (rab2 + d2ik - d2jk) / xy;
  }
  T aterm = pow(0.5 * (term + 1.0), T(alp3));
  return -ca * dampl * aterm / d2jk;
}

// eabxag (src/eabxag.f90:35-156): energy plus Caracal's difference quotients
// (step 1e-6); each atom's three components all get the z-direction quotient.
// The virial (src/eabxag.f90:86-87, 140-153) pairs (r_A - r_X) with A's
// gradient and (r_B - r_X) with the X atom's, raw coordinates.
template <class T>
inline void eabxag(const T* x0, int n, int A, int B, int H, double ca, T* e, T* g, const FF* ffv = nullptr) {
  std::vector<T> x(x0, x0 + 3 * n);
  *e = *e + eabx<T>(x.data(), A, B, H, ca);
  const double step = 1.0e-6;
  const double dum = 1.0 / (2.0 * step);
  const int atoms[3] = {A, B, H};
  T lastq[3];
  for (int ia = 0; ia < 3; ++ia) {
    const int at = atoms[ia];
    T last = 0.0;
    for (int j = 0; j < 3; ++j) {
      x[3 * at + j] = x[3 * at + j] + step;
      T er = eabx<T>(x.data(), A, B, H, ca);
      x[3 * at + j] = x[3 * at + j] - step * 2.0;
      T el = eabx<T>(x.data(), A, B, H, ca);
      x[3 * at + j] = x[3 * at + j] + step;
      last = (er - el) * dum;
    }
    for (int c = 0; c < 3; ++c) g[3 * at + c] += last;
    lastq[ia] = last;
  }
  if (ffv) {
    T vah[3], vbh[3], gA[3], gH[3];
    for (int c = 0; c < 3; ++c) {
      vah[c] = x0[3 * A + c] - x0[3 * H + c];
      vbh[c] = x0[3 * B + c] - x0[3 * H + c];
      gA[c] = lastq[0];
      gH[c] = lastq[2];
    }
    vir_add(*ffv, vah, gA);
    vir_add(*ffv, vbh, gH);
  }
}

// ff_hb (src/ff_hb.f90:36-93) for one molecule: the listed triples, skipped
// beyond 15 bohr between A and B.
template <class T>
inline void ff_hb(const FF& ff, const T* x, T* eh, T* g) {
  for (int k = 0; k < ff.nhb; ++k) {
    const int i1 = ff.hb[3 * k], i2 = ff.hb[3 * k + 1], i = ff.hb[3 * k + 2];
    T rb[3];
    for (int c = 0; c < 3; ++c) rb[c] = x[3 * i1 + c] - x[3 * i2 + c];
    box_image(ff, rb);
    T r = sqrt(rb[0] * rb[0] + rb[1] * rb[1] + rb[2] * rb[2]);
    if (r > 15.0) continue;
    if (ff.at[i] == 1) eabhag<T>(ff, x, i1, i2, i, ff.vhb[2 * k], ff.vhb[2 * k + 1], eh, g);
    else eabxag<T>(x, ff.n, i1, i2, i, ff.vhb[2 * k], eh, g, &ff);
  }
}

// gradient dispatch for one QMDFF (src/gradient.f90:342-358)
template <class T>
inline void egrad(const FF& ff, const T* x, T* V, T* g) {
  T e;
  ff_eg(ff, x, &e, g);
  ff_nonb(ff, x, &e, g);
  ff_hb(ff, x, &e, g);
  *V = e + ff.e_zero;
}

}  // namespace qmdff
}  // namespace orc
