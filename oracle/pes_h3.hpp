// ORACLE (test infrastructure only) -- BKMP2 H3 potential, CPU restatement.
//
// Restates Caracal's src/egrad_h3.f: the Boothroyd-Keogh-Martin-Peterson
// (J. Chem. Phys. 95, 4343 (1991); 104, 7139 (1996)) H3 surface with the
// JUN21/95 parameter set.  Function-by-function map:
//   egrad_h3   src/egrad_h3.f:29-77     distances -> pote -> Cartesian chain rule
//   pote       src/egrad_h3.f:79-248    sum of all parts
//   triplet    src/egrad_h3.f:251-319   TRIPLET95
//   singlet    src/egrad_h3.f:322-416   VH2OPT95 (Schwenke H2 curve)
//   london     src/egrad_h3.f:419-479   H3LOND95
//   vascal     src/egrad_h3.f:482-546   VASCAL95
//   acalc      src/egrad_h3.f:549-573   ACALC95
//   compac     src/egrad_h3.f:576-608   COMPAC95
//   casym      src/egrad_h3.f:611-704   CASYM95
//   csym       src/egrad_h3.f:707-771   CSYM95
//   vbcb       src/egrad_h3.f:774-1429  VBCB95
// CHGEOM (src/egrad_h3.f:1432-1476) only prints warnings (its IVALID
// assignments are commented out), so it has no effect on the result.
//
// Precision: the file is compiled with IMPLICIT DOUBLE PRECISION but without
// -fdefault-real-8 (Makefile:44), so every PARAMETER constant written without
// a D exponent is a REAL(4) literal widened to double.  R4() reproduces that
// widening; D8() marks genuine double constants.  The second derivative that
// VH2OPT95 computes when IDERIV=2 never reaches the outputs and is omitted,
// and TRIPLET95's second VH2OPT95 call on the same distance reuses the value
// from the London term (bitwise the same numbers).
#pragma once
#include <cmath>

#define R4(x) ((double)(x##f))
#define D8(x) ((double)(x))

namespace orc {
namespace h3 {

using std::exp;
using std::pow;
using std::sqrt;
using std::fabs;

// ---- Schwenke H2 singlet curve (VH2OPT95) --------------------------------
// returns E and dE/dR
template <class T>
inline void singlet(T R, T* E, T* dE) {
  const double a[17] = {
      R4(0.03537359271649620),  R4(2.013977588700072),   R4(-2.827452449964767),
      R4(2.713257715593500),    R4(-2.792039234205731),  R4(2.166542078766724),
      R4(-1.272679684173909),   R4(0.5630423099212294),  R4(-0.1879397372273814),
      R4(0.04719891893374140),  R4(-0.008851622656489644), R4(0.001224998776243630),
      D8(-1.227820520228028e-04), D8(8.638783190083473e-06), D8(-4.036967926499151e-07),
      D8(1.123286608335365e-08), D8(-1.406619156782167e-10)};
  const double R0 = D8(3.5284882), DD = D8(0.160979391);
  const double C6 = D8(6.499027), C8 = D8(124.3991), C10 = D8(3285.828);
  T r2 = R * R, r3 = r2 * R, r4 = r3 * R, r5 = r4 * R, r6 = r5 * R, r7 = r6 * R;
  T r8 = r7 * R, r9 = r8 * R, r10 = r9 * R, r11 = r10 * R, r12 = r11 * R;
  T r13 = r12 * R, r14 = r13 * R, r15 = r14 * R;
  double r02 = R0 * R0, r04 = r02 * r02, r06 = r04 * r02;
  T rr2 = r2 + r02, rr4 = r4 + r04, rr6 = r6 + r06;
  T rr25 = rr2 * rr2 * rr2 * rr2 * rr2;
  T alpha = a[0] / R + a[1] + a[2] * R + a[3] * r2 + a[4] * r3 + a[5] * r4 + a[6] * r5 +
            a[7] * r6 + a[8] * r7 + a[9] * r8 + a[10] * r9 + a[11] * r10 + a[12] * r11 +
            a[13] * r12 + a[14] * r13 + a[15] * r14 + a[16] * r15;
  T ea = exp(alpha);
  T vsr = DD * (ea - 1.0) * (ea - 1.0) - DD;
  T vlr = -C6 / rr6 - C8 / (rr4 * rr4) - C10 / rr25;
  *E = vsr + vlr;
  // first derivative (the source recomputes r3, r5 identically)
  T rr26 = rr25 * rr2;
  T rr43 = rr4 * rr4 * rr4;
  T dalpha = -a[0] / r2 + a[2] + 2.0 * a[3] * R + 3.0 * a[4] * r2 + 4.0 * a[5] * r3 +
             5.0 * a[6] * r4 + 6.0 * a[7] * r5 + 7.0 * a[8] * r6 + 8.0 * a[9] * r7 +
             9.0 * a[10] * r8 + 10.0 * a[11] * r9 + 11.0 * a[12] * r10 +
             12.0 * a[13] * r11 + 13.0 * a[14] * r12 + 14.0 * a[15] * r13 +
             15.0 * a[16] * r14;
  T dvsr = 2.0 * DD * (ea - 1.0) * ea * dalpha;
  T dvlr = 6.0 * C6 * r5 / (rr6 * rr6) + 8.0 * C8 * r3 / rr43 + 10.0 * C10 * R / rr26;
  *dE = dvsr + dvlr;
}

// ---- H2 triplet curve (TRIPLET95), given the singlet at the same R --------
template <class T>
inline void triplet(T R, T e1, T de1, T* E3, T* dE3) {
  const double RL = D8(0.95), RR = D8(1.15);
  const double A1 = R4(-0.0298546962), A2 = R4(-23.9604445036), A3 = R4(-42.5185569474);
  const double A4 = R4(2.0382390988), A5 = R4(-11.5214861455), A6 = R4(1.5309487826);
  const double C1 = R4(-0.4106358351531854), C2 = R4(-0.0770355790707090);
  const double C3 = R4(0.4303193846943223);
  if (R >= RR) {
    T exdr = exp(-A4 * R);
    T rsq = R * R;
    T ra6 = pow(R, T(-A6));
    *E3 = A1 * (A2 + R + A3 * rsq + A5 * ra6) * exdr;
    T ra61 = pow(R, T(-A6 - 1.0));
    *dE3 = A1 * exdr *
           (1.0 - A2 * A4 + (2.0 * A3 - A4) * R - A3 * A4 * rsq - A5 * A6 * ra61 -
            A4 * A5 * ra6);
  } else {
    T dr = R - RL;
    if (R <= RL) {
      *E3 = e1 + C2 * dr + C3;
      *dE3 = de1 + C2;
    } else {
      *E3 = e1 + C1 * dr * dr * dr + C2 * dr + C3;
      *dE3 = de1 + 3.0 * C1 * dr * dr + C2;
    }
  }
}

// ---- London term (H3LOND95) ----------------------------------------------
template <class T>
inline void london(const T R[3], T* V, T dV[3]) {
  T e1[3], de1[3], e3[3], de3[3], Q[3], J[3];
  for (int i = 0; i < 3; ++i) {
    singlet(R[i], &e1[i], &de1[i]);
    triplet(R[i], e1[i], de1[i], &e3[i], &de3[i]);
    Q[i] = 0.5 * (e1[i] + e3[i]);
    J[i] = 0.5 * (e1[i] - e3[i]);
  }
  T sumq = Q[0] + Q[1] + Q[2];
  T d21 = fabs(J[1] - J[0]), d32 = fabs(J[2] - J[1]), d31 = fabs(J[2] - J[0]);
  T sumj = d21 * d21 + d32 * d32 + d31 * d31;
  T jt = 0.5 * sumj + D8(1.0e-12);
  T rootjt = sqrt(jt);
  *V = sumq - rootjt;
  dV[0] = 0.5 * (de1[0] + de3[0]) - 0.25 * (2.0 * J[0] - J[1] - J[2]) * (de1[0] - de3[0]) / rootjt;
  dV[1] = 0.5 * (de1[1] + de3[1]) - 0.25 * (2.0 * J[1] - J[2] - J[0]) * (de1[1] - de3[1]) / rootjt;
  dV[2] = 0.5 * (de1[2] + de3[2]) - 0.25 * (2.0 * J[2] - J[0] - J[1]) * (de1[2] - de3[2]) / rootjt;
}

// ---- A = |(r1-r2)(r2-r3)(r3-r1)| and its gradient (ACALC95) ----------------
template <class T>
inline void acalc(T r1, T r2, T r3, T* A, T dA[3]) {
  T a = (r1 - r2) * (r2 - r3) * (r3 - r1);
  dA[0] = (-2.0 * r1 + r2 + r3) * (r2 - r3);
  dA[1] = (-2.0 * r2 + r3 + r1) * (r3 - r1);
  dA[2] = (-2.0 * r3 + r1 + r2) * (r1 - r2);
  if (a < 0.0) {
    a = -a;
    dA[0] = -dA[0];
    dA[1] = -dA[1];
    dA[2] = -dA[2];
  }
  *A = a;
}

// ---- asymmetric correction (VASCAL95) -------------------------------------
template <class T>
inline void vascal(const T Rp[3], T* V, T dV[3]) {
  const double AA1 = R4(0.3788951192E-02), AA2 = R4(0.1478100901E-02);
  const double AA3 = R4(-.1848513849E-03), AA4 = R4(0.9230803609E-05);
  const double AA5 = R4(-.1293180255E-06), AA6 = R4(0.5237179303E+00);
  const double AA7 = R4(-.1112326215E-02);
  T R = Rp[0] + Rp[1] + Rp[2];
  T rsq = R * R;
  T rcu = rsq * R;
  T A, dA[3];
  acalc(Rp[0], Rp[1], Rp[2], &A, dA);
  T a2 = A * A, a3 = a2 * A, a4 = a3 * A, a5 = a4 * A;
  T exp1 = exp(-AA1 * rcu);
  T exp6 = exp(-AA6 * R);
  T S = AA2 * a2 + AA3 * a3 + AA4 * a4 + AA5 * a5;
  *V = S * exp1 + AA7 * a2 * exp6 / R;
  for (int i = 0; i < 3; ++i) {
    T ds = (2.0 * AA2 * A + 3.0 * AA3 * a2 + 4.0 * AA4 * a3 + 5.0 * AA5 * a4) * dA[i];
    dV[i] = -3.0 * AA1 * rsq * S * exp1 + ds * exp1 - AA7 * a2 * exp6 / rsq +
            2.0 * AA7 * A * dA[i] * exp6 / R - AA6 * AA7 * a2 * exp6 / R;
  }
}

// ---- compactness switch (COMPAC95) ---------------------------------------
template <class T>
inline int compac(const T R[3], T t[3], T dt[3]) {
  const double RR = D8(1.15), RP = D8(1.25);
  int nc = 0;
  for (int i = 0; i < 3; ++i) {
    t[i] = 0.0;
    dt[i] = 0.0;
  }
  for (int i = 0; i < 3; ++i)
    if (R[i] < RR) nc++;
  if (nc == 0) return 0;
  for (int i = 0; i < 3; ++i) {
    if (R[i] < RR) {
      T top = RR - R[i];
      T bot = RP - R[i];
      T top2 = top * top, top3 = top2 * top, bot2 = bot * bot;
      t[i] = top3 / bot;
      dt[i] = -3.0 * top2 / bot + top3 / bot2;
    }
  }
  return nc;
}

// ---- compact asymmetric correction (CASYM95) --------------------------------
template <class T>
inline void casym(const T R[3], T* V, T dV[3], const T t[3], const T dt[3]) {
  const double U1 = R4(0.2210243144E+00), U2 = R4(0.4367417579E+00), U3 = R4(0.6994985432E-02);
  const double U4 = R4(0.1491096501E+01), U5 = R4(0.1602896673E+01), U6 = R4(-.2821747323E+01);
  const double U7 = R4(0.4948310833E+00), U8 = R4(-.3540394679E-01), U9 = R4(-.3305809954E+01);
  const double U10 = R4(0.3644382172E+01), U11 = R4(-.9997570970E+00), U12 = R4(0.7989919534E-01);
  const double U13 = R4(-.1075807322E-02);
  T A, dA[3];
  acalc(R[0], R[1], R[2], &A, dA);
  T a2 = A * A;
  T sumt = t[0] + t[1] + t[2];
  T sr = R[0] + R[1] + R[2];
  T pr = R[0] * R[1] * R[2];
  T sr2 = sr * sr, sr3 = sr2 * sr;
  T pr2 = pr * pr, pr3 = pr2 * pr;
  T series = 1.0 + U4 / pr2 + U5 / pr + U6 + U7 * pr + U8 * pr2 +
             A * (U9 / pr2 + U10 / pr + U11 + U12 * pr + U13 * pr2);
  T term1 = U1 / pow(pr, T(U2));
  T eterm = exp(-U3 * sr3);
  *V = sumt * a2 * term1 * series * eterm;
  T dpr[3] = {R[1] * R[2], R[2] * R[0], R[0] * R[1]};
  for (int i = 0; i < 3; ++i) {
    T dterm1 = -1.0 * U1 * U2 * pow(pr, T(-U2 - 1.0)) * dpr[i];
    T determ = eterm * (-3.0 * U3 * sr2);
    T dseries = dpr[i] * (-2.0 * U4 / pr3 - U5 / pr2 + U7 + 2.0 * U8 * pr) +
                dA[i] * (U9 / pr2 + U10 / pr + U11 + U12 * pr + U13 * pr2) +
                A * dpr[i] * (-2.0 * U9 / pr3 - U10 / pr2 + U12 + 2.0 * U13 * pr);
    dV[i] = dt[i] * a2 * term1 * series * eterm + 2.0 * A * dA[i] * sumt * term1 * series * eterm +
            dterm1 * sumt * a2 * series * eterm + dseries * sumt * a2 * term1 * eterm +
            determ * sumt * a2 * term1 * series;
  }
}

// ---- compact symmetric correction (CSYM95) --------------------------------
template <class T>
inline void csym(const T R[3], T* V, T dV[3]) {
  const double RR = D8(1.15), RP = D8(1.25);
  const double V1 = R4(-.2071708868E+00), V2 = R4(-.5672350377E+00), V3 = R4(0.9058780367E-02);
  T sr = R[0] + R[1] + R[2];
  T sr2 = sr * sr;
  T sr3 = sr * sr2;
  T exp3 = exp(-V3 * sr3);
  T dexp3 = -3.0 * V3 * sr2 * exp3;
  T g[3], dg[3];
  for (int i = 0; i < 3; ++i) {
    T ri = R[i];
    T a = RR - ri, a2 = a * a, a3 = a * a2;
    T b = RP - ri, b2 = b * b;
    g[i] = 0.0;
    dg[i] = 0.0;
    T sumv = V1 + V1 * V2 * ri;
    if (ri < RR) {
      g[i] = (a3 / b) * sumv;
      dg[i] = (a3 / b2) * sumv - 3.0 * (a2 / b) * sumv + (a3 / b) * V1 * V2;
    }
  }
  T sumg = g[0] + g[1] + g[2];
  *V = sumg * exp3;
  for (int i = 0; i < 3; ++i) dV[i] = dg[i] * exp3 + sumg * dexp3;
}

// ---- bend terms VBNDA/VBNDB and compact bend terms CBNDA/CBNDB (VBCB95) ----
struct BendCoef {  // one set of VBEND coefficients (A or G)
  double s11, s12, s13, s21, s22, s23, s24, s31, s32, s41, s42, s43, s44, s51, s52, s53;
};
struct CBendCoef {  // one set of CBEND coefficients (C or D)
  double s11, s12, s13, s14, s15, s21, s22, s23, s24, s31, s32, s41, s42, s43, s44;
  double s51, s52, s53, s61, s62, s63, s71, s72, s73, s74, s75, s81, s82, s83, s84;
};

inline const BendCoef& vbend_a() {
  static const BendCoef c = {
      R4(-.1838073394E+03), R4(0.1334593242E+02), R4(-.2358129537E+00), R4(-.4668193478E+01),
      R4(0.7197506670E+01), R4(0.2162004275E+02), R4(0.2106294028E+02), R4(0.4242962586E+01),
      R4(0.4453505045E+01), R4(-.1456918088E+00), R4(-.1692657366E-01), R4(0.1279520698E+01),
      R4(-.4898940075E+00), R4(0.1742295219E+03), R4(0.3142175348E+02), R4(0.5152903406E+01)};
  return c;
}
inline const BendCoef& vbend_b() {
  static const BendCoef c = {
      R4(-.4765732725E+02), R4(0.3648933563E+01), R4(-.7141145244E-01), R4(0.1002349176E-01),
      R4(0.9989856329E-02), R4(-.4161953634E-02), R4(0.9075807910E-03), R4(-.2693628729E+00),
      R4(-.1399065763E-01), R4(-.1417634346E-01), R4(-.4870024792E-03), R4(0.1312231847E+00),
      R4(-.4409850519E-01), R4(0.5382970863E+02), R4(0.4587102824E+01), R4(0.1768550515E+01)};
  return c;
}
inline const CBendCoef& cbend_a() {
  static const CBendCoef c = {
      R4(0.1860299931E+04), R4(-.6134458037E+03), R4(0.7337207161E+02), R4(-.2676717625E+04),
      R4(0.1344099415E+04), R4(0.1538913137E+03), R4(0.4348007369E+02), R4(0.1719720677E+03),
      R4(0.2115963042E+03), R4(-.7026089414E+02), R4(-.1300938992E+03), R4(0.1310273564E+01),
      R4(-.6175149574E+00), R4(-.2679089358E+02), R4(0.5577477171E+01), R4(-.3543353539E+04),
      R4(-.3740709591E+03), R4(0.7979303144E+02), R4(-.1104230585E+04), R4(0.4603572025E+04),
      R4(-.5593496634E+04), R4(-.1069406434E+02), R4(0.1021807153E+01), R4(0.6669828341E-01),
      R4(0.4168542348E+02), R4(0.1751608567E+02), R4(0.9486883238E+02), R4(-.1519334221E+02),
      R4(0.4024697252E+04), R4(-.2225159395E+02)};
  return c;
}
inline const CBendCoef& cbend_b() {
  static const CBendCoef c = {
      R4(0.4203543357E+03), R4(-.4922474096E+02), R4(0.3362942544E+00), R4(-.3827423082E+03),
      R4(0.1746726001E+03), R4(0.1699995737E-01), R4(0.1513036778E-01), R4(0.2659119354E-01),
      R4(-.5760387483E-02), R4(0.1020622621E+02), R4(0.1050536271E-01), R4(0.6836172780E+00),
      R4(-.1627858240E+00), R4(-.6925485045E+01), R4(0.1632567385E+01), R4(0.1083595009E+04),
      R4(0.4641431791E+01), R4(-.8233144461E+00), R4(-.6157225942E+02), R4(0.3094361471E+03),
      R4(-.3299631143E+03), R4(0.8866227120E+01), R4(-.1382126854E+01), R4(0.7620770145E-01),
      R4(-.5145757859E+02), R4(0.2046097265E+01), R4(0.2540775558E+01), R4(-.4889246569E+00),
      R4(-.1127439280E+04), R4(-.2269932295E+01)};
  return c;
}

// Quantities shared by the four bend sums.
template <class T>
struct BendShared {
  T b1a, b1b, db1a[3], db1b[3];
  T R, rsq, b2, b3, b3b, db2[3], db3[6];
  T exp1, exp2, exp7, dexp1, dexp2, dexp7;
};

template <class T>
inline void bend_shared(const T Rp[3], BendShared<T>& s) {
  const double Z58 = D8(0.625), Z38 = D8(0.375);
  const double BETA1 = D8(0.52), BETA2 = D8(0.052), BETA3 = D8(0.79);
  T r1 = Rp[0], r2 = Rp[1], r3 = Rp[2];
  T t1 = r1 * r1 - r2 * r2 - r3 * r3;
  T t2 = r2 * r2 - r3 * r3 - r1 * r1;
  T t3 = r3 * r3 - r1 * r1 - r2 * r2;
  T c1 = t1 / (-2.0 * r2 * r3);
  T c2 = t2 / (-2.0 * r3 * r1);
  T c3 = t3 / (-2.0 * r1 * r2);
  T sum = c1 + c2 + c3;
  s.b1a = 1.0 - sum;
  T c1c = c1 * c1 * c1, c2c = c2 * c2 * c2, c3c = c3 * c3 * c3;
  T cos3t1 = 4.0 * c1c - 3.0 * c1;
  T cos3t2 = 4.0 * c2c - 3.0 * c2;
  T cos3t3 = 4.0 * c3c - 3.0 * c3;
  T sumb = cos3t1 + cos3t2 + cos3t3;
  s.b1b = 1.0 - (Z58 * sumb + Z38 * sum);
  T dc1dr1 = -r1 / (r2 * r3);
  T dc2dr2 = -r2 / (r1 * r3);
  T dc3dr3 = -r3 / (r1 * r2);
  T dc1dr2 = (t1 / (r2 * r2) + 2.0) / (2.0 * r3);
  T dc1dr3 = (t1 / (r3 * r3) + 2.0) / (2.0 * r2);
  T dc2dr1 = (t2 / (r1 * r1) + 2.0) / (2.0 * r3);
  T dc2dr3 = (t2 / (r3 * r3) + 2.0) / (2.0 * r1);
  T dc3dr1 = (t3 / (r1 * r1) + 2.0) / (2.0 * r2);
  T dc3dr2 = (t3 / (r2 * r2) + 2.0) / (2.0 * r1);
  s.db1a[0] = -1.0 * (dc1dr1 + dc2dr1 + dc3dr1);
  s.db1a[1] = -1.0 * (dc1dr2 + dc2dr2 + dc3dr2);
  s.db1a[2] = -1.0 * (dc1dr3 + dc2dr3 + dc3dr3);
  T d1 = 12.0 * c1 * c1 - 3.0;
  T d2 = 12.0 * c2 * c2 - 3.0;
  T d3 = 12.0 * c3 * c3 - 3.0;
  s.db1b[0] = -Z58 * (d1 * dc1dr1 + d2 * dc2dr1 + d3 * dc3dr1) - Z38 * (dc1dr1 + dc2dr1 + dc3dr1);
  s.db1b[1] = -Z58 * (d1 * dc1dr2 + d2 * dc2dr2 + d3 * dc3dr2) - Z38 * (dc1dr2 + dc2dr2 + dc3dr2);
  s.db1b[2] = -Z58 * (d1 * dc1dr3 + d2 * dc2dr3 + d3 * dc3dr3) - Z38 * (dc1dr3 + dc2dr3 + dc3dr3);
  s.R = r1 + r2 + r3;
  s.rsq = s.R * s.R;
  s.b2 = 1.0 / r1 + 1.0 / r2 + 1.0 / r3;
  s.b3 = (r2 - r1) * (r2 - r1) + (r3 - r2) * (r3 - r2) + (r1 - r3) * (r1 - r3);
  s.b3b = sqrt(s.b3 + D8(1.0e-12));
  s.db2[0] = -1.0 / (r1 * r1);
  s.db2[1] = -1.0 / (r2 * r2);
  s.db2[2] = -1.0 / (r3 * r3);
  s.db3[0] = 4.0 * r1 - 2.0 * r2 - 2.0 * r3;
  s.db3[1] = 4.0 * r2 - 2.0 * r3 - 2.0 * r1;
  s.db3[2] = 4.0 * r3 - 2.0 * r1 - 2.0 * r2;
  s.db3[3] = 0.5 * s.db3[0] / s.b3b;
  s.db3[4] = 0.5 * s.db3[1] / s.b3b;
  s.db3[5] = 0.5 * s.db3[2] / s.b3b;
  s.exp1 = exp(-BETA1 * s.R);
  s.exp2 = exp(-BETA2 * s.rsq);
  s.exp7 = exp(-BETA3 * s.R);
  s.dexp1 = -BETA1 * s.exp1;
  s.dexp2 = -2.0 * BETA2 * s.R * s.exp2;
  s.dexp7 = -BETA3 * s.exp7;
}

// One VBEND sum for bend variable B1 (B1A or B1B) with coefficient set k.
template <class T>
inline void vbend(const BendShared<T>& s, T B1, const T dB1[3], const BendCoef& k, T* V, T dV[3]) {
  T R = s.R, rsq = s.rsq;
  T b12 = B1 * B1, b13 = b12 * B1, b14 = b13 * B1, b15 = b14 * B1;
  T asum = k.s11 + k.s12 * R + k.s13 * rsq;
  T bsum = k.s21 * b12 + k.s22 * b13 + k.s23 * b14 + k.s24 * b15;
  T csum = k.s31 * B1 * s.exp1 + k.s32 * b12 * s.exp2;
  T dsum1 = k.s41 * s.exp1 + k.s42 * s.exp2;
  T dsum2 = k.s43 * s.exp1 + k.s44 * s.exp2;
  T fsum = k.s51 + k.s52 * R + k.s53 * rsq;
  T vb1 = B1 * asum * s.exp1;
  T vb2 = bsum * s.exp2;
  T vb3 = s.b2 * csum;
  T vb4 = B1 * s.b3 * dsum1 + B1 * s.b3b * dsum2;
  T vb5 = B1 * fsum * s.exp7;
  *V = vb1 + vb2 + vb3 + vb4 + vb5;
  T dasum = k.s12 + 2.0 * k.s13 * R;
  T dbsum = 2.0 * k.s21 * B1 + 3.0 * k.s22 * b12 + 4.0 * k.s23 * b13 + 5.0 * k.s24 * b14;
  T ddsum1 = k.s41 * s.dexp1 + k.s42 * s.dexp2;
  T ddsum2 = k.s43 * s.dexp1 + k.s44 * s.dexp2;
  T dfsum = k.s52 + 2.0 * k.s53 * R;
  for (int i = 0; i < 3; ++i) {
    T d1 = dB1[i] * asum * s.exp1 + B1 * dasum * s.exp1 + B1 * asum * s.dexp1;
    T d2 = dbsum * dB1[i] * s.exp2 + bsum * s.dexp2;
    T d3 = s.db2[i] * csum + s.b2 * (k.s31 * dB1[i] * s.exp1 + k.s31 * B1 * s.dexp1 +
                                     2.0 * k.s32 * B1 * dB1[i] * s.exp2 + k.s32 * b12 * s.dexp2);
    T d4 = dB1[i] * s.b3 * dsum1 + B1 * s.db3[i] * dsum1 + B1 * s.b3 * ddsum1 +
           dB1[i] * s.b3b * dsum2 + B1 * s.db3[3 + i] * dsum2 + B1 * s.b3b * ddsum2;
    T d5 = dB1[i] * fsum * s.exp7 + B1 * dfsum * s.exp7 + B1 * fsum * s.dexp7;
    dV[i] = d1 + d2 + d3 + d4 + d5;
  }
}

// One CBEND sum (before the SUMT factor) for bend variable B1.
template <class T>
inline void cbend(const BendShared<T>& s, const T Rp[3], T B1, const T dB1[3], const CBendCoef& k,
                  T exp7c, T dexp7c, T* C, T dC[3]) {
  T R = s.R, rsq = s.rsq, rcu = rsq * R;
  T P = Rp[0] * Rp[1] * Rp[2];
  T psq = P * P, pcu = psq * P;
  T dp[3] = {Rp[1] * Rp[2], Rp[2] * Rp[0], Rp[0] * Rp[1]};
  double cx1 = k.s51 + k.s83;  // FEB27/91: new C51 = C51 + C83
  T b12 = B1 * B1, b13 = b12 * B1, b14 = b13 * B1, b15 = b14 * B1;
  T asum = k.s11 + k.s12 * R + k.s13 * rsq + k.s14 / R + k.s15 / rsq;
  T bsum = k.s21 * b12 + k.s22 * b13 + k.s23 * b14 + k.s24 * b15;
  T csum = k.s31 * B1 * s.exp1 + k.s32 * b12 * s.exp2;
  T dsum1 = k.s41 * s.exp1 + k.s42 * s.exp2;
  T dsum2 = k.s43 * s.exp1 + k.s44 * s.exp2;
  T fsum = cx1 + k.s52 * R + k.s53 * rsq;
  T gsum = k.s61 + k.s62 / R + k.s63 / rsq;
  T aasum = k.s71 + k.s72 * P + k.s73 * psq + k.s74 / P + k.s75 / psq;
  T ffsum = k.s81 * P + k.s82 * psq + k.s84 / psq;
  T dasum = k.s12 + 2.0 * k.s13 * R - k.s14 / rsq - 2.0 * k.s15 / rcu;
  T dbsum = 2.0 * k.s21 * B1 + 3.0 * k.s22 * b12 + 4.0 * k.s23 * b13 + 5.0 * k.s24 * b14;
  T ddsum1 = k.s41 * s.dexp1 + k.s42 * s.dexp2;
  T ddsum2 = k.s43 * s.dexp1 + k.s44 * s.dexp2;
  T dfsum = k.s52 + 2.0 * k.s53 * R;
  T dgsum = -k.s62 / rsq - 2.0 * k.s63 / rcu;
  T daasum = k.s72 + 2.0 * k.s73 * P - k.s74 / psq - 2.0 * k.s75 / pcu;
  T dffsum = k.s81 + 2.0 * k.s82 * P - 2.0 * k.s84 / pcu;
  T cb1 = B1 * asum * s.exp1 / P;
  T cb2 = bsum * s.exp2;
  T cb3 = s.b2 * csum;
  T cb4 = B1 * s.b3 * dsum1 + B1 * s.b3b * dsum2;
  T cb5 = B1 * fsum * exp7c / P;
  T cb6 = B1 * gsum * exp7c;
  T cb7 = B1 * aasum * s.exp2;
  T cb8 = B1 * ffsum * exp7c;
  *C = cb1 + cb2 + cb3 + cb4 + cb5 + cb6 + cb7 + cb8;
  for (int i = 0; i < 3; ++i) {
    T d1 = dB1[i] * asum * s.exp1 / P + B1 * dasum * s.exp1 / P + B1 * asum * s.dexp1 / P -
           B1 * asum * s.exp1 * dp[i] / psq;
    T d2 = dbsum * dB1[i] * s.exp2 + bsum * s.dexp2;
    T d3 = s.db2[i] * csum + s.b2 * (k.s31 * dB1[i] * s.exp1 + k.s31 * B1 * s.dexp1 +
                                     k.s32 * 2.0 * B1 * dB1[i] * s.exp2 + k.s32 * b12 * s.dexp2);
    T d4 = dB1[i] * s.b3 * dsum1 + B1 * s.db3[i] * dsum1 + B1 * s.b3 * ddsum1 +
           dB1[i] * s.b3b * dsum2 + B1 * s.db3[3 + i] * dsum2 + B1 * s.b3b * ddsum2;
    T d5 = dB1[i] * fsum * exp7c / P + B1 * dfsum * exp7c / P + B1 * fsum * dexp7c / P -
           B1 * fsum * exp7c * dp[i] / psq;
    T d6 = dB1[i] * gsum * exp7c + B1 * dgsum * exp7c + B1 * gsum * dexp7c;
    T d7 = dB1[i] * aasum * s.exp2 + B1 * daasum * dp[i] * s.exp2 + B1 * aasum * s.dexp2;
    T d8 = dB1[i] * ffsum * exp7c + B1 * dffsum * dp[i] * exp7c + B1 * ffsum * dexp7c;
    dC[i] = d1 + d2 + d3 + d4 + d5 + d6 + d7 + d8;
  }
}

template <class T>
inline void vbcb(const T Rp[3], int ncompact, const T t[3], const T dt[3], T* vbnda, T* vbndb,
                 T dvbnda[3], T dvbndb[3], T* cbnda, T* cbndb, T dcbnda[3], T dcbndb[3]) {
  BendShared<T> s;
  bend_shared(Rp, s);
  vbend(s, s.b1a, s.db1a, vbend_a(), vbnda, dvbnda);
  vbend(s, s.b1b, s.db1b, vbend_b(), vbndb, dvbndb);
  if (ncompact == 0) return;  // CBND* keep the zeros set by the caller
  const double BETA2 = D8(0.052);
  T rcu = s.rsq * s.R;
  T exp7c = exp(-BETA2 * rcu);
  T dexp7c = -3.0 * BETA2 * s.rsq * exp7c;
  T sumt = t[0] + t[1] + t[2];
  T ca, cb, dca[3], dcb[3];
  cbend(s, Rp, s.b1a, s.db1a, cbend_a(), exp7c, dexp7c, &ca, dca);
  cbend(s, Rp, s.b1b, s.db1b, cbend_b(), exp7c, dexp7c, &cb, dcb);
  for (int i = 0; i < 3; ++i) {
    dcbnda[i] = dt[i] * ca + sumt * dca[i];
    dcbndb[i] = dt[i] * cb + sumt * dcb[i];
  }
  *cbnda = sumt * ca;
  *cbndb = sumt * cb;
}

// ---- total potential (POTE) ------------------------------------------------
template <class T>
inline void pote(const T R[3], T* V, T dV[3]) {
  T vlon, dvlon[3], vas, dvas[3];
  T cal = 0.0, cas = 0.0, vbnda = 0.0, vbndb = 0.0, cbnda = 0.0, cbndb = 0.0;
  T dcal[3], dcas[3], dvbnda[3], dvbndb[3], dcbnda[3], dcbndb[3];
  for (int i = 0; i < 3; ++i) {
    dcal[i] = 0.0;
    dcas[i] = 0.0;
    dvbnda[i] = 0.0;
    dvbndb[i] = 0.0;
    dcbnda[i] = 0.0;
    dcbndb[i] = 0.0;
  }
  london(R, &vlon, dvlon);
  vascal(R, &vas, dvas);
  T t[3], dt[3];
  int nc = compac(R, t, dt);
  if (nc >= 1) {
    csym(R, &cal, dcal);
    casym(R, &cas, dcas, t, dt);
  }
  vbcb(R, nc, t, dt, &vbnda, &vbndb, dvbnda, dvbndb, &cbnda, &cbndb, dcbnda, dcbndb);
  *V = vlon + vas + vbnda + vbndb + cal + cas + cbnda + cbndb;
  for (int i = 0; i < 3; ++i)
    dV[i] = dvlon[i] + dvas[i] + dvbnda[i] + dvbndb[i] + dcal[i] + dcas[i] + dcbnda[i] + dcbndb[i];
}

// ---- egrad_h3 for one bead: q(3,3) column-major (x,y,z per atom) ------------
template <class T>
inline void egrad_bead(const T* q, T* V, T* g) {
  T xab = q[3] - q[0], yab = q[4] - q[1], zab = q[5] - q[2];
  T rab = sqrt(xab * xab + yab * yab + zab * zab);
  T xac = q[0] - q[6], yac = q[1] - q[7], zac = q[2] - q[8];
  T rac = sqrt(xac * xac + yac * yac + zac * zac);
  T xbc = q[6] - q[3], ybc = q[7] - q[4], zbc = q[8] - q[5];
  T rbc = sqrt(xbc * xbc + ybc * ybc + zbc * zbc);
  T R[3] = {rab, rac, rbc};
  T dvdr[3];
  pote(R, V, dvdr);
  g[0] = dvdr[1] * xac / rac - dvdr[0] * xab / rab;
  g[1] = dvdr[1] * yac / rac - dvdr[0] * yab / rab;
  g[2] = dvdr[1] * zac / rac - dvdr[0] * zab / rab;
  g[3] = dvdr[0] * xab / rab - dvdr[2] * xbc / rbc;
  g[4] = dvdr[0] * yab / rab - dvdr[2] * ybc / rbc;
  g[5] = dvdr[0] * zab / rab - dvdr[2] * zbc / rbc;
  g[6] = dvdr[2] * xbc / rbc - dvdr[1] * xac / rac;
  g[7] = dvdr[2] * ybc / rbc - dvdr[1] * yac / rac;
  g[8] = dvdr[2] * zbc / rbc - dvdr[1] * zac / rac;
}

}  // namespace h3
}  // namespace orc
