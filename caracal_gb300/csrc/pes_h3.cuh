// BKMP2 H3 potential (Boothroyd, Keogh, Martin, Peterson, J. Chem. Phys. 95,
// 4343 (1991) and 104, 7139 (1996); JUN21/95 parameters) as GB300 device code.
//
// Drop-in for Caracal's egrad_h3 (src/egrad_h3.f:29-77) and its helpers
// (POTE 79, TRIPLET95 251, VH2OPT95 322, H3LOND95 419, VASCAL95 482,
// ACALC95 549, COMPAC95 576, CASYM95 611, CSYM95 707, VBCB95 774).
//
// One thread evaluates one bead.  The compute type F is double for the plain
// form and float for the mixed form.  Caracal compiles this file with
// IMPLICIT DOUBLE PRECISION but default REAL(4) literals, so every PARAMETER
// written without a D exponent is a single-precision value widened to double;
// K4() reproduces that (exact in both forms), K8() marks the genuine doubles.
//
// Restructured for the FP64 pipe (same mathematics, rounding differs at the
// 1e-16 level): Horner form of the Schwenke polynomial and its derivative,
// shared reciprocals instead of repeated divisions, pow(R,-a-1) from
// pow(R,-a)/R, the unused second derivative dropped, and the singlet curve
// evaluated once per distance (TRIPLET95 recomputes it).
#pragma once
#include <cuda_runtime.h>

#define K4(x) (F)(x##f)
#define K8(x) (F)(x)

namespace cr {
namespace h3 {

template <class F> __device__ inline F fexp(F x);
template <> __device__ inline double fexp<double>(double x) { return exp(x); }
template <> __device__ inline float fexp<float>(float x) { return expf(x); }
template <class F> __device__ inline F fpow(F x, F y);
template <> __device__ inline double fpow<double>(double x, double y) { return pow(x, y); }
template <> __device__ inline float fpow<float>(float x, float y) { return powf(x, y); }
template <class F> __device__ inline F fsqrt(F x);
template <> __device__ inline double fsqrt<double>(double x) { return sqrt(x); }
template <> __device__ inline float fsqrt<float>(float x) { return sqrtf(x); }
template <class F> __device__ inline F frcp(F x) { return F(1) / x; }

// Schwenke H2 singlet E(R) and dE/dR (VH2OPT95).
// The polynomial alpha(R) of the Schwenke curve sums terms up to ~1e6 at
// R ~ 12 bohr that cancel to ~-25, so even the rounding of R to float moves
// exp(alpha) by orders of magnitude: alpha and dalpha/dR are always evaluated
// in FP64 from the FP64 distance Rd; the rest follows the compute type F.
template <class F>
__device__ inline void singlet(double Rd, F R, F ir, F& E, F& dE) {
  const F R0 = K8(3.5284882), DD = K8(0.160979391);
  const F C6 = K8(6.499027), C8 = K8(124.3991), C10 = K8(3285.828);
  // polynomial part a1 + a2 R + ... + a16 R^15 and its derivative, Horner
  // form, FP64 (the a_i are the same widened REAL(4)/REAL(8) values)
  const double b0 = (double)(0.03537359271649620f), b1 = (double)(2.013977588700072f),
               b2 = (double)(-2.827452449964767f), b3 = (double)(2.713257715593500f),
               b4 = (double)(-2.792039234205731f), b5 = (double)(2.166542078766724f),
               b6 = (double)(-1.272679684173909f), b7 = (double)(0.5630423099212294f),
               b8 = (double)(-0.1879397372273814f), b9 = (double)(0.04719891893374140f),
               b10 = (double)(-0.008851622656489644f), b11 = (double)(0.001224998776243630f),
               b12 = -1.227820520228028e-04, b13 = 8.638783190083473e-06,
               b14 = -4.036967926499151e-07, b15 = 1.123286608335365e-08,
               b16 = -1.406619156782167e-10;
  double pa = b16, pd = 15.0 * b16;
  pa = pa * Rd + b15; pd = pd * Rd + 14.0 * b15;
  pa = pa * Rd + b14; pd = pd * Rd + 13.0 * b14;
  pa = pa * Rd + b13; pd = pd * Rd + 12.0 * b13;
  pa = pa * Rd + b12; pd = pd * Rd + 11.0 * b12;
  pa = pa * Rd + b11; pd = pd * Rd + 10.0 * b11;
  pa = pa * Rd + b10; pd = pd * Rd + 9.0 * b10;
  pa = pa * Rd + b9;  pd = pd * Rd + 8.0 * b9;
  pa = pa * Rd + b8;  pd = pd * Rd + 7.0 * b8;
  pa = pa * Rd + b7;  pd = pd * Rd + 6.0 * b7;
  pa = pa * Rd + b6;  pd = pd * Rd + 5.0 * b6;
  pa = pa * Rd + b5;  pd = pd * Rd + 4.0 * b5;
  pa = pa * Rd + b4;  pd = pd * Rd + 3.0 * b4;
  pa = pa * Rd + b3;  pd = pd * Rd + 2.0 * b3;
  pa = pa * Rd + b2;  pd = pd * Rd + b2;
  pa = pa * Rd + b1;
  const double ird = 1.0 / Rd;
  F alpha = (F)(b0 * ird + pa);
  F dalpha = (F)(pd - b0 * ird * ird);
  F ea = fexp<F>(alpha);
  F em1 = ea - F(1);
  F r2 = R * R, r4 = r2 * r2, r6 = r4 * r2;
  const F r02 = R0 * R0, r04 = r02 * r02, r06 = r04 * r02;
  F rr2 = r2 + r02, rr4 = r4 + r04, rr6 = r6 + r06;
  F i2 = frcp<F>(rr2), i4 = frcp<F>(rr4), i6 = frcp<F>(rr6);
  F i4s = i4 * i4;
  F i2p5 = i2 * i2; i2p5 = i2p5 * i2p5 * i2;  // rr2^-5
  E = DD * em1 * em1 - DD - C6 * i6 - C8 * i4s - C10 * i2p5;
  dE = F(2) * DD * em1 * ea * dalpha + F(6) * C6 * (r4 * R) * i6 * i6 +
       F(8) * C8 * (r2 * R) * i4s * i4 + F(10) * C10 * R * i2p5 * i2;
}

// H2 triplet E3(R) and dE3/dR (TRIPLET95) given the singlet at R.
template <class F>
__device__ inline void triplet(F R, F ir, F e1, F de1, F& E3, F& dE3) {
  const F RL = K8(0.95), RR = K8(1.15);
  const F A1 = K4(-0.0298546962), A2 = K4(-23.9604445036), A3 = K4(-42.5185569474);
  const F A4 = K4(2.0382390988), A5 = K4(-11.5214861455), A6 = K4(1.5309487826);
  const F C1 = K4(-0.4106358351531854), C2 = K4(-0.0770355790707090);
  const F C3 = K4(0.4303193846943223);
  if (R >= RR) {
    F exdr = fexp<F>(-A4 * R);
    F rsq = R * R;
    F ra6 = fpow<F>(R, -A6);
    F ra61 = ra6 * ir;
    E3 = A1 * (A2 + R + A3 * rsq + A5 * ra6) * exdr;
    dE3 = A1 * exdr *
          (F(1) - A2 * A4 + (F(2) * A3 - A4) * R - A3 * A4 * rsq - A5 * A6 * ra61 - A4 * A5 * ra6);
  } else {
    F dr = R - RL;
    if (R <= RL) {
      E3 = e1 + C2 * dr + C3;
      dE3 = de1 + C2;
    } else {
      E3 = e1 + C1 * dr * dr * dr + C2 * dr + C3;
      dE3 = de1 + F(3) * C1 * dr * dr + C2;
    }
  }
}

// Full BKMP2 V(R1,R2,R3) and dV/dRi (POTE).
template <class F>
__device__ inline void pote(const F (&R)[3], const double (&Rd)[3], F& V, F (&dV)[3]) {
  F ir[3] = {frcp<F>(R[0]), frcp<F>(R[1]), frcp<F>(R[2])};
  // ---- London term (H3LOND95)
  F Q[3], J[3], dQ[3], dJ[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    F e1, de1, e3, de3;
    singlet<F>(Rd[i], R[i], ir[i], e1, de1);
    triplet<F>(R[i], ir[i], e1, de1, e3, de3);
    Q[i] = F(0.5) * (e1 + e3);
    J[i] = F(0.5) * (e1 - e3);
    dQ[i] = F(0.5) * (de1 + de3);
    dJ[i] = de1 - de3;
  }
  F d21 = J[1] - J[0], d32 = J[2] - J[1], d31 = J[2] - J[0];
  F jt = F(0.5) * (d21 * d21 + d32 * d32 + d31 * d31) + K8(1.0e-12);
  F rootjt = fsqrt<F>(jt);
  F irj = F(0.25) / rootjt;
  V = Q[0] + Q[1] + Q[2] - rootjt;
  dV[0] = dQ[0] - (F(2) * J[0] - J[1] - J[2]) * dJ[0] * irj;
  dV[1] = dQ[1] - (F(2) * J[1] - J[2] - J[0]) * dJ[1] * irj;
  dV[2] = dQ[2] - (F(2) * J[2] - J[0] - J[1]) * dJ[2] * irj;

  // ---- A = |(r1-r2)(r2-r3)(r3-r1)| (ACALC95), shared by VASCAL95 and CASYM95
  const F r1 = R[0], r2 = R[1], r3 = R[2];
  F A = (r1 - r2) * (r2 - r3) * (r3 - r1);
  F dA[3] = {(F(-2) * r1 + r2 + r3) * (r2 - r3), (F(-2) * r2 + r3 + r1) * (r3 - r1),
             (F(-2) * r3 + r1 + r2) * (r1 - r2)};
  if (A < F(0)) {
    A = -A;
    dA[0] = -dA[0];
    dA[1] = -dA[1];
    dA[2] = -dA[2];
  }
  const F Rs = r1 + r2 + r3, rsq = Rs * Rs, rcu = rsq * Rs, iRs = frcp<F>(Rs);
  F a2 = A * A;

  // ---- asymmetric correction (VASCAL95)
  {
    const F AA1 = K4(0.3788951192E-02), AA2 = K4(0.1478100901E-02);
    const F AA3 = K4(-.1848513849E-03), AA4 = K4(0.9230803609E-05);
    const F AA5 = K4(-.1293180255E-06), AA6 = K4(0.5237179303E+00);
    const F AA7 = K4(-.1112326215E-02);
    F exp1 = fexp<F>(-AA1 * rcu);
    F exp6 = fexp<F>(-AA6 * Rs);
    F S = a2 * (AA2 + A * (AA3 + A * (AA4 + A * AA5)));
    F dSdA = A * (F(2) * AA2 + A * (F(3) * AA3 + A * (F(4) * AA4 + A * F(5) * AA5)));
    F e6r = AA7 * exp6 * iRs;
    V += S * exp1 + a2 * e6r;
    F common = F(-3) * AA1 * rsq * S * exp1 - a2 * e6r * iRs - AA6 * a2 * e6r;
#pragma unroll
    for (int i = 0; i < 3; ++i) dV[i] += common + (dSdA * exp1 + F(2) * A * e6r) * dA[i];
  }

  // ---- compactness (COMPAC95) and compact corrections (CSYM95, CASYM95)
  const F RRc = K8(1.15), RPc = K8(1.25);
  F t[3], dt[3];
  bool compact = false;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    t[i] = F(0);
    dt[i] = F(0);
    if (R[i] < RRc) {
      compact = true;
      F top = RRc - R[i], bot = RPc - R[i], ib = frcp<F>(bot);
      F top2 = top * top, top3 = top2 * top;
      t[i] = top3 * ib;
      dt[i] = F(-3) * top2 * ib + top3 * ib * ib;
    }
  }
  F sumt = t[0] + t[1] + t[2];
  const F P3 = r1 * r2 * r3, iP = frcp<F>(P3), psq = P3 * P3;
  const F dP[3] = {r2 * r3, r3 * r1, r1 * r2};
  if (compact) {
    // CSYM95
    const F V1 = K4(-.2071708868E+00), V2 = K4(-.5672350377E+00), V3 = K4(0.9058780367E-02);
    F exp3 = fexp<F>(-V3 * rcu);
    F dexp3 = F(-3) * V3 * rsq * exp3;
    F g[3], dg[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      g[i] = F(0);
      dg[i] = F(0);
      if (R[i] < RRc) {
        F a = RRc - R[i], ia = RPc - R[i], ib = frcp<F>(ia);
        F sumv = V1 + V1 * V2 * R[i];
        F a3b = a * a * a * ib;
        g[i] = a3b * sumv;
        dg[i] = a3b * ib * sumv - F(3) * a * a * ib * sumv + a3b * V1 * V2;
      }
    }
    F sumg = g[0] + g[1] + g[2];
    V += sumg * exp3;
#pragma unroll
    for (int i = 0; i < 3; ++i) dV[i] += dg[i] * exp3 + sumg * dexp3;
    // CASYM95
    const F U1 = K4(0.2210243144E+00), U2 = K4(0.4367417579E+00), U3 = K4(0.6994985432E-02);
    const F U4 = K4(0.1491096501E+01), U5 = K4(0.1602896673E+01), U6 = K4(-.2821747323E+01);
    const F U7 = K4(0.4948310833E+00), U8 = K4(-.3540394679E-01), U9 = K4(-.3305809954E+01);
    const F U10 = K4(0.3644382172E+01), U11 = K4(-.9997570970E+00), U12 = K4(0.7989919534E-01);
    const F U13 = K4(-.1075807322E-02);
    F ip2 = iP * iP;
    F ser_b = U9 * ip2 + U10 * iP + U11 + U12 * P3 + U13 * psq;
    F series = F(1) + U4 * ip2 + U5 * iP + U6 + U7 * P3 + U8 * psq + A * ser_b;
    F powp = fpow<F>(P3, -U2);          // PR**(-U2)
    F term1 = U1 * powp;
    F eterm = fexp<F>(-U3 * rcu);
    F cas = sumt * a2 * term1 * series * eterm;
    V += cas;
    F dterm1_dp = F(-1) * U1 * U2 * powp * iP;  // d term1 / dP
    F dser_dp = (F(-2) * U4 * ip2 * iP - U5 * ip2 + U7 + F(2) * U8 * P3) +
                A * (F(-2) * U9 * ip2 * iP - U10 * ip2 + U12 + F(2) * U13 * P3);
    F determ = eterm * (F(-3) * U3 * rsq);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      F dseries = dP[i] * dser_dp + dA[i] * ser_b;
      dV[i] += dt[i] * a2 * term1 * series * eterm + F(2) * A * dA[i] * sumt * term1 * series * eterm +
               dterm1_dp * dP[i] * sumt * a2 * series * eterm + dseries * sumt * a2 * term1 * eterm +
               determ * sumt * a2 * term1 * series;
    }
  }

  // ---- bend variables (VBCB95)
  F t1 = r1 * r1 - r2 * r2 - r3 * r3;
  F t2 = r2 * r2 - r3 * r3 - r1 * r1;
  F t3 = r3 * r3 - r1 * r1 - r2 * r2;
  F c1 = t1 * (F(-0.5) * ir[1] * ir[2]);
  F c2 = t2 * (F(-0.5) * ir[2] * ir[0]);
  F c3 = t3 * (F(-0.5) * ir[0] * ir[1]);
  F csum = c1 + c2 + c3;
  F b1a = F(1) - csum;
  F sumb = (F(4) * c1 * c1 - F(3)) * c1 + (F(4) * c2 * c2 - F(3)) * c2 + (F(4) * c3 * c3 - F(3)) * c3;
  const F Z58 = K8(0.625), Z38 = K8(0.375);
  F b1b = F(1) - (Z58 * sumb + Z38 * csum);
  // dc_i/dr_j
  F dc11 = -r1 * ir[1] * ir[2], dc22 = -r2 * ir[0] * ir[2], dc33 = -r3 * ir[0] * ir[1];
  F dc12 = (t1 * ir[1] * ir[1] + F(2)) * F(0.5) * ir[2];
  F dc13 = (t1 * ir[2] * ir[2] + F(2)) * F(0.5) * ir[1];
  F dc21 = (t2 * ir[0] * ir[0] + F(2)) * F(0.5) * ir[2];
  F dc23 = (t2 * ir[2] * ir[2] + F(2)) * F(0.5) * ir[0];
  F dc31 = (t3 * ir[0] * ir[0] + F(2)) * F(0.5) * ir[1];
  F dc32 = (t3 * ir[1] * ir[1] + F(2)) * F(0.5) * ir[0];
  F db1a[3] = {-(dc11 + dc21 + dc31), -(dc12 + dc22 + dc32), -(dc13 + dc23 + dc33)};
  F d1 = F(12) * c1 * c1 - F(3), d2 = F(12) * c2 * c2 - F(3), d3 = F(12) * c3 * c3 - F(3);
  F db1b[3] = {-Z58 * (d1 * dc11 + d2 * dc21 + d3 * dc31) + Z38 * db1a[0],
               -Z58 * (d1 * dc12 + d2 * dc22 + d3 * dc32) + Z38 * db1a[1],
               -Z58 * (d1 * dc13 + d2 * dc23 + d3 * dc33) + Z38 * db1a[2]};
  F b2 = ir[0] + ir[1] + ir[2];
  F db2[3] = {-ir[0] * ir[0], -ir[1] * ir[1], -ir[2] * ir[2]};
  F b3 = (r2 - r1) * (r2 - r1) + (r3 - r2) * (r3 - r2) + (r1 - r3) * (r1 - r3);
  F b3b = fsqrt<F>(b3 + K8(1.0e-12));
  F ib3b = F(0.5) / b3b;
  F db3[3] = {F(4) * r1 - F(2) * r2 - F(2) * r3, F(4) * r2 - F(2) * r3 - F(2) * r1,
              F(4) * r3 - F(2) * r1 - F(2) * r2};
  const F BETA1 = K8(0.52), BETA2 = K8(0.052), BETA3 = K8(0.79);
  F exp1 = fexp<F>(-BETA1 * Rs), exp2 = fexp<F>(-BETA2 * rsq), exp7 = fexp<F>(-BETA3 * Rs);
  F dexp1 = -BETA1 * exp1, dexp2 = F(-2) * BETA2 * Rs * exp2, dexp7 = -BETA3 * exp7;

  // VBNDA (coefficients A) and VBNDB (coefficients G)
#pragma unroll
  for (int set = 0; set < 2; ++set) {
    const bool sa = (set == 0);
    const F s11 = sa ? K4(-.1838073394E+03) : K4(-.4765732725E+02);
    const F s12 = sa ? K4(0.1334593242E+02) : K4(0.3648933563E+01);
    const F s13 = sa ? K4(-.2358129537E+00) : K4(-.7141145244E-01);
    const F s21 = sa ? K4(-.4668193478E+01) : K4(0.1002349176E-01);
    const F s22 = sa ? K4(0.7197506670E+01) : K4(0.9989856329E-02);
    const F s23 = sa ? K4(0.2162004275E+02) : K4(-.4161953634E-02);
    const F s24 = sa ? K4(0.2106294028E+02) : K4(0.9075807910E-03);
    const F s31 = sa ? K4(0.4242962586E+01) : K4(-.2693628729E+00);
    const F s32 = sa ? K4(0.4453505045E+01) : K4(-.1399065763E-01);
    const F s41 = sa ? K4(-.1456918088E+00) : K4(-.1417634346E-01);
    const F s42 = sa ? K4(-.1692657366E-01) : K4(-.4870024792E-03);
    const F s43 = sa ? K4(0.1279520698E+01) : K4(0.1312231847E+00);
    const F s44 = sa ? K4(-.4898940075E+00) : K4(-.4409850519E-01);
    const F s51 = sa ? K4(0.1742295219E+03) : K4(0.5382970863E+02);
    const F s52 = sa ? K4(0.3142175348E+02) : K4(0.4587102824E+01);
    const F s53 = sa ? K4(0.5152903406E+01) : K4(0.1768550515E+01);
    const F B1 = sa ? b1a : b1b;
    const F* dB1 = sa ? db1a : db1b;
    F b12 = B1 * B1;
    F asum = s11 + s12 * Rs + s13 * rsq;
    F bsum = b12 * (s21 + B1 * (s22 + B1 * (s23 + B1 * s24)));
    F csm = s31 * B1 * exp1 + s32 * b12 * exp2;
    F dsum1 = s41 * exp1 + s42 * exp2;
    F dsum2 = s43 * exp1 + s44 * exp2;
    F fsum = s51 + s52 * Rs + s53 * rsq;
    V += B1 * asum * exp1 + bsum * exp2 + b2 * csm + B1 * (b3 * dsum1 + b3b * dsum2) + B1 * fsum * exp7;
    F dasum = s12 + F(2) * s13 * Rs;
    F dbsum = B1 * (F(2) * s21 + B1 * (F(3) * s22 + B1 * (F(4) * s23 + B1 * F(5) * s24)));
    F ddsum1 = s41 * dexp1 + s42 * dexp2;
    F ddsum2 = s43 * dexp1 + s44 * dexp2;
    F dfsum = s52 + F(2) * s53 * Rs;
    // parts of the derivative that do not depend on i
    F radial = B1 * dasum * exp1 + B1 * asum * dexp1 + bsum * dexp2 +
               b2 * (s31 * B1 * dexp1 + s32 * b12 * dexp2) + B1 * b3 * ddsum1 + B1 * b3b * ddsum2 +
               B1 * dfsum * exp7 + B1 * fsum * dexp7;
    F perB = asum * exp1 + dbsum * exp2 + b2 * (s31 * exp1 + F(2) * s32 * B1 * exp2) + b3 * dsum1 +
             b3b * dsum2 + fsum * exp7;
#pragma unroll
    for (int i = 0; i < 3; ++i)
      dV[i] += radial + dB1[i] * perB + db2[i] * csm + B1 * db3[i] * (dsum1 + ib3b * dsum2);
  }

  if (!compact) return;
  // CBNDA (coefficients C) and CBNDB (coefficients D), scaled by SUMT
  F exp7c = fexp<F>(-BETA2 * rcu);
  F dexp7c = F(-3) * BETA2 * rsq * exp7c;
  F irsq = iRs * iRs, ircu = irsq * iRs;
  F ip2 = iP * iP, ip3 = ip2 * iP;
#pragma unroll
  for (int set = 0; set < 2; ++set) {
    const bool sa = (set == 0);
    const F s11 = sa ? K4(0.1860299931E+04) : K4(0.4203543357E+03);
    const F s12 = sa ? K4(-.6134458037E+03) : K4(-.4922474096E+02);
    const F s13 = sa ? K4(0.7337207161E+02) : K4(0.3362942544E+00);
    const F s14 = sa ? K4(-.2676717625E+04) : K4(-.3827423082E+03);
    const F s15 = sa ? K4(0.1344099415E+04) : K4(0.1746726001E+03);
    const F s21 = sa ? K4(0.1538913137E+03) : K4(0.1699995737E-01);
    const F s22 = sa ? K4(0.4348007369E+02) : K4(0.1513036778E-01);
    const F s23 = sa ? K4(0.1719720677E+03) : K4(0.2659119354E-01);
    const F s24 = sa ? K4(0.2115963042E+03) : K4(-.5760387483E-02);
    const F s31 = sa ? K4(-.7026089414E+02) : K4(0.1020622621E+02);
    const F s32 = sa ? K4(-.1300938992E+03) : K4(0.1050536271E-01);
    const F s41 = sa ? K4(0.1310273564E+01) : K4(0.6836172780E+00);
    const F s42 = sa ? K4(-.6175149574E+00) : K4(-.1627858240E+00);
    const F s43 = sa ? K4(-.2679089358E+02) : K4(-.6925485045E+01);
    const F s44 = sa ? K4(0.5577477171E+01) : K4(0.1632567385E+01);
    const F s51 = sa ? K4(-.3543353539E+04) : K4(0.1083595009E+04);
    const F s52 = sa ? K4(-.3740709591E+03) : K4(0.4641431791E+01);
    const F s53 = sa ? K4(0.7979303144E+02) : K4(-.8233144461E+00);
    const F s61 = sa ? K4(-.1104230585E+04) : K4(-.6157225942E+02);
    const F s62 = sa ? K4(0.4603572025E+04) : K4(0.3094361471E+03);
    const F s63 = sa ? K4(-.5593496634E+04) : K4(-.3299631143E+03);
    const F s71 = sa ? K4(-.1069406434E+02) : K4(0.8866227120E+01);
    const F s72 = sa ? K4(0.1021807153E+01) : K4(-.1382126854E+01);
    const F s73 = sa ? K4(0.6669828341E-01) : K4(0.7620770145E-01);
    const F s74 = sa ? K4(0.4168542348E+02) : K4(-.5145757859E+02);
    const F s75 = sa ? K4(0.1751608567E+02) : K4(0.2046097265E+01);
    const F s81 = sa ? K4(0.9486883238E+02) : K4(0.2540775558E+01);
    const F s82 = sa ? K4(-.1519334221E+02) : K4(-.4889246569E+00);
    const F s83 = sa ? K4(0.4024697252E+04) : K4(-.1127439280E+04);
    const F s84 = sa ? K4(-.2225159395E+02) : K4(-.2269932295E+01);
    const F cx1 = s51 + s83;  // FEB27/91: C51 <- C51 + C83
    const F B1 = sa ? b1a : b1b;
    const F* dB1 = sa ? db1a : db1b;
    F b12 = B1 * B1;
    F asum = s11 + s12 * Rs + s13 * rsq + s14 * iRs + s15 * irsq;
    F bsum = b12 * (s21 + B1 * (s22 + B1 * (s23 + B1 * s24)));
    F csm = s31 * B1 * exp1 + s32 * b12 * exp2;
    F dsum1 = s41 * exp1 + s42 * exp2;
    F dsum2 = s43 * exp1 + s44 * exp2;
    F fsum = cx1 + s52 * Rs + s53 * rsq;
    F gsum = s61 + s62 * iRs + s63 * irsq;
    F aasum = s71 + s72 * P3 + s73 * psq + s74 * iP + s75 * ip2;
    F ffsum = s81 * P3 + s82 * psq + s84 * ip2;
    F dasum = s12 + F(2) * s13 * Rs - s14 * irsq - F(2) * s15 * ircu;
    F dbsum = B1 * (F(2) * s21 + B1 * (F(3) * s22 + B1 * (F(4) * s23 + B1 * F(5) * s24)));
    F ddsum1 = s41 * dexp1 + s42 * dexp2;
    F ddsum2 = s43 * dexp1 + s44 * dexp2;
    F dfsum = s52 + F(2) * s53 * Rs;
    F dgsum = -s62 * irsq - F(2) * s63 * ircu;
    F daasum = s72 + F(2) * s73 * P3 - s74 * ip2 - F(2) * s75 * ip3;
    F dffsum = s81 + F(2) * s82 * P3 - F(2) * s84 * ip3;
    F cbs = B1 * asum * exp1 * iP + bsum * exp2 + b2 * csm + B1 * (b3 * dsum1 + b3b * dsum2) +
            B1 * fsum * exp7c * iP + B1 * gsum * exp7c + B1 * aasum * exp2 + B1 * ffsum * exp7c;
    F radial = B1 * dasum * exp1 * iP + B1 * asum * dexp1 * iP + bsum * dexp2 +
               b2 * (s31 * B1 * dexp1 + s32 * b12 * dexp2) + B1 * b3 * ddsum1 + B1 * b3b * ddsum2 +
               B1 * dfsum * exp7c * iP + B1 * fsum * dexp7c * iP + B1 * dgsum * exp7c +
               B1 * gsum * dexp7c + B1 * aasum * dexp2 + B1 * ffsum * dexp7c;
    F perB = asum * exp1 * iP + dbsum * exp2 + b2 * (s31 * exp1 + F(2) * s32 * B1 * exp2) + b3 * dsum1 +
             b3b * dsum2 + fsum * exp7c * iP + gsum * exp7c + aasum * exp2 + ffsum * exp7c;
    F perP = -B1 * asum * exp1 * ip2 - B1 * fsum * exp7c * ip2 + B1 * daasum * exp2 + B1 * dffsum * exp7c;
    V += sumt * cbs;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      F dcb = radial + dB1[i] * perB + db2[i] * csm + B1 * db3[i] * (dsum1 + ib3b * dsum2) + dP[i] * perP;
      dV[i] += dt[i] * cbs + sumt * dcb;
    }
  }
}

}  // namespace h3

// egrad_h3 for one bead.  q, g: (3,3) column-major per bead, FP64 at the
// boundary.  Distances come from FP64 displacements; the mixed form rounds
// the displacements to float and evaluates the surface in float.
struct PesH3 {
  static constexpr int N = 3;
  template <class F>
  __device__ static inline void egrad(const double (&q)[9], double& V, double (&g)[9]) {
    F d[3][3];  // d[0]=q2-q1 (AB), d[1]=q1-q3 (AC), d[2]=q3-q2 (BC)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      d[0][c] = (F)(q[3 + c] - q[c]);
      d[1][c] = (F)(q[c] - q[6 + c]);
      d[2][c] = (F)(q[6 + c] - q[3 + c]);
    }
    F R[3], iR[3];
    double Rd[3];
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      const int i0 = (b == 0) ? 3 : (b == 1) ? 0 : 6, i1 = (b == 0) ? 0 : (b == 1) ? 6 : 3;
      const double x = q[i0] - q[i1], y = q[i0 + 1] - q[i1 + 1], z = q[i0 + 2] - q[i1 + 2];
      Rd[b] = sqrt(x * x + y * y + z * z);
      R[b] = (F)Rd[b];
      iR[b] = F(1) / R[b];
    }
    F v, dv[3];
    h3::pote<F>(R, Rd, v, dv);
    V = (double)v;
    F u[3] = {dv[0] * iR[0], dv[1] * iR[1], dv[2] * iR[2]};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      g[c] = (double)(u[1] * d[1][c]) - (double)(u[0] * d[0][c]);
      g[3 + c] = (double)(u[0] * d[0][c]) - (double)(u[2] * d[2][c]);
      g[6 + c] = (double)(u[2] * d[2][c]) - (double)(u[1] * d[1][c]);
    }
  }
};

}  // namespace cr

#undef K4
#undef K8
