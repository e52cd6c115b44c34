// Caracal's ANA_OH3 surface (src/egrad_oh3.f): the OH + H2 potential of
// G. C. Schatz and H. Elgersma, Chem. Phys. Lett. 73, 21 (1980), on the
// device.  Atoms O, H1, H2, H3; distances R1 = O-H1, R2 = O-H2, R3 = O-H3,
// R4 = H1-H2, R5 = H1-H3, R6 = H2-H3 (egrad_oh3:60-105).  pot_oh3 sums Morse
// terms on R1, R4, R5, the LEPS three-body term (V3POT) on (R2, R3, R6),
// the water-like terms (VH2O) on (R1, R2, R4) and (R1, R3, R5), the Gaussian
// four-body term (V4POT) on (R2, R3, R4, R5), then -2 DE(2) + DE(3); the
// constants are the BLOCK DATA PTPACM_oh3 (V4POT reads ALP, CLAM, ACON and
// VH2O reads CON through their COMMON layouts).  F is the arithmetic type of
// the surface (double, or float in the mixed form); the distances are formed
// in FP64 and the gradient is assembled in FP64.  Mixed form: the O-H Morse
// of R1 (1 - exp(-b (R - Re)) cancels near its minimum) and the H2 LEPS term
// (its Coulomb and exchange parts cancel) in double-FP32 arithmetic
// (ff32.cuh) from the FP64 distances split into float pairs, the rest FP32.
#pragma once
#include <cuda_runtime.h>

#include <type_traits>

#include "ff32.cuh"

namespace cr {
namespace oh3 {

struct K {
  static constexpr double de[3] = {0.148201, 0.0275690, 0.151548};
  static constexpr double beta[3] = {1.260580, 0.924180, 1.068620};
  static constexpr double re[3] = {1.863300, 2.907700, 1.428600};
  static constexpr double sato = 0.10;
  static constexpr double gam[3] = {2.399700, 1.058350, 2.399700};
  static constexpr double reoh = 1.808090, rehh = 2.861590;
  static constexpr double con[7] = {-.0015920, 0.026963, 0.0014689, 0.080011, 0.085816, -0.063179, 0.101380};
  static constexpr double alp[4] = {4.773, 7.14, 2.938, 5.28};
  static constexpr double clam[4] = {0.10, 0.10, 0.20, 0.03};
  static constexpr double acon[2] = {0.10, 0.009};
};

template <class F>
__device__ inline F sq(F x) { return x * x; }

// Morse D (1 - exp(-B (R - T)))^2 and its derivative
template <class F>
__device__ inline void morse(F d, F b, F t, F r, F& v, F& dv) {
  const F ex = exp(-b * (r - t));
  const F u = F(1) - ex;
  v = d * (u * u);
  dv = F(2) * b * d * u * ex;
}

// LEPS of (R2, R3, R6): DE, BETA, RE = (DE1, DE1, DE3), ...
template <class F>
__device__ inline F v3pot(const F (&r)[3], F (&dedr)[3]) {
  const F z = F(K::sato), zpo = F(1) + z, op3z = F(1) + F(3) * z, top3z = F(2) * op3z, zp3 = z + F(3),
          tzp3 = F(2) * zp3;
  const F de[3] = {F(K::de[0]), F(K::de[0]), F(K::de[2])};
  const F be[3] = {F(K::beta[0]), F(K::beta[0]), F(K::beta[2])};
  const F re[3] = {F(K::re[0]), F(K::re[0]), F(K::re[2])};
  F x[3], exch[3], do4z[3], e = F(0);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    do4z[i] = de[i] / F(4) / zpo;
    x[i] = exp(-be[i] * (r[i] - re[i]));
    e = e + do4z[i] * (zp3 * x[i] - top3z) * x[i];
    exch[i] = do4z[i] * (op3z * x[i] - tzp3) * x[i];
  }
  const F rad = sqrt(sq(exch[0] - exch[1]) + sq(exch[1] - exch[2]) + sq(exch[2] - exch[0]));
  const F is2 = F(0.70710678118654752440);
  e = e - rad * is2;
  const F s = exch[0] + exch[1] + exch[2];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const F b = be[i] * do4z[i] * F(2);
    dedr[i] = b * x[i] * ((F(3) * exch[i] - s) * is2 * (op3z * x[i] - zp3) / rad - zp3 * x[i] + op3z);
  }
  return e;
}

// The same two terms in float-pair arithmetic (mixed form), rounded once.
__device__ inline void morse_ff(double d, double b, double t, ff r, float& v, ff& dv) {
  const ff bb = ff_const(b), dd = ff_const(d);
  const ff ex = ff_exp(-(bb * (r - ff_const(t))));
  const ff u = ff_from(1.f) - ex;
  v = ff_float(dd * (u * u));
  dv = bb * dd * u * ex * 2.f;
}
__device__ inline float v3pot_ff(const ff (&r)[3], ff (&dedr)[3]) {
  constexpr double z = K::sato, zpo = 1.0 + z, op3z = 1.0 + 3.0 * z, top3z = 2.0 * op3z, zp3 = z + 3.0,
                   tzp3 = 2.0 * zp3;
  constexpr double de[3] = {K::de[0], K::de[0], K::de[2]};
  constexpr double be[3] = {K::beta[0], K::beta[0], K::beta[2]};
  constexpr double re[3] = {K::re[0], K::re[0], K::re[2]};
  ff x[3], exch[3], do4z[3], e = ff_from(0.f);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    do4z[i] = ff_const(de[i] / 4.0 / zpo);
    x[i] = ff_exp(-(ff_const(be[i]) * (r[i] - ff_const(re[i]))));
    e += do4z[i] * (ff_const(zp3) * x[i] - ff_const(top3z)) * x[i];
    exch[i] = do4z[i] * (ff_const(op3z) * x[i] - ff_const(tzp3)) * x[i];
  }
  const ff d01 = exch[0] - exch[1], d12 = exch[1] - exch[2], d20 = exch[2] - exch[0];
  const ff rad = ff_sqrt(d01 * d01 + d12 * d12 + d20 * d20);
  constexpr ff is2 = ff_const(0.70710678118654752440);
  e -= rad * is2;
  const ff sx = exch[0] + exch[1] + exch[2];
  const ff irad = ff_recip(rad);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const ff b = ff_const(be[i]) * do4z[i] * 2.f;
    dedr[i] = b * x[i] *
              ((exch[i] * 3.f - sx) * is2 * (ff_const(op3z) * x[i] - ff_const(zp3)) * irad - ff_const(zp3) * x[i] +
               ff_const(op3z));
  }
  return ff_float(e);
}

// Gaussians of (R2, R3, R4, R5)
template <class F>
__device__ inline F v4pot(const F (&r)[4], F (&dedr)[4]) {
  const F a0 = F(K::alp[0]), a1 = F(K::alp[1]), a2 = F(K::alp[2]), a3 = F(K::alp[3]);
  const F c0 = F(K::clam[0]), c1 = F(K::clam[1]), c2 = F(K::clam[2]), c3 = F(K::clam[3]);
  const F t1 = exp(-(c0 * sq(r[0] - a0)) - c0 * sq(r[1] - a0) - c2 * sq(r[2] - a2) - c2 * sq(r[3] - a2)) *
               F(K::acon[0]);
  const F t2 = exp(-(c1 * sq(r[0] - a1)) - c1 * sq(r[1] - a1) - c3 * sq(r[2] - a3) - c3 * sq(r[3] - a3)) *
               F(K::acon[1]);
  dedr[0] = F(-2) * (t1 * c0 * (r[0] - a0) + t2 * c1 * (r[0] - a1));
  dedr[1] = F(-2) * (t1 * c0 * (r[1] - a0) + t2 * c1 * (r[1] - a1));
  dedr[2] = F(-2) * (t1 * c2 * (r[2] - a2) + t2 * c3 * (r[2] - a3));
  dedr[3] = F(-2) * (t1 * c2 * (r[3] - a2) + t2 * c3 * (r[3] - a3));
  return t1 + t2;
}

// Water-like term of (OH, OH', HH): Q1 Q2 Q3 P, Q = 1 - tanh(gam s / 2)
// (2 / (1 + exp(2x)) for 15 <= x < 43, 0 beyond; where Q = 0 the derivative
// is 0); derivatives returned in the argument order
template <class F>
__device__ inline F vh2o(const F (&r)[3], F (&dedr)[3]) {
  const F gam[3] = {F(K::gam[0]), F(K::gam[1]), F(K::gam[2])};
  F s[3], q[3], dq[3];
  s[0] = r[0] - F(K::reoh);
  s[2] = r[1] - F(K::reoh);
  s[1] = r[2] - F(K::rehh);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const F x = F(0.5) * gam[i] * s[i];
    if (x < F(15)) {
      q[i] = F(1) - tanh(x);
    } else if (x < F(43)) {
      q[i] = F(2) / (F(1) + exp(F(2) * x));
    } else {
      q[i] = F(0);
      dq[i] = F(0);
      continue;
    }
    const F ch = cosh(x);
    dq[i] = F(-0.5) * gam[i] / (ch * ch);
  }
  const F c0 = F(K::con[0]), c1 = F(K::con[1]), c2 = F(K::con[2]), c3 = F(K::con[3]), c4 = F(K::con[4]),
          c5 = F(K::con[5]), c6 = F(K::con[6]);
  const F p = c0 + c1 * (s[0] + s[2]) + c2 * s[1] + F(0.5) * c3 * (s[0] * s[0] + s[2] * s[2]) +
              F(0.5) * c4 * s[1] * s[1] + c5 * s[1] * (s[0] + s[2]) + c6 * s[0] * s[2];
  const F e = q[0] * q[1] * q[2] * p;
  const F dp[3] = {c1 + c3 * s[0] + c5 * s[1] + c6 * s[2], c2 + c4 * s[1] + c5 * (s[0] + s[2]),
                   c1 + c3 * s[2] + c5 * s[1] + c6 * s[0]};
  F d[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) d[i] = q[i] == F(0) ? F(0) : e * (dq[i] / q[i] + (dp[i] / p));
  dedr[0] = d[0];
  dedr[1] = d[2];
  dedr[2] = d[1];
  return e;
}

template <class F>
__device__ inline F pot(const F (&R)[6], F (&dv)[6]) {
  F v, m3, m4;
  morse(F(K::de[0]), F(K::beta[0]), F(K::re[0]), R[0], v, dv[0]);
  morse(F(K::de[1]), F(K::beta[1]), F(K::re[1]), R[3], m3, dv[3]);
  morse(F(K::de[1]), F(K::beta[1]), F(K::re[1]), R[4], m4, dv[4]);
  v = v + m3 + m4;
  dv[1] = dv[2] = dv[5] = F(0);
  {
    const F r3[3] = {R[1], R[2], R[5]};
    F d[3];
    v = v + v3pot(r3, d);
    dv[1] += d[0];
    dv[2] += d[1];
    dv[5] += d[2];
  }
  {
    const F r3[3] = {R[0], R[1], R[3]};
    F d[3];
    v = v + vh2o(r3, d);
    dv[0] += d[0];
    dv[1] += d[1];
    dv[3] += d[2];
  }
  {
    const F r3[3] = {R[0], R[2], R[4]};
    F d[3];
    v = v + vh2o(r3, d);
    dv[0] += d[0];
    dv[2] += d[1];
    dv[4] += d[2];
  }
  {
    const F r4[4] = {R[1], R[2], R[3], R[4]};
    F d[4];
    v = v + v4pot(r4, d);
    dv[1] += d[0];
    dv[2] += d[1];
    dv[3] += d[2];
    dv[4] += d[3];
  }
  return v - F(2) * F(K::de[1]) + F(K::de[2]);
}

// Mixed form of pot: the R1 Morse and the H2 LEPS term in float pairs (from
// the FP64 distances), the rest FP32, and dV/dR_k summed as float pairs (the
// terms of one distance can be large and opposite).
__device__ inline float pot_mixed(const float (&R)[6], const double (&Rd)[6], ff (&dv)[6]) {
  ff Rp[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    const float h = __double2float_rn(Rd[k]);
    Rp[k] = ff{h, __double2float_rn(Rd[k] - (double)h)};
  }
  float v, m3, m4, d3, d4;
  constexpr double d1 = K::de[0], b1 = K::beta[0], t1 = K::re[0];
  morse_ff(d1, b1, t1, Rp[0], v, dv[0]);
  constexpr float d2 = (float)K::de[1], b2 = (float)K::beta[1], t2 = (float)K::re[1];
  morse(d2, b2, t2, R[3], m3, d3);
  morse(d2, b2, t2, R[4], m4, d4);
  dv[3] = ff_from(d3);
  dv[4] = ff_from(d4);
  v = v + m3 + m4;
  {
    const ff r3[3] = {Rp[1], Rp[2], Rp[5]};
    ff d[3];
    v = v + v3pot_ff(r3, d);
    dv[1] = d[0];
    dv[2] = d[1];
    dv[5] = d[2];
  }
  {
    const float r3[3] = {R[0], R[1], R[3]};
    float d[3];
    v = v + vh2o(r3, d);
    dv[0] += d[0];
    dv[1] += d[1];
    dv[3] += d[2];
  }
  {
    const float r3[3] = {R[0], R[2], R[4]};
    float d[3];
    v = v + vh2o(r3, d);
    dv[0] += d[0];
    dv[2] += d[1];
    dv[4] += d[2];
  }
  {
    const float r4[4] = {R[1], R[2], R[3], R[4]};
    float d[4];
    v = v + v4pot(r4, d);
    dv[1] += d[0];
    dv[2] += d[1];
    dv[3] += d[2];
    dv[4] += d[3];
  }
  return v - 2.0f * (float)K::de[1] + (float)K::de[2];
}

}  // namespace oh3

struct PesOH3 {
  static constexpr int N = 4;
  template <class F>
  __device__ static inline void egrad(const double (&q)[12], double& V, double (&g)[12]) {
    constexpr int pa[6] = {0, 0, 0, 1, 1, 2}, pb[6] = {1, 2, 3, 2, 3, 3};  // R_k = |q_pb - q_pa|
    double d[6][3], Rd[6];
    F R[6], dv[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
#pragma unroll
      for (int x = 0; x < 3; ++x) d[k][x] = q[3 * pb[k] + x] - q[3 * pa[k] + x];
      Rd[k] = sqrt(d[k][0] * d[k][0] + d[k][1] * d[k][1] + d[k][2] * d[k][2]);
      R[k] = (F)Rd[k];
    }
    double dvd[6];
    if constexpr (std::is_same<F, float>::value) {
      ff dvp[6];
      V = (double)oh3::pot_mixed(R, Rd, dvp);
#pragma unroll
      for (int k = 0; k < 6; ++k) dvd[k] = (double)dvp[k].hi + (double)dvp[k].lo;
    } else {
      V = (double)oh3::pot<F>(R, dv);
#pragma unroll
      for (int k = 0; k < 6; ++k) dvd[k] = (double)dv[k];
    }
#pragma unroll
    for (int x = 0; x < 12; ++x) g[x] = 0.0;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      const double u = dvd[k] / Rd[k];
#pragma unroll
      for (int x = 0; x < 3; ++x) {
        g[3 * pa[k] + x] -= u * d[k][x];
        g[3 * pb[k] + x] += u * d[k][x];
      }
    }
  }
};

}  // namespace cr
