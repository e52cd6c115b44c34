// Caracal's flexible SPC water box (src/egrad_water.f90:36-333, parameters
// src/water_init.f90:74-103, minimum image src/box_image.f90:36-63) on the
// GPU: one CTA per bead, one thread per atom.
//
// Thread w < nwater evaluates molecule w's intramolecular terms (two Morse
// OH stretches with the reference's exp(+a dr), harmonic HH stretch, the
// bond-angle and bond-bond couplings) into a shared gradient array; then
// thread i sums, onto that, the pair forces on atom i from every atom j of
// another molecule, j = 0, 1, ..., n-1.  That is the order in which the
// reference's i < j double loop accumulates into g(i) (a pair's vector for
// the later atom is the exact negation of the earlier one's), so no
// scatter or atomic is needed and the sums run in the reference's order.
// Pair terms:
// point-charge Coulomb (or the Zahn form) and, where the pair's first atom
// (the smaller index) is an oxygen, LJ 12-6 (the reference tests name(i)
// twice).  Periodic: minimum image of every distance vector, pairs at
// r >= coul_cut skipped.  Each pair's energy counts once (thread min(i, j)).
//
// Mixed form: the pairs in FP32 from the (hi, lo) split of the coordinates,
// their forces and energies accumulated as compensated FP32 sums; the
// intramolecular terms stay FP64.
#pragma once
#include <cuda_runtime.h>

namespace cr {
namespace water {

constexpr int kMaxAtoms = 1024;  // one thread per atom
constexpr int kImageIters = 64;  // bound of the minimum-image loop (a NaN or huge vector stops there)

struct Dev {
  int nwater, n, periodic, zahn;
  double len[3], half[3];
  double coul_cut, zahn_a, zahn_par;
  double r0, r0hh, de, a, ktheta, krtheta, krr, eh, eo, sigma, eps;
  float flen[3], fhalf[3], fcut, fzahn_a, fzahn_par, feh, feo, fsigma, feps;
};

__device__ inline void image(const Dev& D, double* d) {
#pragma unroll
  for (int k = 0; k < 3; ++k)
    for (int it = 0; it < kImageIters && fabs(d[k]) > D.half[k]; ++it) d[k] = d[k] - copysign(D.len[k], d[k]);
}
__device__ inline void image(const Dev& D, float* d) {
#pragma unroll
  for (int k = 0; k < 3; ++k)
    for (int it = 0; it < kImageIters && fabsf(d[k]) > D.fhalf[k]; ++it) d[k] = d[k] - copysignf(D.flen[k], d[k]);
}

// Molecule w's intramolecular energy; its gradient into gi (3n doubles).
__device__ inline double intra(const Dev& D, const double* x, int w, double* gi) {
  const int o = 3 * w, h1 = 3 * w + 1, h2 = 3 * w + 2;
  double oh1[3], oh2[3], hh[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    oh1[k] = x[3 * o + k] - x[3 * h1 + k];
    oh2[k] = x[3 * o + k] - x[3 * h2 + k];
    hh[k] = x[3 * h1 + k] - x[3 * h2 + k];
  }
  if (D.periodic) {
    image(D, oh1);
    image(D, oh2);
    image(D, hh);
  }
  const double r1 = sqrt(oh1[0] * oh1[0] + oh1[1] * oh1[1] + oh1[2] * oh1[2]);
  const double d1 = r1 - D.r0;
  const double r2 = sqrt(oh2[0] * oh2[0] + oh2[1] * oh2[1] + oh2[2] * oh2[2]);
  const double d2 = r2 - D.r0;
  const double rh = sqrt(hh[0] * hh[0] + hh[1] * hh[1] + hh[2] * hh[2]);
  const double dh = rh - D.r0hh;
  const double ex1 = exp(D.a * d1), ex2 = exp(D.a * d2);
  double e = D.de * (1.0 - ex1) * (1.0 - ex1);
  e = e + D.de * (1.0 - ex2) * (1.0 - ex2);
  double go[3] = {0.0, 0.0, 0.0}, g1[3] = {0.0, 0.0, 0.0}, g2[3] = {0.0, 0.0, 0.0};
  const double de1 = -2.0 * D.a * D.de * ex1 * (1.0 - ex1) / r1;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double ga = de1 * oh1[k];
    g1[k] = g1[k] - ga;
    go[k] = go[k] + ga;
  }
  const double de2 = -2.0 * D.a * D.de * ex2 * (1.0 - ex2) / r2;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double ga = de2 * oh2[k];
    g2[k] = g2[k] - ga;
    go[k] = go[k] + ga;
  }
  e = e + 0.5 * D.ktheta * dh * dh;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double ga = D.ktheta * hh[k] * dh / rh;
    g1[k] = g1[k] + ga;
    g2[k] = g2[k] - ga;
  }
  e = e + D.krtheta * dh * (d1 + d2);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double ga = dh / r1 * oh1[k] * D.krtheta;
    const double gb = dh / r2 * oh2[k] * D.krtheta;
    const double gh = D.krtheta * 1.0 * (d1 + d2) / rh * hh[k];
    g1[k] = g1[k] + gh - ga;
    g2[k] = g2[k] - gh - gb;
    go[k] = go[k] + ga + gb;
  }
  e = e + D.krr * d1 * d2;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double ga = D.krr * (d2 / r1 * oh1[k]);
    const double gb = D.krr * (d1 / r2 * oh2[k]);
    g1[k] = g1[k] - ga;
    g2[k] = g2[k] - gb;
    go[k] = go[k] + gb + ga;
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    gi[3 * o + k] = go[k];
    gi[3 * h1 + k] = g1[k];
    gi[3 * h2 + k] = g2[k];
  }
  return e;
}

// Pair forces on atom i (plain form), added to f in j order; returns the
// energy of the pairs (i, j > i).
__device__ inline double pairs_plain(const Dev& D, const double* x, int i, double (&f)[3]) {
  const double qi = (i % 3 == 0) ? D.eo : D.eh;
  const double xi[3] = {x[3 * i], x[3 * i + 1], x[3 * i + 2]};
  double e = 0.0;
  for (int j = 0; j < D.n; ++j) {
    if (j / 3 == i / 3) continue;
    const double qj = (j % 3 == 0) ? D.eo : D.eh;
    double d[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) d[k] = xi[k] - x[3 * j + k];
    if (D.periodic) image(D, d);
    const double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    if (!(r < D.coul_cut || !D.periodic)) continue;
    const double oner = 1.0 / r;
    double e0;
    if (D.zahn) e0 = qi * qj * ((erfc(D.zahn_a * r) * oner) - D.zahn_par * (r - D.coul_cut));
    else e0 = qi * qj * oner;
    if (j > i) e += e0;
#pragma unroll
    for (int k = 0; k < 3; ++k) f[k] = f[k] - e0 * oner * oner * d[k];
    if ((i < j ? i : j) % 3 == 0) {
      const double sr = D.sigma * oner;
      const double sr2 = sr * sr;
      const double s6 = sr2 * sr2 * sr2;
      if (j > i) e += 4.0 * D.eps * (s6 * s6 - s6);
#pragma unroll
      for (int k = 0; k < 3; ++k) f[k] = f[k] - 24.0 * D.eps * oner * oner * d[k] * s6 * (2.0 * s6 - 1.0);
    }
  }
  return e;
}

// Error-free FP32 sum (Knuth's TwoSum): s + e == a + b exactly.
__device__ inline void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// The same in FP32 from the (hi, lo) coordinates; forces and energy summed
// as compensated FP32 pairs (sum + compensation, TwoSum per term), which
// keeps the FP64-quality sums on the FP32 pipes.
// The truncated Coulomb sum jumps by q_i q_j / r_cut where a pair crosses the
// cutoff, so the cutoff decision must be the plain form's: where the FP32 r
// lies within 1e-5 of the cutoff, the FP64 distance (same image loop, same
// sqrt) decides.
__device__ inline double pairs_mixed(const Dev& D, const double* x, const float2* hl, int i, double (&f)[3]) {
  const float qi = (i % 3 == 0) ? D.feo : D.feh;
  float2 xi[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) xi[k] = hl[3 * i + k];
  float es = 0.f, ec = 0.f, fs[3] = {0.f, 0.f, 0.f}, fc[3] = {0.f, 0.f, 0.f};
  for (int j = 0; j < D.n; ++j) {
    if (j / 3 == i / 3) continue;
    const float qj = (j % 3 == 0) ? D.feo : D.feh;
    float d[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float2 xj = hl[3 * j + k];
      d[k] = (xi[k].x - xj.x) + (xi[k].y - xj.y);
    }
    if (D.periodic) image(D, d);
    const float r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    float oner = rsqrtf(r2);
    oner = fmaf(0.5f * oner, fmaf(-r2 * oner, oner, 1.0f), oner);  // one Newton step
    const float r = r2 * oner;
    if (D.periodic) {
      bool inside = r < D.fcut;
      if (fabsf(r - D.fcut) < 1e-5f * D.fcut) {
        double dd[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) dd[k] = x[3 * i + k] - x[3 * j + k];
        image(D, dd);
        inside = sqrt(dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2]) < D.coul_cut;
      }
      if (!inside) continue;
    }
    const float ir2 = oner * oner;
    float e0;
    if (D.zahn) e0 = qi * qj * ((erfcf(D.fzahn_a * r) * oner) - D.fzahn_par * (r - D.fcut));
    else e0 = qi * qj * oner;
    float s = e0 * ir2, ep = e0;
    if ((i < j ? i : j) % 3 == 0) {
      const float sr2 = D.fsigma * D.fsigma * ir2;
      const float s6 = sr2 * sr2 * sr2;
      ep += 4.0f * D.feps * (s6 * s6 - s6);
      s += 24.0f * D.feps * ir2 * s6 * (2.0f * s6 - 1.0f);
    }
    if (j > i) {
      float t, r;
      two_sum(es, ep, t, r);
      es = t;
      ec += r;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      float t, r;
      two_sum(fs[k], -(s * d[k]), t, r);
      fs[k] = t;
      fc[k] += r;
    }
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) f[k] += (double)fs[k] + (double)fc[k];
  return (double)es + (double)ec;
}

}  // namespace water
}  // namespace cr
