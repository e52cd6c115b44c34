// ORACLE (test infrastructure only) -- counter-based Gaussian stream.
//
// Caracal draws thermostat noise from gfortran's intrinsic `random_number`
// (src/andersen.f90:121-126) through a Marsaglia polar transform
// (src/andersen.f90:84-113).  That generator lives in libgfortran and cannot
// be reproduced, so the engine and this oracle share their own stream:
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC'11), restated here from the published description,
// followed by a Box-Muller transform.  Parity of the noise against Caracal
// itself is therefore unpinned; parity between the CUDA engine and this
// oracle is exact up to libm rounding.
//
// Stream layout (shared with the CUDA engine):
//   key     = (seed low 32 bits, global trajectory index)
//   counter = (pair index i, bead j, step s, tag)
//   one call -> two doubles u_a, u_b in [0,1) (53-bit) -> two normals,
//   which are the normals of coordinates 2i and 2i+1 of bead j, coordinates
//   numbered c = dim + 3*atom (Fortran order of q(3,natoms)).
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

namespace orc {

struct Philox4 {
  uint32_t v[4];
};

inline void philox_mulhilo(uint32_t a, uint32_t b, uint32_t* hi, uint32_t* lo) {
  uint64_t p = (uint64_t)a * (uint64_t)b;
  *hi = (uint32_t)(p >> 32);
  *lo = (uint32_t)p;
}

// Ten rounds of Philox4x32 on counter c with key (k0, k1).
inline Philox4 philox4x32_10(const uint32_t c_in[4], uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
  uint32_t c0 = c_in[0], c1 = c_in[1], c2 = c_in[2], c3 = c_in[3];
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0, lo0, hi1, lo1;
    philox_mulhilo(M0, c0, &hi0, &lo0);
    philox_mulhilo(M1, c2, &hi1, &lo1);
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n1 = lo1;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    uint32_t n3 = lo0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += W0;
    k1 += W1;
  }
  Philox4 out;
  out.v[0] = c0; out.v[1] = c1; out.v[2] = c2; out.v[3] = c3;
  return out;
}

// Tags separating the independent uses of the stream.
enum NoiseTag : uint32_t {
  TAG_INIT_MOMENTA = 0,   // mdinit: Andersen draw at step 0
  TAG_ANDERSEN = 1,       // Andersen resample at step s
  TAG_PILE_A = 2,         // PILE half step before the first kick
  TAG_PILE_B = 3,         // PILE half step after the second kick
  TAG_BEAD_JITTER = 4,    // initial-geometry jitter of the beads
  TAG_CHILD_MOMENTA = 5,  // recrossing child momenta
};

// Gaussian deviates as the engine draws them: Box-Muller in FP32 on two
// 24-bit uniforms, with ln and sin/cos as explicit polynomials in single
// rounded FP32 operations (std::fma where the engine uses an FMA; this file
// is compiled with -ffp-contract=off), so the deviates match the GPU's bit
// for bit.  ln m = 2 atanh((m-1)/(m+1)) for m in [sqrt(1/2), sqrt(2)), odd
// series to t^9; sin/cos by quadrant and Taylor series to theta^9 / theta^10.
inline float bm_log(float u) {
  int32_t i;
  std::memcpy(&i, &u, 4);
  int e = ((i >> 23) & 0xff) - 127;
  const int32_t mb = (i & 0x7fffff) | 0x3f800000;
  float m;
  std::memcpy(&m, &mb, 4);
  if (m > 0x1.6a09e6p+0f) {
    m = m * 0.5f;
    e += 1;
  }
  const float t = (m - 1.f) / (m + 1.f);
  const float t2 = t * t;
  float p = std::fma(t2, 0x1.c71c72p-4f, 0x1.24924ap-3f);
  p = std::fma(t2, p, 0x1.99999ap-3f);
  p = std::fma(t2, p, 0x1.555556p-2f);
  p = std::fma(t2, p, 1.f);
  const float lnm = (2.f * t) * p;
  const float fe = (float)e;
  return std::fma(fe, 0x1.62ep-1f, std::fma(fe, 0x1.0bfbe8p-15f, lnm));
}

inline void bm_sincos2pi(float v, float* sn, float* cs) {
  const float x = 4.f * v;
  const int q = (int)std::nearbyint(x);
  const float th = (x - (float)q) * 0x1.921fb6p+0f;
  const float t2 = th * th;
  float ps = std::fma(t2, 0x1.71de3ap-19f, -0x1.a01a02p-13f);
  ps = std::fma(t2, ps, 0x1.111112p-7f);
  ps = std::fma(t2, ps, -0x1.555556p-3f);
  const float s = std::fma(th * t2, ps, th);
  float pc = std::fma(t2, -0x1.27e4fcp-22f, 0x1.a01a02p-16f);
  pc = std::fma(t2, pc, -0x1.6c16c2p-10f);
  pc = std::fma(t2, pc, 0x1.555556p-5f);
  pc = std::fma(t2, pc, -0.5f);
  const float c = std::fma(t2, pc, 1.f);
  switch (q & 3) {
    case 0: *sn = s; *cs = c; break;
    case 1: *sn = c; *cs = -s; break;
    case 2: *sn = -s; *cs = -c; break;
    default: *sn = -c; *cs = s; break;
  }
}

inline void bm_pair(uint32_t wa, uint32_t wb, double* z0, double* z1) {
  const float u = (float)((wa >> 8) + 1u) * 0x1.0p-24f;
  const float v = (float)(wb >> 8) * 0x1.0p-24f;
  const float rad = std::sqrt(-2.f * bm_log(u));
  float sn, cs;
  bm_sincos2pi(v, &sn, &cs);
  *z0 = (double)(rad * cs);
  *z1 = (double)(rad * sn);
}

// Deviates 2 pair and 2 pair + 1 of (traj, bead, step, tag); Philox block
// pair / 2, words 0-1 for an even pair, 2-3 for an odd one.
inline void normal_pair(uint32_t seed, uint32_t traj, uint32_t pair, uint32_t bead,
                        uint32_t step, uint32_t tag, double* z0, double* z1) {
  uint32_t c[4] = {pair >> 1, bead, step, tag};
  Philox4 r = philox4x32_10(c, seed, traj);
  if (pair & 1u) bm_pair(r.v[2], r.v[3], z0, z1);
  else bm_pair(r.v[0], r.v[1], z0, z1);
}

// Deviates for all 3*natoms coordinates of one bead (coordinate c = deviate c).
inline void normals_bead(uint32_t seed, uint32_t traj, uint32_t bead, uint32_t step,
                         uint32_t tag, int ncoord, double* z) {
  for (int i = 0; 2 * i < ncoord; ++i) {
    double a, b;
    normal_pair(seed, traj, (uint32_t)i, bead, step, tag, &a, &b);
    z[2 * i] = a;
    if (2 * i + 1 < ncoord) z[2 * i + 1] = b;
  }
}

}  // namespace orc
