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

// Two standard normals for (traj, bead, step, tag, pair).
inline void normal_pair(uint32_t seed, uint32_t traj, uint32_t pair, uint32_t bead,
                        uint32_t step, uint32_t tag, double* z0, double* z1) {
  uint32_t c[4] = {pair, bead, step, tag};
  Philox4 r = philox4x32_10(c, seed, traj);
  uint64_t a = ((uint64_t)r.v[1] << 32) | r.v[0];
  uint64_t b = ((uint64_t)r.v[3] << 32) | r.v[2];
  double ua = (double)(a >> 11) * 0x1.0p-53;
  double ub = (double)(b >> 11) * 0x1.0p-53;
  double rad = std::sqrt(-2.0 * std::log(1.0 - ua));
  double th = 2.0 * M_PI * ub;
  *z0 = rad * std::cos(th);
  *z1 = rad * std::sin(th);
}

// Normals for all 3*natoms coordinates of one bead.
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
