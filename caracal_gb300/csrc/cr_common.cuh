// Common device helpers of the GB300 RPMD engine: error codes, the Philox
// Gaussian stream, compensated sums, and group reductions.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/caracal_gb300.h"

namespace cr {

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), written from the paper.
// Stream layout: key = (seed, global trajectory), counter = (pair, bead, step,
// tag); one call gives the normals of coordinates 2*pair and 2*pair+1 of one
// bead (coordinate c = dim + 3*atom, Fortran order of q(3,natoms)).
// ---------------------------------------------------------------------------
enum NoiseTag : uint32_t {
  TAG_INIT_MOMENTA = 0,
  TAG_ANDERSEN = 1,
  TAG_PILE_A = 2,
  TAG_PILE_B = 3,
  TAG_BEAD_JITTER = 4,
  TAG_CHILD_MOMENTA = 5,
};

__host__ __device__ inline uint4 philox4x32_10(uint4 c, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
#ifdef __CUDA_ARCH__
    uint32_t hi0 = __umulhi(M0, c.x), lo0 = M0 * c.x;
    uint32_t hi1 = __umulhi(M1, c.z), lo1 = M1 * c.z;
#else
    uint64_t p0 = (uint64_t)M0 * c.x, p1 = (uint64_t)M1 * c.z;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
#endif
    c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
    k0 += W0;
    k1 += W1;
  }
  return c;
}

// Two N(0,1) deviates by Box-Muller on two 53-bit uniforms, FP64 throughout.
__device__ inline void normal_pair_f64(uint32_t seed, uint32_t traj, uint32_t pair,
                                       uint32_t bead, uint32_t step, uint32_t tag,
                                       double& z0, double& z1) {
  uint4 r = philox4x32_10(make_uint4(pair, bead, step, tag), seed, traj);
  uint64_t a = ((uint64_t)r.y << 32) | r.x;
  uint64_t b = ((uint64_t)r.w << 32) | r.z;
  double ua = (double)(a >> 11) * 0x1.0p-53;
  double ub = (double)(b >> 11) * 0x1.0p-53;
  double rad = sqrt(-2.0 * log(1.0 - ua));
  double s, c;
  sincospi(2.0 * ub, &s, &c);
  z0 = rad * c;
  z1 = rad * s;
}

// Fills z[0..NC) with the normals of one bead.
template <int NC>
__device__ inline void normals_bead(uint32_t seed, uint32_t traj, uint32_t bead,
                                    uint32_t step, uint32_t tag, double (&z)[NC]) {
#pragma unroll
  for (int i = 0; 2 * i < NC; ++i) {
    double a, b;
    normal_pair_f64(seed, traj, (uint32_t)i, bead, step, tag, a, b);
    z[2 * i] = a;
    if (2 * i + 1 < NC) z[2 * i + 1] = b;
  }
}

// ---------------------------------------------------------------------------
// Compensated (Neumaier) accumulation for the mixed form.
// ---------------------------------------------------------------------------
template <class F>
struct NeumaierSum {
  F s = F(0), c = F(0);
  __device__ inline void add(F x) {
    F t = s + x;
    if (fabs(s) >= fabs(x)) c += (s - t) + x;
    else c += (x - t) + s;
    s = t;
  }
  __device__ inline F value() const { return s + c; }
};

}  // namespace cr
