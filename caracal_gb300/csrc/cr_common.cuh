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

// Gaussian deviates: Box-Muller in FP32 on two 24-bit uniforms from two
// 32-bit Philox words, with the logarithm and the sine/cosine written out as
// polynomials in explicitly rounded FP32 operations (__fmaf_rn, __fmul_rn,
// ...: the compiler may not contract or reorder them), so the host oracle
// reproduces every bit with std::fma.  A deviate has 24-bit resolution (the
// tails reach 5.8 sigma) and costs a few dozen FP32 operations, where FP64
// log/sincos cost hundreds of FP64-pipe slots; the thermostat arithmetic
// that uses it stays FP64.
//   ln u, u in (0, 1]: u = m 2^e with m in [sqrt(1/2), sqrt(2)),
//     ln m = 2 atanh(t), t = (m-1)/(m+1), |t| <= 0.172, odd series to t^9;
//   sin/cos(2 pi v): quadrant q = rint(4v), theta = (4v - q) pi/2 in
//     [-pi/4, pi/4], Taylor series to theta^9 (sin) and theta^10 (cos).
__device__ inline float bm_log(float u) {
  const int i = __float_as_int(u);
  int e = ((i >> 23) & 0xff) - 127;
  float m = __int_as_float((i & 0x7fffff) | 0x3f800000);
  if (m > 0x1.6a09e6p+0f) {
    m = __fmul_rn(m, 0.5f);
    e += 1;
  }
  const float t = __fdiv_rn(__fsub_rn(m, 1.f), __fadd_rn(m, 1.f));
  const float t2 = __fmul_rn(t, t);
  float p = __fmaf_rn(t2, 0x1.c71c72p-4f, 0x1.24924ap-3f);
  p = __fmaf_rn(t2, p, 0x1.99999ap-3f);
  p = __fmaf_rn(t2, p, 0x1.555556p-2f);
  p = __fmaf_rn(t2, p, 1.f);
  const float lnm = __fmul_rn(__fmul_rn(2.f, t), p);
  const float fe = (float)e;
  return __fmaf_rn(fe, 0x1.62ep-1f, __fmaf_rn(fe, 0x1.0bfbe8p-15f, lnm));
}

__device__ inline void bm_sincos2pi(float v, float& sn, float& cs) {
  const float x = __fmul_rn(4.f, v);
  const int q = __float2int_rn(x);
  const float th = __fmul_rn(__fsub_rn(x, (float)q), 0x1.921fb6p+0f);
  const float t2 = __fmul_rn(th, th);
  float ps = __fmaf_rn(t2, 0x1.71de3ap-19f, -0x1.a01a02p-13f);
  ps = __fmaf_rn(t2, ps, 0x1.111112p-7f);
  ps = __fmaf_rn(t2, ps, -0x1.555556p-3f);
  const float s = __fmaf_rn(__fmul_rn(th, t2), ps, th);
  float pc = __fmaf_rn(t2, -0x1.27e4fcp-22f, 0x1.a01a02p-16f);
  pc = __fmaf_rn(t2, pc, -0x1.6c16c2p-10f);
  pc = __fmaf_rn(t2, pc, 0x1.555556p-5f);
  pc = __fmaf_rn(t2, pc, -0.5f);
  const float c = __fmaf_rn(t2, pc, 1.f);
  switch (q & 3) {
    case 0: sn = s; cs = c; break;
    case 1: sn = c; cs = -s; break;
    case 2: sn = -s; cs = -c; break;
    default: sn = -c; cs = s; break;
  }
}

__device__ inline void bm_pair(uint32_t wa, uint32_t wb, double& z0, double& z1) {
  const float u = __fmul_rn((float)((wa >> 8) + 1u), 0x1.0p-24f);  // (0, 1]
  const float v = __fmul_rn((float)(wb >> 8), 0x1.0p-24f);         // [0, 1)
  const float rad = __fsqrt_rn(__fmul_rn(-2.f, bm_log(u)));
  float sn, cs;
  bm_sincos2pi(v, sn, cs);
  z0 = (double)__fmul_rn(rad, cs);
  z1 = (double)__fmul_rn(rad, sn);
}

// Deviates 2 pair and 2 pair + 1 of (traj, bead, step, tag): one Philox
// block (counter pair / 2) gives two pairs.
__device__ inline void normal_pair(uint32_t seed, uint32_t traj, uint32_t pair, uint32_t bead, uint32_t step,
                                   uint32_t tag, double& z0, double& z1) {
  const uint4 r = philox4x32_10(make_uint4(pair >> 1, bead, step, tag), seed, traj);
  if (pair & 1u) bm_pair(r.z, r.w, z0, z1);
  else bm_pair(r.x, r.y, z0, z1);
}

// Deviates for all NC coordinates of one bead (coordinate c = deviate c).
template <int NC>
__device__ inline void normals_bead(uint32_t seed, uint32_t traj, uint32_t bead,
                                    uint32_t step, uint32_t tag, double (&z)[NC]) {
#pragma unroll
  for (int i = 0; 4 * i < NC; ++i) {
    const uint4 r = philox4x32_10(make_uint4((uint32_t)i, bead, step, tag), seed, traj);
    double a, b;
    bm_pair(r.x, r.y, a, b);
    z[4 * i] = a;
    if (4 * i + 1 < NC) z[4 * i + 1] = b;
    if (4 * i + 2 < NC) {
      bm_pair(r.z, r.w, a, b);
      z[4 * i + 2] = a;
      if (4 * i + 3 < NC) z[4 * i + 3] = b;
    }
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
