// QMDFF force field on the GB300: one warp per bead.
//
// Drop-in for Caracal's per-bead QMDFF gradient (src/gradient.f90:342-358:
// ff_eg src/ff_eg.f90:41-629, ff_nonb src/ff_nonb.f90:34-889, E_zero shift),
// non-periodic, one molecule.  A bead's coordinates and gradient live in the
// warp's shared memory.  The host packs the terms of each kind into batches
// of 32 (one term per lane) and colours each batch so that no atom appears
// twice within a colour; a lane computes its term, then the warp scatters the
// term gradients colour by colour.  No atomics, fixed accumulation order:
// results are deterministic run to run.
//
// Precision: the plain form computes every term in FP64 with Caracal's
// formulas (divisions by a shared denominator taken as one reciprocal).  The
// mixed form splits each FP64 coordinate once per bead into an FP32 pair
// x = hi + lo; a displacement (hi_a - hi_b) + (lo_a - lo_b) is then within
// about one FP32 ulp of the exact difference without any FP64 work per term.
// Terms run in FP32 with cancellation-free rewrites where the FP64 formula
// subtracts nearly equal numbers (bond stretch from an FP64 r^2 - r0^2,
// dihedral angle from atan2 instead of acos); gradient and energy are
// accumulated with compensated (Neumaier) FP32 sums.
#pragma once
#include <cuda_runtime.h>

#include <type_traits>

#include "../../include/caracal_gb300.h"
#include "dual.cuh"

namespace cr {
namespace qmdff {

constexpr int kMaxAtoms = 1024;
constexpr int kVAngl = 4;   // theta0, k, cos(theta0), linear flag
constexpr int kVPair = 8;   // R0, C6, sr42, zab, alpha, eps2, qq (eps1 q_i q_j or q_i q_j), 0

// Per-term parameter tables in the arithmetic type of the form.
template <class F>
struct Tables {
  const F* rad;    // covalent radius per atom (bohr)
  const F* vbond;  // 3 per bond: r0, k, a
  const F* vangl;  // kVAngl per angle
  const F* vtors;  // 14 per torsion: phi0, V, (rn, phase, Vn) x 4
  const F* vpair;  // kVPair per NCI pair
};

constexpr int kKinds = 5;  // bonds, angles, torsions, NCI pairs, H/halogen bonds

// Warp schedule of the terms: batches of 32 slots (one term per lane) with
// the colour of each slot; no atom appears twice within a colour.
struct Schedule {
  int nb[kKinds];    // batches per kind
  int boff[kKinds];  // first batch of each kind
  const int* slot;             // [batches][32]: term index or -1
  const unsigned char* color;  // [batches][32]
  const unsigned char* ncol;   // [batches]
};

// A periodic box (src/box_image.f90): edges and halves in bohr, and for the
// mixed form the edges as (hi, lo) float pairs and the halves in FP32.
struct PBox {
  double len[3], half[3];
  float flen[3], flen_lo[3], fhalf[3], fhalf_lo[3];
  float fhalf_dn[3], fhalf_up[3];  // half -+ 4 ulps: outside, the hi part decides the image
};
__host__ __device__ inline PBox make_box(const double* len) {
  PBox b;
  for (int k = 0; k < 3; ++k) {
    b.len[k] = len[k];
    b.half[k] = len[k] * 0.5;
    b.flen[k] = (float)len[k];
    b.flen_lo[k] = (float)(len[k] - (double)b.flen[k]);
    b.fhalf[k] = (float)b.half[k];
    b.fhalf_lo[k] = (float)(b.half[k] - (double)b.fhalf[k]);
    b.fhalf_dn[k] = (float)(b.half[k] * (1.0 - 4.8e-7));
    b.fhalf_up[k] = (float)(b.half[k] * (1.0 + 4.8e-7));
  }
  return b;
}

struct Dev {
  int n;
  // [0] plain form: full 32-term batches, as many colours as needed (an FP64
  // term costs far more than a scatter round); [1] mixed form: NCI pairs in
  // round-robin matchings (one colour), bonds up to 3 colours, angles 4,
  // torsions 6, H/halogen bonds 2.
  Schedule sched[2];
  const int* bond;   // 2 per bond (0-based)
  const int* angl;   // 3 per angle (centre, i, k)
  const int* tors;   // 6 per torsion: i, j, k, l, nt, type
  const int* pair;   // 2 per NCI pair
  const int* hb;     // 4 per H/halogen bond: A, B, H, type (1 hydrogen bond, 2 halogen bond)
  const double* vhb; // 2 per H/halogen bond: ca, cb
  Tables<double> d;
  Tables<float> f;
  double coul_cut, zahn_a, zahn_par, e_zero;
  float fcoul_cut, fzahn_a, fzahn_par;  // the same in FP32 (mixed form)
  int zahn;
  // periodic box (src/set_periodic.f90, src/box_image.f90) and the
  // dispersion/repulsion cutoff, bohr
  int periodic;
  PBox box;
  double vdw_cut;
  float fvdw_cut;
  // NpT, set per launch: the box of each trajectory (3 edges, bohr) for
  // beads [t tbox_beads, (t + 1) tbox_beads) in place of `box`, and the
  // virial trace of each bead out (src/ff_eg.f90, ff_nonb.f90, eabhag.f90,
  // eabxag.f90 `vir_ten`); NULL otherwise
  const double* tbox;
  int tbox_beads;
  double* vir;
  int distinct;  // 1: every term's atoms are pairwise distinct
  int nterm[kKinds];  // terms per kind
  // mixed form, bond stretch gradient as a double-FP32 polynomial (see
  // bond_mixed): per bond kBondSer (hi, lo) pairs: 1/r0^2, r0^2, (use flag,
  // 0), the kBondPoly coefficients
  const float2* bser;
  // mixed form, NCI pairs with their constants folded (pair_mixed): per pair
  // kVPair floats R0^6, R0^8, eps2 C6, eps2 C6 sr42, eps2 zab,
  // alpha log2(e), qq, alpha, each rounded once from FP64
  const float* fpair;
};

constexpr int kBondPoly = 24;             // polynomial of degree 23
constexpr int kBondSer = kBondPoly + 3;
constexpr double kBondSerMaxT = 0.45;     // used for |r^2/r0^2 - 1| <= this

// Double-FP32 ("float-float") numbers hi + lo, |lo| <= ulp(hi)/2: about 44
// bits of significand from FP32 operations (error-free sum of Knuth, product
// split by FMA).  Used where FP32 rounding would set the mixed form's error.
struct FF {
  float hi, lo;
};
__device__ inline FF ff_norm(float s, float e) {
  const float h = s + e;
  return FF{h, e - (h - s)};
}
__device__ inline FF ff_add(FF a, FF b) {
  const float s = a.hi + b.hi, bb = s - a.hi;
  const float e = (a.hi - (s - bb)) + (b.hi - bb);
  return ff_norm(s, e + (a.lo + b.lo));
}
__device__ inline FF ff_mul(FF a, FF b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
  return ff_norm(p, e);
}
__device__ inline FF ff_of(float2 v) { return FF{v.x, v.y}; }

template <class F> __device__ inline F q_sqrt(F x);
template <> __device__ inline double q_sqrt<double>(double x) { return sqrt(x); }
template <> __device__ inline float q_sqrt<float>(float x) { return sqrtf(x); }
template <class F> __device__ inline F q_exp(F x);
template <> __device__ inline double q_exp<double>(double x) { return exp(x); }
template <> __device__ inline float q_exp<float>(float x) { return expf(x); }
template <class F> __device__ inline F q_acos(F x);
template <> __device__ inline double q_acos<double>(double x) { return acos(x); }
template <> __device__ inline float q_acos<float>(float x) { return acosf(x); }
template <class F> __device__ inline F q_asin(F x);
template <> __device__ inline double q_asin<double>(double x) { return asin(x); }
template <> __device__ inline float q_asin<float>(float x) { return asinf(x); }
template <class F> __device__ inline F q_erf(F x);
template <> __device__ inline double q_erf<double>(double x) { return erf(x); }
template <> __device__ inline float q_erf<float>(float x) { return erff(x); }
template <class F> __device__ inline F q_erfc(F x);
template <> __device__ inline double q_erfc<double>(double x) { return erfc(x); }
template <> __device__ inline float q_erfc<float>(float x) { return erfcf(x); }
template <class F> __device__ inline F q_sin(F x);
template <> __device__ inline double q_sin<double>(double x) { return sin(x); }
template <> __device__ inline float q_sin<float>(float x) { return sinf(x); }
template <class F> __device__ inline F q_cos(F x);
template <> __device__ inline double q_cos<double>(double x) { return cos(x); }
template <> __device__ inline float q_cos<float>(float x) { return cosf(x); }
template <class F> __device__ inline F q_pow(F x, double p);
template <> __device__ inline double q_pow<double>(double x, double p) { return pow(x, p); }
// dual coordinates (Hessian-vector products of the plain form)
template <> __device__ inline Dual q_sqrt<Dual>(Dual x) { return sqrt(x); }
template <> __device__ inline Dual q_exp<Dual>(Dual x) { return exp(x); }
template <> __device__ inline Dual q_acos<Dual>(Dual x) { return acos(x); }
template <> __device__ inline Dual q_asin<Dual>(Dual x) { return asin(x); }
template <> __device__ inline Dual q_erf<Dual>(Dual x) { return erf(x); }
template <> __device__ inline Dual q_erfc<Dual>(Dual x) { return erfc(x); }
template <> __device__ inline Dual q_sin<Dual>(Dual x) { return sin(x); }
template <> __device__ inline Dual q_cos<Dual>(Dual x) { return cos(x); }
template <> __device__ inline Dual q_pow<Dual>(Dual x, double p) { return pow(x, p); }

// |x| < 1e-14 and |x| > 1e-14 as the reference tests its FP64 denominators;
// for FP32 the same sets of values without a conversion (1e-14 is not a
// float: |x| < 1e-14 holds exactly for |x| <= 1e-14f).
template <class F> __device__ inline bool below_1em14(F x) { return fabs((double)ad::val(x)) < 1e-14; }
template <> __device__ inline bool below_1em14<float>(float x) { return fabsf(x) <= 1e-14f; }
template <class F> __device__ inline bool above_1em14(F x) { return fabs((double)ad::val(x)) > 1e-14; }
template <> __device__ inline bool above_1em14<float>(float x) { return fabsf(x) > 1e-14f; }

// Parameter type of a term evaluated in arithmetic type F (dual coordinates
// read FP64 parameters).
template <class F> struct ParamOf { using type = F; };
template <> struct ParamOf<Dual> { using type = double; };

template <class F>
__device__ inline void cross(const F* a, const F* b, F* c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}
template <class F>
__device__ inline F dot3(const F* a, const F* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// Gradient contribution of one term: up to four atoms.
template <class F>
struct Contrib {
  int na;
  int a[4];
  F g[4][3];
};

// Gradient accumulator of one bead in shared memory: FP64 in the plain form,
// compensated FP32 (sum and compensation arrays) in the mixed form.
template <class F>
struct Grad;
template <>
struct Grad<double> {
  double* g;
  __device__ inline void add(int i, double v) { g[i] += v; }
  __device__ inline double get(int i) const { return g[i]; }
};
template <>
struct Grad<float> {
  float2* sk;  // (sum, compensation) per coordinate: one 8-byte access each
  float* pr;   // NCI pair contributions, a plain FP32 sum: they are ~1 % of
               // the valence forces, so their own rounding stays below the
               // compensated sum's, and keeping them apart leaves that sum
               // free of many small additions
  __device__ inline void add(int i, float v) {
    float2 c = sk[i];
    const float t = c.x + v;
    c.y += (fabsf(c.x) >= fabsf(v)) ? ((c.x - t) + v) : ((v - t) + c.x);
    c.x = t;
    sk[i] = c;
  }
  __device__ inline double get(int i) const { return ((double)sk[i].x + (double)sk[i].y) + (double)pr[i]; }
};

// Adds a term's gradient for its NA atoms (compile-time count).  Mixed form
// with distinct atoms (checked on the host, `Dev::distinct`): all loads are
// issued before the stores, so the shared-memory round trips overlap.  The
// FP64 form is bound by the FP64 pipe, not by these round trips, and keeps
// the sequential adds (fewer live registers).
template <int NA>
__device__ inline void scatter(const Contrib<double>& c, Grad<double>& G, bool) {
#pragma unroll
  for (int m = 0; m < NA; ++m)
#pragma unroll
    for (int d = 0; d < 3; ++d) G.add(3 * c.a[m] + d, c.g[m][d]);
}
// bond of the mixed form: (hi, lo) parts in g[0..1] and g[2..3]
__device__ inline void scatter_bond(const Contrib<float>& c, Grad<float>& G) {
#pragma unroll
  for (int m = 0; m < 2; ++m)
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      G.add(3 * c.a[m] + d, c.g[m][d]);
      G.add(3 * c.a[m] + d, c.g[m + 2][d]);
    }
}
template <int NA>
__device__ inline void scatter_pair(const Contrib<float>& c, Grad<float>& G) {
  float a[NA][3];
#pragma unroll
  for (int m = 0; m < NA; ++m)
#pragma unroll
    for (int d = 0; d < 3; ++d) a[m][d] = G.pr[3 * c.a[m] + d];
#pragma unroll
  for (int m = 0; m < NA; ++m)
#pragma unroll
    for (int d = 0; d < 3; ++d) G.pr[3 * c.a[m] + d] = a[m][d] + c.g[m][d];
}
template <int NA>
__device__ inline void scatter(const Contrib<float>& c, Grad<float>& G, bool distinct) {
  if (distinct) {
    float2 a[NA][3];
#pragma unroll
    for (int m = 0; m < NA; ++m)
#pragma unroll
      for (int d = 0; d < 3; ++d) a[m][d] = G.sk[3 * c.a[m] + d];
#pragma unroll
    for (int m = 0; m < NA; ++m)
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const float v = c.g[m][d], s0 = a[m][d].x, t = s0 + v;
        const float k = a[m][d].y + ((fabsf(s0) >= fabsf(v)) ? ((s0 - t) + v) : ((v - t) + s0));
        G.sk[3 * c.a[m] + d] = make_float2(t, k);
      }
  } else {
#pragma unroll
    for (int m = 0; m < NA; ++m)
#pragma unroll
      for (int d = 0; d < 3; ++d) G.add(3 * c.a[m] + d, c.g[m][d]);
  }
}

// abdamp (src/abdamp.f90:36-51); the cutoff prefactor is the REAL(4) product 3.0*3.5710642
template <class F>
__device__ inline void abdamp(F radi, F radj, F r2, F& damp, F& ddamp) {
  const F pre = (F)(double)(3.0f * 3.5710642f);
  const F s = radi + radj;
  const F rcut = pre * (s * s);
  const F x = r2 / rcut;
  const F rr = x * x;
  if constexpr (std::is_same<F, float>::value) damp = __frcp_rn(1.0f + rr);  // = 1/(1 + rr), correctly rounded
  else damp = F(1) / (F(1) + rr);
  ddamp = F(-4) * rr * (damp * damp) / r2;
}

// A bead's coordinates: FP64, and (mixed form) the FP32 split x = hi + lo.
struct BeadPos {
  const double* x;
  const float2* hl;  // (hi, lo) per coordinate (mixed form only)
  const double* w;   // tangent direction (dual coordinates only)
  const PBox* pbc;   // the bead's box where periodic, else NULL
};

// box_image (src/box_image.f90:36-63): subtract the edge while a component
// exceeds half of it; bounded (a non-finite or absurd vector stops after
// kImageIters subtractions and the step's NaN check reports it).  In FP32
// the vector is a (hi, lo) pair and the edge is subtracted as one.
constexpr int kImageIters = 64;
__device__ inline double image1(double v, double len, double half) {
  for (int it = 0; it < kImageIters && fabs(v) > half; ++it) v = v - copysign(len, v);
  return v;
}
// FP32: the difference of two (hi, lo) coordinates as an exact float pair
// first (atoms a box edge apart are not close enough for the hi parts to
// subtract exactly), the edge subtracted as a pair, then rounded once.
// |d| > half, so that the choice of image agrees with FP64's except within
// ~1e-14 of half the edge: the hi part decides unless it lies within 4 ulps
// of half, where |d| - half is formed as a float pair.
static __device__ __noinline__ bool beyond_half_pair(FF d, float half, float half_lo) {
  const FF a = d.hi < 0.0f ? FF{-d.hi, -d.lo} : d;
  const FF t = ff_add(a, FF{-half, -half_lo});
  return t.hi > 0.0f || (t.hi == 0.0f && t.lo > 0.0f);
}
__device__ inline bool beyond_half(FF d, const PBox& b, int k) {
  const float ah = fabsf(d.hi);
  if (ah > b.fhalf_up[k]) return true;
  if (ah < b.fhalf_dn[k]) return false;
  return beyond_half_pair(d, b.fhalf[k], b.fhalf_lo[k]);  // out of line: rarely taken
}
__device__ inline float image1(FF d, const PBox& b, int k) {
  const float len = b.flen[k], len_lo = b.flen_lo[k];
  for (int it = 0; it < kImageIters && beyond_half(d, b, k); ++it) {
    const float s = copysignf(1.0f, d.hi);
    d = ff_add(d, FF{-s * len, -s * len_lo});
  }
  return d.hi + d.lo;
}

template <class F>
__device__ inline void disp(const BeadPos& X, int a, int b, F* v);
template <>
__device__ inline void disp<double>(const BeadPos& X, int a, int b, double* v) {
  v[0] = X.x[3 * a] - X.x[3 * b];
  v[1] = X.x[3 * a + 1] - X.x[3 * b + 1];
  v[2] = X.x[3 * a + 2] - X.x[3 * b + 2];
  if (X.pbc) {
#pragma unroll
    for (int d = 0; d < 3; ++d) v[d] = image1(v[d], X.pbc->len[d], X.pbc->half[d]);
  }
}
template <>
__device__ inline void disp<Dual>(const BeadPos& X, int a, int b, Dual* v) {
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    double x = X.x[3 * a + d] - X.x[3 * b + d];
    if (X.pbc) x = image1(x, X.pbc->len[d], X.pbc->half[d]);
    v[d] = Dual(x, X.w[3 * a + d] - X.w[3 * b + d]);
  }
}
template <>
__device__ inline void disp<float>(const BeadPos& X, int a, int b, float* v) {
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float2 u = X.hl[3 * a + d], w = X.hl[3 * b + d];
    if (X.pbc)
      v[d] = image1(ff_add(FF{u.x, u.y}, FF{-w.x, -w.y}), *X.pbc, d);
    else v[d] = (u.x - w.x) + (u.y - w.y);
  }
}

// Bond stretch, generalised Lennard-Jones (src/ff_eg.f90:87-163):
// e = k (1 + (r0/r)^a - 2 (r0/r)^(a/2)).
template <class F>
__device__ inline F bond_plain(const Dev& D, const Tables<typename ParamOf<F>::type>& T, const BeadPos& x, int m,
                               Contrib<F>& c) {
  const int i = D.bond[2 * m], j = D.bond[2 * m + 1];
  F rb[3];
  disp<F>(x, i, j, rb);
  const F r2 = rb[0] * rb[0] + rb[1] * rb[1] + rb[2] * rb[2];
  const F r = q_sqrt<F>(r2);
  const auto* v = &T.vbond[3 * m];
  const double rij = v[0], kij = v[1], aai = v[2];
  const F pa2 = q_pow<F>(rij / r, aai / 2), pa = pa2 * pa2;
  const F fac = aai * kij * (-pa + pa2) / r2;
  c.na = 2;
  c.a[0] = i;
  c.a[1] = j;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    c.g[0][d] = fac * rb[d];
    c.g[1][d] = -fac * rb[d];
  }
  return kij * (1. + pa - 2. * pa2);
}

// Mixed form: with u = (r0/r)^(a/2) = exp(-(a/2) log1p(x)), x = (r - r0)/r0
// taken from the FP64 r^2 - r0^2, e = k (1 - u)^2 and the gradient factor
// a k u (1 - u) / r^2 are free of the cancellation in 1 + u^2 - 2u.
// Bond stretches carry the largest forces of a molecule, so FP32 roundings
// of their gradient set the form's force error (~4e-7 of the largest force;
// angles, torsions and pairs stay below 7e-8).  The gradient is therefore
// taken in double-FP32 arithmetic without transcendentals: with
// t = r^2/r0^2 - 1,
// a k u (1 - u) / r^2 = (a k / r0^2) [(1+t)^-(a/4+1) - (1+t)^-(a/2+1)]
//                     = t H(t),
// H a degree-23 polynomial in t / kBondSerMaxT (Chebyshev interpolation of
// H on |t| <= kBondSerMaxT, fitted per bond on the host, relative error
// below 1e-10 for exponents a <= 16), summed by Horner; the displacement
// comes exactly from the (hi, lo) coordinates and the gradient is scattered
// as its (hi, lo) pair.  Beyond that range, and for the energy, the FP32
// formula above (the FP64 pipe would cost more than the whole FP32 term).
__device__ inline float bond_mixed(const Dev& D, const BeadPos& x, int m, Contrib<float>& c) {
  const int i = D.bond[2 * m], j = D.bond[2 * m + 1];
  const float2* ser = D.bser + (size_t)kBondSer * m;
  // displacement as double-FP32 from the (hi, lo) coordinates
  FF dv[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float2 a = x.hl[3 * i + d], b = x.hl[3 * j + d];
    dv[d] = ff_add(FF{a.x, a.y}, FF{-b.x, -b.y});
    if (x.pbc) {
      for (int it = 0; it < kImageIters && beyond_half(dv[d], *x.pbc, d); ++it) {
        const float sg = copysignf(1.0f, dv[d].hi);
        dv[d] = ff_add(dv[d], FF{-sg * x.pbc->flen[d], -sg * x.pbc->flen_lo[d]});
      }
    }
  }
  FF r2f = ff_mul(dv[0], dv[0]);
  r2f = ff_add(r2f, ff_mul(dv[1], dv[1]));
  r2f = ff_add(r2f, ff_mul(dv[2], dv[2]));
  const FF r0sq = ff_of(__ldg(ser + 1));
  const float r2 = r2f.hi;
  const float r = sqrtf(r2);
  const float r0 = D.f.vbond[3 * m];
  const FF d2 = ff_add(r2f, FF{-r0sq.hi, -r0sq.lo});
  const float dr = (d2.hi + d2.lo) / (r + r0);  // r - r0
  const float kij = D.f.vbond[3 * m + 1], aai = D.f.vbond[3 * m + 2];
  const float lg = -0.5f * aai * log1pf(dr / r0);
  const float omu = -expm1f(lg);  // 1 - u
  const float u = 1.0f - omu;
  const float fac = aai * kij * u * omu / r2;  // a k (u - u^2) / r^2
  c.na = 2;
  c.a[0] = i;
  c.a[1] = j;
  const FF t = ff_add(ff_mul(r2f, ff_of(__ldg(ser))), FF{-1.0f, 0.0f});
  if (__ldg(ser + 2).x != 0.0f && fabsf(t.hi) <= (float)kBondSerMaxT) {
    // 1 / kBondSerMaxT = 20/9 as a double-FP32 constant
    const FF xs = ff_mul(t, FF{2.22222232818603515625f, -1.0596381372e-07f});
    FF h = ff_of(__ldg(ser + 3 + kBondPoly - 1));
#pragma unroll
    for (int k = kBondPoly - 2; k >= 0; --k) h = ff_add(ff_mul(h, xs), ff_of(__ldg(ser + 3 + k)));
    const FF f = ff_mul(t, h);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const FF g = ff_mul(f, dv[d]);
      c.g[0][d] = g.hi;
      c.g[1][d] = -g.hi;
      c.g[2][d] = g.lo;
      c.g[3][d] = -g.lo;
    }
  } else {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const float rb = dv[d].hi;
      c.g[0][d] = fac * rb;
      c.g[1][d] = -fac * rb;
      c.g[2][d] = 0.0f;
      c.g[3][d] = 0.0f;
    }
  }
  return kij * omu * omu;
}

// Angle bend with abdamp damping (src/ff_eg.f90:167-299).
template <class F>
__device__ inline F angle_term(const Dev& D, const Tables<typename ParamOf<F>::type>& T, const BeadPos& x, int m,
                               Contrib<F>& c) {
  const int j = D.angl[3 * m], i = D.angl[3 * m + 1], k = D.angl[3 * m + 2];
  const auto* v = &T.vangl[kVAngl * m];
  const F c0 = v[0], kijk = v[1], cc0 = v[2];
  F vab[3], vcb[3], vp[3];
  disp<F>(x, i, j, vab);
  disp<F>(x, k, j, vcb);
  const F rab2 = dot3(vab, vab), rcb2 = dot3(vcb, vcb);
  cross(vcb, vab, vp);
  const F vpl = dot3(vp, vp);
  const F rp = (vpl > F(0) ? q_sqrt<F>(vpl) : F(0)) + F(1e-14);
  const F al = q_sqrt<F>(rab2), bl = q_sqrt<F>(rcb2);
  F cosa = (al > F(0) && bl > F(0)) ? dot3(vab, vcb) / (al * bl) : F(0);
  cosa = fmin(F(1), fmax(F(-1), cosa));
  // FP32: theta only for linear reference angles; sin(theta) of the
  // harmonic-cosine form as sqrt((1 - c)(1 + c)), free of cancellation away
  // from c = +-1 (where the linear form is used)
  F theta = F(0);
  if (!std::is_same<F, float>::value || v[3] != F(0)) theta = q_acos<F>(cosa);
  F dampij, damp2ij, dampjk, damp2jk;
  abdamp<F>(T.rad[i], T.rad[j], rab2, dampij, damp2ij);
  abdamp<F>(T.rad[k], T.rad[j], rcb2, dampjk, damp2jk);
  const F damp = dampij * dampjk;
  F ea, deddt;
  if (v[3] != F(0)) {  // linear reference angle: harmonic in theta
    const F dt = theta - c0;
    ea = kijk * (dt * dt);
    deddt = F(2) * kijk * dt;
  } else {
    const F dd = cosa - cc0;
    ea = kijk * (dd * dd);
    F sth;
    if constexpr (std::is_same<F, float>::value) sth = sqrtf((1.0f - cosa) * (1.0f + cosa));
    else sth = q_sin<F>(theta);
    deddt = F(2) * kijk * sth * (cc0 - cosa);
  }
  F deda[3], dedc[3];
  cross(vab, vp, deda);
  cross(vcb, vp, dedc);
  const F rmul1 = -deddt / (rab2 * rp), rmul2 = deddt / (rcb2 * rp);
  c.na = 3;
  c.a[0] = i;
  c.a[1] = j;
  c.a[2] = k;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const F da = deda[d] * rmul1, dc = dedc[d] * rmul2;
    const F t1 = ea * damp2ij * dampjk * vab[d];
    const F t2 = ea * damp2jk * dampij * vcb[d];
    c.g[0][d] = da * damp + t1;
    c.g[1][d] = -(da + dc) * damp - t1 - t2;
    c.g[2][d] = dc * damp + t2;
  }
  return ea * damp;
}

// Torsion angle phi in [0, pi] of i-j-k-l (valijkl, src/valijkl.f90) with
// its cosine and sine.  FP64: Caracal's acos of the normalised plane normals.
// FP32: atan2(|rb| |na . rc|, na . nb), accurate near 0 and pi.
template <class F>
__device__ inline F dihedral(const F* ra, const F* rb, const F* rc, F* na, F* nb, F& nan_, F& nbn,
                             F& cosphi, F& sinphi) {
  cross(ra, rb, na);
  cross(rb, rc, nb);
  nan_ = q_sqrt<F>(dot3(na, na));
  nbn = q_sqrt<F>(dot3(nb, nb));
  F phi;
  if constexpr (!std::is_same<F, float>::value) {
    F a[3] = {na[0], na[1], na[2]}, b[3] = {nb[0], nb[1], nb[2]};
    if (fabs(ad::val(nan_)) > 1e-14) {
      const F o = 1.0 / nan_;
      a[0] *= o;
      a[1] *= o;
      a[2] *= o;
    }
    if (fabs(ad::val(nbn)) > 1e-14) {
      const F o = 1.0 / nbn;
      b[0] *= o;
      b[1] *= o;
      b[2] *= o;
    }
    F s = a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
    if (fabs(fabs(ad::val(s)) - 1.0) < 1e-14) s = ad::val(s) >= 0 ? F(1.0) : F(-1.0);
    phi = q_acos<F>(s);
    cosphi = q_cos<F>(phi);
    sinphi = q_sin<F>(phi);
  } else {
    const float cn = dot3(na, nb);
    const float sn = sqrtf(dot3(rb, rb)) * fabsf(dot3(na, rc));
    phi = atan2f(sn, cn);
    const float den = nan_ * nbn;
    const float id = den > 0.f ? __frcp_rn(den) : 0.f;
    cosphi = den > 0.f ? cn * id : 1.f;
    sinphi = den > 0.f ? sn * id : 0.f;
  }
  return phi;
}

// vab.g_a + vcb.(g_c + g_d) + vdc.g_d with the term's own vectors: the
// torsions' and inversions' vir_ten (src/ff_eg.f90:420-440, 583-603).
template <class F>
__device__ inline F tors_virial(const F* vab, const F* vcb, const F* vdc, const Contrib<F>& c) {
  const F gcd[3] = {c.g[2][0] + c.g[3][0], c.g[2][1] + c.g[3][1], c.g[2][2] + c.g[3][2]};
  return dot3(vab, c.g[0]) + dot3(vcb, gcd) + dot3(vdc, c.g[3]);
}

// Torsions (erf-blended cosine series, src/ff_eg.f90:303-440) and
// inversions (tors type 2, src/ff_eg.f90:441-618).
template <class F>
__device__ inline F torsion_term(const Dev& D, const Tables<typename ParamOf<F>::type>& T, const BeadPos& x, int m,
                                 Contrib<F>& c, F* vir = nullptr) {
  const F pi = (F)3.1415926535897932384626433832795029;
  const F pi2 = (F)6.28318530717958623199592693708837;
  const F spi = (F)1.77245385090551599275151910313925;
  const int i = D.tors[6 * m], j = D.tors[6 * m + 1], k = D.tors[6 * m + 2], l = D.tors[6 * m + 3];
  const int nt = D.tors[6 * m + 4], type = D.tors[6 * m + 5];
  const auto* vt = &T.vtors[14 * m];
  const F phi0 = vt[0];
  F vab[3], vcb[3], vdc[3], dda[3], ddb[3], ddc[3], ddd[3];
  F et, dij, dampij, dampjk, dampX, d2ij, d2jk, d2X;
  c.na = 4;
  c.a[0] = i;
  c.a[1] = j;
  c.a[2] = k;
  c.a[3] = l;
  if (type != 2) {
    disp<F>(x, i, j, vab);
    disp<F>(x, j, k, vcb);
    disp<F>(x, k, l, vdc);
    abdamp<F>(T.rad[i], T.rad[j], dot3(vab, vab), dampij, d2ij);
    abdamp<F>(T.rad[k], T.rad[j], dot3(vcb, vcb), dampjk, d2jk);
    abdamp<F>(T.rad[k], T.rad[l], dot3(vdc, vdc), dampX, d2X);
    // dphidr (src/dphidr.f90): ra = r_j - r_i, rb = r_k - r_j, rc = r_l - r_k
    const F ra[3] = {-vab[0], -vab[1], -vab[2]}, rb[3] = {-vcb[0], -vcb[1], -vcb[2]};
    const F rc[3] = {-vdc[0], -vdc[1], -vdc[2]};
    F na[3], nb[3], nan_, nbn, cosphi, sinphi;
    const F phi = dihedral<F>(ra, rb, rc, na, nb, nan_, nbn, cosphi, sinphi);
    const F nenner = nan_ * nbn * sinphi;
    if constexpr (std::is_same<F, float>::value) {
      // FP32: dphi/dr without the division by sin(phi) of dphidr.f90, whose
      // numerator cancels as phi -> 0 or pi (planar groups); the same
      // derivative, written with the plane normals (Blondel and Karplus,
      // J. Comput. Chem. 17, 1132 (1996)):
      //   dphi/dr_i = -s |rb| na / |na|^2,  dphi/dr_l = s |rb| nb / |nb|^2,
      //   dphi/dr_j = -dphi/dr_i + s (u + v),  dphi/dr_k = -dphi/dr_l - s (u + v),
      //   u = (ra.rb) na / (|na|^2 |rb|),  v = (rc.rb) nb / (|nb|^2 |rb|),
      // s = sign(na.rc) (phi is the unsigned angle)
      const float a2 = dot3(na, na), b2 = dot3(nb, nb), tr = dot3(na, rc);
      const float sg = (tr > 0.f) ? 1.f : ((tr < 0.f) ? -1.f : 0.f);
      if (!(a2 > 0.f) || !(b2 > 0.f)) {
#pragma unroll
        for (int d = 0; d < 3; ++d) dda[d] = ddb[d] = ddc[d] = ddd[d] = 0.f;
      } else {
        const float L = sqrtf(dot3(rb, rb)), ia2 = __frcp_rn(a2), ib2 = __frcp_rn(b2), iL = __frcp_rn(L);
        const float fa = sg * L * ia2, fb = sg * L * ib2;
        const float fu = sg * dot3(ra, rb) * ia2 * iL, fv = sg * dot3(rc, rb) * ib2 * iL;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          const float uv = fu * na[d] + fv * nb[d];
          dda[d] = -fa * na[d];
          ddd[d] = fb * nb[d];
          ddb[d] = fa * na[d] + uv;
          ddc[d] = -fb * nb[d] - uv;
        }
      }
    } else if (below_1em14(nenner)) {
#pragma unroll
      for (int d = 0; d < 3; ++d) dda[d] = ddb[d] = ddc[d] = ddd[d] = F(0);
    } else {
      F on, rba_, rab_;
      if constexpr (std::is_same<F, float>::value) {
        on = __frcp_rn(nenner);
        rba_ = nbn * __frcp_rn(nan_);
        rab_ = nan_ * __frcp_rn(nbn);
      } else {
        on = F(1) / nenner;
        rba_ = nbn / nan_;
        rab_ = nan_ / nbn;
      }
      const F rapb[3] = {ra[0] + rb[0], ra[1] + rb[1], ra[2] + rb[2]};
      const F rbpc[3] = {rb[0] + rc[0], rb[1] + rc[1], rb[2] + rc[2]};
      F t_rab[3], t_rba[3], t_rac[3], t_rbb[3], t_rbc[3], t_raa[3], rapba[3], rapbb[3], rbpca[3], rbpcb[3];
      cross(na, rb, t_rab);
      cross(nb, ra, t_rba);
      cross(na, rc, t_rac);
      cross(nb, rb, t_rbb);
      cross(nb, rc, t_rbc);
      cross(na, ra, t_raa);
      cross(rapb, na, rapba);
      cross(rapb, nb, rapbb);
      cross(rbpc, na, rbpca);
      cross(rbpc, nb, rbpcb);
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        dda[d] = on * (cosphi * rba_ * t_rab[d] - t_rbb[d]);
        ddb[d] = on * (cosphi * (rba_ * rapba[d] + rab_ * t_rbc[d]) - (t_rac[d] + rapbb[d]));
        ddc[d] = on * (cosphi * (rba_ * t_raa[d] + rab_ * rbpcb[d]) - (t_rba[d] + rbpca[d]));
        ddd[d] = on * (cosphi * rab_ * t_rbb[d] - t_rab[d]);
      }
    }
    et = F(0);
    dij = F(0);
    const F phipi = phi - pi;
    const F ef = q_erf<F>(phipi);
    F expo;
    if constexpr (std::is_same<F, float>::value) expo = q_exp<F>(-(phipi * phipi)) * 0.564189583547756286948f;  // 1/sqrt(pi)
    else expo = q_exp<F>(-(phipi * phipi)) / spi;
    for (int it = 0; it < nt; ++it) {
      const F rn = vt[2 + 3 * it], ph = vt[3 + 3 * it], vn = vt[4 + 3 * it];
      const F c1 = rn * (phi - phi0) + ph;
      const F c2 = rn * (phi + phi0 - pi2) + ph;
      F x1cos, x2cos, x1sin, x2sin;
      if constexpr (std::is_same<F, float>::value) {
        sincosf(c1, &x1sin, &x1cos);
        sincosf(c2, &x2sin, &x2cos);
      } else {
        x1cos = q_cos<F>(c1);
        x2cos = q_cos<F>(c2);
        x1sin = q_sin<F>(c1);
        x2sin = q_sin<F>(c2);
      }
      const F e1 = vn * (F(1) + x1cos), e2 = vn * (F(1) + x2cos);
      et = et + F(0.5) * (F(1) - ef) * e1 + (F(0.5) + F(0.5) * ef) * e2;
      dij = dij - expo * e1 - F(0.5) * (F(1) - ef) * vn * x1sin * rn + expo * e2 -
            (F(0.5) + F(0.5) * ef) * vn * x2sin * rn;
    }
    et = et * vt[1];
    const F damp = dampjk * dampij * dampX;
    dij = dij * vt[1] * damp;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const F t1 = et * d2ij * dampjk * dampX * vab[d];
      const F t2 = et * d2jk * dampij * dampX * vcb[d];
      const F t3 = et * d2X * dampij * dampjk * vdc[d];
      c.g[0][d] = dij * dda[d] + t1;
      c.g[1][d] = dij * ddb[d] - t1 + t2;
      c.g[2][d] = dij * ddc[d] + t3 - t2;
      c.g[3][d] = dij * ddd[d] - t3;
    }
    if (vir) *vir = tors_virial(vab, vcb, vdc, c);
    return et * damp;
  }
  // inversion: omega (src/omega.f90) and domegadr (src/domegadr.f90)
  disp<F>(x, j, i, vab);
  disp<F>(x, j, k, vcb);
  disp<F>(x, j, l, vdc);
  abdamp<F>(T.rad[i], T.rad[j], dot3(vab, vab), dampij, d2ij);
  abdamp<F>(T.rad[k], T.rad[j], dot3(vcb, vcb), dampjk, d2jk);
  abdamp<F>(T.rad[j], T.rad[l], dot3(vdc, vdc), dampX, d2X);
  const F re[3] = {-vab[0], -vab[1], -vab[2]};  // r_i - r_j
  const F rd[3] = {-vcb[0], -vcb[1], -vcb[2]};  // r_k - r_j
  F rv[3];
  disp<F>(x, l, i, rv);                          // r_l - r_i
  F rn[3];
  cross(re, rd, rn);
  const F rnn = q_sqrt<F>(dot3(rn, rn)), rvn = q_sqrt<F>(dot3(rv, rv));
  F om;
  if constexpr (!std::is_same<F, float>::value) {
    F a[3] = {rn[0], rn[1], rn[2]}, b[3] = {rv[0], rv[1], rv[2]};
    if (fabs(ad::val(rnn)) > 1e-14) {
      const F o = 1.0 / rnn;
      a[0] *= o;
      a[1] *= o;
      a[2] *= o;
    }
    if (fabs(ad::val(rvn)) > 1e-14) {
      const F o = 1.0 / rvn;
      b[0] *= o;
      b[1] *= o;
      b[2] *= o;
    }
    om = q_asin<F>(a[0] * b[0] + a[1] * b[1] + a[2] * b[2]);
  } else {
    om = q_asin<F>(fmin(F(1), fmax(F(-1), dot3(rn, rv) / (rnn * rvn))));
  }
  const F sinom = q_sin<F>(om), cosom = q_cos<F>(om);
  const F rdme[3] = {rd[0] - re[0], rd[1] - re[1], rd[2] - re[2]};
  F rve[3], rne[3], rdv[3], rdn[3], rvdme[3], rndme[3];
  cross(rv, re, rve);
  cross(rn, re, rne);
  cross(rd, rv, rdv);
  cross(rd, rn, rdn);
  cross(rv, rdme, rvdme);
  cross(rn, rdme, rndme);
  const F nenner = rnn * rvn * cosom;
  if (above_1em14(nenner)) {
    const F on = F(1) / nenner;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      dda[d] = on * (rdv[d] - rn[d] - sinom * (rvn / rnn * rdn[d] - rnn / rvn * rv[d]));
      ddb[d] = on * (rvdme[d] - sinom * rvn / rnn * rndme[d]);
      ddc[d] = on * (rve[d] - sinom * rvn / rnn * rne[d]);
      ddd[d] = on * (rn[d] - sinom * rnn / rvn * rv[d]);
    }
  } else {
#pragma unroll
    for (int d = 0; d < 3; ++d) dda[d] = ddb[d] = ddc[d] = ddd[d] = F(0);
  }
  const F damp = dampjk * dampij * dampX;
  if constexpr (std::is_same<F, float>::value) {
    // FP32: the differences of cosines as products of sines, cos a - cos b
    // = -2 sin((a+b)/2) sin((a-b)/2) and 1 - cos a = 2 sin^2(a/2): near
    // omega = phi0 the reference's forms cancel to a few bits in float,
    // which the large inversion barriers of planar centres (tens of Eh)
    // turn into force errors of 1e-6
    const float h = 0.5f * (om - phi0), sh = sinf(h);
    if (vt[2] > 1e-6f) {
      et = 2.f * sh * sh * vt[1];
      dij = sinf(om - phi0) * vt[1] * damp;
    } else {
      const float dd = -2.f * sinf(0.5f * (om + phi0)) * sh;  // cos(om) - cos(phi0)
      et = vt[1] * (dd * dd);
      dij = -2.f * vt[1] * sinf(om) * dd * damp;
    }
  } else if (vt[2] > F(1e-6)) {
    const F c1 = (om - phi0) + pi;
    et = (F(1) + q_cos<F>(c1)) * vt[1];
    dij = -q_sin<F>(c1) * vt[1] * damp;
  } else {
    const F dd = q_cos<F>(om) - q_cos<F>(phi0);
    et = vt[1] * (dd * dd);
    dij = F(2) * vt[1] * q_sin<F>(om) * (q_cos<F>(phi0) - q_cos<F>(om)) * damp;
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const F t1 = et * d2ij * dampjk * dampX * vab[d];
    const F t2 = et * d2jk * dampij * dampX * vcb[d];
    const F t3 = et * d2X * dampij * dampjk * vdc[d];
    c.g[0][d] = dij * dda[d] - t1;
    c.g[1][d] = dij * ddb[d] + t1 + t2 + t3;
    c.g[2][d] = dij * ddc[d] - t2;
    c.g[3][d] = dij * ddd[d] - t3;
  }
  if (vir) *vir = tors_virial(vab, vcb, vdc, c);
  return et * damp;
}

// kVPair parameters of one pair with 16-byte loads (rows are 32 / 64 bytes).
__device__ inline void load_pair_params(const float* p, float* v) {
  const float4 a = __ldg(reinterpret_cast<const float4*>(p)), b = __ldg(reinterpret_cast<const float4*>(p) + 1);
  v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
  v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
}
__device__ inline void load_pair_params(const double* p, double* v) {
  const double2* q = reinterpret_cast<const double2*>(p);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const double2 t = __ldg(q + k);
    v[2 * k] = t.x;
    v[2 * k + 1] = t.y;
  }
}
__device__ inline void load_pair_params(const double* p, Dual* v) {
  double t[kVPair];
  load_pair_params(p, t);
#pragma unroll
  for (int k = 0; k < kVPair; ++k) v[k] = Dual(t[k]);
}

// One NCI pair (src/ff_nonb.f90): BJ-damped C6/C8 dispersion and, for
// r < 25 bohr, exponential repulsion, both times eps2 (:79-193); Coulomb
// within coul_cut (:337-416), eps1 q_i q_j / r or the Zahn form.
template <class F>
__device__ inline F pair_term(const Dev& D, const Tables<typename ParamOf<F>::type>& T, const BeadPos& x, int kp,
                              Contrib<F>& c) {
  const int2 ij = __ldg(reinterpret_cast<const int2*>(D.pair) + kp);
  const int i1 = ij.x, i2 = ij.y;
  F v[kVPair];
  load_pair_params(&T.vpair[kVPair * kp], v);
  F vab[3];
  disp<F>(x, i1, i2, vab);
  const F r2 = dot3(vab, vab);
  F r, oner, it6, it8;
  const F R0 = v[0], c6 = v[1], eps2 = v[5];
  const F r4 = r2 * r2, r6 = r4 * r2;
  const F R02 = R0 * R0, r06 = R02 * R02 * R02;
  const F t6 = r6 + r06;
  const F t8 = r6 * r2 + r06 * R0 * R0;
  if constexpr (std::is_same<F, float>::value) {
    // hardware approximations (a few ulp): the pair forces are ~1 % of the
    // valence forces, far below the form's error budget
    oner = rsqrtf(r2);
    r = r2 * oner;
    it6 = __fdividef(1.0f, t6);
    it8 = __fdividef(1.0f, t8);
  } else {
    r = q_sqrt<F>(r2);
    oner = F(1) / r;
    it6 = F(1) / t6;
    it8 = F(1) / t8;
  }
  const F ir2 = oner * oner;
  const F c6t6 = c6 * it6, c6t8 = c6 * it8;
  const F t27 = v[2] * c6t8;
  // periodic: dispersion and repulsion only within vdw_cut (src/ff_nonb.f90:107)
  const bool vdw = !x.pbc || !(r > (std::is_same<F, float>::value ? F(D.fvdw_cut) : F(D.vdw_cut)));
  F e = vdw ? -(c6t6 + t27) * eps2 : F(0);
  F drij = vdw ? eps2 * (c6t6 * F(6) * r4 * it6 + F(8) * t27 * r6 * it8) : F(0);
  if (vdw && r < F(25)) {
    const F alpha = v[4];
    F ex;
    if constexpr (std::is_same<F, float>::value) ex = __expf(-alpha * r);
    else ex = q_exp<F>(-alpha * r);
    const F t = v[3] * ex;
    e = e + t * oner * eps2;
    drij = drij - eps2 * t * (alpha * r + F(1)) * oner * ir2;
  }
  const F cut = std::is_same<F, float>::value ? F(D.fcoul_cut) : F(D.coul_cut);
  if (!(r > cut)) {
    F e0;
    if (D.zahn) {
      const F za = std::is_same<F, float>::value ? F(D.fzahn_a) : F(D.zahn_a);
      const F zp = std::is_same<F, float>::value ? F(D.fzahn_par) : F(D.zahn_par);
      e0 = v[6] * ((q_erfc<F>(za * r) * oner) - zp * (r - cut));
    }
    else e0 = v[6] * oner;
    e = e + e0;
    drij = drij - e0 * ir2;
  }
  c.na = 2;
  c.a[0] = i1;
  c.a[1] = i2;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    c.g[0][d] = vab[d] * drij;
    c.g[1][d] = -vab[d] * drij;
  }
  return e;
}

// FP32 hardware approximations (PTX rsqrt / rcp / ex2 .approx.ftz, relative
// error about 2^-22): inputs here are normal numbers far from the limits.
__device__ inline float rsqrt_approx(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ inline float rcp_approx(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ inline float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// One NCI pair in the mixed form: the formulas of pair_term with the
// per-pair constants folded into the table Dev::fpair (R0^6 and R0^8 of the
// BJ damping, eps2 into the C6 / C8 and repulsion prefactors, alpha log2(e)
// for a base-2 exponential).  The pair forces are ~1 % of the valence
// forces, so hardware approximations stay far below the form's error budget.
__device__ inline float pair_mixed_v(const Dev& D, const BeadPos& x, int i1, int i2, const float (&v)[kVPair],
                                     Contrib<float>& c, float* vir = nullptr) {
  float vab[3];
  disp<float>(x, i1, i2, vab);
  const float r2 = dot3(vab, vab);
  const float oner = rsqrt_approx(r2), r = r2 * oner, ir2 = oner * oner;
  const float r4 = r2 * r2, r6 = r4 * r2;
  const float it6 = rcp_approx(r6 + v[0]), it8 = rcp_approx(r6 * r2 + v[1]);
  const float d6 = v[2] * it6, d8 = v[3] * it8;
  const bool vdw = !x.pbc || !(r > D.fvdw_cut);
  float e = vdw ? -(d6 + d8) : 0.0f;
  float drij = vdw ? 6.0f * d6 * (r4 * it6) + 8.0f * d8 * (r6 * it8) : 0.0f;
  if (vdw && r < 25.0f) {
    const float t = v[4] * ex2_approx(-v[5] * r) * oner;
    e += t;
    drij = fmaf(-t * ir2, fmaf(v[7], r, 1.0f), drij);
  }
  if (!(r > D.fcoul_cut)) {
    float e0;
    if (D.zahn) e0 = v[6] * ((q_erfc<float>(D.fzahn_a * r) * oner) - D.fzahn_par * (r - D.fcoul_cut));
    else e0 = v[6] * oner;
    e += e0;
    drij = fmaf(-e0, ir2, drij);
  }
  c.na = 2;
  c.a[0] = i1;
  c.a[1] = i2;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    c.g[0][d] = vab[d] * drij;
    c.g[1][d] = -vab[d] * drij;
  }
  if (vir) *vir = r2 * drij;  // vab . g_i1 with g_i1 = vab drij (NpT)
  return e;
}

__device__ inline float pair_mixed(const Dev& D, const BeadPos& x, int kp, Contrib<float>& c) {
  const int2 ij = __ldg(reinterpret_cast<const int2*>(D.pair) + kp);
  float v[kVPair];
  load_pair_params(&D.fpair[kVPair * kp], v);
  return pair_mixed_v(D, x, ij.x, ij.y, v, c);
}

// x^5, x^6, x^12 by products (the reference's real-exponent ** operators)
template <class F>
__device__ inline F pow6(F x) {
  const F x2 = x * x;
  return x2 * x2 * x2;
}

// eabhag (src/eabhag.f90:35-220): hydrogen bond A...H-B; nothing if the
// energy is above -1e-8 (the reference returns before its gradient).
template <class F>
__device__ inline F hbond_term(const BeadPos& X, int A, int B, int H, F ca, F cb, Contrib<F>& c) {
  const F longcut = F(8.0), alp7 = F(12.0), alp3 = F(6.0);
  F drah[3], drbh[3], drab[3];
  disp<F>(X, A, H, drah);
  disp<F>(X, B, H, drbh);
  disp<F>(X, A, B, drab);
  c.a[0] = A;
  c.a[1] = B;
  c.a[2] = H;
  const F rab2 = dot3(drab, drab), rab = q_sqrt<F>(rab2);
  const F rah2 = dot3(drah, drah), rah = q_sqrt<F>(rah2);
  const F rbh2 = dot3(drbh, drbh), rbh = q_sqrt<F>(rbh2);
  const F q6 = pow6<F>(rab / longcut);
  const F ratio = q6 * q6;
  F rdampl = F(1) / (F(1) + ratio);
  rdampl = rdampl / rab2 / rab;
  const bool far_a = rah2 > rbh2;
  F cosabh, aprod;
  if (far_a) {
    aprod = F(1) / rbh / rab;
    cosabh = -dot3(drbh, drab) * aprod;
  } else {
    aprod = F(1) / rah / rab;
    cosabh = dot3(drah, drab) * aprod;
  }
  F aterm = F(0.5) * (cosabh + F(1));
  const F a2 = aterm * aterm;
  F apref = a2 * a2 * aterm;  // aterm**(alp3-1)
  aterm = aterm * apref;
  apref = alp3 * F(0.5) * apref;
  const F rah4 = rah2 * rah2, rbh4 = rbh2 * rbh2;
  const F denom = F(1) / (rah4 + rbh4);
  const F da = (ca * rah4 + cb * rbh4) * denom;
  const F eabh = -da * rdampl * aterm;
#pragma unroll
  for (int m = 0; m < 3; ++m)
#pragma unroll
    for (int d = 0; d < 3; ++d) c.g[m][d] = F(0);
  if (eabh > F(-1.0e-8)) return F(0);
  F ga[3], gb[3], gh[3];
  F gi = F(4) * (ca - cb) * rah2 * rbh4 * denom * denom;
  gi = -gi * rdampl * aterm;
  F gj = F(4) * (cb - ca) * rbh2 * rah4 * denom * denom;
  gj = -gj * rdampl * aterm;
  F gl = rdampl * rdampl * rab * (F(3) + (F(3) + alp7) * ratio);
  gl = gl * da * aterm;
  const F gn = -da * rdampl * apref;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    ga[d] = gi * drah[d];
    gb[d] = gj * drbh[d];
    gh[d] = -ga[d] - gb[d];
    const F dl = gl * drab[d];
    ga[d] += dl;
    gb[d] -= dl;
    if (far_a) {
      const F dg = gn * (-aprod * drbh[d] - cosabh * drab[d] / rab2);
      const F dg2 = gn * (aprod * drab[d] + cosabh * drbh[d] / rbh2);
      ga[d] += dg;
      gh[d] += dg2;
      gb[d] = gb[d] - dg - dg2;
    } else {
      const F dg = gn * (-aprod * drah[d] + cosabh * drab[d] / rab2);
      const F dg2 = gn * (-aprod * drab[d] + cosabh * drah[d] / rah2);
      gb[d] += dg;
      gh[d] += dg2;
      ga[d] = ga[d] - dg - dg2;
    }
    c.g[0][d] = ga[d];
    c.g[1][d] = gb[d];
    c.g[2][d] = gh[d];
  }
  return eabh;
}

// eabx (src/eabx.f90:34-111) on the three atoms' coordinates xa, xb, xh.
__device__ inline double eabx(const double* xa, const double* xb, const double* xh, double ca) {
  double rb[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) rb[d] = xa[d] - xb[d];
  const double rab2 = rb[0] * rb[0] + rb[1] * rb[1] + rb[2] * rb[2];
  const double dampl = 1.0 / (1.0 + pow6<double>(rab2 / 120.0));
#pragma unroll
  for (int d = 0; d < 3; ++d) rb[d] = xa[d] - xh[d];
  const double d2ik = rb[0] * rb[0] + rb[1] * rb[1] + rb[2] * rb[2];
#pragma unroll
  for (int d = 0; d < 3; ++d) rb[d] = xh[d] - xb[d];
  const double d2jk = rb[0] * rb[0] + rb[1] * rb[1] + rb[2] * rb[2];
  double term;
  if (d2ik > d2jk) term = 0.5 * (rab2 + d2jk - d2ik) / sqrt(rab2 * d2jk);
  else term = 0.5 * (rab2 + d2ik - d2jk) / sqrt(rab2 * d2ik);
  const double aterm = pow6<double>(0.5 * (term + 1.0));
  return -ca * dampl * aterm / d2jk;
}

// eabxag (src/eabxag.f90:35-156): halogen bond A...X-B, energy and Caracal's
// central-difference gradient (step 1e-6), FP64 in both forms.  As in the
// reference, each atom's three components all receive the z quotient.
template <class F>
__device__ inline F xbond_term(const BeadPos& X, int A, int B, int H, double ca, Contrib<F>& c) {
  double p[3][3];
  const int at[3] = {A, B, H};
#pragma unroll
  for (int m = 0; m < 3; ++m)
#pragma unroll
    for (int d = 0; d < 3; ++d) p[m][d] = X.x[3 * at[m] + d];
  const double e = eabx(p[0], p[1], p[2], ca);
  const double step = 1.0e-6, dum = 1.0 / (2.0 * step);
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    double last = 0.0;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      p[m][j] = p[m][j] + step;
      const double er = eabx(p[0], p[1], p[2], ca);
      p[m][j] = p[m][j] - step * 2.0;
      const double el = eabx(p[0], p[1], p[2], ca);
      p[m][j] = p[m][j] + step;
      last = (er - el) * dum;
    }
    c.a[m] = at[m];
#pragma unroll
    for (int d = 0; d < 3; ++d) c.g[m][d] = (F)last;
  }
  return (F)e;
}

// One entry of ff_hb (src/ff_hb.f90:55-79): skipped beyond 15 bohr A-B.
// Out of line (a handful of terms per molecule) to keep the register count
// of the frequent terms.
template <class F>
__device__ __noinline__ F hb_term(const Dev& D, const Tables<F>&, const BeadPos& X, int k, Contrib<F>& c) {
  const int4 t = __ldg(reinterpret_cast<const int4*>(D.hb) + k);
  double rb[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    rb[d] = X.x[3 * t.x + d] - X.x[3 * t.y + d];
    if (X.pbc) rb[d] = image1(rb[d], X.pbc->len[d], X.pbc->half[d]);  // src/ff_hb.f90:64-66
  }
  const double r2 = rb[0] * rb[0] + rb[1] * rb[1] + rb[2] * rb[2];
  c.a[0] = t.x;
  c.a[1] = t.y;
  c.a[2] = t.z;
  if (sqrt(r2) > 15.0) {
#pragma unroll
    for (int m = 0; m < 3; ++m)
#pragma unroll
      for (int d = 0; d < 3; ++d) c.g[m][d] = F(0);
    return F(0);
  }
  if (t.w == 1) return hbond_term<F>(X, t.x, t.y, t.z, (F)D.vhb[2 * k], (F)D.vhb[2 * k + 1], c);
  return xbond_term<F>(X, t.x, t.y, t.z, D.vhb[2 * k], c);
}

// Energy of one term of kind `kind` (0 bond, 1 angle, 2 torsion, 3 pair, 4 H/halogen bond).
template <bool MIXED>
__device__ inline typename std::conditional<MIXED, float, double>::type term(
    const Dev& D, int kind, const BeadPos& x, int m, Contrib<typename std::conditional<MIXED, float, double>::type>& c) {
  if constexpr (MIXED) {
    switch (kind) {
      case 0: return bond_mixed(D, x, m, c);
      case 1: return angle_term<float>(D, D.f, x, m, c);
      case 2: return torsion_term<float>(D, D.f, x, m, c);
      case 3: return pair_mixed(D, x, m, c);
      default: return hb_term<float>(D, D.f, x, m, c);
    }
  } else {
    switch (kind) {
      case 0: return bond_plain<double>(D, D.d, x, m, c);
      case 1: return angle_term<double>(D, D.d, x, m, c);
      case 2: return torsion_term<double>(D, D.d, x, m, c);
      case 3: return pair_term<double>(D, D.d, x, m, c);
      default: return hb_term<double>(D, D.d, x, m, c);
    }
  }
}

// All batches of one term kind (NA atoms per term): each lane evaluates its
// slot's term, then the warp scatters colour by colour.
// The virial trace of one term as the reference accumulates `vir_ten` for
// NpT: bonds (src/ff_eg.f90:133-150) rbond.g_i, rbond = r_i - r_j; angles
// (:270-281) vab.g_i + vcb.g_k about the centre j; torsions (:317-320,
// 420-440) vab.g_i + vcb.(g_k + g_l) + vdc.g_l with vab = r_i - r_j,
// vcb = r_j - r_k, vdc = r_k - r_l, and inversions (:503-505, 583-603) the
// same formula with vab = r_j - r_i, vcb = r_j - r_k, vdc = r_j - r_l (for
// neither is it the sum of (r - r_j).g over the term's atoms); NCI pairs
// (src/ff_nonb.f90:180-190, 318-328, 405-415, 495-505) vab.g_i1, vab = r_i1 - r_i2; hydrogen bonds
// (src/eabhag.f90:54, 203-216) drah.g_A + drbh.g_B about H; halogen bonds
// (src/eabxag.f90:86-87, 140-153) (r_A - r_X).g_A + (r_B - r_X).g_X, the
// X atom's gradient with the B vector.  Vectors minimum-imaged as the
// terms' own.  Mixed-form bonds carry g_i as (hi, lo) in g[0] and g[2].
template <class F, int KIND>
__device__ inline F term_virial(const Dev& D, const BeadPos& X, int m, const Contrib<F>& c) {
  F u[3], v[3], w[3];
  if constexpr (KIND == 0) {
    disp<F>(X, c.a[0], c.a[1], u);
    F g[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) g[d] = std::is_same<F, float>::value ? c.g[0][d] + c.g[2][d] : c.g[0][d];
    return dot3(u, g);
  } else if constexpr (KIND == 1) {
    disp<F>(X, c.a[0], c.a[1], u);
    disp<F>(X, c.a[2], c.a[1], v);
    return dot3(u, c.g[0]) + dot3(v, c.g[2]);
  } else if constexpr (KIND == 2) {
    const int i = c.a[0], j = c.a[1], k = c.a[2], l = c.a[3];
    if (D.tors[6 * m + 5] != 2) {
      disp<F>(X, i, j, u);
      disp<F>(X, j, k, v);
      disp<F>(X, k, l, w);
    } else {
      disp<F>(X, j, i, u);
      disp<F>(X, j, k, v);
      disp<F>(X, j, l, w);
    }
    F gkl[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) gkl[d] = c.g[2][d] + c.g[3][d];
    return dot3(u, c.g[0]) + dot3(v, gkl) + dot3(w, c.g[3]);
  } else if constexpr (KIND == 3) {
    disp<F>(X, c.a[0], c.a[1], u);
    return dot3(u, c.g[0]);
  } else {
    disp<F>(X, c.a[0], c.a[2], u);
    disp<F>(X, c.a[1], c.a[2], v);
    const bool halogen = D.hb[4 * m + 3] != 1;
    return dot3(u, c.g[0]) + dot3(v, halogen ? c.g[2] : c.g[1]);
  }
}

// Box modes of the force kernel, compile-time so the free molecule's kernel
// carries no imaging code: kFree (no box), kBox (the force field's periodic
// box), kNpt (each trajectory's box from Dev::tbox, and the virial).
constexpr int kFree = 0, kBox = 1, kNpt = 2;

template <bool MIXED, int KIND, int NA, int MODE>
__device__ inline void kind_batches(const Dev& D, const BeadPos& X,
                                    Grad<typename std::conditional<MIXED, float, double>::type>& G,
                                    typename std::conditional<MIXED, float, double>::type& es,
                                    typename std::conditional<MIXED, float, double>::type& ec,
                                    typename std::conditional<MIXED, float, double>::type& wv, int lane) {
  using F = typename std::conditional<MIXED, float, double>::type;
  const Schedule& S = D.sched[MIXED ? 1 : 0];
  const int b0 = S.boff[KIND], nb = S.nb[KIND];
  const bool distinct = D.distinct != 0;
  for (int b = b0; b < b0 + nb; ++b) {
    const int m = S.slot[32 * b + lane];
    const int col = S.color[32 * b + lane];
    const int ncol = S.ncol[b];
    Contrib<F> c;
    if (m >= 0) {
      F v;
      if constexpr (MODE == kNpt && KIND == 2) {  // the torsion's own vectors give its virial
        F w;
        if constexpr (MIXED) v = torsion_term<float>(D, D.f, X, m, c, &w);
        else v = torsion_term<double>(D, D.d, X, m, c, &w);
        wv += w;
      } else {
        v = term<MIXED>(D, KIND, X, m, c);
        if constexpr (MODE == kNpt) wv += term_virial<F, KIND>(D, X, m, c);
      }
      if constexpr (MIXED) {  // compensated FP32 lane sum
        const F t = es + v;
        ec += (fabs(es) >= fabs(v)) ? ((es - t) + v) : ((v - t) + es);
        es = t;
      } else {
        es += v;
      }
    }
    for (int k = 0; k < ncol; ++k) {
      if (m >= 0 && col == k) {
        if constexpr (MIXED && KIND == 3) scatter_pair<NA>(c, G);
        else if constexpr (MIXED && KIND == 0) scatter_bond(c, G);
        else scatter<NA>(c, G, distinct);
      }
      __syncwarp();
    }
  }
}

// Mixed-form NCI pairs: every batch is one matching (one colour), so each
// lane scatters right after its term; the next batch's slot, atom pair and
// parameters are loaded before the current batch's arithmetic, so the L1
// latency of the term tables overlaps the work.
template <int MODE>
__device__ inline void pair_batches_mixed(const Dev& D, const BeadPos& X, Grad<float>& G, float& es, float& ec,
                                          float& wv, int lane) {
  const Schedule& S = D.sched[1];
  const int b0 = S.boff[3], nb = S.nb[3];
  if (nb <= 0) return;
  int m = S.slot[32 * b0 + lane];
  int2 ij = m >= 0 ? __ldg(reinterpret_cast<const int2*>(D.pair) + m) : make_int2(0, 0);
  float4 pa = m >= 0 ? __ldg(reinterpret_cast<const float4*>(&D.fpair[kVPair * m])) : make_float4(0, 0, 0, 0);
  float4 pb = m >= 0 ? __ldg(reinterpret_cast<const float4*>(&D.fpair[kVPair * m]) + 1) : make_float4(0, 0, 0, 0);
  for (int b = b0; b < b0 + nb; ++b) {
    const int mc = m;
    const int2 ijc = ij;
    const float v[kVPair] = {pa.x, pa.y, pa.z, pa.w, pb.x, pb.y, pb.z, pb.w};
    if (b + 1 < b0 + nb) {
      m = S.slot[32 * (b + 1) + lane];
      if (m >= 0) {
        ij = __ldg(reinterpret_cast<const int2*>(D.pair) + m);
        pa = __ldg(reinterpret_cast<const float4*>(&D.fpair[kVPair * m]));
        pb = __ldg(reinterpret_cast<const float4*>(&D.fpair[kVPair * m]) + 1);
      }
    }
    if (mc >= 0) {
      Contrib<float> c;
      float w = 0.0f;
      const float e = pair_mixed_v(D, X, ijc.x, ijc.y, v, c, MODE == kNpt ? &w : nullptr);
      const float t = es + e;
      ec += (fabsf(es) >= fabsf(e)) ? ((es - t) + e) : ((e - t) + es);
      es = t;
      if constexpr (MODE == kNpt) wv += w;
      scatter_pair<2>(c, G);
    }
    __syncwarp();
  }
}

// Shared memory per warp (bytes): coordinates (3n doubles), the FP32 split
// (hi, lo) (3n float pairs) and the gradient (3n doubles, or (sum,
// compensation) float pairs and the 3n floats of the pair sum).
__host__ __device__ inline size_t warp_smem_bytes(int n) { return (size_t)3 * n * (8 + 4 + 4 + 8 + 4); }

// Energy (with E_zero) and gradient (times gscale) of one bead by one warp.
// ws: the warp's shared memory with the bead's FP64 coordinates in its first
// 3n doubles; gout: the gradient destination.  Returns the energy on every lane.
template <bool MIXED, int MODE = kFree>
__device__ inline double warp_egrad(const Dev& D, double* ws, double* gout, double gscale, int lane, int bead = 0) {
  // MODE (kFree, kBox, kNpt): with kNpt the bead's trajectory box from D.tbox
  // and the virial trace into D.vir
  using F = typename std::conditional<MIXED, float, double>::type;
  const int n3 = 3 * D.n;
  double* xs = ws;
  float2* hl = (float2*)(ws + n3);
  void* gs = hl + n3;
  // the box as a local copy: taking the address of the kernel parameter D
  // would move all of it from the constant bank to local memory
  PBox tb;
  const PBox* pb = nullptr;
  if constexpr (MODE == kNpt) {  // this trajectory's box
    tb = make_box(D.tbox + 3 * (size_t)(bead / D.tbox_beads));
    pb = &tb;
  } else if constexpr (MODE == kBox) {
    tb = D.box;
    pb = &tb;
  }
  BeadPos X{xs, hl, nullptr, pb};
  Grad<F> G;
  if constexpr (MIXED) {
    for (int a = lane; a < n3; a += 32) {
      const double v = xs[a];
      const float h = __double2float_rn(v);
      hl[a] = make_float2(h, __double2float_rn(v - (double)h));
    }
    G.sk = (float2*)gs;
    G.pr = (float*)(G.sk + n3);
    for (int a = lane; a < n3; a += 32) {
      G.sk[a] = make_float2(0.f, 0.f);
      G.pr[a] = 0.f;
    }
  } else {
    G.g = (double*)gs;
    for (int a = lane; a < n3; a += 32) G.g[a] = 0.0;
  }
  __syncwarp();
  F es = F(0), ec = F(0);  // compensated lane sum of term energies
  F wv = F(0);             // lane sum of the terms' virial traces (NpT)
  kind_batches<MIXED, 0, 2, MODE>(D, X, G, es, ec, wv, lane);
  kind_batches<MIXED, 1, 3, MODE>(D, X, G, es, ec, wv, lane);
  kind_batches<MIXED, 2, 4, MODE>(D, X, G, es, ec, wv, lane);
  if constexpr (MIXED) pair_batches_mixed<MODE>(D, X, G, es, ec, wv, lane);
  else kind_batches<MIXED, 3, 2, MODE>(D, X, G, es, ec, wv, lane);
  kind_batches<MIXED, 4, 3, MODE>(D, X, G, es, ec, wv, lane);
  for (int a = lane; a < n3; a += 32) gout[a] = gscale * G.get(a);
  double e = (double)es + (double)ec;
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
  if constexpr (MODE == kNpt) {
    double w = (double)wv;
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) w += __shfl_xor_sync(0xffffffffu, w, o);
    if (lane == 0) D.vir[bead] = w;
  }
  return e + D.e_zero;
}

// ---------------------------------------------------------------------------
// Derivatives for the adjoint (plain form only; bonds, angles, torsions and
// NCI pairs).
// ---------------------------------------------------------------------------

// Gradient value and tangent (H w) of one bead in shared memory.
struct GradDual {
  double* g;
  double* h;
  __device__ inline void add(int i, const Dual& v) {
    g[i] += v.v;
    h[i] += v.d;
  }
};

__device__ inline Dual term_dual(const Dev& D, int kind, const BeadPos& x, int m, Contrib<Dual>& c) {
  switch (kind) {
    case 0: return bond_plain<Dual>(D, D.d, x, m, c);
    case 1: return angle_term<Dual>(D, D.d, x, m, c);
    case 2: return torsion_term<Dual>(D, D.d, x, m, c);
    default: return pair_term<Dual>(D, D.d, x, m, c);
  }
}

// The plain form's schedule (sched[0]) with dual coordinates.
template <int KIND, int NA>
__device__ inline void kind_batches_dual(const Dev& D, const BeadPos& X, GradDual& G, Dual& es, int lane) {
  const Schedule& S = D.sched[0];
  const int b0 = S.boff[KIND], nb = S.nb[KIND];
  for (int b = b0; b < b0 + nb; ++b) {
    const int m = S.slot[32 * b + lane];
    const int col = S.color[32 * b + lane];
    const int ncol = S.ncol[b];
    Contrib<Dual> c;
    if (m >= 0) es += term_dual(D, KIND, X, m, c);
    for (int k = 0; k < ncol; ++k) {
      if (m >= 0 && col == k) {
#pragma unroll
        for (int a = 0; a < NA; ++a)
#pragma unroll
          for (int d = 0; d < 3; ++d) G.add(3 * c.a[a] + d, c.g[a][d]);
      }
      __syncwarp();
    }
  }
}

// Shared memory per warp of warp_hvp: x, w, gradient, H w (3n doubles each).
__host__ __device__ inline size_t warp_hvp_smem_bytes(int n) { return (size_t)12 * n * sizeof(double); }

// Energy (with E_zero), gradient and Hessian-vector product H w of one bead
// by one warp.  ws: the warp's shared memory holding x (3n doubles) then w
// (3n doubles).  dew receives the directional derivative w . grad E.
__device__ inline double warp_hvp(const Dev& D, double* ws, double* gout, double* hout, double& dew, int lane) {
  const int n3 = 3 * D.n;
  double* xs = ws;
  double* w = ws + n3;
  GradDual G{w + n3, w + 2 * n3};
  for (int a = lane; a < n3; a += 32) {
    G.g[a] = 0.0;
    G.h[a] = 0.0;
  }
  __syncwarp();
  PBox tb;
  if (D.periodic) tb = D.box;
  BeadPos X{xs, nullptr, w, D.periodic ? &tb : nullptr};
  Dual es(0.0);
  kind_batches_dual<0, 2>(D, X, G, es, lane);
  kind_batches_dual<1, 3>(D, X, G, es, lane);
  kind_batches_dual<2, 4>(D, X, G, es, lane);
  kind_batches_dual<3, 2>(D, X, G, es, lane);
  for (int a = lane; a < n3; a += 32) {
    if (gout) gout[a] = G.g[a];
    hout[a] = G.h[a];
  }
  double e = es.v, de = es.d;
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
    e += __shfl_xor_sync(0xffffffffu, e, o);
    de += __shfl_xor_sync(0xffffffffu, de, o);
  }
  dew = de;
  return e + D.e_zero;
}

// Linear parameters of the force field (the loss gradients of the adjoint are
// taken with respect to these): bond force constant k (vbond[1]), angle force
// constant k (vangl[1]), torsion barrier V (vtors[1]) and the NCI pair's
// Coulomb product qq (vpair[6]: eps1 q_i q_j, or q_i q_j in the Zahn form).
// Every term is linear in its parameter, so d/dtheta_t (v . grad E) is v .
// grad E_t evaluated with theta_t = 1; the tables U hold the parameters with
// those entries set to 1 (and, for pairs, eps2 = 0: Coulomb only).
// Per term, out receives alpha * (v . grad E_t|unit) + beta * E_t|unit.
__device__ inline void warp_param_vjp(const Dev& D, const Tables<double>& U, const double* xs, const double* vs,
                                      double alpha, double beta, double* out, int lane) {
  PBox tb;
  if (D.periodic) tb = D.box;
  const BeadPos X{xs, nullptr, nullptr, D.periodic ? &tb : nullptr};
  int off = 0;
#pragma unroll 1
  for (int kind = 0; kind < 4; ++kind) {
    const int nt = D.nterm[kind];
    for (int m = lane; m < nt; m += 32) {
      Contrib<double> c;
      double e;
      switch (kind) {
        case 0: e = bond_plain<double>(D, U, X, m, c); break;
        case 1: e = angle_term<double>(D, U, X, m, c); break;
        case 2: e = torsion_term<double>(D, U, X, m, c); break;
        default: e = pair_term<double>(D, U, X, m, c); break;
      }
      double s = 0.0;
      for (int a = 0; a < c.na; ++a)
#pragma unroll
        for (int d = 0; d < 3; ++d) s += vs[3 * c.a[a] + d] * c.g[a][d];
      out[off + m] = alpha * s + beta * e;
    }
    off += nt;
  }
}

}  // namespace qmdff
}  // namespace cr
