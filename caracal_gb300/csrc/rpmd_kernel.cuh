// Persistent RPMD step kernel: many trajectories, all steps of a run in one
// launch, every bead's q, p, f held in registers across steps.
//
// Drop-in for the per-step work of Caracal's `verlet` (src/verlet.f90:65-1308)
// on the gas-phase path: 1/2 kick, free ring-polymer propagation in Caracal's
// cosine "normal modes", forces, 1/2 kick, Andersen or PILE thermostat,
// NaN check, `transrot`.
//
// Thread layout: a trajectory owns a group of G = next_pow2(P) consecutive
// threads, bead j on lane j of the group (lanes j >= P idle).  Groups of
// G <= 32 live inside one warp; G = 64 or 128 span 2 or 4 warps.
//
// Bead coupling.  Caracal applies C = sqrt(1/P) cos(2 pi j k/P) (src/rfft.f90,
// src/irfft.f90), a per-mode 2x2 rotation (src/verlet.f90:405-454), and C
// again.  The composite is linear: p' = K1 p + m K2 q, q' = K3 p / m + K1 q
// with K = C diag(poly) C.  Since poly(k) = poly(P-k), K[j][l] = K[-j][l] =
// K[j][-l]: beads j and P-j get the same output and only the P/2+1
// symmetrised inputs s_l = x_l + x_{-l} matter.  For even P (M = P/2),
// C[M-r][k] = (-1)^k C[r][k], so with K = Ke + Ko split by mode parity,
// K[r] = Ke[r] + Ko[r] and K[M-r] = Ke[r] - Ko[r]; Ke is even and Ko odd
// under l -> M-l.  One pass over u_l = s_l + s_{M-l}, v_l = s_l - s_{M-l}
// gives rows r and M-r together.  The group's lanes share the (coordinate,
// row pair) tasks, so each unique output is computed once: per coordinate
// 4 (M/2+1)(M+1) FP64 FMAs for the whole ring polymer, against 4 P (M+1)
// when every bead computes its own row.
//
// PILE (new; Caracal has Andersen and Nose-Hoover only) uses the orthonormal
// real normal modes; O^T diag(c) O is circulant, so each half step is two
// length-P circular convolutions: p' = a * p + sqrt(mP/beta) b * eta.
#pragma once
#include <cuda_runtime.h>

#include "cr_common.cuh"

namespace cr {

constexpr int kMaxBeads = 128;
constexpr int kMaxAtoms = 7;

// BIMOLEC reaction coordinate of Caracal's recrossing (calc_xi mode 2,
// src/calc_xi.f90:63-279): xi = xi_ideal*s1 + (1-xi_ideal)*s0 with
// s1 = (r_break - break_ref) - (r_form - form_ref), s0 = R_inf - |COM2 - COM1|.
struct XiDev {
  int nreac1, reac1[8], nreac2, reac2[8];  // 0-based atoms
  int form0, form1, brk0, brk1;
  double form_ref, break_ref, r_inf, xi_ideal;
  double mreac1, mreac2;
  double w1[8], w2[8];  // mass / mreac of each reactant atom (the step kernel's xi)
};

template <int N>
__host__ __device__ inline double xi_bimolec(const XiDev& x, const double* c, const double* mass,
                                             double* dxi) {
  double Rf[3], Rb[3];
  for (int d = 0; d < 3; ++d) {
    Rf[d] = c[3 * x.form0 + d] - c[3 * x.form1 + d];
    Rb[d] = c[3 * x.brk0 + d] - c[3 * x.brk1 + d];
  }
  const double rf = sqrt(Rf[0] * Rf[0] + Rf[1] * Rf[1] + Rf[2] * Rf[2]);
  const double rb = sqrt(Rb[0] * Rb[0] + Rb[1] * Rb[1] + Rb[2] * Rb[2]);
  const double s1 = (rb - x.break_ref) - (rf - x.form_ref);
  double c1[3] = {0, 0, 0}, c2[3] = {0, 0, 0};
  for (int k = 0; k < x.nreac1; ++k)
    for (int d = 0; d < 3; ++d) c1[d] += mass[x.reac1[k]] * c[3 * x.reac1[k] + d] / x.mreac1;
  for (int k = 0; k < x.nreac2; ++k)
    for (int d = 0; d < 3; ++d) c2[d] += mass[x.reac2[k]] * c[3 * x.reac2[k] + d] / x.mreac2;
  const double Red[3] = {c2[0] - c1[0], c2[1] - c1[1], c2[2] - c1[2]};
  const double reds = sqrt(Red[0] * Red[0] + Red[1] * Red[1] + Red[2] * Red[2]);
  const double s0 = x.r_inf - reds;
  if (dxi) {
    const double a = x.xi_ideal, b = 1.0 - x.xi_ideal;
    for (int i = 0; i < 3 * N; ++i) dxi[i] = 0.0;
    for (int d = 0; d < 3; ++d) {
      dxi[3 * x.form0 + d] -= a * Rf[d] / rf;
      dxi[3 * x.form1 + d] += a * Rf[d] / rf;
      dxi[3 * x.brk0 + d] += a * Rb[d] / rb;
      dxi[3 * x.brk1 + d] -= a * Rb[d] / rb;
    }
    for (int k = 0; k < x.nreac1; ++k)
      for (int d = 0; d < 3; ++d) dxi[3 * x.reac1[k] + d] += b * Red[d] / reds * mass[x.reac1[k]] / x.mreac1;
    for (int k = 0; k < x.nreac2; ++k)
      for (int d = 0; d < 3; ++d) dxi[3 * x.reac2[k] + d] -= b * Red[d] / reds * mass[x.reac2[k]] / x.mreac2;
  }
  return x.xi_ideal * s1 + (1.0 - x.xi_ideal) * s0;
}

// xi alone (no derivative) for the side bit of a recrossing child: the same
// formula as xi_bimolec with the reactant weights m / m_reac precomputed, so
// the COMs cost multiplications only (FP64 divisions take ~10 FP64-pipe
// instructions each on this GPU).
template <int N>
__device__ inline double xi_bimolec_value(const XiDev& x, const double* c) {
  double Rf[3], Rb[3], c1[3] = {0, 0, 0}, c2[3] = {0, 0, 0};
  for (int d = 0; d < 3; ++d) {
    Rf[d] = c[3 * x.form0 + d] - c[3 * x.form1 + d];
    Rb[d] = c[3 * x.brk0 + d] - c[3 * x.brk1 + d];
  }
  for (int k = 0; k < x.nreac1; ++k)
    for (int d = 0; d < 3; ++d) c1[d] = fma(x.w1[k], c[3 * x.reac1[k] + d], c1[d]);
  for (int k = 0; k < x.nreac2; ++k)
    for (int d = 0; d < 3; ++d) c2[d] = fma(x.w2[k], c[3 * x.reac2[k] + d], c2[d]);
  const double Red[3] = {c2[0] - c1[0], c2[1] - c1[1], c2[2] - c1[2]};
  const double rf = sqrt(Rf[0] * Rf[0] + Rf[1] * Rf[1] + Rf[2] * Rf[2]);
  const double rb = sqrt(Rb[0] * Rb[0] + Rb[1] * Rb[1] + Rb[2] * Rb[2]);
  const double reds = sqrt(Red[0] * Red[0] + Red[1] * Red[1] + Red[2] * Red[2]);
  const double s1 = (rb - x.break_ref) - (rf - x.form_ref);
  return x.xi_ideal * s1 + (1.0 - x.xi_ideal) * (x.r_inf - reds);
}

// Shape of the parity-split propagator blocks for P beads.
struct PropDims {
  int M;      // P / 2
  int split;  // 1: even P, parity-split blocks; 0: odd P, unique rows only
  int nr;     // task rows
  int nu;     // length of u (even part)
  int nv;     // length of v (odd part)
  int su, sv; // padded (odd) shared-memory strides of u and v
};

__host__ __device__ inline PropDims prop_dims(int P) {
  PropDims d;
  d.M = P / 2;
  d.split = (P % 2 == 0) ? 1 : 0;
  if (d.split) {
    d.nr = d.M / 2 + 1;
    d.nu = d.M / 2 + 1;
    d.nv = d.M - d.M / 2;
  } else {
    d.nr = P / 2 + 1;
    d.nu = d.nr;
    d.nv = 0;
  }
  d.su = d.nu | 1;
  d.sv = d.nv > 0 ? (d.nv | 1) : 0;
  return d;
}

__device__ inline double sym_at(const double* x, int l, int P) {
  return (l == 0 || 2 * l == P) ? x[l] : x[l] + x[P - l];
}

// Nose-Hoover chain constants of one engine (src/nhc.f90:35-171 with the
// masses of src/mdinit.f90:128-147), precomputed on the host.
struct NhcParams {
  double ekt;     // nhc's kT: the REAL(4) quotient 1.380649E-23/4.3597447E-18 times kelvin
  double qnh[4];  // chain masses: 3N Q, Q, Q, Q with Q = k_B T nose_q^2
  double dtc;     // dt / nc
  double w[3];    // Suzuki-Yoshida weights
  int nfree;      // 3N
};

// One nhc call on a trajectory whose kinetic sum (centroid-normalised, as
// Caracal: sum p.p/(2m)/P/P) is eksum: advances the chain velocities vnh and
// returns the factor every momentum is scaled by.  Same operation order as
// the reference loop (nc = 5 passes of ns = 3 weights).
__host__ __device__ inline double nhc_scale(const NhcParams& c, double eksum, double (&vnh)[4]) {
  double gnh[4];
  double scale = 1.0;
  for (int ic = 0; ic < 5; ++ic)
    for (int j = 0; j < 3; ++j) {
      const double dts = c.w[j] * c.dtc;
      const double dt2 = 0.5 * dts, dt4 = 0.25 * dts, dt8 = 0.125 * dts;
      double ex;
      gnh[3] = (c.qnh[2] * vnh[2] * vnh[2] - c.ekt) / c.qnh[3];
      vnh[3] = vnh[3] + gnh[3] * dt4;
      gnh[2] = (c.qnh[1] * vnh[1] * vnh[1] - c.ekt) / c.qnh[2];
      ex = exp(-vnh[3] * dt8);
      vnh[2] = ex * (vnh[2] * ex + gnh[2] * dt4);
      gnh[1] = (c.qnh[0] * vnh[0] * vnh[0] - c.ekt) / c.qnh[1];
      ex = exp(-vnh[2] * dt8);
      vnh[1] = ex * (vnh[1] * ex + gnh[1] * dt4);
      gnh[0] = (2.0 * eksum - (double)c.nfree * c.ekt) / c.qnh[0];
      ex = exp(-vnh[1] * dt8);
      vnh[0] = ex * (vnh[0] * ex + gnh[0] * dt4);
      ex = exp(-vnh[0] * dt2);
      scale = scale * ex;
      eksum = eksum * ex * ex;
      gnh[0] = (2.0 * eksum - (double)c.nfree * c.ekt) / c.qnh[0];
      ex = exp(-vnh[1] * dt8);
      vnh[0] = ex * (vnh[0] * ex + gnh[0] * dt4);
      gnh[1] = (c.qnh[0] * vnh[0] * vnh[0] - c.ekt) / c.qnh[1];
      ex = exp(-vnh[2] * dt8);
      vnh[1] = ex * (vnh[1] * ex + gnh[1] * dt4);
      gnh[2] = (c.qnh[1] * vnh[1] * vnh[1] - c.ekt) / c.qnh[2];
      ex = exp(-vnh[3] * dt8);
      vnh[2] = ex * (vnh[2] * ex + gnh[2] * dt4);
      gnh[3] = (c.qnh[2] * vnh[2] * vnh[2] - c.ekt) / c.qnh[3];
      vnh[3] = vnh[3] + gnh[3] * dt4;
    }
  return scale;
}

struct StepParams {
  int T;           // trajectories in the launch
  int P;           // beads
  int G;           // threads per trajectory (power of two >= P)
  int H;           // P/2 + 1
  int thermostat;  // CR_THERMO_*
  int andersen_step;
  int transrot;
  uint32_t seed;
  uint32_t traj0;  // global index of trajectory 0 (noise key)
  double dt;
  double half_dt;
  double beta;
  double totmass;  // Caracal's transrot total mass (P^2 sum m)
  double mass[kMaxAtoms];
  double inv_mass[kMaxAtoms];
  double sigma[kMaxAtoms];    // sqrt(m P / beta): Andersen / PILE noise scale
  PropDims pd;
  const double* ke;    // [3][nr][nu]: K1, K2, K3 (unit mass), even-mode part (odd P: unique rows)
  const double* ko;    // [3][nr][nv]: odd-mode part
  const double* pile;  // [2][P]: circulant a (c1) and b (c2)
  NhcParams nhc;
  double* vnh;         // [T][4] Nose-Hoover chain velocities
  double* q;           // [T][P][N][3]
  double* p;
  double* f;
  double* epot;        // [T]
  int* status;         // [T]
  // recrossing children: after each step, side[t*side_stride + istep-side_step0-1]
  // records xi(centroid) > 0 (src/recross.f90:596-602)
  int xi_on;
  int side_step0;
  int side_stride;
  unsigned char* side;
  XiDev xi;
  // step counter on the device (a launch replayed from a CUDA graph reads its
  // first step index here); NULL: the launch argument
  const int* istep_dev;
  int pow2_P;     // P is a power of two: centroids multiply by inv_P (exact)
  double inv_P;
  // nm_mode 1 (orthonormal normal modes): K1, K2, K3 are circulant, row j
  // holds circ[w][(j - l) mod P] (unit mass); loaded where Ke sits in shared memory
  int nm_mode;
  const double* circ;  // [3][P]
};

// Sum over the G lanes of a group (deterministic tree).  red: per-group
// shared scratch of (G/32) * NV doubles, used only when G > 32.
template <int NV>
__device__ inline void group_sum(double (&v)[NV], int G, double* red, int lane_in_group) {
  const int w = G < 32 ? G : 32;
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
    if (o < w) {
#pragma unroll
      for (int i = 0; i < NV; ++i) v[i] += __shfl_xor_sync(0xffffffffu, v[i], o);
    }
  }
  if (G > 32) {
    const int nw = G / 32, wid = lane_in_group / 32;
    __syncthreads();
    if ((lane_in_group & 31) == 0) {
#pragma unroll
      for (int i = 0; i < NV; ++i) red[wid * NV + i] = v[i];
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      double s = red[i];
      for (int k = 1; k < nw; ++k) s += red[k * NV + i];
      v[i] = s;
    }
  }
}

// Allreduce over a group of G <= 32 lanes by reduce-scatter and all-gather:
// at each butterfly level (offset O = G/2 .. 1) a lane keeps half of the
// values it holds (the lower half if its bit O is clear) and adds the
// partner's copy of that half, so the FP64 adds per lane total about NV
// instead of NV log2(G); each sum is then read from the lane holding it.
// The summation order is fixed (deterministic), not that of group_sum.
template <int N, int O, int NV>
__device__ __forceinline__ void rs_levels(double (&v)[NV], int lane) {
  if constexpr (O >= 1) {
    constexpr int H = (N + 1) / 2;
    const bool b = (lane & O) != 0;
#pragma unroll
    for (int i = 0; i < H; ++i) {
      const double hi = (i < N - H) ? v[H + i] : 0.0;
      const double send = b ? v[i] : hi;
      const double keep = b ? hi : v[i];
      v[i] = keep + __shfl_xor_sync(0xffffffffu, send, O);
    }
    rs_levels<H, O / 2, NV>(v, lane);
  }
}

struct RsSrc {
  int lane, idx;
};
// Which lane (within the group) ends up holding the sum of value c, and at
// which slot, after rs_levels<NV, G/2>.  Every level halves the held set to
// ceil(n/2) slots on both sides of the split (the upper half of an odd set
// carries one empty slot), as rs_levels does.
__host__ __device__ constexpr RsSrc rs_src(int NV, int G, int c) {
  int n = NV, lo = 0, lane = 0;
  for (int o = G / 2; o >= 1; o /= 2) {
    const int h = (n + 1) / 2;
    if (c - lo >= h) {
      lane |= o;
      lo += h;
    }
    n = h;
  }
  return RsSrc{lane, c - lo};
}

template <int NV, int G>
__device__ inline void rs_allreduce(double (&v)[NV], int lane_in_group) {
  rs_levels<NV, G / 2, NV>(v, lane_in_group);
  const int base = (int)(threadIdx.x & 31u) & ~(G - 1);
  double out[NV];
#pragma unroll
  for (int c = 0; c < NV; ++c) {
    const RsSrc src = rs_src(NV, G, c);
    out[c] = __shfl_sync(0xffffffffu, v[src.idx], base + src.lane);
  }
#pragma unroll
  for (int c = 0; c < NV; ++c) v[c] = out[c];
}

// Sum over the G lanes of a group, on every lane: reduce-scatter for groups
// inside one warp, the tree of group_sum for groups spanning warps.
template <int NV>
__device__ inline void group_allreduce(double (&v)[NV], int G, double* red, int lane_in_group) {
  switch (G) {
    case 32: rs_allreduce<NV, 32>(v, lane_in_group); return;
    case 16: rs_allreduce<NV, 16>(v, lane_in_group); return;
    case 8: rs_allreduce<NV, 8>(v, lane_in_group); return;
    case 4: rs_allreduce<NV, 4>(v, lane_in_group); return;
    case 2: rs_allreduce<NV, 2>(v, lane_in_group); return;
    case 1: return;
    default: group_sum<NV>(v, G, red, lane_in_group);
  }
}

// Non-finite test on the exponent bits (integer pipe, no FP64 compare).
__device__ inline bool nonfinite_bits(double x) { return (__double2hiint(x) & 0x7ff00000) == 0x7ff00000; }

__device__ inline void group_sync(int G) {
  if (G > 32) __syncthreads();
  else __syncwarp();
}

// Gauss-Jordan inverse with full pivoting of a 3x3 matrix (the algorithm of
// Caracal's invert, src/invert.f90:38-124).  Returns false if singular.
__device__ inline bool invert3(double (&a)[3][3]) {
  int ipiv[3] = {0, 0, 0}, indxr[3], indxc[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    double big = 0.0;
    int irow = 0, icol = 0;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      if (ipiv[j] != 1) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          if (ipiv[k] == 0 && fabs(a[j][k]) >= big) {
            big = fabs(a[j][k]);
            irow = j;
            icol = k;
          }
        }
      }
    }
    ipiv[icol] += 1;
    if (irow != icol) {
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        double t = a[irow][j];
        a[irow][j] = a[icol][j];
        a[icol][j] = t;
      }
    }
    indxr[i] = irow;
    indxc[i] = icol;
    if (a[icol][icol] == 0.0) return false;
    double ipivot = 1.0 / a[icol][icol];
    a[icol][icol] = 1.0;
#pragma unroll
    for (int j = 0; j < 3; ++j) a[icol][j] *= ipivot;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      if (j != icol) {
        double t = a[j][icol];
        a[j][icol] = 0.0;
#pragma unroll
        for (int k = 0; k < 3; ++k) a[j][k] -= a[icol][k] * t;
      }
    }
  }
#pragma unroll
  for (int i = 2; i >= 0; --i) {
    if (indxr[i] != indxc[i]) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        double t = a[k][indxr[i]];
        a[k][indxr[i]] = a[k][indxc[i]];
        a[k][indxc[i]] = t;
      }
    }
  }
  return true;
}

// Dynamic shared memory layout (doubles):
//   [0, 3 nr (nu + nv))            propagator blocks Ke, Ko of K1, K2, K3
//   then 2P                        PILE circulant vectors a, b
//   then per group: xs[2 NC][G] (reused as the outputs [2 NC][P/2+1]),
//                   u[2 NC][su], v[2 NC][sv], red[(GT/32) * 32] with GT = G TPB
__host__ __device__ inline size_t step_group_doubles(int P, int G, int NC, int tpb = 1) {
  const PropDims d = prop_dims(P);
  return (size_t)2 * NC * G + (size_t)2 * NC * (d.su + d.sv) + (size_t)((G * tpb + 31) / 32) * 32;
}
__host__ __device__ inline size_t step_smem_doubles(int P, int G, int NC, int groups, int tpb = 1) {
  const PropDims d = prop_dims(P);
  return (size_t)3 * d.nr * (d.nu + d.nv) + 2 * (size_t)P + step_group_doubles(P, G, NC, tpb) * groups;
}

// Threads per bead (TPB = 1, 2, 4).  A trajectory owns GT = G TPB
// consecutive threads: thread l of the group serves bead j = l mod G as its
// sub-thread s = l / G.  Sub-thread s owns the atoms a with a mod TPB = s:
// their q, p, f stay in its registers (slot 3 (a / TPB) + d), and it does
// their share of every per-coordinate stage (kicks, the PILE convolutions,
// the propagator's output rows, Andersen, the NaN check, the transrot moment
// sums), so those stages cost 1/TPB per thread; the propagator's
// (coordinate, row) tasks are shared by all GT threads.  The surface needs
// the whole bead, so every sub-thread gathers the bead's coordinates
// through shared memory and evaluates it (the same instructions side by
// side; no exchange of forces).  Worth it where the batch is too small to
// fill the GPU and the integrator dominates the bead's work (H3, OH + H2);
// TPB = 1 is the one-thread-per-bead kernel.
template <int TPB>
__host__ __device__ constexpr int own_slot(int c) { return 3 * ((c / 3) / TPB) + c % 3; }

template <class PES, bool MIXED, int TPB>
__global__ void __launch_bounds__(256) rpmd_run_kernel(StepParams prm, int istep_arg, int nsteps) {
  const int istep0 = prm.istep_dev ? *prm.istep_dev : istep_arg;
  constexpr int N = PES::N;
  constexpr int NC = 3 * N;
  constexpr int NL = 3 * ((N + TPB - 1) / TPB);  // coordinate slots per sub-thread
  extern __shared__ double smem[];
  const int P = prm.P, G = prm.G, H = prm.H;
  const int GT = G * TPB;
  const int groups = blockDim.x / GT;
  const int grp = threadIdx.x / GT;
  const int lg = threadIdx.x % GT;          // thread within the group
  const int j = (TPB == 1) ? lg : lg % G;   // bead
  const int sub = (TPB == 1) ? 0 : lg / G;  // sub-thread
  const int t = blockIdx.x * groups + grp;
  const bool active = (t < prm.T) && (j < P);
  // does this sub-thread own coordinate c (c a compile-time loop index)
  auto mine = [&](int c) { return TPB == 1 || (c / 3) % TPB == sub; };

  const PropDims pd = prm.pd;
  const int nke = 3 * pd.nr * pd.nu, nko = 3 * pd.nr * pd.nv;
  double* s_ke = smem;
  double* s_ko = s_ke + nke;
  double* s_pile = s_ko + nko;
  double* s_grp = s_pile + 2 * P + step_group_doubles(P, G, NC, TPB) * grp;
  double* xs = s_grp;                      // [2][NC][G]; after the fold: outputs [2][NC][H]
  double* su = xs + 2 * NC * G;            // [2 NC][su]
  double* sv = su + 2 * NC * pd.su;        // [2 NC][sv]
  double* red = sv + 2 * NC * pd.sv;       // [(GT/32)][32]

  if (prm.nm_mode) {
    for (int x = threadIdx.x; x < 3 * P; x += blockDim.x) s_ke[x] = prm.circ[x];  // 3 P <= nke
  } else {
    for (int x = threadIdx.x; x < nke; x += blockDim.x) s_ke[x] = prm.ke[x];
    for (int x = threadIdx.x; x < nko; x += blockDim.x) s_ko[x] = prm.ko[x];
  }
  if (prm.thermostat == CR_THERMO_PILE)
    for (int x = threadIdx.x; x < 2 * P; x += blockDim.x) s_pile[x] = prm.pile[x];

  double q[NL], p[NL], f[NL];
#pragma unroll
  for (int k = 0; k < NL; ++k) { q[k] = 0.0; p[k] = 0.0; f[k] = 0.0; }
  const size_t base = ((size_t)t * P + j) * NC;
  if (active) {
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      if (!mine(c)) continue;
      q[own_slot<TPB>(c)] = prm.q[base + c];
      p[own_slot<TPB>(c)] = prm.p[base + c];
      f[own_slot<TPB>(c)] = prm.f[base + c];
    }
  }
  const uint32_t traj_key = prm.traj0 + (uint32_t)t;
  int status = 0;
  double vbead = 0.0;
  const bool nhc = prm.thermostat == CR_THERMO_NHC;
  double vnh[4] = {0.0, 0.0, 0.0, 0.0};
  if (nhc && t < prm.T) {
#pragma unroll
    for (int k = 0; k < 4; ++k) vnh[k] = prm.vnh[4 * (size_t)t + k];
  }
  __syncthreads();

  // nhc (src/nhc.f90): group sum of p.p/(2m)/P/P, the chain, one scale.
  auto nhc_half = [&]() {
    double ek[1] = {0.0};
    if (active) {
#pragma unroll
      for (int i = 0; i < N; ++i) {
        if (!mine(3 * i)) continue;
        const int k = own_slot<TPB>(3 * i);
        const double pp = p[k] * p[k] + p[k + 1] * p[k + 1] + p[k + 2] * p[k + 2];
        ek[0] = ek[0] + pp / (2.0 * prm.mass[i]) / P / P;
      }
    }
    group_sum<1>(ek, GT, red, lg);
    const double sc = nhc_scale(prm.nhc, ek[0], vnh);
#pragma unroll
    for (int k = 0; k < NL; ++k) p[k] = sc * p[k];
  };

  // PILE half step on p (in place); eta from the per-bead Gaussian stream.
  auto pile_half = [&](uint32_t step, uint32_t tag) {
    double eta[NC];
    normals_bead<NC>(prm.seed, traj_key, (uint32_t)j, step, tag, eta);
    group_sync(GT);
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      if (!mine(c)) continue;
      xs[c * G + j] = p[own_slot<TPB>(c)];
      xs[(NC + c) * G + j] = active ? eta[c] : 0.0;
    }
    group_sync(GT);
    const double* a = s_pile;
    const double* b = s_pile + P;
    if (j < P) {
      double acc_p[NL], acc_e[NL];
#pragma unroll
      for (int k = 0; k < NL; ++k) { acc_p[k] = 0.0; acc_e[k] = 0.0; }
      int m = j;  // (j - l) mod P
      for (int l = 0; l < P; ++l) {
        const double al = a[m], bl = b[m];
#pragma unroll
        for (int c = 0; c < NC; ++c) {
          if (!mine(c)) continue;
          const int k = own_slot<TPB>(c);
          acc_p[k] = fma(al, xs[c * G + l], acc_p[k]);
          acc_e[k] = fma(bl, xs[(NC + c) * G + l], acc_e[k]);
        }
        m = (m == 0) ? P - 1 : m - 1;
      }
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        if (!mine(c)) continue;
        const int k = own_slot<TPB>(c);
        p[k] = acc_p[k] + prm.sigma[c / 3] * acc_e[k];
      }
    }
  };

  for (int n = 1; n <= nsteps; ++n) {
    const int istep = istep0 + n;
    if (nhc) nhc_half();  // src/verlet.f90:186-208
    if (prm.thermostat == CR_THERMO_PILE) pile_half((uint32_t)istep, TAG_PILE_A);

    // 1/2 kick (src/verlet.f90:216-218)
#pragma unroll
    for (int k = 0; k < NL; ++k) p[k] = p[k] - prm.half_dt * f[k];

    // free ring polymer (src/verlet.f90:377-463): Caracal's cosine modes, or
    // orthonormal normal modes where nm_mode is set
    group_sync(GT);
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      if (!mine(c)) continue;
      xs[c * G + j] = p[own_slot<TPB>(c)];
      xs[(NC + c) * G + j] = q[own_slot<TPB>(c)];
    }
    group_sync(GT);
    if (prm.nm_mode) {
      // orthonormal normal modes: bead j's row of the circulant K1, K2, K3
      if (j < P) {
        const double* c1 = s_ke;
        const double* c2 = s_ke + P;
        const double* c3 = s_ke + 2 * P;
#pragma unroll
        for (int c = 0; c < NC; ++c) {
          if (!mine(c)) continue;
          double a1p = 0.0, a1q = 0.0, a2q = 0.0, a3p = 0.0;
          int m = j;  // (j - l) mod P
          for (int l = 0; l < P; ++l) {
            const double xp = xs[c * G + l], xq = xs[(NC + c) * G + l];
            a1p = fma(c1[m], xp, a1p);
            a1q = fma(c1[m], xq, a1q);
            a2q = fma(c2[m], xq, a2q);
            a3p = fma(c3[m], xp, a3p);
            m = (m == 0) ? P - 1 : m - 1;
          }
          p[own_slot<TPB>(c)] = fma(prm.mass[c / 3], a2q, a1p);
          q[own_slot<TPB>(c)] = fma(prm.inv_mass[c / 3], a3p, a1q);
        }
      }
    } else {
      // Caracal's transform: fold each coordinate's P values into u (and v): tasks (cc, l)
      for (int idx = lg; idx < 2 * NC * pd.nu; idx += GT) {
        const int cc = idx / pd.nu, l = idx - cc * pd.nu;
        const double* x = xs + cc * G;
        const double a = sym_at(x, l, P);
        if (pd.split && 2 * l != pd.M) {
          const double b = sym_at(x, pd.M - l, P);
          su[cc * pd.su + l] = a + b;
          if (l < pd.nv) sv[cc * pd.sv + l] = a - b;
        } else {
          su[cc * pd.su + l] = a;
        }
      }
      group_sync(GT);
      // row pairs (r, M - r) of every coordinate: tasks (c, r); outputs into xs
      for (int idx = lg; idx < NC * pd.nr; idx += GT) {
        const int c = idx / pd.nr, r = idx - c * pd.nr;
        const double* k1e = s_ke + (0 * pd.nr + r) * pd.nu;
        const double* k2e = s_ke + (1 * pd.nr + r) * pd.nu;
        const double* k3e = s_ke + (2 * pd.nr + r) * pd.nu;
        const double* up = su + c * pd.su;
        const double* uq = su + (NC + c) * pd.su;
        double e1q = 0.0, e1p = 0.0, e2q = 0.0, e3p = 0.0;
        for (int l = 0; l < pd.nu; ++l) {
          const double a1 = k1e[l], a2 = k2e[l], a3 = k3e[l], xq = uq[l], xp = up[l];
          e1q = fma(a1, xq, e1q);
          e1p = fma(a1, xp, e1p);
          e2q = fma(a2, xq, e2q);
          e3p = fma(a3, xp, e3p);
        }
        double o1q = 0.0, o1p = 0.0, o2q = 0.0, o3p = 0.0;
        if (pd.nv > 0) {
          const double* k1o = s_ko + (0 * pd.nr + r) * pd.nv;
          const double* k2o = s_ko + (1 * pd.nr + r) * pd.nv;
          const double* k3o = s_ko + (2 * pd.nr + r) * pd.nv;
          const double* vp = sv + c * pd.sv;
          const double* vq = sv + (NC + c) * pd.sv;
          for (int l = 0; l < pd.nv; ++l) {
            const double a1 = k1o[l], a2 = k2o[l], a3 = k3o[l], xq = vq[l], xp = vp[l];
            o1q = fma(a1, xq, o1q);
            o1p = fma(a1, xp, o1p);
            o2q = fma(a2, xq, o2q);
            o3p = fma(a3, xp, o3p);
          }
        }
        const double m = prm.mass[c / 3], im = prm.inv_mass[c / 3];
        xs[c * H + r] = fma(m, e2q + o2q, e1p + o1p);
        xs[(NC + c) * H + r] = fma(im, e3p + o3p, e1q + o1q);
        if (pd.split && 2 * r != pd.M) {
          xs[c * H + pd.M - r] = fma(m, e2q - o2q, e1p - o1p);
          xs[(NC + c) * H + pd.M - r] = fma(im, e3p - o3p, e1q - o1q);
        }
      }
      group_sync(GT);
      if (j < P) {
        const int row = (j <= P - j) ? j : P - j;
#pragma unroll
        for (int c = 0; c < NC; ++c) {
          if (!mine(c)) continue;
          p[own_slot<TPB>(c)] = xs[c * H + row];
          q[own_slot<TPB>(c)] = xs[(NC + c) * H + row];
        }
      }
    }

    // per-bead forces (src/verlet.f90:772-777); with TPB > 1 the bead's
    // coordinates are first gathered from its sub-threads
    double g[NC];
    if constexpr (TPB == 1) {
      if (MIXED) PES::template egrad<float>(q, vbead, g);
      else PES::template egrad<double>(q, vbead, g);
#pragma unroll
      for (int c = 0; c < NC; ++c) f[c] = active ? g[c] : 0.0;
    } else {
      group_sync(GT);
#pragma unroll
      for (int c = 0; c < NC; ++c)
        if (mine(c)) xs[c * G + j] = q[own_slot<TPB>(c)];
      group_sync(GT);
      double qb[NC];
#pragma unroll
      for (int c = 0; c < NC; ++c) qb[c] = xs[c * G + j];
      if (MIXED) PES::template egrad<float>(qb, vbead, g);
      else PES::template egrad<double>(qb, vbead, g);
#pragma unroll
      for (int c = 0; c < NC; ++c)
        if (mine(c)) f[own_slot<TPB>(c)] = active ? g[c] : 0.0;
      if (sub != 0) vbead = 0.0;  // the bead's energy counts once
    }
    if (!active) vbead = 0.0;

    // reaction coordinate of the centroid (umbrella mode 1 of a child step,
    // src/verlet.f90:1049-1050 -> src/umbrella.f90:115-117)
    if (prm.xi_on) {
      double cq[NC];
#pragma unroll
      for (int c = 0; c < NC; ++c) cq[c] = (active && mine(c)) ? q[own_slot<TPB>(c)] : 0.0;
      group_allreduce<NC>(cq, GT, red, lg);
      if (active && lg == 0) {
        // centroid: a multiplication by 1/P where P is a power of two (exact), else the division
#pragma unroll
        for (int c = 0; c < NC; ++c) cq[c] = prm.pow2_P ? cq[c] * prm.inv_P : cq[c] / P;
        const double xi = xi_bimolec_value<N>(prm.xi, cq);
        prm.side[(size_t)t * prm.side_stride + (istep - prm.side_step0 - 1)] = xi > 0.0 ? 1 : 0;
      }
    }

    // 1/2 kick (src/verlet.f90:1060-1062)
#pragma unroll
    for (int k = 0; k < NL; ++k) p[k] = p[k] - prm.half_dt * f[k];

    if (nhc) nhc_half();  // src/verlet.f90:1085-1106

    // Andersen (src/verlet.f90:1159-1165): full resample every andersen_step
    if (prm.thermostat == CR_THERMO_ANDERSEN && (istep % prm.andersen_step) == 0) {
      double z[NC];
      normals_bead<NC>(prm.seed, traj_key, (uint32_t)j, (uint32_t)istep, TAG_ANDERSEN, z);
#pragma unroll
      for (int c = 0; c < NC; ++c)
        if (mine(c)) p[own_slot<TPB>(c)] = active ? z[c] * prm.sigma[c / 3] : 0.0;
    }
    if (prm.thermostat == CR_THERMO_PILE) pile_half((uint32_t)istep, TAG_PILE_B);

    // NaN / Inf check (src/verlet.f90:1256-1275)
#pragma unroll
    for (int k = 0; k < NL; ++k)
      if (nonfinite_bits(q[k])) status |= CR_TRAJ_NONFINITE;

    // transrot (src/transrot.f90:36-237): removed COM velocity and rotation
    // centre both carry Caracal's extra 1/P (total mass P^2 sum m).
    if (prm.transrot) {
      double vel[NL];
#pragma unroll
      for (int c = 0; c < NC; ++c)
        if (mine(c)) vel[own_slot<TPB>(c)] = p[own_slot<TPB>(c)] * prm.inv_mass[c / 3];
      double s1[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll
      for (int i = 0; i < N; ++i) {
        if (!mine(3 * i)) continue;
        const int k = own_slot<TPB>(3 * i);
        const double w = prm.mass[i];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          s1[d] = fma(vel[k + d], w, s1[d]);
          s1[3 + d] = fma(q[k + d], w, s1[3 + d]);
        }
      }
      if (!active) {
#pragma unroll
        for (int k = 0; k < 6; ++k) s1[k] = 0.0;
      }
      group_allreduce<6>(s1, GT, red, lg);
      const double itm = 1.0 / prm.totmass;
      const double vt[3] = {s1[0] * itm, s1[1] * itm, s1[2] * itm};
      const double xt[3] = {s1[3] * itm, s1[4] * itm, s1[5] * itm};
      double s2[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
      for (int i = 0; i < N; ++i) {
        if (!mine(3 * i)) continue;
        const int k = own_slot<TPB>(3 * i);
        const double w = prm.mass[i];
        const double* qq = &q[k];
        const double* vv = &vel[k];
        s2[0] = fma(qq[1] * vv[2] - qq[2] * vv[1], w, s2[0]);
        s2[1] = fma(qq[2] * vv[0] - qq[0] * vv[2], w, s2[1]);
        s2[2] = fma(qq[0] * vv[1] - qq[1] * vv[0], w, s2[2]);
        const double xd = qq[0] - xt[0], yd = qq[1] - xt[1], zd = qq[2] - xt[2];
        s2[3] = fma(xd * xd, w, s2[3]);
        s2[4] = fma(xd * yd, w, s2[4]);
        s2[5] = fma(xd * zd, w, s2[5]);
        s2[6] = fma(yd * yd, w, s2[6]);
        s2[7] = fma(yd * zd, w, s2[7]);
        s2[8] = fma(zd * zd, w, s2[8]);
      }
      if (!active) {
#pragma unroll
        for (int k = 0; k < 9; ++k) s2[k] = 0.0;
      }
      group_allreduce<9>(s2, GT, red, lg);
      const double tm = prm.totmass;
      double mang[3] = {s2[0] - (xt[1] * vt[2] - xt[2] * vt[1]) * tm,
                        s2[1] - (xt[2] * vt[0] - xt[0] * vt[2]) * tm,
                        s2[2] - (xt[0] * vt[1] - xt[1] * vt[0]) * tm};
      double ten[3][3] = {{s2[6] + s2[8], -s2[4], -s2[5]},
                          {-s2[4], s2[3] + s2[8], -s2[7]},
                          {-s2[5], -s2[7], s2[3] + s2[6]}};
      if (N <= 2) {
        ten[0][0] += 0.000001;
        ten[1][1] += 0.000001;
        ten[2][2] += 0.000001;
      }
      if (!invert3(ten)) {
        status |= CR_TRAJ_SINGULAR_INERTIA;
      } else {
        double va[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) va[a] = ten[a][0] * mang[0] + ten[a][1] * mang[1] + ten[a][2] * mang[2];
#pragma unroll
        for (int i = 0; i < N; ++i) {
          if (!mine(3 * i)) continue;
          double* vv = &vel[own_slot<TPB>(3 * i)];
          const double* qq = &q[own_slot<TPB>(3 * i)];
          vv[0] -= vt[0];
          vv[1] -= vt[1];
          vv[2] -= vt[2];
          const double xd = qq[0] - xt[0], yd = qq[1] - xt[1], zd = qq[2] - xt[2];
          vv[0] = vv[0] - va[1] * zd + va[2] * yd;
          vv[1] = vv[1] - va[2] * xd + va[0] * zd;
          vv[2] = vv[2] - va[0] * yd + va[1] * xd;
        }
#pragma unroll
        for (int c = 0; c < NC; ++c)
          if (mine(c)) p[own_slot<TPB>(c)] = active ? vel[own_slot<TPB>(c)] * prm.mass[c / 3] : 0.0;
      }
    }
  }

  // potential energy of the last step, summed over beads
  double e[1] = {vbead};
  group_sum<1>(e, GT, red, lg);
  if (active) {
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      if (!mine(c)) continue;
      prm.q[base + c] = q[own_slot<TPB>(c)];
      prm.p[base + c] = p[own_slot<TPB>(c)];
      prm.f[base + c] = f[own_slot<TPB>(c)];
    }
    if (lg == 0) prm.epot[t] = e[0];
    if (lg == 0 && nhc) {
#pragma unroll
      for (int k = 0; k < 4; ++k) prm.vnh[4 * (size_t)t + k] = vnh[k];
    }
    if (status) atomicOr(&prm.status[t], status);
  }
}

// One thread per bead: V and dV/dq.
template <class PES, bool MIXED>
__global__ void egrad_kernel(int nbeads_total, const double* q, double* V, double* g) {
  constexpr int NC = 3 * PES::N;
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nbeads_total) return;
  double qq[NC], gg[NC], v;
#pragma unroll
  for (int c = 0; c < NC; ++c) qq[c] = q[(size_t)b * NC + c];
  if (MIXED) PES::template egrad<float>(qq, v, gg);
  else PES::template egrad<double>(qq, v, gg);
  V[b] = v;
#pragma unroll
  for (int c = 0; c < NC; ++c) g[(size_t)b * NC + c] = gg[c];
}

}  // namespace cr
