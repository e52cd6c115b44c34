// Step kernels of the RPMD engine for molecules too large to keep a bead's
// state in registers (QMDFF): the state stays in HBM, laid out
// q[traj][bead][atom][3], and one step is a short chain of kernels captured
// in a CUDA graph:
//   split_nhc_kernel     Nose-Hoover chain (NHC only)
//   split_drift_kernel   PILE half (if PILE), 1/2 kick, free ring polymer
//   (force kernel)       dV/dq and V of every bead
//   split_kick_kernel    1/2 kick, Andersen resample or PILE half
//   split_nhc_kernel     Nose-Hoover chain (NHC only)
//   split_finish_kernel  NaN check, transrot, epot per trajectory
//   split_advance_kernel step counter + 1
// The order is Caracal's verlet (src/verlet.f90:216-218, 377-463, 772-777,
// 1060-1062, 1159-1165, 1256-1306).  The step index lives on the device so a
// captured step can be replayed.
//
// Free ring-polymer propagation.  Caracal's composite map K = C diag(poly) C
// (C = sqrt(1/P) cos(2 pi j k/P), src/rfft.f90 and src/irfft.f90 applied as
// the normal-mode transform) satisfies K[j][l] = K[-j][l] = K[j][-l], so the
// outputs of beads j and P-j coincide and only the P/2+1 symmetrised inputs
// s_l = x_l + x_{P-l} matter.  For even P, with M = P/2,
// C[M-r][k] = (-1)^k C[r][k]: splitting K = Ke + Ko by mode parity gives
// K[r] = Ke[r] + Ko[r] and K[M-r] = Ke[r] - Ko[r], with Ke even and Ko odd
// under l -> M-l.  One pass over u_l = s_l + s_{M-l} and v_l = s_l - s_{M-l}
// therefore yields rows r and M-r together: 4 (M/2+1)(M+1) FMAs per
// coordinate and trajectory for the four blocks, against 4 (M+1)^2 for the
// unique rows and 4 P (M+1) for one row per bead.
#pragma once
#include <cuda_runtime.h>

#include "cr_common.cuh"
#include "dual.cuh"
#include "rpmd_kernel.cuh"

namespace cr {

// Umbrella windows (verlet with constrain = 0, src/umbrella.f90 mode 0).
struct UmbrellaDev {
  const double* center;  // [T] xi of each trajectory's window
  const double* kforce;  // [T] force constant (Eh)
  double beta;           // 1 / (k_B T) of the fs term
  const int* sampling;   // device flag: 1 while the statistics are collected
  double* xsum;          // [T] sum of xi over the sampled steps
  double* xsum2;         // [T] sum of xi^2
  int nbins;             // histogram of xi over [lo, hi) (0: none)
  double lo, hi;
  double* hist;          // [T][nbins]
};

struct SplitParams {
  int T, P, N, NC;
  int M;          // P / 2
  int split;      // 1: even P, parity-split blocks; 0: odd P, unique rows only
  int nr, nu, nv; // task rows, u length, v length
  int su, sv;     // padded smem row strides of u and v
  int thermostat, andersen_step, transrot;
  uint32_t seed, traj0;
  double half_dt, totmass;
  const double* mass;      // [N]
  const double* inv_mass;  // [N]
  const double* sigma;     // [N] sqrt(m P / beta)
  const double* ke;        // [3][nr][nu]: K1, K2, K3 (unit mass), even-mode part (or full rows)
  const double* ko;        // [3][nr][nv]: odd-mode part
  const double* pile;      // [2][P] circulant a, b
  double* q;
  double* p;
  double* f;               // dV/dq
  double* V;               // [T][P] bead energies
  double* epot;            // [T]
  int* status;             // [T]
  int* istep;              // device step counter (last completed step)
  NhcParams nhc;
  double* vnh;             // [T][4] Nose-Hoover chain velocities
  // constrained parent (verlet with constrain = 1)
  int constrain;
  XiDev xi;
  double* dxi;             // [T][NC] dxi_act
  double* cq;              // [T][NC] centroid before SHAKE
  int* shake_fail;         // [T]
  int umbrella;            // 1: bias towards the trajectory's window after the forces
  UmbrellaDev umb;
};

constexpr int kSplitBlock = 128;
constexpr int kFinishBlock = 256;

__host__ __device__ inline int split_chunk(int P) { return P <= 64 ? 32 : 16; }

// shared-memory doubles of split_drift_kernel / split_kick_kernel
__host__ __device__ inline size_t split_smem_doubles(const SplitParams& s, bool pile) {
  const int cw = split_chunk(s.P), sp = s.P + 1;
  size_t n = (size_t)3 * s.nr * (s.nu + s.nv);        // tables
  n += (size_t)2 * cw * sp;                            // xq, xp
  n += (size_t)2 * cw * (s.su + s.sv);                 // u, v (q and p)
  if (pile) n += (size_t)2 * cw * sp + 2 * (size_t)s.P;  // eta, tmp, circulants
  return n;
}

// Deterministic block sum of NV values per thread (fixed tree); red holds
// NV * blockDim.x doubles.  The result is returned on every thread.
template <int NV>
__device__ inline void block_sum(double (&v)[NV], double* red) {
  __syncthreads();
#pragma unroll
  for (int i = 0; i < NV; ++i) red[i * blockDim.x + threadIdx.x] = v[i];
  __syncthreads();
  for (int w = blockDim.x / 2; w >= 1; w >>= 1) {
    if ((int)threadIdx.x < w) {
#pragma unroll
      for (int i = 0; i < NV; ++i) red[i * blockDim.x + threadIdx.x] += red[i * blockDim.x + threadIdx.x + w];
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < NV; ++i) v[i] = red[i * blockDim.x];
}

// Normals of coordinates [c0, c0+cw) of every bead into eta[c][j] (row stride sp).
__device__ inline void chunk_normals(const SplitParams& s, uint32_t traj, uint32_t step, uint32_t tag, int c0,
                                     int cw, double* eta, int sp) {
  const int npair = (cw + 1) / 2;
  for (int idx = threadIdx.x; idx < s.P * npair; idx += blockDim.x) {
    const int j = idx / npair, ip = idx % npair;
    const int c = 2 * ip;
    double z0, z1;
    normal_pair_f64(s.seed, traj, (uint32_t)((c0 + c) / 2), (uint32_t)j, step, tag, z0, z1);
    eta[c * sp + j] = z0;
    if (c + 1 < cw) eta[(c + 1) * sp + j] = z1;
  }
}

// PILE half step on xp (chunk of cw coordinates): p <- a * p + sigma b * eta.
__device__ inline void chunk_pile(const SplitParams& s, uint32_t traj, uint32_t step, uint32_t tag, int c0, int cw,
                                  double* xp, double* eta, double* tmp, const double* sa, const double* sb,
                                  int sp) {
  chunk_normals(s, traj, step, tag, c0, cw, eta, sp);
  __syncthreads();
  const int P = s.P;
  for (int idx = threadIdx.x; idx < P * cw; idx += blockDim.x) {
    const int c = idx % cw, j = idx / cw;
    const double* x = xp + c * sp;
    const double* e = eta + c * sp;
    double ap = 0.0, ae = 0.0;
    int m = j;  // (j - l) mod P
    for (int l = 0; l < P; ++l) {
      ap = fma(sa[m], x[l], ap);
      ae = fma(sb[m], e[l], ae);
      m = (m == 0) ? P - 1 : m - 1;
    }
    tmp[c * sp + j] = ap + s.sigma[(c0 + c) / 3] * ae;
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < P * cw; idx += blockDim.x) {
    const int c = idx % cw, j = idx / cw;
    xp[c * sp + j] = tmp[c * sp + j];
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kSplitBlock) split_drift_kernel(SplitParams s) {
  extern __shared__ double sm[];
  const int P = s.P, NC = s.NC, cw_max = split_chunk(P), sp = P + 1;
  const int t = blockIdx.y, c0 = blockIdx.x * cw_max;
  const int cw = min(cw_max, NC - c0);
  const uint32_t istep = (uint32_t)(*s.istep + 1);
  const bool pile = s.thermostat == CR_THERMO_PILE;
  const int nke = 3 * s.nr * s.nu, nko = 3 * s.nr * s.nv;
  double* ske = sm;
  double* sko = ske + nke;
  double* xq = sko + nko;
  double* xp = xq + cw_max * sp;
  double* uq = xp + cw_max * sp;
  double* up = uq + cw_max * s.su;
  double* vq = up + cw_max * s.su;
  double* vp = vq + cw_max * s.sv;
  double* eta = vp + cw_max * s.sv;
  double* tmp = eta + cw_max * sp;
  double* sa = tmp + cw_max * sp;
  double* sb = sa + P;
  for (int x = threadIdx.x; x < nke; x += blockDim.x) ske[x] = s.ke[x];
  for (int x = threadIdx.x; x < nko; x += blockDim.x) sko[x] = s.ko[x];
  if (pile)
    for (int x = threadIdx.x; x < 2 * P; x += blockDim.x) sa[x] = s.pile[x];
  const size_t tb = (size_t)t * P * NC + c0;
  for (int idx = threadIdx.x; idx < P * cw; idx += blockDim.x) {
    const int c = idx % cw, j = idx / cw;
    const size_t g = tb + (size_t)j * NC + c;
    xq[c * sp + j] = s.q[g];
    xp[c * sp + j] = pile ? s.p[g] : s.p[g] - s.half_dt * s.f[g];
  }
  __syncthreads();
  if (pile) {
    chunk_pile(s, s.traj0 + (uint32_t)t, istep, TAG_PILE_A, c0, cw, xp, eta, tmp, sa, sb, sp);
    for (int idx = threadIdx.x; idx < P * cw; idx += blockDim.x) {
      const int c = idx % cw, j = idx / cw;
      xp[c * sp + j] = xp[c * sp + j] - s.half_dt * s.f[tb + (size_t)j * NC + c];
    }
    __syncthreads();
  }
  // fold into u (and v)
  const int M = s.M;
  for (int idx = threadIdx.x; idx < cw * s.nu; idx += blockDim.x) {
    const int c = idx % cw, l = idx / cw;
    const double* a = xq + c * sp;
    const double* b = xp + c * sp;
    const double aq = sym_at(a, l, P), ap = sym_at(b, l, P);
    if (s.split && 2 * l != M) {
      const double bq = sym_at(a, M - l, P), bp = sym_at(b, M - l, P);
      uq[c * s.su + l] = aq + bq;
      up[c * s.su + l] = ap + bp;
      if (l < s.nv) {
        vq[c * s.sv + l] = aq - bq;
        vp[c * s.sv + l] = ap - bp;
      }
    } else {
      uq[c * s.su + l] = aq;
      up[c * s.su + l] = ap;
    }
  }
  __syncthreads();
  // rows r (and M - r): q' = K1 q + K3 p / m, p' = K1 p + m K2 q
  const int nr = s.nr, nu = s.nu, nv = s.nv;
  for (int idx = threadIdx.x; idx < cw * nr; idx += blockDim.x) {
    const int c = idx % cw, r = idx / cw;
    const double* k1e = ske + (0 * nr + r) * nu;
    const double* k2e = ske + (1 * nr + r) * nu;
    const double* k3e = ske + (2 * nr + r) * nu;
    const double* uqc = uq + c * s.su;
    const double* upc = up + c * s.su;
    double e1q = 0.0, e1p = 0.0, e2q = 0.0, e3p = 0.0;
    for (int l = 0; l < nu; ++l) {
      const double a1 = k1e[l], a2 = k2e[l], a3 = k3e[l];
      const double xq_ = uqc[l], xp_ = upc[l];
      e1q = fma(a1, xq_, e1q);
      e1p = fma(a1, xp_, e1p);
      e2q = fma(a2, xq_, e2q);
      e3p = fma(a3, xp_, e3p);
    }
    double o1q = 0.0, o1p = 0.0, o2q = 0.0, o3p = 0.0;
    if (nv > 0) {
      const double* k1o = sko + (0 * nr + r) * nv;
      const double* k2o = sko + (1 * nr + r) * nv;
      const double* k3o = sko + (2 * nr + r) * nv;
      const double* vqc = vq + c * s.sv;
      const double* vpc = vp + c * s.sv;
      for (int l = 0; l < nv; ++l) {
        const double a1 = k1o[l], a2 = k2o[l], a3 = k3o[l];
        const double xq_ = vqc[l], xp_ = vpc[l];
        o1q = fma(a1, xq_, o1q);
        o1p = fma(a1, xp_, o1p);
        o2q = fma(a2, xq_, o2q);
        o3p = fma(a3, xp_, o3p);
      }
    }
    const int atom = (c0 + c) / 3;
    const double m = s.mass[atom], im = s.inv_mass[atom];
    const double qa = fma(im, e3p + o3p, e1q + o1q);
    const double pa = fma(m, e2q + o2q, e1p + o1p);
    int rows[2] = {r, -1};
    double qv[2] = {qa, 0.0}, pv[2] = {pa, 0.0};
    if (s.split && 2 * r != M) {
      rows[1] = M - r;
      qv[1] = fma(im, e3p - o3p, e1q - o1q);
      pv[1] = fma(m, e2q - o2q, e1p - o1p);
    }
    for (int k = 0; k < 2; ++k) {
      const int row = rows[k];
      if (row < 0) continue;
      const size_t g = tb + (size_t)row * NC + c;
      s.q[g] = qv[k];
      s.p[g] = pv[k];
      if (row != 0 && 2 * row != P) {
        const size_t g2 = tb + (size_t)(P - row) * NC + c;
        s.q[g2] = qv[k];
        s.p[g2] = pv[k];
      }
    }
  }
}

// mode 0: 1/2 kick and thermostat; 1: 1/2 kick only; 2: thermostat only (the
// constrained parent runs RATTLE between the two).
__global__ void __launch_bounds__(kSplitBlock) split_kick_kernel(SplitParams s, int mode) {
  extern __shared__ double sm[];
  const int P = s.P, NC = s.NC, cw_max = split_chunk(P), sp = P + 1;
  const int t = blockIdx.y, c0 = blockIdx.x * cw_max;
  const int cw = min(cw_max, NC - c0);
  const int istep = *s.istep + 1;
  const size_t tb = (size_t)t * P * NC + c0;
  const uint32_t traj = s.traj0 + (uint32_t)t;
  const double hdt = mode == 2 ? 0.0 : s.half_dt;
  if (mode == 1) {
    for (int idx = threadIdx.x; idx < P * cw; idx += blockDim.x) {
      const int c = idx % cw, j = idx / cw;
      const size_t g = tb + (size_t)j * NC + c;
      s.p[g] = s.p[g] - s.half_dt * s.f[g];
    }
    return;
  }
  if (s.thermostat == CR_THERMO_PILE) {
    double* xp = sm;
    double* eta = xp + cw_max * sp;
    double* tmp = eta + cw_max * sp;
    double* sa = tmp + cw_max * sp;
    double* sb = sa + P;
    for (int x = threadIdx.x; x < 2 * P; x += blockDim.x) sa[x] = s.pile[x];
    for (int idx = threadIdx.x; idx < P * cw; idx += blockDim.x) {
      const int c = idx % cw, j = idx / cw;
      const size_t g = tb + (size_t)j * NC + c;
      xp[c * sp + j] = s.p[g] - hdt * s.f[g];
    }
    __syncthreads();
    chunk_pile(s, traj, (uint32_t)istep, TAG_PILE_B, c0, cw, xp, eta, tmp, sa, sb, sp);
    for (int idx = threadIdx.x; idx < P * cw; idx += blockDim.x) {
      const int c = idx % cw, j = idx / cw;
      s.p[tb + (size_t)j * NC + c] = xp[c * sp + j];
    }
    return;
  }
  if (s.thermostat == CR_THERMO_ANDERSEN && (istep % s.andersen_step) == 0) {
    // full resample (src/andersen.f90:37-71); the kick is overwritten
    const int npair = (cw + 1) / 2;
    for (int idx = threadIdx.x; idx < P * npair; idx += blockDim.x) {
      const int j = idx / npair, ip = idx % npair;
      const int c = 2 * ip;
      double z0, z1;
      normal_pair_f64(s.seed, traj, (uint32_t)((c0 + c) / 2), (uint32_t)j, (uint32_t)istep, TAG_ANDERSEN, z0, z1);
      s.p[tb + (size_t)j * NC + c] = z0 * s.sigma[(c0 + c) / 3];
      if (c + 1 < cw) s.p[tb + (size_t)j * NC + c + 1] = z1 * s.sigma[(c0 + c + 1) / 3];
    }
    return;
  }
  if (mode == 2) return;
  for (int idx = threadIdx.x; idx < P * cw; idx += blockDim.x) {
    const int c = idx % cw, j = idx / cw;
    const size_t g = tb + (size_t)j * NC + c;
    s.p[g] = s.p[g] - s.half_dt * s.f[g];
  }
}

// ---- constrained parent (src/constrain_q.f90, src/constrain_p.f90) ----------
// One block per trajectory.  SHAKE: the centroid c (kept for the next dxi),
// Newton iterations for the multiplier on thread 0 (at most 200; the
// tolerances 1.0E-8 and 1.0E-10 are REAL(4) literals), then every bead moves:
// q by the coefficient of the last iteration's start, p by the updated
// multiplier.  A failed SHAKE leaves q, p unchanged and is flagged.
template <int N>
__global__ void split_shake_kernel(SplitParams s) {
  constexpr int NC = 3 * N;
  __shared__ double cq[NC], dxa[NC], res[3];
  const int t = blockIdx.x, P = s.P;
  const size_t tb = (size_t)t * P * NC;
  for (int c = threadIdx.x; c < NC; c += blockDim.x) {
    double acc = 0.0;
    for (int k = 0; k < P; ++k) acc = acc + s.q[tb + (size_t)k * NC + c];
    cq[c] = acc / P;
    dxa[c] = s.dxi[(size_t)t * NC + c];
    s.cq[(size_t)t * NC + c] = cq[c];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const double dt = 2.0 * s.half_dt;
    double mult = 0.0, coeff = 0.0, qt[NC], dxn[NC];
    int ok = 0;
    for (int iter = 1; iter <= 200; ++iter) {
      coeff = mult * dt * dt / P;
      for (int c = 0; c < NC; ++c) qt[c] = cq[c] + coeff * dxa[c] / s.mass[c / 3];
      const double sigma = xi_bimolec<N>(s.xi, qt, s.mass, dxn);
      double dsigma = 0.0;
      for (int c = 0; c < NC; ++c) dsigma = dsigma + dxn[c] * dt * dt * dxa[c] / (s.mass[c / 3] * P);
      const double dx = sigma / dsigma;
      mult = mult - dx;
      if (fabs(dx) < (double)1.0E-8f || fabs(sigma) < (double)1.0E-10f) {
        ok = 1;
        break;
      }
    }
    res[0] = coeff;
    res[1] = mult;
    res[2] = ok;
    s.shake_fail[t] = ok ? 0 : 1;
  }
  __syncthreads();
  if (res[2] == 0.0) return;
  const double coeff = res[0], mult = res[1], dt = 2.0 * s.half_dt;
  for (int idx = threadIdx.x; idx < P * NC; idx += blockDim.x) {
    const int c = idx % NC;
    const double m = s.mass[c / 3];
    s.q[tb + idx] = s.q[tb + idx] + coeff / m * dxa[c];
    s.p[tb + idx] = s.p[tb + idx] + mult * dt / P * dxa[c];
  }
}

// dxi_act <- dxi at the pre-SHAKE centroid (umbrella mode 1, src/verlet.f90:
// 1047-1049), then RATTLE: p -= (sum dxi.p/m) / (sum dxi^2/m) / P * dxi.
template <int N>
__global__ void split_rattle_kernel(SplitParams s) {
  constexpr int NC = 3 * N;
  __shared__ double dxa[NC], red[kFinishBlock];
  const int t = blockIdx.x, P = s.P;
  const size_t tb = (size_t)t * P * NC;
  if (threadIdx.x == 0) {
    double cq[NC], d[NC];
    for (int c = 0; c < NC; ++c) cq[c] = s.cq[(size_t)t * NC + c];
    xi_bimolec<N>(s.xi, cq, s.mass, d);
    for (int c = 0; c < NC; ++c) {
      dxa[c] = d[c];
      s.dxi[(size_t)t * NC + c] = d[c];
    }
  }
  __syncthreads();
  double c1[1] = {0.0};
  for (int idx = threadIdx.x; idx < P * NC; idx += blockDim.x) {
    const int c = idx % NC;
    c1[0] = c1[0] + dxa[c] * s.p[tb + idx] / s.mass[c / 3];
  }
  block_sum<1>(c1, red);
  double c2 = 0.0;
  for (int c = 0; c < NC; ++c) c2 = c2 + dxa[c] * dxa[c] / s.mass[c / 3];
  const double lambdas = -c1[0] / c2 / P;
  for (int idx = threadIdx.x; idx < P * NC; idx += blockDim.x) s.p[tb + idx] = s.p[tb + idx] + lambdas * dxa[idx % NC];
}

// initial dxi_act of each parent at its current centroid
template <int N>
__global__ void split_parent_init_kernel(SplitParams s) {
  constexpr int NC = 3 * N;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= s.T) return;
  double cq[NC], d[NC];
  for (int c = 0; c < NC; ++c) {
    double acc = 0.0;
    for (int k = 0; k < s.P; ++k) acc = acc + s.q[((size_t)t * s.P + k) * NC + c];
    cq[c] = acc / s.P;
  }
  xi_bimolec<N>(s.xi, cq, s.mass, d);
  for (int c = 0; c < NC; ++c) s.dxi[(size_t)t * NC + c] = d[c];
  s.shake_fail[t] = 0;
}

// NaN check (src/verlet.f90:1256-1275), transrot (src/transrot.f90:36-237,
// COM velocity and rotation centre with Caracal's total mass P^2 sum m) and
// the potential energy summed over beads.  One block per trajectory.
__global__ void __launch_bounds__(kFinishBlock) split_finish_kernel(SplitParams s) {
  __shared__ double red[9 * kFinishBlock];
  __shared__ double sva[4];
  const int t = blockIdx.x, P = s.P, N = s.N, NC = s.NC;
  const size_t tb = (size_t)t * P * NC;
  const int items = P * N;
  int status = 0;
  double s1[7] = {0, 0, 0, 0, 0, 0, 0};
  for (int idx = threadIdx.x; idx < items; idx += blockDim.x) {
    const int a = idx % N;
    const double* qq = s.q + tb + 3 * (size_t)idx;
    const double* pp = s.p + tb + 3 * (size_t)idx;
    const double w = s.mass[a], iw = s.inv_mass[a];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      if (!isfinite(qq[d])) status |= CR_TRAJ_NONFINITE;
      s1[d] = fma(pp[d] * iw, w, s1[d]);
      s1[3 + d] = fma(qq[d], w, s1[3 + d]);
    }
  }
  for (int j = threadIdx.x; j < P; j += blockDim.x) s1[6] += s.V[(size_t)t * P + j];
  block_sum<7>(s1, red);
  __shared__ int sstat;
  if (threadIdx.x == 0) sstat = 0;
  __syncthreads();
  if (status) atomicOr(&sstat, status);
  __syncthreads();
  status = sstat;
  if (s.constrain && s.shake_fail[t]) status |= CR_TRAJ_SHAKE_FAILED;
  if (threadIdx.x == 0) s.epot[t] = s1[6] + ((s.constrain && s.shake_fail[t]) ? 100000.0 : 0.0);
  if (s.transrot) {
    const double itm = 1.0 / s.totmass;
    const double vt[3] = {s1[0] * itm, s1[1] * itm, s1[2] * itm};
    const double xt[3] = {s1[3] * itm, s1[4] * itm, s1[5] * itm};
    double s2[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int idx = threadIdx.x; idx < items; idx += blockDim.x) {
      const int a = idx % N;
      const double* qq = s.q + tb + 3 * (size_t)idx;
      const double* pp = s.p + tb + 3 * (size_t)idx;
      const double w = s.mass[a], iw = s.inv_mass[a];
      const double vv[3] = {pp[0] * iw, pp[1] * iw, pp[2] * iw};
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
    block_sum<9>(s2, red);
    if (threadIdx.x == 0) {
      const double tm = s.totmass;
      const double mang[3] = {s2[0] - (xt[1] * vt[2] - xt[2] * vt[1]) * tm,
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
        sva[3] = 1.0;
      } else {
        sva[3] = 0.0;
        for (int a = 0; a < 3; ++a) sva[a] = ten[a][0] * mang[0] + ten[a][1] * mang[1] + ten[a][2] * mang[2];
      }
    }
    __syncthreads();
    if (sva[3] != 0.0) {
      status |= CR_TRAJ_SINGULAR_INERTIA;
    } else {
      const double va[3] = {sva[0], sva[1], sva[2]};
      for (int idx = threadIdx.x; idx < items; idx += blockDim.x) {
        const int a = idx % N;
        const double* qq = s.q + tb + 3 * (size_t)idx;
        double* pp = s.p + tb + 3 * (size_t)idx;
        const double w = s.mass[a], iw = s.inv_mass[a];
        double vv[3] = {pp[0] * iw - vt[0], pp[1] * iw - vt[1], pp[2] * iw - vt[2]};
        const double xd = qq[0] - xt[0], yd = qq[1] - xt[1], zd = qq[2] - xt[2];
        const double v0 = vv[0] - va[1] * zd + va[2] * yd;
        const double v1 = vv[1] - va[2] * xd + va[0] * zd;
        const double v2 = vv[2] - va[0] * yd + va[1] * xd;
        pp[0] = v0 * w;
        pp[1] = v1 * w;
        pp[2] = v2 * w;
      }
    }
  }
  if (threadIdx.x == 0 && status) atomicOr(&s.status[t], status);
}

// nhc (src/nhc.f90:35-171) on one trajectory per block: the kinetic sum
// p.p/(2m)/P/P over beads and atoms, the chain, one scale of every momentum.
__global__ void __launch_bounds__(kFinishBlock) split_nhc_kernel(SplitParams s) {
  __shared__ double red[kFinishBlock];
  __shared__ double ssc;
  const int t = blockIdx.x, P = s.P, N = s.N, NC = s.NC;
  const size_t tb = (size_t)t * P * NC;
  double ek[1] = {0.0};
  for (int idx = threadIdx.x; idx < P * N; idx += blockDim.x) {
    const double* pp = s.p + tb + 3 * (size_t)idx;
    const double w = s.mass[idx % N];
    ek[0] = ek[0] + (pp[0] * pp[0] + pp[1] * pp[1] + pp[2] * pp[2]) / (2.0 * w) / P / P;
  }
  block_sum<1>(ek, red);
  if (threadIdx.x == 0) {
    double v[4];
    for (int k = 0; k < 4; ++k) v[k] = s.vnh[4 * (size_t)t + k];
    ssc = nhc_scale(s.nhc, ek[0], v);
    for (int k = 0; k < 4; ++k) s.vnh[4 * (size_t)t + k] = v[k];
  }
  __syncthreads();
  const double sc = ssc;
  for (int x = threadIdx.x; x < P * NC; x += blockDim.x) s.p[tb + x] = sc * s.p[tb + x];
}

__global__ void split_advance_kernel(int* istep) { *istep += 1; }
__global__ void advance_by_kernel(int* istep, int n) { *istep += n; }

// mdinit-style initial state for any atom count: per (trajectory, bead, pair).
__global__ void split_init_positions_kernel(int T, int P, int NC, uint32_t seed, uint32_t traj0, const double* q0,
                                            double sigma, double* q) {
  const int npair = (NC + 1) / 2;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)T * P * npair) return;
  const int ip = (int)(idx % npair);
  const long long b = idx / npair;
  const int t = (int)(b / P), k = (int)(b % P);
  double z0, z1;
  normal_pair_f64(seed, traj0 + (uint32_t)t, (uint32_t)ip, (uint32_t)k, 0u, TAG_BEAD_JITTER, z0, z1);
  const int c = 2 * ip;
  q[(size_t)b * NC + c] = q0[c] + sigma * z0;
  if (c + 1 < NC) q[(size_t)b * NC + c + 1] = q0[c + 1] + sigma * z1;
}

__global__ void split_init_momenta_kernel(int T, int P, int NC, uint32_t seed, uint32_t traj0, const double* sig,
                                          int zero, double* p) {
  const int npair = (NC + 1) / 2;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)T * P * npair) return;
  const int ip = (int)(idx % npair);
  const long long b = idx / npair;
  const int t = (int)(b / P), k = (int)(b % P);
  const int c = 2 * ip;
  double z0 = 0.0, z1 = 0.0;
  if (!zero) normal_pair_f64(seed, traj0 + (uint32_t)t, (uint32_t)ip, (uint32_t)k, 0u, TAG_INIT_MOMENTA, z0, z1);
  p[(size_t)b * NC + c] = z0 * sig[c / 3];
  if (c + 1 < NC) p[(size_t)b * NC + c + 1] = z1 * sig[(c + 1) / 3];
}

// epot[t] = sum of the bead energies (after a force evaluation outside a step)
__global__ void split_sum_beads_kernel(int T, int P, const double* V, double* epot) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  double s = 0.0;
  for (int k = 0; k < P; ++k) s += V[(size_t)t * P + k];
  epot[t] = s;
}


// BIMOLEC reaction coordinate of umbrella sampling (calc_xi mode 1,
// src/calc_xi.f90:63-279): xi = s0 / (s0 - s1) and its gradient
// (s0 ds1 - s1 ds0) / (s0 - s1)^2.  T = Dual gives, with dual coordinates
// c + eps u, the Hessian-vector product in the eps parts of dxi.
template <int N, class T>
__device__ inline T xi_umbrella(const XiDev& x, const T* c, const double* mass, T* dxi) {
  constexpr int NC = 3 * N;
  T Rf[3], Rb[3];
  for (int d = 0; d < 3; ++d) {
    Rf[d] = c[3 * x.form0 + d] - c[3 * x.form1 + d];
    Rb[d] = c[3 * x.brk0 + d] - c[3 * x.brk1 + d];
  }
  const T rf = sqrt(Rf[0] * Rf[0] + Rf[1] * Rf[1] + Rf[2] * Rf[2]);
  const T rb = sqrt(Rb[0] * Rb[0] + Rb[1] * Rb[1] + Rb[2] * Rb[2]);
  T s1 = T(0.0);
  s1 = s1 + (rb - x.break_ref) / 1.0;
  s1 = s1 - (rf - x.form_ref) / 1.0;
  T c1[3] = {T(0.0), T(0.0), T(0.0)}, c2[3] = {T(0.0), T(0.0), T(0.0)};
  for (int k = 0; k < x.nreac1; ++k)
    for (int d = 0; d < 3; ++d) c1[d] = c1[d] + mass[x.reac1[k]] * c[3 * x.reac1[k] + d] / x.mreac1;
  for (int k = 0; k < x.nreac2; ++k)
    for (int d = 0; d < 3; ++d) c2[d] = c2[d] + mass[x.reac2[k]] * c[3 * x.reac2[k] + d] / x.mreac2;
  const T Red[3] = {c2[0] - c1[0], c2[1] - c1[1], c2[2] - c1[2]};
  const T reds = sqrt(Red[0] * Red[0] + Red[1] * Red[1] + Red[2] * Red[2]);
  T s0 = T(0.0);
  s0 = s0 + (x.r_inf - reds);
  s0 = s0 / 1.0;
  T ds1[NC], ds0[NC];
  for (int i = 0; i < NC; ++i) ds1[i] = ds0[i] = T(0.0);
  T ri = 1.0 / rf;
  for (int d = 0; d < 3; ++d) {
    ds1[3 * x.form0 + d] = ds1[3 * x.form0 + d] - Rf[d] * ri / 1.0;
    ds1[3 * x.form1 + d] = ds1[3 * x.form1 + d] + Rf[d] * ri / 1.0;
  }
  ri = 1.0 / rb;
  for (int d = 0; d < 3; ++d) {
    ds1[3 * x.brk0 + d] = ds1[3 * x.brk0 + d] + Rb[d] * ri / 1.0;
    ds1[3 * x.brk1 + d] = ds1[3 * x.brk1 + d] - Rb[d] * ri / 1.0;
  }
  ri = 1.0 / reds;
  for (int k = 0; k < x.nreac1; ++k) {
    const int a = x.reac1[k];
    for (int d = 0; d < 3; ++d) ds0[3 * a + d] = ds0[3 * a + d] + Red[d] * ri * mass[a] / x.mreac1 / 1.0;
  }
  for (int k = 0; k < x.nreac2; ++k) {
    const int a = x.reac2[k];
    for (int d = 0; d < 3; ++d) ds0[3 * a + d] = ds0[3 * a + d] + (-1.0) * Red[d] * ri * mass[a] / x.mreac2 / 1.0;
  }
  const T D = s0 - s1;
  for (int i = 0; i < NC; ++i) dxi[i] = (s0 * ds1[i] - s1 * ds0[i]) / (D * D);
  return s0 / D;
}

// Umbrella bias after the forces (src/umbrella.f90:100-176): at the centroid,
// every bead's gradient gets k (xi - xi0) dxi, then the gradient of
// -(1/beta) log fs, (-1/beta) / (2 pi beta fs^2) H dxi/m with H the Hessian
// of xi (a dual-number pass along u = dxi/m).  One block per trajectory.
template <int N>
__global__ void split_umbrella_kernel(SplitParams s) {
  constexpr int NC = 3 * N;
  __shared__ double cq[NC], ka[NC], kb[NC];
  const int t = blockIdx.x, P = s.P;
  const size_t tb = (size_t)t * P * NC;
  for (int c = threadIdx.x; c < NC; c += blockDim.x) {
    double acc = 0.0;
    for (int k = 0; k < P; ++k) acc = acc + s.q[tb + (size_t)k * NC + c];
    cq[c] = acc / P;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double dxi[NC];
    const double xi = xi_umbrella<N, double>(s.xi, cq, s.mass, dxi);
    Dual cd[NC], hd[NC];
    for (int c = 0; c < NC; ++c) cd[c] = Dual(cq[c], dxi[c] / s.mass[c / 3]);
    xi_umbrella<N, Dual>(s.xi, cd, s.mass, hd);
    const double delta = xi - s.umb.center[t], kf = s.umb.kforce[t];
    const double pi = 3.1415926535897932384;
    double fs2 = 0.0;
    for (int l = 0; l < 3; ++l)
      for (int m = 0; m < N; ++m) fs2 = fs2 + dxi[3 * m + l] * dxi[3 * m + l] / s.mass[m];
    const double coeff1 = 2.0 * pi * s.umb.beta;
    fs2 = fs2 / coeff1;
    const double coeff2 = -1.0 / s.umb.beta;
    for (int c = 0; c < NC; ++c) {
      ka[c] = kf * delta * dxi[c];
      kb[c] = hd[c].d * coeff2 / (coeff1 * fs2);
    }
    if (*s.umb.sampling) {
      s.umb.xsum[t] = s.umb.xsum[t] + xi;
      s.umb.xsum2[t] = s.umb.xsum2[t] + xi * xi;
      if (s.umb.nbins > 0) {
        const double u = (xi - s.umb.lo) / (s.umb.hi - s.umb.lo) * s.umb.nbins;
        if (u >= 0.0 && u < s.umb.nbins) s.umb.hist[(size_t)t * s.umb.nbins + (int)u] += 1.0;
      }
    }
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < P * NC; idx += blockDim.x) {
    const int c = idx % NC;
    s.f[tb + idx] = (s.f[tb + idx] + ka[c]) + kb[c];
  }
}

}  // namespace cr
