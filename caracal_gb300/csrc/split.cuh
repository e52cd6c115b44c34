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
  double wsum;             // sum of the masses over beads and atoms (P sum m)
  const double* mass;      // [N]
  const double* inv_mass;  // [N]
  const double* sigma;     // [N] sqrt(m P / beta)
  const double* ke;        // [3][nr][nu]: K1, K2, K3 (unit mass), even-mode part (or full rows)
  const double* ko;        // [3][nr][nv]: odd-mode part
  const double* pile;      // [2][P] circulant a, b
  const double* fdrift;    // split_drift_fast_kernel: [3][M+1] mode coefficients, then M Lee factors
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
  // nm_mode 1: orthonormal normal modes, K1, K2, K3 circulant: circ[w][(j - l) mod P]
  int nm_mode;
  const double* circ;      // [3][P]
  // transrot / energy scratch of split_moments_kernel and split_solve_kernel
  double* fsum;            // [T][S][16] partial sums per slice
  int* fstat;              // [T][S] status bits per slice
  double* fmove;           // [T][10] vt, xt, va, skip flag
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
  n += (size_t)cw;                                     // q shifts
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
    normal_pair(s.seed, traj, (uint32_t)((c0 + c) / 2), (uint32_t)j, step, tag, z0, z1);
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
  double* shq = vp + cw_max * s.sv;  // per-coordinate q shift
  double* eta = shq + cw_max;
  double* tmp = eta + cw_max * sp;
  double* sa = tmp + cw_max * sp;
  double* sb = sa + P;
  if (s.nm_mode) {
    for (int x = threadIdx.x; x < 3 * P; x += blockDim.x) ske[x] = s.circ[x];  // 3 P <= nke
  } else {
    for (int x = threadIdx.x; x < nke; x += blockDim.x) ske[x] = s.ke[x];
    for (int x = threadIdx.x; x < nko; x += blockDim.x) sko[x] = s.ko[x];
  }
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
  // q relative to its bead-0 value (the constant vector is the centroid
  // mode: K1 keeps it, K2 drops it; the products then round on bead spreads)
  for (int c = threadIdx.x; c < cw; c += blockDim.x) shq[c] = xq[c * sp];
  __syncthreads();
  for (int idx = threadIdx.x; idx < P * cw; idx += blockDim.x) {
    const int c = idx % cw, j = idx / cw;
    xq[c * sp + j] -= shq[c];
  }
  __syncthreads();
  if (s.nm_mode) {
    // orthonormal normal modes: row j of the circulant K1, K2, K3 (the
    // constant vector is an eigenvector of all three, so the q shift holds)
    for (int idx = threadIdx.x; idx < P * cw; idx += blockDim.x) {
      const int c = idx % cw, j = idx / cw;
      const double* xqc = xq + c * sp;
      const double* xpc = xp + c * sp;
      double a1p = 0.0, a1q = 0.0, a2q = 0.0, a3p = 0.0;
      int m = j;  // (j - l) mod P
      for (int l = 0; l < P; ++l) {
        const double c1 = ske[m], c2 = ske[P + m], c3 = ske[2 * P + m];
        a1p = fma(c1, xpc[l], a1p);
        a1q = fma(c1, xqc[l], a1q);
        a2q = fma(c2, xqc[l], a2q);
        a3p = fma(c3, xpc[l], a3p);
        m = (m == 0) ? P - 1 : m - 1;
      }
      const int atom = (c0 + c) / 3;
      const size_t g = tb + (size_t)j * NC + c;
      s.q[g] = fma(s.inv_mass[atom], a3p, a1q) + shq[c];
      s.p[g] = fma(s.mass[atom], a2q, a1p);
    }
    return;
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
    const double qa = fma(im, e3p + o3p, e1q + o1q) + shq[c];
    const double pa = fma(m, e2q + o2q, e1p + o1p);
    int rows[2] = {r, -1};
    double qv[2] = {qa, 0.0}, pv[2] = {pa, 0.0};
    if (s.split && 2 * r != M) {
      rows[1] = M - r;
      qv[1] = fma(im, e3p - o3p, e1q - o1q) + shq[c];
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

// ---- free ring polymer by fast cosine transforms (even P = 2M, M = 4..32) ----
// Caracal's map y = C D C x (C = sqrt(1/P) cos(2 pi j k / P)) depends on x
// only through the fold s_0 = x_0, s_M = x_M, s_l = x_l + x_{P-l}, and
// C x = T_M(s) / sqrt(P) with the type-I cosine transform
//   T_M(s)_k = s_0 + (-1)^k s_M + sum_{l=1}^{M-1} s_l cos(pi k l / M),  k = 0..M.
// The output is y_j = y_{P-j} = T_M(z)_j / sqrt(P), z_k = w_k D_k (C x)_k with
// w_0 = w_M = 1, w_k = 2 otherwise.  T_M splits by the parity of k into
// T_{M/2} of u_l = s_l + s_{M-l} (even k) and the type-III transform of size
// M/2 of v_l = s_l - s_{M-l} (odd k); the type-III transform
//   X_k = sum_{n<N} x_n cos(pi (2k+1) n / (2N))
// follows Lee's recursion (B. G. Lee, IEEE Trans. ASSP 32 (1984) 1243):
// G = (size N/2 of x_{2m}), H' = (size N/2 of x_{2m+1} + x_{2m-1}),
// X_k = G_k + H'_k / (2 cos(pi (2k+1) / (2N))), X_{N-1-k} = G_k - (same).
// For M = 32 that is ~210 FP64 operations per transform against 33^2 for the
// matrix; the rounding error measured against extended precision is below
// the matrix form's.
template <int N>
struct Dct3 {
  __device__ static inline void run(const double (&x)[N], double (&X)[N], const double* lee) {
    constexpr int H = N / 2;
    double xe[H], z[H], G[H], Hh[H];
#pragma unroll
    for (int m = 0; m < H; ++m) {
      xe[m] = x[2 * m];
      z[m] = m > 0 ? x[2 * m + 1] + x[2 * m - 1] : x[1];
    }
    Dct3<H>::run(xe, G, lee);
    Dct3<H>::run(z, Hh, lee);
#pragma unroll
    for (int k = 0; k < H; ++k) {
      const double h = Hh[k] * lee[H - 1 + k];  // 1 / (2 cos(pi (2k+1) / (2N)))
      X[k] = G[k] + h;
      X[N - 1 - k] = G[k] - h;
    }
  }
};
template <>
struct Dct3<1> {
  __device__ static inline void run(const double (&x)[1], double (&X)[1], const double*) { X[0] = x[0]; }
};

template <int M>
struct Dct1 {
  __device__ static inline void run(const double (&s)[M + 1], double (&y)[M + 1], const double* lee) {
    constexpr int N = M / 2;
    double u[N + 1], v[N], ye[N + 1], yo[N];
    u[0] = s[0] + s[M];
    v[0] = s[0] - s[M];
#pragma unroll
    for (int l = 1; l < N; ++l) {
      u[l] = s[l] + s[M - l];
      v[l] = s[l] - s[M - l];
    }
    u[N] = s[N];
    Dct1<N>::run(u, ye, lee);
    Dct3<N>::run(v, yo, lee);
#pragma unroll
    for (int k = 0; k <= N; ++k) y[2 * k] = ye[k];
#pragma unroll
    for (int k = 0; k < N; ++k) y[2 * k + 1] = yo[k];
  }
};
template <>
struct Dct1<2> {
  __device__ static inline void run(const double (&s)[3], double (&y)[3], const double*) {
    const double a = s[0] + s[2];
    y[0] = a + s[1];
    y[1] = s[0] - s[2];
    y[2] = a - s[1];
  }
};

// Entries of the fast-drift table for even P = 2M: A_k = w_k cos(w_k dt) / P,
// B_k = w_k sin(w_k dt) / (w_k P) and C_k = -w_k w_k sin(w_k dt) / P per mode
// k = 0..M (w the mode weight above), then the Lee factors of every size N
// <= M/2 at [N/2 - 1 + k].
__host__ __device__ inline int fast_drift_doubles(int M) { return 3 * (M + 1) + M; }

// Free ring-polymer step of even P = 2M beads with the 1/2 kick before it
// (no PILE): each warp takes 16 coordinates of one trajectory, lanes 0-15
// transforming q and lanes 16-31 transforming p - dt/2 dV/dq of the same
// coordinates; the 2x2 mode update exchanges the partner's coefficient by a
// shuffle.  Block: 4 warps = 64 coordinates; grid (ceil(NC / 64), T).
template <int M>
__global__ void __launch_bounds__(128) split_drift_fast_kernel(SplitParams s) {
  constexpr int P = 2 * M;
  constexpr int kTab = 3 * (M + 1) + M;
  __shared__ double tab[kTab];
  for (int i = threadIdx.x; i < kTab; i += blockDim.x) tab[i] = s.fdrift[i];
  __syncthreads();
  const double* lee = tab + 3 * (M + 1);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int NC = s.NC, t = blockIdx.y;
  const int c = (blockIdx.x * 4 + warp) * 16 + (lane & 15);
  const bool isp = lane >= 16, active = c < NC;
  const int atom = active ? c / 3 : 0;
  const size_t tb = (size_t)t * P * NC + c;
  // q enters relative to its bead-0 value: the constant vector is mode 0
  // (K1 keeps it, K2 drops it), and the transforms then round on bead
  // spreads instead of absolute positions
  double x[M + 1], shift = 0.0;
#pragma unroll
  for (int l = 0; l <= M; ++l) x[l] = 0.0;
  if (active) {
    const double* src = isp ? s.p : s.q;
    const double hdt = isp ? s.half_dt : 0.0;
    if (!isp) shift = src[tb];
#pragma unroll
    for (int j = 0; j < P; ++j) {
      const size_t g = tb + (size_t)j * NC;
      const double v = fma(-hdt, s.f[g], src[g]) - shift;
      x[j <= M ? j : P - j] += v;
    }
  }
  double X[M + 1];
  Dct1<M>::run(x, X, lee);
  // q' = A q + B p / m (lanes 0-15), p' = A p + C m q (lanes 16-31)
  const double msc = isp ? s.mass[atom] : s.inv_mass[atom];
  const double* coef = tab + (isp ? 2 : 1) * (M + 1);
#pragma unroll
  for (int k = 0; k <= M; ++k) {
    const double other = __shfl_xor_sync(0xffffffffu, X[k], 16);
    X[k] = fma(coef[k] * msc, other, tab[k] * X[k]);
  }
  Dct1<M>::run(X, x, lee);
  if (!active) return;
  double* dst = isp ? s.p : s.q;
#pragma unroll
  for (int j = 0; j <= M; ++j) {
    const double y = x[j] + shift;
    dst[tb + (size_t)j * NC] = y;
    if (j > 0 && j < M) dst[tb + (size_t)(P - j) * NC] = y;
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
      normal_pair(s.seed, traj, (uint32_t)((c0 + c) / 2), (uint32_t)j, (uint32_t)istep, TAG_ANDERSEN, z0, z1);
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
// the potential energy summed over beads, as three kernels:
//   split_moments_kernel  grid (S, T): slice g of trajectory t's (bead, atom)
//                         items -> 15 moment sums (sum w v, sum w x,
//                         sum w x cross v, sum w x x^T), the bead energies
//                         (slice 0), the NaN bits; fixed-order block sums
//   split_solve_kernel    one thread per trajectory: the S partials summed in
//                         order, epot, status, and the 3x3 system for the
//                         angular velocity (Gauss-Jordan, full pivoting)
//   split_apply_kernel    every item: p <- m (v - vt - va x (x - xt)),
//                         evaluated as p - m (b + va x x), b = vt - va x xt
// The second moments about Caracal's rotation centre xt come from the raw
// ones by the parallel-axis identity C = S - xt Sx^T - Sx xt^T + W xt xt^T,
// W = sum w.  Traffic: q and p read twice, p written once.
constexpr int kMomentThreads = 256;
constexpr int kFinishSums = 16;   // 15 moments + sum of bead energies
constexpr int kMoveDoubles = 10;  // b = vt - va x xt, va, (unused), skip flag per trajectory

// slices per trajectory of split_moments_kernel: about 4 items per thread
__host__ __device__ inline int finish_slices(int items) {
  const int s = (items + 4 * kMomentThreads - 1) / (4 * kMomentThreads);
  return s < 1 ? 1 : (s > 16 ? 16 : s);
}

// Not NaN or infinite: exponent bits below all-ones (integer pipe only).
__device__ inline bool finite_bits(double x) { return (__double2hiint(x) & 0x7ff00000) != 0x7ff00000; }

// Moment sums of one (bead, atom) item.  On this GPU the FP64 pipe bounds the
// finish, so the sums use w v = p (momentum) and w x once: 21 FP64
// operations per item.
__device__ inline void finish_accumulate(const SplitParams& s, int a, const double (&q)[3], const double (&p)[3],
                                         double (&acc)[kFinishSums], int& status) {
  const double w = s.mass[a];
  const double wq[3] = {w * q[0], w * q[1], w * q[2]};
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    if (!finite_bits(q[d])) status |= CR_TRAJ_NONFINITE;
    acc[d] += p[d];
    acc[3 + d] += wq[d];
  }
  acc[6] = fma(q[1], p[2], fma(-q[2], p[1], acc[6]));
  acc[7] = fma(q[2], p[0], fma(-q[0], p[2], acc[7]));
  acc[8] = fma(q[0], p[1], fma(-q[1], p[0], acc[8]));
  acc[9] = fma(wq[0], q[0], acc[9]);
  acc[10] = fma(wq[0], q[1], acc[10]);
  acc[11] = fma(wq[0], q[2], acc[11]);
  acc[12] = fma(wq[1], q[1], acc[12]);
  acc[13] = fma(wq[1], q[2], acc[13]);
  acc[14] = fma(wq[2], q[2], acc[14]);
}

// Warp sum of 16 values per lane as a reduce-scatter butterfly: at each of
// the first four levels a lane keeps half of its values and adds the
// partner's copy of that half (8 + 4 + 2 + 1 FP64 adds instead of 16 x 5),
// then one exchange finishes.  Lane l returns the warp sum of value l >> 1.
// Fixed order: deterministic.
__device__ inline double warp_sum16(double (&v)[16], int lane) {
#pragma unroll
  for (int level = 0; level < 4; ++level) {
    const int half = 8 >> level;  // values kept per lane after this level
    const bool up = (lane >> (4 - level)) & 1;
#pragma unroll
    for (int j = 0; j < half; ++j) {
      const double keep = up ? v[half + j] : v[j];
      const double give = up ? v[j] : v[half + j];
      v[j] = keep + __shfl_xor_sync(0xffffffffu, give, 16 >> level);
    }
  }
  return v[0] + __shfl_xor_sync(0xffffffffu, v[0], 1);
}

__global__ void __launch_bounds__(kMomentThreads) split_moments_kernel(SplitParams s) {
  constexpr int kWarps = kMomentThreads / 32;
  __shared__ double wpart[kWarps][kFinishSums];
  __shared__ int wstat[kWarps];
  const int S = gridDim.x, g = blockIdx.x, t = blockIdx.y, P = s.P, N = s.N;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const size_t tb = (size_t)t * P * s.NC;
  const int items = P * N;
  const int lo = (int)((long long)items * g / S), hi = (int)((long long)items * (g + 1) / S);
  double acc[kFinishSums];
#pragma unroll
  for (int j = 0; j < kFinishSums; ++j) acc[j] = 0.0;
  int status = 0;
  for (int i = lo + threadIdx.x; i < hi; i += kMomentThreads) {
    double q[3], p[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      q[d] = s.q[tb + 3 * (size_t)i + d];
      p[d] = s.p[tb + 3 * (size_t)i + d];
    }
    finish_accumulate(s, i % N, q, p, acc, status);
  }
  if (g == 0)
    for (int j = threadIdx.x; j < P; j += kMomentThreads) acc[15] += s.V[(size_t)t * P + j];
  const double ws = warp_sum16(acc, lane);
  status = __reduce_or_sync(0xffffffffu, status);
  if ((lane & 1) == 0) wpart[warp][lane >> 1] = ws;
  if (lane == 0) wstat[warp] = status;
  __syncthreads();
  const size_t slot = (size_t)t * S + g;
  if (threadIdx.x < kFinishSums) {
    double v = 0.0;
    for (int w = 0; w < kWarps; ++w) v += wpart[w][threadIdx.x];
    s.fsum[slot * kFinishSums + threadIdx.x] = v;
  } else if (threadIdx.x == kFinishSums) {
    int st = 0;
    for (int w = 0; w < kWarps; ++w) st |= wstat[w];
    s.fstat[slot] = st;
  }
}

__global__ void split_solve_kernel(SplitParams s, int S) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= s.T) return;
  double tot[kFinishSums];
  int status = 0;
#pragma unroll
  for (int j = 0; j < kFinishSums; ++j) tot[j] = 0.0;
  for (int g = 0; g < S; ++g) {
    const size_t slot = (size_t)t * S + g;
#pragma unroll
    for (int j = 0; j < kFinishSums; ++j) tot[j] += s.fsum[slot * kFinishSums + j];
    status |= s.fstat[slot];
  }
  const bool shake_fail = s.constrain && s.shake_fail[t];
  if (shake_fail) status |= CR_TRAJ_SHAKE_FAILED;
  s.epot[t] = tot[15] + (shake_fail ? 100000.0 : 0.0);
  double* mv = s.fmove + (size_t)t * kMoveDoubles;
  if (s.transrot) {
    const double itm = 1.0 / s.totmass, tm = s.totmass, W = s.wsum;
    const double vt[3] = {tot[0] * itm, tot[1] * itm, tot[2] * itm};
    const double xt[3] = {tot[3] * itm, tot[4] * itm, tot[5] * itm};
    // centred second moments xx, xy, xz, yy, yz, zz
    const double cxx = tot[9] - 2.0 * xt[0] * tot[3] + W * xt[0] * xt[0];
    const double cxy = tot[10] - xt[0] * tot[4] - tot[3] * xt[1] + W * xt[0] * xt[1];
    const double cxz = tot[11] - xt[0] * tot[5] - tot[3] * xt[2] + W * xt[0] * xt[2];
    const double cyy = tot[12] - 2.0 * xt[1] * tot[4] + W * xt[1] * xt[1];
    const double cyz = tot[13] - xt[1] * tot[5] - tot[4] * xt[2] + W * xt[1] * xt[2];
    const double czz = tot[14] - 2.0 * xt[2] * tot[5] + W * xt[2] * xt[2];
    const double mang[3] = {tot[6] - (xt[1] * vt[2] - xt[2] * vt[1]) * tm,
                            tot[7] - (xt[2] * vt[0] - xt[0] * vt[2]) * tm,
                            tot[8] - (xt[0] * vt[1] - xt[1] * vt[0]) * tm};
    double ten[3][3] = {{cyy + czz, -cxy, -cxz}, {-cxy, cxx + czz, -cyz}, {-cxz, -cyz, cxx + cyy}};
    if (s.N <= 2) {
      ten[0][0] += 0.000001;
      ten[1][1] += 0.000001;
      ten[2][2] += 0.000001;
    }
    if (!invert3(ten)) {
      status |= CR_TRAJ_SINGULAR_INERTIA;
      mv[9] = 1.0;
    } else {
      double va[3];
      for (int a = 0; a < 3; ++a) va[a] = ten[a][0] * mang[0] + ten[a][1] * mang[1] + ten[a][2] * mang[2];
      // p <- m (v - vt - va x (x - xt)) = p - m (b + va x x), b = vt - va x xt
      mv[0] = vt[0] - (va[1] * xt[2] - va[2] * xt[1]);
      mv[1] = vt[1] - (va[2] * xt[0] - va[0] * xt[2]);
      mv[2] = vt[2] - (va[0] * xt[1] - va[1] * xt[0]);
      for (int a = 0; a < 3; ++a) mv[3 + a] = va[a];
      mv[9] = 0.0;
    }
  }
  if (status) s.status[t] |= status;
}

__global__ void __launch_bounds__(kMomentThreads) split_apply_kernel(SplitParams s) {
  const int N = s.N, items = s.P * N;
  const size_t total = (size_t)s.T * items;
  for (size_t idx = (size_t)blockIdx.x * kMomentThreads + threadIdx.x; idx < total;
       idx += (size_t)gridDim.x * kMomentThreads) {
    const int t = (int)(idx / items), a = (int)(idx % items) % N;
    const double* mv = s.fmove + (size_t)t * kMoveDoubles;
    if (mv[9] != 0.0) continue;
    const double* qq = s.q + 3 * idx;
    double* pp = s.p + 3 * idx;
    const double w = s.mass[a];
    const double u0 = mv[0] + fma(mv[4], qq[2], -mv[5] * qq[1]);
    const double u1 = mv[1] + fma(mv[5], qq[0], -mv[3] * qq[2]);
    const double u2 = mv[2] + fma(mv[3], qq[1], -mv[4] * qq[0]);
    pp[0] = fma(-w, u0, pp[0]);
    pp[1] = fma(-w, u1, pp[1]);
    pp[2] = fma(-w, u2, pp[2]);
  }
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

// NpT with the Berendsen barostat (src/verlet.f90:1111-1151), one block per
// trajectory, after the second half kick: the pressure from the beads' virial
// traces (the reference's kinetic stress tensor stays zero, so
// p = (1/V)(0 - tr W)/3 with V the box at the start of the step), the scale
// (1 + rate (p - p0))^(1/3) with rate = dt compress / taupres, then the box
// and every bead's coordinates scaled.  A non-finite scale reaches the
// coordinates and the step's NaN check.
struct NptStep {
  double* box;        // [T][3] edges, bohr
  double* press;      // [T][2] the step's pressure and the running sum, a.u.
  const double* vir;  // [T][P] virial trace per bead
  double pressure;    // target, a.u.
  double rate;        // dt compress / taupres
};
__global__ void split_berendsen_kernel(SplitParams s, NptStep n) {
  const int t = blockIdx.x;
  const int P = s.P, nq = P * s.NC;
  __shared__ double scale;
  if (threadIdx.x == 0) {
    double w = 0.0;
    for (int b = 0; b < P; ++b) w += n.vir[(size_t)t * P + b];
    double* L = n.box + 3 * (size_t)t;
    const double factor = 1.0 / (L[0] * L[1] * L[2]);
    const double pr = (factor * (0.0 - w)) / 3.0;
    const double sc = pow(1.0 + n.rate * (pr - n.pressure), 1.0 / 3.0);
    for (int k = 0; k < 3; ++k) L[k] = L[k] * sc;
    n.press[2 * (size_t)t] = pr;
    n.press[2 * (size_t)t + 1] += pr;  // press_avg (src/verlet.f90:1171-1173)
    scale = sc;
  }
  __syncthreads();
  double* q = s.q + (size_t)t * nq;
  for (int i = threadIdx.x; i < nq; i += blockDim.x) q[i] = q[i] * scale;
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
  normal_pair(seed, traj0 + (uint32_t)t, (uint32_t)ip, (uint32_t)k, 0u, TAG_BEAD_JITTER, z0, z1);
  const int c = 2 * ip;
  q[(size_t)b * NC + c] = q0[c] + sigma * z0;
  if (c + 1 < NC) q[(size_t)b * NC + c + 1] = q0[c + 1] + sigma * z1;
}

__global__ void split_init_momenta_kernel(int T, int P, int NC, uint32_t seed, uint32_t traj0, const double* sig,
                                          int zero, uint32_t draw, double* p) {
  const int npair = (NC + 1) / 2;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)T * P * npair) return;
  const int ip = (int)(idx % npair);
  const long long b = idx / npair;
  const int t = (int)(b / P), k = (int)(b % P);
  const int c = 2 * ip;
  double z0 = 0.0, z1 = 0.0;
  if (!zero) normal_pair(seed, traj0 + (uint32_t)t, (uint32_t)ip, (uint32_t)k, draw, TAG_INIT_MOMENTA, z0, z1);
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
