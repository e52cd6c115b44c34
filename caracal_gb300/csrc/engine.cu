// Host side of the GB300 RPMD engine and its C-ABI (include/caracal_gb300.h).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/caracal_gb300.h"
#include "cr_common.cuh"
#include "pes_runs.h"
#include "rpmd_kernel.cuh"
#include "host_util.h"
#include "qmdff_host.h"
#include "water_host.h"
#include "split.cuh"

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

#define CR_CUDA(call)                                                                 \
  do {                                                                                \
    cudaError_t _e = (call);                                                          \
    if (_e != cudaSuccess)                                                            \
      return fail(CR_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e));   \
  } while (0)

constexpr double kPi = 3.1415926535897932384626433832795029;

int next_pow2(int x) {
  int g = 1;
  while (g < x) g <<= 1;
  return g;
}

int pes_natoms(int pes) {
  switch (pes) {
    case CR_PES_H3:
    case CR_PES_BRH2: return 3;
    case CR_PES_CH4H: return 6;
    case CR_PES_CH4OH:
    case CR_PES_GEH4OH: return 7;
    case CR_PES_OH3: return 4;
    default: return -1;
  }
}

}  // namespace

int cr_set_error(int code, const std::string& msg) { return fail(code, msg); }

// ---------------------------------------------------------------------------
// Device kernels outside the step loop
// ---------------------------------------------------------------------------
namespace cr {

// q[t][k] = q0 + sigma * N(0,1) per coordinate (tag TAG_BEAD_JITTER, step 0)
template <int NC>
__global__ void init_positions_kernel(int T, int P, uint32_t seed, uint32_t traj0, const double* q0,
                                      double sigma, double* q) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= T * P) return;
  int t = idx / P, k = idx % P;
  double z[NC];
  normals_bead<NC>(seed, traj0 + t, (uint32_t)k, 0u, TAG_BEAD_JITTER, z);
#pragma unroll
  for (int c = 0; c < NC; ++c) q[(size_t)idx * NC + c] = q0[c] + sigma * z[c];
}

// mdinit Andersen draw: p = sqrt(m P / beta) N(0,1) (tag TAG_INIT_MOMENTA,
// counter `draw`: 0 for the first mdinit of a run, then one per later call)
template <int NC>
__global__ void init_momenta_kernel(int T, int P, uint32_t seed, uint32_t traj0, StepParams prm,
                                    int zero, uint32_t draw, double* p) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= T * P) return;
  int t = idx / P, k = idx % P;
  if (zero) {
#pragma unroll
    for (int c = 0; c < NC; ++c) p[(size_t)idx * NC + c] = 0.0;
    return;
  }
  double z[NC];
  normals_bead<NC>(seed, traj0 + t, (uint32_t)k, draw, TAG_INIT_MOMENTA, z);
#pragma unroll
  for (int c = 0; c < NC; ++c) p[(size_t)idx * NC + c] = z[c] * prm.sigma[c / 3];
}

// Recrossing children (src/recross.f90:540-561): q = parent ring polymer,
// p = Andersen draw keyed by the pair (trajectories 2i and 2i+1 share it),
// the odd member gets -p.
template <int NC>
__global__ void init_children_kernel(int T, int P, uint32_t seed, uint32_t traj0, StepParams prm,
                                     const double* qpar, double* q, double* p) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= T * P) return;
  int t = idx / P, k = idx % P;
  double z[NC];
  normals_bead<NC>(seed, traj0 + (uint32_t)(t & ~1), (uint32_t)k, 0u, TAG_CHILD_MOMENTA, z);
  const double sgn = (t & 1) ? -1.0 : 1.0;
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    q[(size_t)idx * NC + c] = qpar[(size_t)k * NC + c];
    p[(size_t)idx * NC + c] = sgn * (z[c] * prm.sigma[c / 3]);
  }
}

// Flux weight of each child (src/recross.f90:562-590): vs = dxi . sum_k p_k / m / P,
// fs = sqrt(sum dxi^2 / m / (2 pi beta)), w = vs / fs, wpos = vs > 0.
template <int N>
__global__ void child_flux_kernel(int T, int P, StepParams prm, const double* q, const double* p,
                                  double* w, int* wpos) {
  constexpr int NC = 3 * N;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  double c[NC], dxi[NC];
  for (int x = 0; x < NC; ++x) {
    double acc = 0.0;
    for (int k = 0; k < P; ++k) acc += q[((size_t)t * P + k) * NC + x];
    c[x] = acc / P;
  }
  xi_bimolec<N>(prm.xi, c, prm.mass, dxi);
  double vs = 0.0;
  for (int l = 0; l < 3; ++l)
    for (int m = 0; m < N; ++m)
      for (int o = 0; o < P; ++o) vs += dxi[3 * m + l] * p[((size_t)t * P + o) * NC + 3 * m + l] / prm.mass[m];
  vs = vs / P;
  double fs = 0.0;
  for (int l = 0; l < 3; ++l)
    for (int m = 0; m < N; ++m) fs += dxi[3 * m + l] * dxi[3 * m + l] / prm.mass[m];
  fs = sqrt(fs / (2.0 * 3.1415926535897932384 * prm.beta));
  w[t] = vs / fs;
  wpos[t] = vs > 0.0 ? 1 : 0;
}

// kappa(t) numerator and denominator, summed over trajectories in index order
// (deterministic): num[s] = sum_t w[t] [xi_t > 0 after step s+1].
__global__ void kappa_kernel(int T, int nsteps, int stride, const unsigned char* side, const double* w,
                             const int* wpos, double* num, double* denom) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < nsteps) {
    double acc = 0.0;
    for (int t = 0; t < T; ++t)
      if (side[(size_t)t * stride + s]) acc += w[t];
    num[s] = acc;
  } else if (s == nsteps) {
    double acc = 0.0;
    for (int t = 0; t < T; ++t)
      if (wpos[t]) acc += w[t];
    *denom = acc;
  }
}

// epot[t] = sum over beads of V[t][k]
__global__ void sum_beads_kernel(int T, int P, const double* V, double* epot) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  double s = 0.0;
  for (int k = 0; k < P; ++k) s += V[(size_t)t * P + k];
  epot[t] = s;
}

}  // namespace cr

// ---------------------------------------------------------------------------
// Engine
// ---------------------------------------------------------------------------
constexpr int kHostGroups = 8;  // most trajectory groups of the pipelined host-buffer step

struct cr_engine {
  cr_config cfg{};
  std::vector<double> mass;
  int N = 0, NC = 0, P = 0, T = 0, G = 1, H = 1;
  int block = 32, grid = 1;
  int tpb = 1;  // threads per bead of the persistent step kernel
  size_t smem = 0;
  int istep = 0;
  int launches = 0;
  float last_ms = 0.f;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double *d_q = nullptr, *d_p = nullptr, *d_f = nullptr, *d_epot = nullptr, *d_V = nullptr;
  double *d_pile = nullptr, *d_q0 = nullptr;
  double* d_circ = nullptr;  // [3][P] circulant propagator rows (nm_mode 1)
  int* d_status = nullptr;
  // recrossing children
  int xi_on = 0, side_cap = 0, side_step0 = 0;
  unsigned char* d_side = nullptr;
  double *d_w = nullptr, *d_kappa = nullptr, *d_qpar = nullptr;
  int* d_wpos = nullptr;
  cr::StepParams prm{};
  // large-molecule path (QMDFF): state in HBM, a captured graph per step
  cr_qmdff* ff = nullptr;
  cr_evb* evb = nullptr;               // dE-EVB of two force fields (ff = the first)
  cr_water* water = nullptr;           // flexible SPC water box
  double *d_V2 = nullptr, *d_f2 = nullptr;  // second force field's energies / gradients
  bool split = false;
  cr::SplitParams sp{};
  double *d_mass = nullptr, *d_inv_mass = nullptr, *d_sigma = nullptr, *d_ke = nullptr, *d_ko = nullptr;
  int* d_istep = nullptr;
  int h_istep = 0;
  double* d_vnh = nullptr;  // [T][4] Nose-Hoover chain velocities
  // constrained parent (analytic surfaces through the graph path)
  bool parent = false;
  int step_launches = 5;  // kernels per step of the graph path
  double *d_dxi = nullptr, *d_cq = nullptr;
  int* d_shake_fail = nullptr;
  size_t smem_drift = 0, smem_kick = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  bool split_ready = false;  // split_prepare done
  // umbrella windows (graph path, analytic surfaces)
  double *d_umb = nullptr;   // [T] centres, [T] force constants, [T] xsum, [T] xsum2, [T][nbins] histogram
  int* d_umb_flag = nullptr; // [2]: sampling switch, constant 0
  int umb_sampling = 0;      // host copy of the sampling switch
  double* d_fdrift = nullptr;  // split_drift_fast_kernel table (SplitParams::fdrift)
  int fast_M = 0;              // P / 2 when the drift runs by fast cosine transforms, else 0
  double *d_fsum = nullptr, *d_fmove = nullptr;  // split finish scratch (SplitParams::fsum, fmove)
  int* d_fstat = nullptr;
  // host-buffer step (cr_engine_step_host): trajectory groups whose copies in,
  // step and copies out overlap on separate streams
  cudaStream_t hs_in = nullptr, hs_out = nullptr, hs_c[kHostGroups] = {};
  // asynchronous trajectory dumps (cr_engine_run_dump_async): two snapshot
  // slots, each a device copy of q, p, epot and the status words, and its
  // page-locked host copy
  cudaStream_t ds = nullptr;
  char* d_snap[2] = {nullptr, nullptr};
  char* h_snap[2] = {nullptr, nullptr};
  cudaEvent_t ev_snap[2] = {nullptr, nullptr}, ev_copied[2] = {nullptr, nullptr};
  cudaEvent_t hev_in[kHostGroups] = {}, hev_c[kHostGroups] = {}, hev_out = nullptr;
  // NpT with the Berendsen barostat (periodic QMDFF): per-trajectory box
  // edges [T][3] (bohr), the last step's pressure [T] (a.u.) and the beads'
  // virial traces [T][P]
  bool npt = false;
  double npt_pressure = 0.0, npt_rate = 0.0;
  double *d_box = nullptr, *d_press = nullptr, *d_vir = nullptr;
};

namespace {

// Caracal's cosine transform C = sqrt(1/P) cos(2 pi j k / P) and the per-mode
// coefficients of the free ring polymer at unit mass (src/verlet.f90:405-429):
// pc = cos(w dt), pq = -w sin(w dt), pd = sin(w dt) / w (mode 0: 1, 0, dt).
void mode_tables(int P, double beta, double dt, std::vector<double>& C, std::vector<double> (&diag)[3]) {
  C.assign((size_t)P * P, 0.0);
  const double factor = std::sqrt(1.0 / P);
  for (int j = 0; j < P; ++j)
    for (int k = 0; k < P; ++k) {
      long long m = ((long long)j * k) % P;
      C[(size_t)j * P + k] = factor * std::cos(2.0 * kPi * (double)m / P);
    }
  std::vector<double> pc(P, 1.0), pq(P, 0.0), pd(P, dt);
  if (P > 1) {
    const double beta_n = beta / P, twown = 2.0 / beta_n, pi_n = kPi / P;
    for (int k = 1; k <= P / 2; ++k) {
      double wk = twown * std::sin(k * pi_n);
      double wt = wk * dt;
      pc[k] = std::cos(wt);
      pq[k] = -wk * std::sin(wt);
      pd[k] = std::sin(wt) / wk;
    }
    for (int k = 1; k <= (P - 1) / 2; ++k) {
      pc[P - k] = pc[k];
      pq[P - k] = pq[k];
      pd[P - k] = pd[k];
    }
  }
  diag[0] = pc;
  diag[1] = pq;
  diag[2] = pd;
}

// sum over modes k (of parity `par`: 0 even, 1 odd, -1 all) of C[r][k] D[k] C[k][l]
double kentry(const std::vector<double>& C, const std::vector<double>& D, int P, int r, int l, int par) {
  double s = 0.0;
  for (int k = 0; k < P; ++k)
    if (par < 0 || (k & 1) == par) s += C[(size_t)r * P + k] * D[k] * C[(size_t)k * P + l];
  return s;
}

// Parity-split propagator blocks (both step paths): for even P, Ke[w][r][l]
// (even modes, l < nu) and Ko[w][r][l] (odd modes, l < nv), r < nr; for odd P
// the unique rows of K (nr = nu = P/2+1, nv = 0).
// Orthonormal normal modes (nm_mode 1): K_w = O^T diag(D_w) O is circulant,
// K_w[j][l] = circ[w][(j - l) mod P] = (1/P) sum_k D_w[k] cos(2 pi k (j - l) / P)
// with Caracal's per-mode coefficients D (mode k and P - k share a frequency).
void build_circulant(int P, double beta, double dt, std::vector<double>& circ) {
  std::vector<double> C, diag[3];
  mode_tables(P, beta, dt, C, diag);
  circ.assign((size_t)3 * P, 0.0);
  for (int w = 0; w < 3; ++w)
    for (int d = 0; d < P; ++d) {
      double acc = 0.0;
      for (int k = 0; k < P; ++k) {
        const long long m = ((long long)k * d) % P;
        acc += diag[w][(size_t)k] * std::cos(2.0 * kPi * (double)m / P);
      }
      circ[(size_t)w * P + d] = acc / P;
    }
}

void build_split_propagator(int P, double beta, double dt, const cr::PropDims& d, std::vector<double>& ke,
                            std::vector<double>& ko) {
  std::vector<double> C, diag[3];
  mode_tables(P, beta, dt, C, diag);
  ke.assign((size_t)3 * d.nr * d.nu, 0.0);
  ko.assign((size_t)3 * d.nr * (d.nv > 0 ? d.nv : 1), 0.0);
  for (int w = 0; w < 3; ++w)
    for (int r = 0; r < d.nr; ++r) {
      for (int l = 0; l < d.nu; ++l)
        ke[((size_t)w * d.nr + r) * d.nu + l] = kentry(C, diag[w], P, r, l, d.split ? 0 : -1);
      for (int l = 0; l < d.nv; ++l) ko[((size_t)w * d.nr + r) * d.nv + l] = kentry(C, diag[w], P, r, l, 1);
    }
}

// Table of split_drift_fast_kernel for even P = 2M: per mode k = 0..M the
// weights w_k / P (w_0 = w_M = 1, else 2) times pc, pd, pq of mode_tables,
// then the factors 1 / (2 cos(pi (2k+1) / (2N))) of Lee's type-III recursion
// for N = 2, 4, ..., M/2 at [N/2 - 1 + k].
void build_fast_drift(int P, double beta, double dt, std::vector<double>& tab) {
  const int M = P / 2;
  std::vector<double> C, diag[3];
  mode_tables(P, beta, dt, C, diag);
  tab.assign((size_t)cr::fast_drift_doubles(M), 0.0);
  for (int k = 0; k <= M; ++k) {
    const double w = (k == 0 || k == M) ? 1.0 / P : 2.0 / P;
    tab[(size_t)k] = w * diag[0][(size_t)k];
    tab[(size_t)(M + 1) + k] = w * diag[2][(size_t)k];
    tab[(size_t)2 * (M + 1) + k] = w * diag[1][(size_t)k];
  }
  for (int N = 2; N <= M / 2; N *= 2)
    for (int k = 0; k < N / 2; ++k)
      tab[(size_t)3 * (M + 1) + N / 2 - 1 + k] = 1.0 / (2.0 * std::cos(kPi * (2 * k + 1) / (2.0 * N)));
}


// PILE-L circulant vectors a (friction) and b (noise) of O^T diag(c) O with O
// the orthonormal real normal-mode matrix; gamma_0 = 1/tau0, gamma_k = 2 w_k.
void build_pile(int P, double beta, double dt, double tau0, std::vector<double>& out) {
  std::vector<double> O((size_t)P * P);
  for (int k = 0; k < P; ++k)
    for (int j = 0; j < P; ++j) {
      long long m = ((long long)j * k) % P;
      double ang = 2.0 * kPi * (double)m / P, v;
      if (k == 0) v = std::sqrt(1.0 / P);
      else if (2 * k < P) v = std::sqrt(2.0 / P) * std::cos(ang);
      else if (2 * k == P) v = ((j % 2) == 0 ? 1.0 : -1.0) * std::sqrt(1.0 / P);
      else v = std::sqrt(2.0 / P) * std::sin(ang);
      O[(size_t)k * P + j] = v;
    }
  std::vector<double> c1(P), c2(P);
  const double twown = 2.0 * P / beta;
  for (int k = 0; k < P; ++k) {
    int kk = (2 * k <= P) ? k : P - k;
    double gamma = (k == 0) ? 1.0 / tau0 : 2.0 * twown * std::sin(kk * kPi / P);
    c1[k] = std::exp(-0.5 * dt * gamma);
    c2[k] = std::sqrt(1.0 - c1[k] * c1[k]);
  }
  out.assign((size_t)2 * P, 0.0);
  for (int m = 0; m < P; ++m) {
    double a = 0.0, b = 0.0;
    for (int k = 0; k < P; ++k) {
      a += O[(size_t)k * P + m] * c1[k] * O[(size_t)k * P + 0];
      b += O[(size_t)k * P + m] * c2[k] * O[(size_t)k * P + 0];
    }
    out[m] = a;
    out[P + m] = b;
  }
}

// Persistent run of nsteps steps.  dev_step: the first step index is read
// from the device counter, which a second launch then advances (so the pair
// can be replayed from a graph); the shared-memory limit is then set by the
// caller before the capture.
int launch_run(cr_engine* e, int nsteps, bool dev_step = false) {
  const cr::PesRuns* r = cr::pes_runs(e->cfg.pes);
  if (!r) return fail(CR_ERR_UNSUPPORTED, "PES not built");
  const bool mixed = e->cfg.precision == CR_PREC_MIXED;
  if (!dev_step) {
    CR_CUDA(r->set_smem(mixed, e->tpb, e->smem));
    CR_CUDA(r->run(e->prm, mixed, e->tpb, e->grid, e->block, e->smem, e->stream, e->istep, nsteps));
    return CR_OK;
  }
  cr::StepParams prm = e->prm;
  prm.istep_dev = e->d_istep;
  CR_CUDA(r->run(prm, mixed, e->tpb, e->grid, e->block, e->smem, e->stream, 0, nsteps));
  cr::advance_by_kernel<<<1, 1, 0, e->stream>>>(e->d_istep, nsteps);
  CR_CUDA(cudaGetLastError());
  return CR_OK;
}

// One step of trajectories [t0, t0 + tn) by the persistent kernel on stream
// st (the shared-memory limit is set by the caller): per-trajectory arrays
// offset, the noise key of trajectory t0, the step index from the host.
int launch_group(cr_engine* e, int t0, int tn, cudaStream_t st) {
  const cr::PesRuns* r = cr::pes_runs(e->cfg.pes);
  if (!r) return fail(CR_ERR_UNSUPPORTED, "PES not built");
  cr::StepParams prm = e->prm;
  const size_t off = (size_t)t0 * e->P * e->NC;
  prm.istep_dev = nullptr;
  prm.T = tn;
  prm.traj0 += (uint32_t)t0;
  prm.q += off;
  prm.p += off;
  prm.f += off;
  prm.epot += t0;
  prm.status += t0;
  prm.vnh += 4 * (size_t)t0;
  if (prm.side) prm.side += (size_t)t0 * prm.side_stride;
  const int groups = e->block / (e->G * e->tpb);
  CR_CUDA(r->run(prm, e->cfg.precision == CR_PREC_MIXED, e->tpb, (tn + groups - 1) / groups, e->block, e->smem, st,
                 e->istep, 1));
  return CR_OK;
}

int set_run_smem(cr_engine* e) {
  const cr::PesRuns* r = cr::pes_runs(e->cfg.pes);
  if (!r) return fail(CR_ERR_UNSUPPORTED, "PES not built");
  CR_CUDA(r->set_smem(e->cfg.precision == CR_PREC_MIXED, e->tpb, e->smem));
  return CR_OK;
}

int launch_forces(cr_engine* e) {
  const cr::PesRuns* r = cr::pes_runs(e->cfg.pes);
  if (!r) return fail(CR_ERR_UNSUPPORTED, "PES not built");
  CR_CUDA(r->egrad(e->cfg.precision == CR_PREC_MIXED, e->T * e->P, e->d_q, e->d_V, e->d_f, e->stream));
  cr::sum_beads_kernel<<<(e->T + 127) / 128, 128, 0, e->stream>>>(e->T, e->P, e->d_V, e->d_epot);
  CR_CUDA(cudaGetLastError());
  return CR_OK;
}

// Forces of the large-molecule path from an analytic surface (constrained
// parents and umbrella windows step through the graph path).
int egrad_launch(cr_engine* e, double* V, double* f) {
  const cr::PesRuns* r = cr::pes_runs(e->cfg.pes);
  if (!r) return fail(CR_ERR_UNSUPPORTED, "PES not built");
  CR_CUDA(r->egrad(e->cfg.precision == CR_PREC_MIXED, e->T * e->P, e->d_q, V, f, e->stream));
  return CR_OK;
}

// Forces of trajectories [t0, t0 + tn) on stream st (V, f: that range's
// outputs).  The analytic surfaces go through here only for constrained
// parents, which always cover every trajectory.
int split_forces_range(cr_engine* e, int t0, int tn, double* V, double* f, cudaStream_t st) {
  const size_t off = (size_t)t0 * e->P * e->NC;
  if (e->evb)
    return evb_launch(e->evb, e->d_q + off, tn * e->P, V, f, e->d_V2 + (size_t)t0 * e->P, e->d_f2 + off,
                      e->cfg.precision, st);
  if (e->ff && e->npt) {
    const QmdffNpt np{e->d_box + 3 * (size_t)t0, e->P, e->d_vir + (size_t)t0 * e->P};
    return qmdff_launch(e->ff, e->d_q + off, tn * e->P, V, f, e->cfg.precision, st, &np);
  }
  if (e->ff) return qmdff_launch(e->ff, e->d_q + off, tn * e->P, V, f, e->cfg.precision, st);
  if (e->water) return water_launch(e->water, e->d_q + off, tn * e->P, V, f, e->cfg.precision, st);
  if (t0 != 0 || tn != e->T || st != e->stream) return fail(CR_ERR_UNSUPPORTED, "analytic forces cover every trajectory");
  return egrad_launch(e, V, f);
}

int split_forces(cr_engine* e, double* V, double* f) { return split_forces_range(e, 0, e->T, V, f, e->stream); }

// SHAKE / RATTLE of the constrained parent (template on the atom count)
int parent_kernel(cr_engine* e, int which) {
  const int T = e->T;
  switch (e->N) {
    case 3:
      if (which == 0) cr::split_shake_kernel<3><<<T, 32, 0, e->stream>>>(e->sp);
      else if (which == 1) cr::split_rattle_kernel<3><<<T, cr::kFinishBlock, 0, e->stream>>>(e->sp);
      else cr::split_parent_init_kernel<3><<<(T + 63) / 64, 64, 0, e->stream>>>(e->sp);
      break;
    case 6:
      if (which == 0) cr::split_shake_kernel<6><<<T, 32, 0, e->stream>>>(e->sp);
      else if (which == 1) cr::split_rattle_kernel<6><<<T, cr::kFinishBlock, 0, e->stream>>>(e->sp);
      else cr::split_parent_init_kernel<6><<<(T + 63) / 64, 64, 0, e->stream>>>(e->sp);
      break;
    case 7:
      if (which == 0) cr::split_shake_kernel<7><<<T, 32, 0, e->stream>>>(e->sp);
      else if (which == 1) cr::split_rattle_kernel<7><<<T, cr::kFinishBlock, 0, e->stream>>>(e->sp);
      else cr::split_parent_init_kernel<7><<<(T + 63) / 64, 64, 0, e->stream>>>(e->sp);
      break;
    case 4:
      if (which == 0) cr::split_shake_kernel<4><<<T, 32, 0, e->stream>>>(e->sp);
      else if (which == 1) cr::split_rattle_kernel<4><<<T, cr::kFinishBlock, 0, e->stream>>>(e->sp);
      else cr::split_parent_init_kernel<4><<<(T + 63) / 64, 64, 0, e->stream>>>(e->sp);
      break;
    default: return fail(CR_ERR_UNSUPPORTED, "constrained parents are built for the analytic surfaces");
  }
  CR_CUDA(cudaGetLastError());
  return CR_OK;
}

// The engine's graph-path parameters restricted to trajectories
// [t0, t0 + tn): per-trajectory arrays offset, the noise key of trajectory t0.
cr::SplitParams split_params_range(const cr_engine* e, int t0, int tn) {
  cr::SplitParams s = e->sp;
  const size_t off = (size_t)t0 * e->P * e->NC;
  s.T = tn;
  s.traj0 += (uint32_t)t0;
  s.q += off;
  s.p += off;
  s.f += off;
  s.V += (size_t)t0 * e->P;
  s.epot += t0;
  s.status += t0;
  s.vnh += 4 * (size_t)t0;
  const int S = cr::finish_slices(e->P * e->N);
  s.fsum += (size_t)t0 * S * cr::kFinishSums;
  s.fstat += (size_t)t0 * S;
  s.fmove += (size_t)t0 * cr::kMoveDoubles;
  return s;
}

// The kernels of one step of the large-molecule path for the trajectories
// of s (s = split_params_range(e, t0, tn)) on stream st; the caller advances
// the device step counter.  Constrained parents and umbrella windows step
// every trajectory at once on e->stream.  *nl counts the launches.
int split_group_launches(cr_engine* e, const cr::SplitParams& s, int t0, int tn, cudaStream_t st, int* nl) {
  const bool whole = t0 == 0 && tn == e->T && st == e->stream;
  if ((e->parent || s.umbrella) && !whole)
    return fail(CR_ERR_UNSUPPORTED, "constrained parents and umbrella windows step every trajectory at once");
  const int cw = cr::split_chunk(e->P);
  const dim3 grid((e->NC + cw - 1) / cw, tn);
  // under the Berendsen barostat the reference applies no Nose-Hoover chain
  // (src/verlet.f90:189-208, 1088-1106)
  const bool nhc = e->cfg.thermostat == CR_THERMO_NHC && !e->npt;
  int n = 0;
  if (nhc) {
    cr::split_nhc_kernel<<<tn, cr::kFinishBlock, 0, st>>>(s);
    CR_CUDA(cudaGetLastError());
    ++n;
  }
  switch (e->fast_M) {
    case 4: cr::split_drift_fast_kernel<4><<<dim3((e->NC + 63) / 64, tn), 128, 0, st>>>(s); break;
    case 8: cr::split_drift_fast_kernel<8><<<dim3((e->NC + 63) / 64, tn), 128, 0, st>>>(s); break;
    case 16: cr::split_drift_fast_kernel<16><<<dim3((e->NC + 63) / 64, tn), 128, 0, st>>>(s); break;
    case 32: cr::split_drift_fast_kernel<32><<<dim3((e->NC + 63) / 64, tn), 128, 0, st>>>(s); break;
    default: cr::split_drift_kernel<<<grid, cr::kSplitBlock, e->smem_drift, st>>>(s);
  }
  CR_CUDA(cudaGetLastError());
  ++n;
  int rc;
  if (e->parent && (rc = parent_kernel(e, 0))) return rc;  // SHAKE (src/verlet.f90:746-757)
  rc = split_forces_range(e, t0, tn, s.V, s.f, st);
  if (rc) return rc;
  n += e->evb ? 3 : 1;
  if (s.umbrella) {  // src/verlet.f90:1043-1046
    switch (e->N) {
      case 3: cr::split_umbrella_kernel<3><<<tn, 64, 0, st>>>(s); break;
      case 6: cr::split_umbrella_kernel<6><<<tn, 64, 0, st>>>(s); break;
      case 7: cr::split_umbrella_kernel<7><<<tn, 64, 0, st>>>(s); break;
      case 4: cr::split_umbrella_kernel<4><<<tn, 64, 0, st>>>(s); break;
      default: return fail(CR_ERR_UNSUPPORTED, "umbrella windows are built for the analytic surfaces");
    }
    CR_CUDA(cudaGetLastError());
    ++n;
  }
  if (e->parent) {
    // 1/2 kick, RATTLE (src/verlet.f90:1080-1082), NHC, then Andersen / PILE
    cr::split_kick_kernel<<<grid, cr::kSplitBlock, 0, st>>>(s, 1);
    CR_CUDA(cudaGetLastError());
    if ((rc = parent_kernel(e, 1))) return rc;
    if (nhc) {
      cr::split_nhc_kernel<<<tn, cr::kFinishBlock, 0, st>>>(s);
      CR_CUDA(cudaGetLastError());
    }
    if (e->cfg.thermostat == CR_THERMO_ANDERSEN || e->cfg.thermostat == CR_THERMO_PILE) {
      cr::split_kick_kernel<<<grid, cr::kSplitBlock, e->smem_kick, st>>>(s, 2);
      CR_CUDA(cudaGetLastError());
    }
  } else {
    cr::split_kick_kernel<<<grid, cr::kSplitBlock, e->smem_kick, st>>>(s, 0);
    CR_CUDA(cudaGetLastError());
    ++n;
    if (nhc) {
      cr::split_nhc_kernel<<<tn, cr::kFinishBlock, 0, st>>>(s);
      CR_CUDA(cudaGetLastError());
      ++n;
    }
  }
  if (e->npt) {  // pressure and Berendsen scaling (src/verlet.f90:1111-1151)
    const cr::NptStep np{e->d_box + 3 * (size_t)t0, e->d_press + 2 * (size_t)t0, e->d_vir + (size_t)t0 * e->P,
                         e->npt_pressure, e->npt_rate};
    cr::split_berendsen_kernel<<<tn, 128, 0, st>>>(s, np);
    CR_CUDA(cudaGetLastError());
    ++n;
  }
  {
    // NaN check, transrot, epot: moments per slice, a solve per trajectory,
    // the momentum update per item
    const int S = cr::finish_slices(e->P * e->N);
    cr::split_moments_kernel<<<dim3(S, tn), cr::kMomentThreads, 0, st>>>(s);
    CR_CUDA(cudaGetLastError());
    cr::split_solve_kernel<<<(tn + 127) / 128, 128, 0, st>>>(s, S);
    CR_CUDA(cudaGetLastError());
    n += 2;
    if (s.transrot) {
      const long long items = (long long)tn * e->P * e->N;
      const int grid = (int)std::min<long long>((items + cr::kMomentThreads - 1) / cr::kMomentThreads, 152LL * 16);
      cr::split_apply_kernel<<<grid, cr::kMomentThreads, 0, st>>>(s);
      CR_CUDA(cudaGetLastError());
      ++n;
    }
  }
  if (nl) *nl += n;
  return CR_OK;
}

// One step of the large-molecule path as kernel launches on e->stream
// (recorded once into a CUDA graph).
int split_step_launches(cr_engine* e) {
  int rc = split_group_launches(e, e->sp, 0, e->T, e->stream, nullptr);
  if (rc) return rc;
  cr::split_advance_kernel<<<1, 1, 0, e->stream>>>(e->d_istep);
  CR_CUDA(cudaGetLastError());
  return CR_OK;
}

// Everything the graph path needs before its launches can be captured:
// shared-memory limits and the force kernel's autotuned variant.
int split_prepare(cr_engine* e) {
  if (e->split_ready) return CR_OK;
  CR_CUDA(cudaFuncSetAttribute(cr::split_drift_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)e->smem_drift));
  CR_CUDA(cudaFuncSetAttribute(cr::split_kick_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)e->smem_kick));
  // the force kernels set their shared-memory limits outside the capture
  int rc = CR_OK;
  if (e->evb) rc = evb_launch(e->evb, e->d_q, 0, e->d_V, e->d_f, e->d_V2, e->d_f2, e->cfg.precision, e->stream);
  else if (e->ff) rc = qmdff_launch(e->ff, e->d_q, 0, e->d_V, e->d_f, e->cfg.precision, e->stream);
  else if (e->water) rc = water_launch(e->water, e->d_q, 0, e->d_V, e->d_f, e->cfg.precision, e->stream);
  if (rc) return rc;
  // let the autotuner pick the force-kernel variant on this batch before it
  // is frozen into the graph; the gradient goes to scratch so f is untouched
  const size_t nall = (size_t)e->T * e->P * e->NC;
  double* scratch = nullptr;
  if (e->ff && cudaMalloc(&scratch, nall * sizeof(double)) == cudaSuccess) {
    rc = split_forces(e, e->d_V, scratch);
    cudaStreamSynchronize(e->stream);
    cudaFree(scratch);
    if (rc) return rc;
  }
  e->split_ready = true;
  return CR_OK;
}

int split_run(cr_engine* e, int nsteps) {
  if (!e->graph_exec) {
    int rc = split_prepare(e);
    if (rc) return rc;
    CR_CUDA(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
    rc = split_step_launches(e);
    cudaGraph_t g = nullptr;
    cudaError_t ce = cudaStreamEndCapture(e->stream, &g);
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (ce != cudaSuccess) return fail(CR_ERR_CUDA, std::string("stream capture: ") + cudaGetErrorString(ce));
    e->graph = g;
    size_t nodes = 0;
    CR_CUDA(cudaGraphGetNodes(e->graph, nullptr, &nodes));
    e->step_launches = (int)nodes;
    CR_CUDA(cudaGraphInstantiate(&e->graph_exec, e->graph, 0));
  }
  e->h_istep = e->istep;
  CR_CUDA(cudaMemcpyAsync(e->d_istep, &e->h_istep, sizeof(int), cudaMemcpyHostToDevice, e->stream));
  for (int n = 0; n < nsteps; ++n) CR_CUDA(cudaGraphLaunch(e->graph_exec, e->stream));
  return CR_OK;
}

int dispatch_run(cr_engine* e, int nsteps) {
  if (e->split) return split_run(e, nsteps);
  return launch_run(e, nsteps);
}

int dispatch_forces(cr_engine* e) {
  if (e->split) {
    int rc = split_forces(e, e->d_V, e->d_f);
    if (rc) return rc;
    cr::split_sum_beads_kernel<<<(e->T + 127) / 128, 128, 0, e->stream>>>(e->T, e->P, e->d_V, e->d_epot);
    CR_CUDA(cudaGetLastError());
    return CR_OK;
  }
  return launch_forces(e);
}

// Launch shape for `block` threads per block and `tpb` threads per bead
// (block a multiple of G tpb, at most 256): false if the surface has no such
// variant or the group scratch of block/(G tpb) trajectories does not fit.
bool set_launch_shape(cr_engine* e, int block, int tpb) {
  const cr::PesRuns* r = cr::pes_runs(e->cfg.pes);
  if (!r || (tpb != 1 && tpb != 2 && tpb != 4) || tpb > r->max_tpb) return false;
  const int GT = e->G * tpb;
  if (block < GT || block % GT || block > 256) return false;
  const size_t smem = cr::step_smem_doubles(e->P, e->G, e->NC, block / GT, tpb) * sizeof(double);
  if (smem > 200 * 1024) return false;
  e->block = block;
  e->tpb = tpb;
  e->grid = (e->T + block / GT - 1) / (block / GT);
  e->smem = smem;
  return true;
}

// Launch shape: a tiny batch is latency-bound, so it is spread one warp per
// SM; a large batch uses 128-thread blocks, shrunk until the shared memory
// fits; one thread per bead.
void choose_launch(cr_engine* e) {
  const int G = e->G;
  int sms = 152;
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long threads = (long long)e->T * G;
  int block = (threads <= (long long)sms * 128) ? 32 : 128;
  if (block < G) block = G;
  if (block > 256) block = 256;
  while (block > G && cr::step_smem_doubles(e->P, G, e->NC, block / G) * 8 > 200 * 1024) block /= 2;
  e->block = block;
  e->tpb = 1;
  const int groups = block / G;
  e->grid = (e->T + groups - 1) / groups;
  e->smem = cr::step_smem_doubles(e->P, G, e->NC, groups) * sizeof(double);
}

}  // namespace

// ---------------------------------------------------------------------------
// C-ABI
// ---------------------------------------------------------------------------
static int egrad_device_impl(int pes, const double* d_q, int npts, double* d_V, double* d_dVdq, int precision,
                             cudaStream_t s) {
  const cr::PesRuns* r = cr::pes_runs(pes);
  if (!r) return fail(CR_ERR_UNSUPPORTED, "PES not built");
  if (precision != CR_PREC_MIXED && precision != CR_PREC_FP64) return fail(CR_ERR_ARG, "unknown precision");
  CR_CUDA(r->egrad(precision == CR_PREC_MIXED, npts, d_q, d_V, d_dVdq, s));
  return CR_OK;
}

extern "C" int cr_egrad_device(int pes, const double* d_q, int npts, double* d_V, double* d_dVdq,
                               int precision, void* stream);

// Host-pointer egrad for any PES: stage through device buffers, one launch.
static int egrad_host(int pes, int natoms_expected, const double* q, int natoms, int nbeads, double* V,
                      double* dVdq, int* info) {
  if (info) *info = 0;
  if (natoms != natoms_expected) return fail(CR_ERR_ARG, "natoms does not match the PES");
  if (nbeads < 0 || (nbeads > 0 && (!q || !V || !dVdq))) return fail(CR_ERR_ARG, "bad egrad arguments");
  if (nbeads == 0) return CR_OK;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(CR_ERR_NO_DEVICE, "no CUDA device");
  const size_t nq = (size_t)3 * natoms * nbeads;
  double *d_q = nullptr, *d_V = nullptr, *d_g = nullptr;
  CR_CUDA(cudaMalloc(&d_q, nq * sizeof(double)));
  cudaError_t e1 = cudaMalloc(&d_V, (size_t)nbeads * sizeof(double));
  cudaError_t e2 = cudaMalloc(&d_g, nq * sizeof(double));
  int rc = CR_OK;
  if (e1 != cudaSuccess || e2 != cudaSuccess) {
    rc = fail(CR_ERR_CUDA, "cudaMalloc failed in egrad");
  } else if (cudaMemcpy(d_q, q, nq * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) {
    rc = fail(CR_ERR_CUDA, "copy of q failed");
  } else if ((rc = cr_egrad_device(pes, d_q, nbeads, d_V, d_g, CR_PREC_FP64, nullptr)) == CR_OK) {
    if (cudaMemcpy(V, d_V, (size_t)nbeads * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(dVdq, d_g, nq * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = fail(CR_ERR_CUDA, "copy of results failed");
  }
  cudaFree(d_q);
  cudaFree(d_V);
  cudaFree(d_g);
  return rc;
}

extern "C" {

const char* cr_error_string(int code) {
  switch (code) {
    case CR_OK: return "ok";
    case CR_ERR_ARG: return "invalid argument";
    case CR_ERR_CUDA: return "CUDA runtime error";
    case CR_ERR_NO_DEVICE: return "no CUDA device";
    case CR_ERR_UNSUPPORTED: return "unsupported configuration";
    case CR_ERR_TRAJECTORY: return "trajectory became non-finite";
    case CR_ERR_IO: return "I/O error";
    default: return "unknown status";
  }
}

int cr_last_error_detail(char* buf, int len) {
  if (!buf || len <= 0) return CR_ERR_ARG;
  std::snprintf(buf, (size_t)len, "%s", g_last_error.c_str());
  return CR_OK;
}

int cr_device_count(int* n) {
  if (!n) return fail(CR_ERR_ARG, "n is NULL");
  int c = 0;
  cudaError_t err = cudaGetDeviceCount(&c);
  if (err != cudaSuccess) {
    *n = 0;
    return fail(CR_ERR_NO_DEVICE, cudaGetErrorString(err));
  }
  *n = c;
  return CR_OK;
}

int cr_egrad_device(int pes, const double* d_q, int npts, double* d_V, double* d_dVdq, int precision,
                    void* stream) {
  if (npts < 0 || (npts > 0 && (!d_q || !d_V || !d_dVdq))) return fail(CR_ERR_ARG, "bad egrad arguments");
  if (npts == 0) return CR_OK;
  cudaStream_t s = (cudaStream_t)stream;
  return egrad_device_impl(pes, d_q, npts, d_V, d_dVdq, precision, s);
}

int cr_egrad_h3_device(const double* d_q, int npts, double* d_V, double* d_dVdq, int precision,
                       void* stream) {
  return cr_egrad_device(CR_PES_H3, d_q, npts, d_V, d_dVdq, precision, stream);
}

int cr_egrad_ch4h(const double* q, int natoms, int nbeads, double* V, double* dVdq, int* info) {
  return egrad_host(CR_PES_CH4H, 6, q, natoms, nbeads, V, dVdq, info);
}

int cr_initialize_ch4h(void) { return CR_OK; }

int cr_egrad_ch4oh(const double* q, int natoms, int nbeads, double* V, double* dVdq, int* info) {
  return egrad_host(CR_PES_CH4OH, 7, q, natoms, nbeads, V, dVdq, info);
}

int cr_initialize_ch4oh(void) { return CR_OK; }

int cr_egrad_geh4oh(const double* q, int natoms, int nbeads, double* V, double* dVdq, int* info) {
  return egrad_host(CR_PES_GEH4OH, 7, q, natoms, nbeads, V, dVdq, info);
}

int cr_initialize_geh4oh(void) { return CR_OK; }

int cr_egrad_brh2(const double* q, int natoms, int nbeads, double* V, double* dVdq, int* info) {
  return egrad_host(CR_PES_BRH2, 3, q, natoms, nbeads, V, dVdq, info);
}

int cr_initialize_brh2(void) { return CR_OK; }

int cr_egrad_oh3(const double* q, int natoms, int nbeads, double* V, double* dVdq, int* info) {
  return egrad_host(CR_PES_OH3, 4, q, natoms, nbeads, V, dVdq, info);
}

int cr_egrad_h3(const double* q, int natoms, int nbeads, double* V, double* dVdq, int* info) {
  if (info) *info = 0;
  if (natoms != 3) return fail(CR_ERR_ARG, "egrad_h3 needs natoms = 3");
  if (nbeads < 0 || (nbeads > 0 && (!q || !V || !dVdq))) return fail(CR_ERR_ARG, "bad egrad_h3 arguments");
  if (nbeads == 0) return CR_OK;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(CR_ERR_NO_DEVICE, "no CUDA device");
  const size_t nq = (size_t)9 * nbeads;
  double *d_q = nullptr, *d_V = nullptr, *d_g = nullptr;
  CR_CUDA(cudaMalloc(&d_q, nq * sizeof(double)));
  cudaError_t e1 = cudaMalloc(&d_V, (size_t)nbeads * sizeof(double));
  cudaError_t e2 = cudaMalloc(&d_g, nq * sizeof(double));
  int rc = CR_OK;
  if (e1 != cudaSuccess || e2 != cudaSuccess) {
    rc = fail(CR_ERR_CUDA, "cudaMalloc failed in cr_egrad_h3");
  } else if (cudaMemcpy(d_q, q, nq * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) {
    rc = fail(CR_ERR_CUDA, "copy of q failed");
  } else if ((rc = cr_egrad_h3_device(d_q, nbeads, d_V, d_g, CR_PREC_FP64, nullptr)) == CR_OK) {
    if (cudaMemcpy(V, d_V, (size_t)nbeads * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(dVdq, d_g, nq * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = fail(CR_ERR_CUDA, "copy of results failed");
  }
  cudaFree(d_q);
  cudaFree(d_V);
  cudaFree(d_g);
  return rc;
}

}  // extern "C"

// Validation and set-up shared by both engine paths; ff != NULL selects the
// large-molecule (QMDFF) path.
static int engine_create(const cr_config* cfg, cr_qmdff* ff, cr_evb* evb, cr_water* water, cr_engine** out) {
  if (!cfg || !out) return fail(CR_ERR_ARG, "NULL argument");
  *out = nullptr;
  int N = -1;
  if (water) {
    if (cfg->pes != CR_PES_WATER) return fail(CR_ERR_ARG, "cr_engine_create_water needs pes = CR_PES_WATER");
    N = water->dev.n;
  } else if (evb) {
    if (cfg->pes != CR_PES_EVB) return fail(CR_ERR_ARG, "cr_engine_create_evb needs pes = CR_PES_EVB");
    ff = evb_first(evb);
    N = ff->n;
  } else if (ff) {
    if (cfg->pes != CR_PES_QMDFF) return fail(CR_ERR_ARG, "cr_engine_create_qmdff needs pes = CR_PES_QMDFF");
    N = ff->n;
  } else {
    if (cfg->pes == CR_PES_QMDFF || cfg->pes == CR_PES_EVB || cfg->pes == CR_PES_WATER)
      return fail(CR_ERR_ARG, "force-field engines are created with cr_engine_create_qmdff / _evb / _water");
    N = pes_natoms(cfg->pes);
    if (N < 0) return fail(CR_ERR_UNSUPPORTED, "PES not available in this engine");
  }
  if (cfg->natoms != N) return fail(CR_ERR_ARG, "natoms does not match the PES");
  if (cfg->nbeads < 1 || cfg->nbeads > cr::kMaxBeads) return fail(CR_ERR_ARG, "nbeads must be 1..128");
  if (cfg->ntraj < 1) return fail(CR_ERR_ARG, "ntraj must be >= 1");
  if ((ff || water) && (long long)cfg->ntraj * cfg->nbeads > (1LL << 26))
    return fail(CR_ERR_ARG, "ntraj * nbeads must be <= 2^26 on the force-field path");
  if (!(cfg->dt > 0.0)) return fail(CR_ERR_ARG, "dt must be > 0");
  if (cfg->thermostat == CR_THERMO_NHC && !(cfg->nose_q > 0.0 && std::isfinite(cfg->nose_q)))
    return fail(CR_ERR_ARG, "the Nose-Hoover chain needs nose_q > 0");
  if (cfg->thermostat != CR_THERMO_NONE && cfg->thermostat != CR_THERMO_ANDERSEN &&
      cfg->thermostat != CR_THERMO_NHC && cfg->thermostat != CR_THERMO_PILE)
    return fail(CR_ERR_ARG, "unknown thermostat");
  if (cfg->precision != CR_PREC_FP64 && cfg->precision != CR_PREC_MIXED)
    return fail(CR_ERR_ARG, "unknown precision");
  if (cfg->nm_mode != 0 && cfg->nm_mode != 1) return fail(CR_ERR_ARG, "nm_mode must be 0 or 1");
  // P > 1 needs a finite beta for the free ring-polymer frequencies.  Caracal's
  // dynamic.x in NVE sets kelvin = 0 (src/dynamic.f90:338), making beta = +Inf
  // and the P > 1 propagator 0/0; the engine refuses that instead.
  if (cfg->nbeads > 1 && !(cfg->beta > 0.0 && std::isfinite(cfg->beta)))
    return fail(CR_ERR_ARG, "nbeads > 1 needs a finite temperature (beta)");
  if (cfg->thermostat != CR_THERMO_NONE && !(cfg->beta > 0.0 && std::isfinite(cfg->beta)))
    return fail(CR_ERR_ARG, "a thermostat needs a finite temperature (beta)");
  if (cfg->thermostat == CR_THERMO_ANDERSEN && cfg->andersen_step < 1)
    return fail(CR_ERR_ARG, "andersen_step must be >= 1");
  if (cfg->thermostat == CR_THERMO_PILE && !(cfg->pile_tau0 > 0.0))
    return fail(CR_ERR_ARG, "PILE needs tau0 > 0");
  if (!cfg->mass) return fail(CR_ERR_ARG, "mass is NULL");
  for (int i = 0; i < N; ++i)
    if (!(cfg->mass[i] > 0.0)) return fail(CR_ERR_ARG, "masses must be > 0");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(CR_ERR_NO_DEVICE, "no CUDA device");

  cr_engine* e = new cr_engine();
  e->cfg = *cfg;
  e->mass.assign(cfg->mass, cfg->mass + N);
  e->cfg.mass = e->mass.data();
  e->ff = ff;
  e->evb = evb;
  e->water = water;
  e->split = ff != nullptr || water != nullptr;
  e->N = N;
  e->NC = 3 * N;
  e->P = cfg->nbeads;
  e->T = cfg->ntraj;
  e->G = next_pow2(e->P);
  e->H = e->P / 2 + 1;
  if (!e->split) choose_launch(e);

  auto cleanup_fail = [&](int code) {
    cr_engine_destroy(e);
    return code;
  };
  const size_t nall = (size_t)e->T * e->P * e->NC;
  if (cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&e->ev0) != cudaSuccess || cudaEventCreate(&e->ev1) != cudaSuccess)
    return cleanup_fail(fail(CR_ERR_CUDA, "stream/event creation failed"));
  if (cudaMalloc(&e->d_q, nall * 8) != cudaSuccess || cudaMalloc(&e->d_p, nall * 8) != cudaSuccess ||
      cudaMalloc(&e->d_f, nall * 8) != cudaSuccess ||
      cudaMalloc(&e->d_epot, (size_t)e->T * 8) != cudaSuccess ||
      cudaMalloc(&e->d_V, (size_t)e->T * e->P * 8) != cudaSuccess ||
      cudaMalloc(&e->d_status, (size_t)e->T * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&e->d_q0, (size_t)e->NC * 8) != cudaSuccess)
    return cleanup_fail(fail(CR_ERR_CUDA, "device allocation of the state failed"));
  if (evb && (cudaMalloc(&e->d_V2, (size_t)e->T * e->P * 8) != cudaSuccess ||
              cudaMalloc(&e->d_f2, nall * 8) != cudaSuccess))
    return cleanup_fail(fail(CR_ERR_CUDA, "device allocation of the EVB buffers failed"));
  cudaMemsetAsync(e->d_q, 0, nall * 8, e->stream);
  cudaMemsetAsync(e->d_p, 0, nall * 8, e->stream);
  cudaMemsetAsync(e->d_f, 0, nall * 8, e->stream);
  cudaMemsetAsync(e->d_V, 0, (size_t)e->T * e->P * 8, e->stream);
  cudaMemsetAsync(e->d_status, 0, (size_t)e->T * sizeof(int), e->stream);

  const cr::PropDims pd = cr::prop_dims(e->P);
  std::vector<double> ke, ko, pile;
  build_split_propagator(e->P, cfg->beta, cfg->dt, pd, ke, ko);
  if (cfg->thermostat == CR_THERMO_PILE) build_pile(e->P, cfg->beta, cfg->dt, cfg->pile_tau0, pile);
  else pile.assign((size_t)2 * e->P, 0.0);
  std::vector<double> circ;
  if (cfg->nm_mode == 1) build_circulant(e->P, cfg->beta, cfg->dt, circ);
  else circ.assign((size_t)3 * e->P, 0.0);
  if (cudaMalloc(&e->d_ke, ke.size() * 8) != cudaSuccess || cudaMalloc(&e->d_ko, ko.size() * 8) != cudaSuccess ||
      cudaMalloc(&e->d_pile, pile.size() * 8) != cudaSuccess || cudaMalloc(&e->d_circ, circ.size() * 8) != cudaSuccess)
    return cleanup_fail(fail(CR_ERR_CUDA, "device allocation of the tables failed"));
  if (cudaMemcpyAsync(e->d_ke, ke.data(), ke.size() * 8, cudaMemcpyHostToDevice, e->stream) != cudaSuccess ||
      cudaMemcpyAsync(e->d_ko, ko.data(), ko.size() * 8, cudaMemcpyHostToDevice, e->stream) != cudaSuccess ||
      cudaMemcpyAsync(e->d_pile, pile.data(), pile.size() * 8, cudaMemcpyHostToDevice, e->stream) != cudaSuccess ||
      cudaMemcpyAsync(e->d_circ, circ.data(), circ.size() * 8, cudaMemcpyHostToDevice, e->stream) != cudaSuccess ||
      cudaStreamSynchronize(e->stream) != cudaSuccess)
    return cleanup_fail(fail(CR_ERR_CUDA, "upload of the tables failed"));

  // Nose-Hoover chain constants (src/mdinit.f90:128-147, src/nhc.f90:47-54)
  cr::NhcParams nhc{};
  if (cfg->thermostat == CR_THERMO_NHC) {
    const double kB = 0.316679e-5;  // src/dynamic.f90:79
    const double kelvin = 1.0 / (cfg->beta * kB);
    const double qterm = kB * kelvin * cfg->nose_q * cfg->nose_q;
    nhc.nfree = 3 * N;
    nhc.qnh[0] = (double)nhc.nfree * qterm;
    nhc.qnh[1] = nhc.qnh[2] = nhc.qnh[3] = qterm;
    nhc.ekt = (double)(1.380649E-23f / 4.3597447E-18f) * kelvin;
    nhc.dtc = cfg->dt / 5.0;
    nhc.w[0] = 1.0 / (2.0 - std::pow(2.0, 1.0 / 3.0));
    nhc.w[1] = 1.0 - 2.0 * nhc.w[0];
    nhc.w[2] = nhc.w[0];
  }
  if (cudaMalloc(&e->d_vnh, (size_t)e->T * 4 * sizeof(double)) != cudaSuccess ||
      cudaMemset(e->d_vnh, 0, (size_t)e->T * 4 * sizeof(double)) != cudaSuccess)
    return cleanup_fail(fail(CR_ERR_CUDA, "device allocation of the chain state failed"));

  double tm = 0.0;  // src/transrot.f90:72-79
  for (int i = 0; i < N; ++i)
    for (int k = 0; k < e->P; ++k) tm = tm + e->mass[i];
  const double totmass = tm * e->P;
  std::vector<double> sig((size_t)N), inv((size_t)N);
  for (int i = 0; i < N; ++i) {
    inv[(size_t)i] = 1.0 / e->mass[i];
    sig[(size_t)i] = (cfg->beta > 0.0 && std::isfinite(cfg->beta)) ? std::sqrt(e->mass[i] / (cfg->beta / e->P)) : 0.0;
  }

  {
    // graph-path parameters: always set up (a constrained parent of an
    // analytic surface also steps through the graph path)
    cr::SplitParams& s = e->sp;
    s.M = pd.M;
    s.split = pd.split;
    s.nr = pd.nr;
    s.nu = pd.nu;
    s.nv = pd.nv;
    s.su = pd.su;
    s.sv = pd.sv;
    if (cudaMalloc(&e->d_mass, (size_t)N * 8) != cudaSuccess || cudaMalloc(&e->d_inv_mass, (size_t)N * 8) != cudaSuccess ||
        cudaMalloc(&e->d_sigma, (size_t)N * 8) != cudaSuccess || cudaMalloc(&e->d_istep, sizeof(int)) != cudaSuccess)
      return cleanup_fail(fail(CR_ERR_CUDA, "device allocation of the split tables failed"));
    if (cudaMemcpy(e->d_mass, e->mass.data(), (size_t)N * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(e->d_inv_mass, inv.data(), (size_t)N * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(e->d_sigma, sig.data(), (size_t)N * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(e->d_istep, 0, sizeof(int)) != cudaSuccess)
      return cleanup_fail(fail(CR_ERR_CUDA, "upload of the split tables failed"));
    const size_t nsl = (size_t)e->T * cr::finish_slices(e->P * N);
    if (cudaMalloc(&e->d_fsum, nsl * cr::kFinishSums * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&e->d_fstat, nsl * sizeof(int)) != cudaSuccess ||
        cudaMalloc(&e->d_fmove, (size_t)e->T * cr::kMoveDoubles * sizeof(double)) != cudaSuccess)
      return cleanup_fail(fail(CR_ERR_CUDA, "device allocation of the finish scratch failed"));
    // the free ring polymer by fast cosine transforms where P is 8..64, a
    // power of two, and no PILE half step runs inside the drift
    const int P = e->P;
    if (pd.split && P >= 8 && P <= 64 && (P & (P - 1)) == 0 && cfg->thermostat != CR_THERMO_PILE &&
        cfg->nm_mode == 0) {
      std::vector<double> tab;
      build_fast_drift(P, cfg->beta, cfg->dt, tab);
      if (cudaMalloc(&e->d_fdrift, tab.size() * 8) != cudaSuccess ||
          cudaMemcpy(e->d_fdrift, tab.data(), tab.size() * 8, cudaMemcpyHostToDevice) != cudaSuccess)
        return cleanup_fail(fail(CR_ERR_CUDA, "upload of the fast drift table failed"));
      e->fast_M = P / 2;
    }
    s.T = e->T;
    s.P = e->P;
    s.N = N;
    s.NC = e->NC;
    s.nm_mode = cfg->nm_mode;
    s.circ = e->d_circ;
    s.thermostat = cfg->thermostat;
    s.andersen_step = cfg->andersen_step > 0 ? cfg->andersen_step : 1;
    s.transrot = cfg->transrot ? 1 : 0;
    s.seed = cfg->seed;
    s.traj0 = cfg->traj0;
    s.half_dt = 0.5 * cfg->dt;
    s.totmass = totmass;
    s.wsum = tm;
    s.mass = e->d_mass;
    s.inv_mass = e->d_inv_mass;
    s.sigma = e->d_sigma;
    s.ke = e->d_ke;
    s.ko = e->d_ko;
    s.pile = e->d_pile;
    s.q = e->d_q;
    s.p = e->d_p;
    s.f = e->d_f;
    s.V = e->d_V;
    s.epot = e->d_epot;
    s.status = e->d_status;
    s.istep = e->d_istep;
    s.nhc = nhc;
    s.vnh = e->d_vnh;
    s.fsum = e->d_fsum;
    s.fdrift = e->d_fdrift;
    s.fstat = e->d_fstat;
    s.fmove = e->d_fmove;
    const bool pl = cfg->thermostat == CR_THERMO_PILE;
    const int cw = cr::split_chunk(e->P), sp1 = e->P + 1;
    e->smem_drift = cr::split_smem_doubles(s, pl) * sizeof(double);
    e->smem_kick = pl ? ((size_t)3 * cw * sp1 + 2 * (size_t)e->P) * sizeof(double) : 0;
    if (e->split && e->smem_drift > 200 * 1024)
      return cleanup_fail(fail(CR_ERR_UNSUPPORTED, "bead count too large for the split path"));
    if (e->split) {
      e->block = cr::kSplitBlock;
      e->grid = ((e->NC + cw - 1) / cw) * e->T;
      e->smem = e->smem_drift;
      *out = e;
      return CR_OK;
    }
  }
  if (N > cr::kMaxAtoms) return cleanup_fail(fail(CR_ERR_UNSUPPORTED, "too many atoms for the persistent kernel"));

  cr::StepParams& s = e->prm;
  s.T = e->T;
  s.P = e->P;
  s.G = e->G;
  s.H = e->H;
  s.thermostat = cfg->thermostat;
  s.andersen_step = cfg->andersen_step > 0 ? cfg->andersen_step : 1;
  s.transrot = cfg->transrot ? 1 : 0;
  s.seed = cfg->seed;
  s.traj0 = cfg->traj0;
  s.dt = cfg->dt;
  s.half_dt = 0.5 * cfg->dt;
  s.beta = cfg->beta;
  s.totmass = totmass;
  for (int i = 0; i < cr::kMaxAtoms; ++i) {
    double m = i < N ? e->mass[i] : 1.0;
    s.mass[i] = m;
    s.inv_mass[i] = 1.0 / m;
    s.sigma[i] = i < N ? sig[(size_t)i] : 0.0;
  }
  s.nhc = nhc;
  s.vnh = e->d_vnh;
  s.pd = pd;
  s.pow2_P = (e->P & (e->P - 1)) == 0 ? 1 : 0;
  s.inv_P = 1.0 / e->P;
  s.nm_mode = cfg->nm_mode;
  s.circ = e->d_circ;
  s.ke = e->d_ke;
  s.ko = e->d_ko;
  s.pile = e->d_pile;
  s.q = e->d_q;
  s.p = e->d_p;
  s.f = e->d_f;
  s.epot = e->d_epot;
  s.status = e->d_status;
  *out = e;
  return CR_OK;
}

extern "C" {

int cr_engine_create(const cr_config* cfg, cr_engine** out) { return engine_create(cfg, nullptr, nullptr, nullptr, out); }

int cr_engine_create_qmdff(const cr_config* cfg, cr_qmdff* ff, cr_engine** out) {
  if (!ff) return fail(CR_ERR_ARG, "NULL force field");
  return engine_create(cfg, ff, nullptr, nullptr, out);
}

int cr_engine_create_evb(const cr_config* cfg, cr_evb* evb, cr_engine** out) {
  if (!evb) return fail(CR_ERR_ARG, "NULL EVB");
  return engine_create(cfg, nullptr, evb, nullptr, out);
}

int cr_engine_create_water(const cr_config* cfg, cr_water* w, cr_engine** out) {
  if (!w) return fail(CR_ERR_ARG, "NULL water box");
  return engine_create(cfg, nullptr, nullptr, w, out);
}

int cr_engine_destroy(cr_engine* e) {
  if (!e) return CR_OK;
  if (e->stream) cudaStreamSynchronize(e->stream);
  cudaFree(e->d_box);
  cudaFree(e->d_press);
  cudaFree(e->d_vir);
  cudaFree(e->d_q);
  cudaFree(e->d_p);
  cudaFree(e->d_f);
  cudaFree(e->d_epot);
  cudaFree(e->d_V);
  cudaFree(e->d_status);
  cudaFree(e->d_q0);
  cudaFree(e->d_pile);
  cudaFree(e->d_side);
  cudaFree(e->d_w);
  cudaFree(e->d_kappa);
  cudaFree(e->d_qpar);
  cudaFree(e->d_wpos);
  cudaFree(e->d_mass);
  cudaFree(e->d_inv_mass);
  cudaFree(e->d_sigma);
  cudaFree(e->d_ke);
  cudaFree(e->d_ko);
  cudaFree(e->d_circ);
  cudaFree(e->d_istep);
  cudaFree(e->d_vnh);
  cudaFree(e->d_V2);
  cudaFree(e->d_f2);
  cudaFree(e->d_dxi);
  cudaFree(e->d_cq);
  cudaFree(e->d_shake_fail);
  cudaFree(e->d_umb);
  cudaFree(e->d_umb_flag);
  cudaFree(e->d_fsum);
  cudaFree(e->d_fdrift);
  cudaFree(e->d_fstat);
  cudaFree(e->d_fmove);
  if (e->graph_exec) cudaGraphExecDestroy(e->graph_exec);
  if (e->graph) cudaGraphDestroy(e->graph);
  if (e->ev0) cudaEventDestroy(e->ev0);
  if (e->ev1) cudaEventDestroy(e->ev1);
  if (e->hs_in) {
    cudaStreamSynchronize(e->hs_in);
    cudaStreamSynchronize(e->hs_out);
    cudaStreamDestroy(e->hs_in);
    cudaStreamDestroy(e->hs_out);
    cudaEventDestroy(e->hev_out);
    for (int g = 0; g < kHostGroups; ++g) {
      cudaStreamSynchronize(e->hs_c[g]);
      cudaStreamDestroy(e->hs_c[g]);
      cudaEventDestroy(e->hev_in[g]);
      cudaEventDestroy(e->hev_c[g]);
    }
  }
  if (e->ds) {
    cudaStreamSynchronize(e->ds);
    cudaStreamDestroy(e->ds);
    for (int k = 0; k < 2; ++k) {
      cudaFree(e->d_snap[k]);
      cudaFreeHost(e->h_snap[k]);
      cudaEventDestroy(e->ev_snap[k]);
      cudaEventDestroy(e->ev_copied[k]);
    }
  }
  if (e->stream) cudaStreamDestroy(e->stream);
  delete e;
  return CR_OK;
}

int cr_engine_init_positions(cr_engine* e, const double* q0, double sigma) {
  if (!e || !q0) return fail(CR_ERR_ARG, "NULL argument");
  if (!(sigma >= 0.0)) return fail(CR_ERR_ARG, "sigma must be >= 0");
  CR_CUDA(cudaMemcpyAsync(e->d_q0, q0, (size_t)e->NC * 8, cudaMemcpyHostToDevice, e->stream));
  const int nb = e->T * e->P;
  if (e->split) {
    const long long n = (long long)nb * ((e->NC + 1) / 2);
    cr::split_init_positions_kernel<<<(unsigned)((n + 127) / 128), 128, 0, e->stream>>>(
        e->T, e->P, e->NC, e->cfg.seed, e->cfg.traj0, e->d_q0, sigma, e->d_q);
    CR_CUDA(cudaGetLastError());
    CR_CUDA(cudaStreamSynchronize(e->stream));
    return CR_OK;
  }
  switch (e->cfg.pes) {
    case CR_PES_H3:
    case CR_PES_BRH2:
      cr::init_positions_kernel<9><<<(nb + 127) / 128, 128, 0, e->stream>>>(
          e->T, e->P, e->cfg.seed, e->cfg.traj0, e->d_q0, sigma, e->d_q);
      break;
    case CR_PES_CH4H:
      cr::init_positions_kernel<18><<<(nb + 127) / 128, 128, 0, e->stream>>>(
          e->T, e->P, e->cfg.seed, e->cfg.traj0, e->d_q0, sigma, e->d_q);
      break;
    case CR_PES_CH4OH:
    case CR_PES_GEH4OH:
      cr::init_positions_kernel<21><<<(nb + 127) / 128, 128, 0, e->stream>>>(
          e->T, e->P, e->cfg.seed, e->cfg.traj0, e->d_q0, sigma, e->d_q);
      break;
    case CR_PES_OH3:
      cr::init_positions_kernel<12><<<(nb + 127) / 128, 128, 0, e->stream>>>(
          e->T, e->P, e->cfg.seed, e->cfg.traj0, e->d_q0, sigma, e->d_q);
      break;
    default: return fail(CR_ERR_UNSUPPORTED, "PES not built");
  }
  CR_CUDA(cudaGetLastError());
  CR_CUDA(cudaStreamSynchronize(e->stream));
  return CR_OK;
}

// Momenta of mdinit with Gaussian stream `draw` (see init_momenta_kernel).
static int init_momenta_draw(cr_engine* e, int zero, uint32_t draw) {
  if (!zero && !(e->cfg.beta > 0.0 && std::isfinite(e->cfg.beta)))
    return fail(CR_ERR_ARG, "Andersen momenta need a finite temperature");
  // mdinit also starts the Nose-Hoover chain at rest (src/mdinit.f90:140-145)
  CR_CUDA(cudaMemsetAsync(e->d_vnh, 0, (size_t)e->T * 4 * sizeof(double), e->stream));
  const int nb = e->T * e->P;
  if (e->split) {
    const long long n = (long long)nb * ((e->NC + 1) / 2);
    cr::split_init_momenta_kernel<<<(unsigned)((n + 127) / 128), 128, 0, e->stream>>>(
        e->T, e->P, e->NC, e->cfg.seed, e->cfg.traj0, e->d_sigma, zero, draw, e->d_p);
    CR_CUDA(cudaGetLastError());
    return CR_OK;
  }
  switch (e->cfg.pes) {
    case CR_PES_H3:
    case CR_PES_BRH2:
      cr::init_momenta_kernel<9><<<(nb + 127) / 128, 128, 0, e->stream>>>(
          e->T, e->P, e->cfg.seed, e->cfg.traj0, e->prm, zero, draw, e->d_p);
      break;
    case CR_PES_CH4H:
      cr::init_momenta_kernel<18><<<(nb + 127) / 128, 128, 0, e->stream>>>(
          e->T, e->P, e->cfg.seed, e->cfg.traj0, e->prm, zero, draw, e->d_p);
      break;
    case CR_PES_CH4OH:
    case CR_PES_GEH4OH:
      cr::init_momenta_kernel<21><<<(nb + 127) / 128, 128, 0, e->stream>>>(
          e->T, e->P, e->cfg.seed, e->cfg.traj0, e->prm, zero, draw, e->d_p);
      break;
    case CR_PES_OH3:
      cr::init_momenta_kernel<12><<<(nb + 127) / 128, 128, 0, e->stream>>>(
          e->T, e->P, e->cfg.seed, e->cfg.traj0, e->prm, zero, draw, e->d_p);
      break;
    default: return fail(CR_ERR_UNSUPPORTED, "PES not built");
  }
  CR_CUDA(cudaGetLastError());
  return CR_OK;
}

int cr_engine_init_momenta(cr_engine* e, int zero) {
  if (!e) return fail(CR_ERR_ARG, "NULL engine");
  int rc = init_momenta_draw(e, zero, 0u);
  if (rc) return rc;
  CR_CUDA(cudaStreamSynchronize(e->stream));
  return CR_OK;
}

int cr_engine_compute_forces(cr_engine* e) {
  if (!e) return fail(CR_ERR_ARG, "NULL engine");
  int rc = dispatch_forces(e);
  if (rc) return rc;
  CR_CUDA(cudaStreamSynchronize(e->stream));
  return CR_OK;
}

int cr_engine_set_state(cr_engine* e, const double* q, const double* p, const double* f) {
  if (!e || !q || !p) return fail(CR_ERR_ARG, "NULL argument");
  const size_t bytes = (size_t)e->T * e->P * e->NC * 8;
  CR_CUDA(cudaMemcpyAsync(e->d_q, q, bytes, cudaMemcpyHostToDevice, e->stream));
  CR_CUDA(cudaMemcpyAsync(e->d_p, p, bytes, cudaMemcpyHostToDevice, e->stream));
  if (f) {
    CR_CUDA(cudaMemcpyAsync(e->d_f, f, bytes, cudaMemcpyHostToDevice, e->stream));
  } else {
    int rc = dispatch_forces(e);
    if (rc) return rc;
  }
  CR_CUDA(cudaStreamSynchronize(e->stream));
  return CR_OK;
}

int cr_engine_get_state(cr_engine* e, double* q, double* p, double* f, double* epot, int* status) {
  if (!e) return fail(CR_ERR_ARG, "NULL engine");
  const size_t bytes = (size_t)e->T * e->P * e->NC * 8;
  if (q) CR_CUDA(cudaMemcpyAsync(q, e->d_q, bytes, cudaMemcpyDeviceToHost, e->stream));
  if (p) CR_CUDA(cudaMemcpyAsync(p, e->d_p, bytes, cudaMemcpyDeviceToHost, e->stream));
  if (f) CR_CUDA(cudaMemcpyAsync(f, e->d_f, bytes, cudaMemcpyDeviceToHost, e->stream));
  if (epot) CR_CUDA(cudaMemcpyAsync(epot, e->d_epot, (size_t)e->T * 8, cudaMemcpyDeviceToHost, e->stream));
  if (status)
    CR_CUDA(cudaMemcpyAsync(status, e->d_status, (size_t)e->T * sizeof(int), cudaMemcpyDeviceToHost, e->stream));
  CR_CUDA(cudaStreamSynchronize(e->stream));
  return CR_OK;
}

static int engine_run_async(cr_engine* e, int nsteps) {
  CR_CUDA(cudaEventRecord(e->ev0, e->stream));
  int rc = dispatch_run(e, nsteps);
  if (rc) return rc;
  CR_CUDA(cudaEventRecord(e->ev1, e->stream));
  e->istep += nsteps;
  e->launches = e->split ? e->step_launches * nsteps : 1;
  return CR_OK;
}

static int engine_finish(cr_engine* e) {
  CR_CUDA(cudaStreamSynchronize(e->stream));
  CR_CUDA(cudaEventElapsedTime(&e->last_ms, e->ev0, e->ev1));
  std::vector<int> st((size_t)e->T);
  CR_CUDA(cudaMemcpy(st.data(), e->d_status, st.size() * sizeof(int), cudaMemcpyDeviceToHost));
  for (int v : st)
    if (v) return fail(CR_ERR_TRAJECTORY, "a trajectory reported a non-finite coordinate or singular inertia");
  return CR_OK;
}

int cr_engine_run(cr_engine* e, int nsteps) {
  if (!e) return fail(CR_ERR_ARG, "NULL engine");
  if (nsteps < 0) return fail(CR_ERR_ARG, "nsteps must be >= 0");
  if (e->xi_on && e->istep + nsteps - e->side_step0 > e->side_cap)
    return fail(CR_ERR_ARG, "run exceeds the recrossing step capacity set by cr_engine_set_recross");
  if (nsteps == 0) return CR_OK;
  int rc = engine_run_async(e, nsteps);
  if (rc) return rc;
  return engine_finish(e);
}

int cr_engine_run_dump(cr_engine* e, int nsteps, int every, cr_dump_fn dump, void* user, double* q, double* p,
                       double* epot) {
  if (!e || !dump || !q || !p || !epot) return fail(CR_ERR_ARG, "NULL argument");
  if (nsteps < 0 || every < 1) return fail(CR_ERR_ARG, "nsteps must be >= 0 and every >= 1");
  int done = 0;
  while (done < nsteps) {
    const int n = std::min(every - e->istep % every, nsteps - done);
    int rc = cr_engine_run(e, n);
    if (rc) return rc;
    done += n;
    if (e->istep % every == 0) {
      if ((rc = cr_engine_get_state(e, q, p, nullptr, epot, nullptr))) return rc;
      if (dump(user, e->istep, q, p, epot) != 0) return fail(CR_ERR_ARG, "the dump callback stopped the run");
    }
  }
  return CR_OK;
}

// Bytes of one dump snapshot: q and p (T P 3N doubles each), epot (T
// doubles), the status words (T ints).
static size_t dump_snapshot_bytes(const cr_engine* e) {
  return (2 * (size_t)e->T * e->P * e->NC + (size_t)e->T) * sizeof(double) + (size_t)e->T * sizeof(int);
}

static int dump_slots_init(cr_engine* e) {
  if (e->ds) return CR_OK;
  const size_t n = dump_snapshot_bytes(e);
  CR_CUDA(cudaStreamCreateWithFlags(&e->ds, cudaStreamNonBlocking));
  for (int k = 0; k < 2; ++k) {
    CR_CUDA(cudaMalloc(&e->d_snap[k], n));
    CR_CUDA(cudaMallocHost(&e->h_snap[k], n));
    CR_CUDA(cudaEventCreateWithFlags(&e->ev_snap[k], cudaEventDisableTiming));
    CR_CUDA(cudaEventCreateWithFlags(&e->ev_copied[k], cudaEventDisableTiming));
  }
  return CR_OK;
}

int cr_engine_run_dump_async(cr_engine* e, int nsteps, int every, cr_dump_fn dump, void* user) {
  if (!e || !dump) return fail(CR_ERR_ARG, "NULL argument");
  if (nsteps < 0 || every < 1) return fail(CR_ERR_ARG, "nsteps must be >= 0 and every >= 1");
  if (e->xi_on && e->istep + nsteps - e->side_step0 > e->side_cap)
    return fail(CR_ERR_ARG, "run exceeds the recrossing step capacity set by cr_engine_set_recross");
  if (nsteps == 0) return CR_OK;
  int rc = dump_slots_init(e);
  if (rc) return rc;
  const size_t nq = (size_t)e->T * e->P * e->NC;
  const size_t nbytes = dump_snapshot_bytes(e);
  // hand the host the snapshot of slot k once its copy has landed; a
  // trajectory that went non-finite by then ends the run before its frame
  // is written
  auto deliver = [&](int k, int istep) -> int {
    CR_CUDA(cudaEventSynchronize(e->ev_copied[k]));
    const double* h = reinterpret_cast<const double*>(e->h_snap[k]);
    const int* st = reinterpret_cast<const int*>(h + 2 * nq + e->T);
    for (int t = 0; t < e->T; ++t)
      if (st[t]) return fail(CR_ERR_TRAJECTORY, "a trajectory reported a non-finite coordinate or singular inertia");
    if (dump(user, istep, h, h + nq, h + 2 * nq) != 0) return fail(CR_ERR_ARG, "the dump callback stopped the run");
    return CR_OK;
  };
  int pending = -1, pending_step = 0, slot = 0, done = 0;
  while (done < nsteps) {
    const int n = std::min(every - e->istep % every, nsteps - done);
    if ((rc = engine_run_async(e, n))) return rc;
    done += n;
    if (e->istep % every != 0) continue;
    // snapshot on the engine stream, copy out on the dump stream: the next
    // steps are queued behind the snapshot while the host writes the frame
    // before it.  Slot `slot` was last read by the callback two dumps ago,
    // which returned before this point.
    char* d = e->d_snap[slot];
    CR_CUDA(cudaMemcpyAsync(d, e->d_q, nq * 8, cudaMemcpyDeviceToDevice, e->stream));
    CR_CUDA(cudaMemcpyAsync(d + nq * 8, e->d_p, nq * 8, cudaMemcpyDeviceToDevice, e->stream));
    CR_CUDA(cudaMemcpyAsync(d + 2 * nq * 8, e->d_epot, (size_t)e->T * 8, cudaMemcpyDeviceToDevice, e->stream));
    CR_CUDA(cudaMemcpyAsync(d + (2 * nq + e->T) * 8, e->d_status, (size_t)e->T * sizeof(int),
                            cudaMemcpyDeviceToDevice, e->stream));
    CR_CUDA(cudaEventRecord(e->ev_snap[slot], e->stream));
    CR_CUDA(cudaStreamWaitEvent(e->ds, e->ev_snap[slot], 0));
    CR_CUDA(cudaMemcpyAsync(e->h_snap[slot], d, nbytes, cudaMemcpyDeviceToHost, e->ds));
    CR_CUDA(cudaEventRecord(e->ev_copied[slot], e->ds));
    if (pending >= 0 && (rc = deliver(pending, pending_step))) {
      cudaStreamSynchronize(e->stream);
      return rc;
    }
    pending = slot;
    pending_step = e->istep;
    slot ^= 1;
  }
  if (pending >= 0 && (rc = deliver(pending, pending_step))) {
    cudaStreamSynchronize(e->stream);
    return rc;
  }
  return engine_finish(e);
}

// Trajectory groups of the pipelined host-buffer step: about 2 MB of each
// state array per group, at most kHostGroups; 1 (copy in, step, copy out in
// sequence) where a group would be too small to pay for its launches, and
// for constrained parents and umbrella windows.
static int host_groups(const cr_engine* e) {
  if (e->parent || (e->split && e->sp.umbrella)) return 1;
  const size_t bytes = (size_t)e->T * e->P * e->NC * 8;
  const size_t ng = bytes / (2u << 20);
  return (int)std::max<size_t>(1, std::min<size_t>({ng, (size_t)kHostGroups, (size_t)e->T}));
}

static int host_pipeline_init(cr_engine* e) {
  if (e->hs_in) return CR_OK;
  CR_CUDA(cudaStreamCreateWithFlags(&e->hs_in, cudaStreamNonBlocking));
  CR_CUDA(cudaStreamCreateWithFlags(&e->hs_out, cudaStreamNonBlocking));
  CR_CUDA(cudaEventCreateWithFlags(&e->hev_out, cudaEventDisableTiming));
  for (int g = 0; g < kHostGroups; ++g) {
    CR_CUDA(cudaStreamCreateWithFlags(&e->hs_c[g], cudaStreamNonBlocking));
    CR_CUDA(cudaEventCreateWithFlags(&e->hev_in[g], cudaEventDisableTiming));
    CR_CUDA(cudaEventCreateWithFlags(&e->hev_c[g], cudaEventDisableTiming));
  }
  return CR_OK;
}

// The step of every group g: on hs_c[g] after its copies in, before its
// copies out.
static int host_group_step(cr_engine* e, int t0, int tn, cudaStream_t st, int* nl) {
  if (e->split) return split_group_launches(e, split_params_range(e, t0, tn), t0, tn, st, nl);
  ++*nl;
  return launch_group(e, t0, tn, st);
}

int cr_engine_step_host(cr_engine* e, double* q, double* p, double* f, double* epot) {
  if (!e || !q || !p || !f) return fail(CR_ERR_ARG, "NULL argument");
  if (e->xi_on && e->istep + 1 - e->side_step0 > e->side_cap)
    return fail(CR_ERR_ARG, "step exceeds the recrossing step capacity set by cr_engine_set_recross");
  const int ng = host_groups(e);
  const size_t per_traj = (size_t)e->P * e->NC;
  if (ng <= 1) {
    const size_t bytes = (size_t)e->T * per_traj * 8;
    CR_CUDA(cudaMemcpyAsync(e->d_q, q, bytes, cudaMemcpyHostToDevice, e->stream));
    CR_CUDA(cudaMemcpyAsync(e->d_p, p, bytes, cudaMemcpyHostToDevice, e->stream));
    CR_CUDA(cudaMemcpyAsync(e->d_f, f, bytes, cudaMemcpyHostToDevice, e->stream));
    int rc = engine_run_async(e, 1);
    if (rc) return rc;
    CR_CUDA(cudaMemcpyAsync(q, e->d_q, bytes, cudaMemcpyDeviceToHost, e->stream));
    CR_CUDA(cudaMemcpyAsync(p, e->d_p, bytes, cudaMemcpyDeviceToHost, e->stream));
    CR_CUDA(cudaMemcpyAsync(f, e->d_f, bytes, cudaMemcpyDeviceToHost, e->stream));
    if (epot) CR_CUDA(cudaMemcpyAsync(epot, e->d_epot, (size_t)e->T * 8, cudaMemcpyDeviceToHost, e->stream));
    return engine_finish(e);
  }
  // Pipelined: group g's copies in (hs_in), its step (hs_c[g]) and its
  // copies out (hs_out) overlap the other groups' work; the device step
  // counter is set before and advanced after every group.
  int rc = host_pipeline_init(e);
  if (rc) return rc;
  if (e->split) {
    if ((rc = split_prepare(e))) return rc;
    e->h_istep = e->istep;
    CR_CUDA(cudaMemcpyAsync(e->d_istep, &e->h_istep, sizeof(int), cudaMemcpyHostToDevice, e->stream));
  } else {
    rc = set_run_smem(e);
    if (rc) return rc;
  }
  CR_CUDA(cudaEventRecord(e->ev0, e->stream));
  CR_CUDA(cudaStreamWaitEvent(e->hs_in, e->ev0, 0));
  for (int g = 0; g < ng; ++g) {
    const int t0 = (int)((long long)e->T * g / ng), t1 = (int)((long long)e->T * (g + 1) / ng);
    const size_t off = (size_t)t0 * per_traj, bytes = (size_t)(t1 - t0) * per_traj * 8;
    CR_CUDA(cudaMemcpyAsync(e->d_q + off, q + off, bytes, cudaMemcpyHostToDevice, e->hs_in));
    CR_CUDA(cudaMemcpyAsync(e->d_p + off, p + off, bytes, cudaMemcpyHostToDevice, e->hs_in));
    CR_CUDA(cudaMemcpyAsync(e->d_f + off, f + off, bytes, cudaMemcpyHostToDevice, e->hs_in));
    CR_CUDA(cudaEventRecord(e->hev_in[g], e->hs_in));
  }
  int nl = 0;
  for (int g = 0; g < ng; ++g) {
    const int t0 = (int)((long long)e->T * g / ng), t1 = (int)((long long)e->T * (g + 1) / ng);
    CR_CUDA(cudaStreamWaitEvent(e->hs_c[g], e->hev_in[g], 0));
    if ((rc = host_group_step(e, t0, t1 - t0, e->hs_c[g], &nl))) return rc;
    CR_CUDA(cudaEventRecord(e->hev_c[g], e->hs_c[g]));
    CR_CUDA(cudaStreamWaitEvent(e->hs_out, e->hev_c[g], 0));
    const size_t off = (size_t)t0 * per_traj, bytes = (size_t)(t1 - t0) * per_traj * 8;
    CR_CUDA(cudaMemcpyAsync(q + off, e->d_q + off, bytes, cudaMemcpyDeviceToHost, e->hs_out));
    CR_CUDA(cudaMemcpyAsync(p + off, e->d_p + off, bytes, cudaMemcpyDeviceToHost, e->hs_out));
    CR_CUDA(cudaMemcpyAsync(f + off, e->d_f + off, bytes, cudaMemcpyDeviceToHost, e->hs_out));
  }
  // epot (often pageable: such a copy returns only when done) once, last
  if (epot) CR_CUDA(cudaMemcpyAsync(epot, e->d_epot, (size_t)e->T * 8, cudaMemcpyDeviceToHost, e->hs_out));
  for (int g = 0; g < ng; ++g) CR_CUDA(cudaStreamWaitEvent(e->stream, e->hev_c[g], 0));
  if (e->split) {
    cr::split_advance_kernel<<<1, 1, 0, e->stream>>>(e->d_istep);
    CR_CUDA(cudaGetLastError());
    ++nl;
  }
  CR_CUDA(cudaEventRecord(e->hev_out, e->hs_out));
  CR_CUDA(cudaStreamWaitEvent(e->stream, e->hev_out, 0));
  CR_CUDA(cudaEventRecord(e->ev1, e->stream));
  e->istep += 1;
  e->launches = nl;
  return engine_finish(e);
}

int cr_engine_last_kernel_ms(const cr_engine* e, float* ms) {
  if (!e || !ms) return fail(CR_ERR_ARG, "NULL argument");
  *ms = e->last_ms;
  return CR_OK;
}

int cr_engine_launch_info(const cr_engine* e, int* grid, int* block, int* smem_bytes, int* launches) {
  if (!e) return fail(CR_ERR_ARG, "NULL engine");
  if (grid) *grid = e->grid;
  if (block) *block = e->block;
  if (smem_bytes) *smem_bytes = (int)e->smem;
  if (launches) *launches = e->launches;
  return CR_OK;
}

int cr_engine_device_state(cr_engine* e, double** q, double** p, double** f) {
  if (!e) return fail(CR_ERR_ARG, "NULL engine");
  if (q) *q = e->d_q;
  if (p) *p = e->d_p;
  if (f) *f = e->d_f;
  return CR_OK;
}

int cr_host_alloc(void** ptr, unsigned long long bytes) {
  if (!ptr) return fail(CR_ERR_ARG, "NULL argument");
  CR_CUDA(cudaMallocHost(ptr, (size_t)bytes));
  return CR_OK;
}

int cr_host_free(void* ptr) {
  if (ptr) CR_CUDA(cudaFreeHost(ptr));
  return CR_OK;
}

int cr_host_register(void* ptr, unsigned long long bytes) {
  if (!ptr || bytes == 0) return fail(CR_ERR_ARG, "NULL pointer or zero size");
  CR_CUDA(cudaHostRegister(ptr, (size_t)bytes, cudaHostRegisterDefault));
  return CR_OK;
}

int cr_host_unregister(void* ptr) {
  if (ptr) CR_CUDA(cudaHostUnregister(ptr));
  return CR_OK;
}

}  // extern "C"

// BIMOLEC reaction coordinate of a cr_recross definition (1-based atoms).
static int make_xidev(const cr_engine* e, const cr_recross* rc, cr::XiDev& x) {
  auto bad_atom = [&](int a) { return a < 1 || a > e->N; };
  if (rc->nreac1 < 1 || rc->nreac1 > 8 || rc->nreac2 < 1 || rc->nreac2 > 8)
    return fail(CR_ERR_ARG, "reactants need 1..8 atoms each");
  x.nreac1 = rc->nreac1;
  x.nreac2 = rc->nreac2;
  x.mreac1 = 0.0;
  x.mreac2 = 0.0;
  for (int k = 0; k < rc->nreac1; ++k) {
    if (bad_atom(rc->reac1[k])) return fail(CR_ERR_ARG, "reactant atom out of range");
    x.reac1[k] = rc->reac1[k] - 1;
    x.mreac1 = x.mreac1 + e->mass[(size_t)x.reac1[k]];
  }
  for (int k = 0; k < rc->nreac2; ++k) {
    if (bad_atom(rc->reac2[k])) return fail(CR_ERR_ARG, "reactant atom out of range");
    x.reac2[k] = rc->reac2[k] - 1;
    x.mreac2 = x.mreac2 + e->mass[(size_t)x.reac2[k]];
  }
  if (bad_atom(rc->bond_form[0]) || bad_atom(rc->bond_form[1]) || bad_atom(rc->bond_break[0]) ||
      bad_atom(rc->bond_break[1]))
    return fail(CR_ERR_ARG, "bond atom out of range");
  x.form0 = rc->bond_form[0] - 1;
  x.form1 = rc->bond_form[1] - 1;
  x.brk0 = rc->bond_break[0] - 1;
  x.brk1 = rc->bond_break[1] - 1;
  x.form_ref = rc->form_ref;
  x.break_ref = rc->break_ref;
  x.r_inf = rc->r_inf;
  x.xi_ideal = rc->xi_ideal;
  for (int k = 0; k < 8; ++k) {
    x.w1[k] = k < x.nreac1 ? e->mass[(size_t)x.reac1[k]] / x.mreac1 : 0.0;
    x.w2[k] = k < x.nreac2 ? e->mass[(size_t)x.reac2[k]] / x.mreac2 : 0.0;
  }
  return CR_OK;
}

extern "C" {

int cr_engine_set_parent(cr_engine* e, const cr_recross* rc) {
  if (!e || !rc) return fail(CR_ERR_ARG, "NULL argument");
  if (e->ff || e->evb || e->water)
    return fail(CR_ERR_UNSUPPORTED, "constrained parents are built for the analytic surfaces");
  if (e->xi_on) return fail(CR_ERR_ARG, "a recrossing-children engine cannot be a parent");
  cr::XiDev x{};
  int rcode = make_xidev(e, rc, x);
  if (rcode) return rcode;
  if (!e->d_dxi) {
    CR_CUDA(cudaMalloc(&e->d_dxi, (size_t)e->T * e->NC * sizeof(double)));
    CR_CUDA(cudaMalloc(&e->d_cq, (size_t)e->T * e->NC * sizeof(double)));
    CR_CUDA(cudaMalloc(&e->d_shake_fail, (size_t)e->T * sizeof(int)));
  }
  e->parent = true;
  e->split = true;
  e->sp.constrain = 1;
  e->sp.xi = x;
  e->sp.transrot = 0;  // verlet calls transrot only for constrain <= 0
  e->sp.dxi = e->d_dxi;
  e->sp.cq = e->d_cq;
  e->sp.shake_fail = e->d_shake_fail;
  if (e->graph_exec) {
    cudaGraphExecDestroy(e->graph_exec);
    e->graph_exec = nullptr;
  }
  if (e->graph) {
    cudaGraphDestroy(e->graph);
    e->graph = nullptr;
  }
  rcode = parent_kernel(e, 2);
  if (rcode) return rcode;
  CR_CUDA(cudaStreamSynchronize(e->stream));
  return CR_OK;
}

int cr_engine_set_umbrella(cr_engine* e, const cr_recross* rc, const double* centers, const double* kforce,
                           int nbins, double lo, double hi) {
  if (!e || !rc || !centers || !kforce) return fail(CR_ERR_ARG, "NULL argument");
  if (e->ff || e->evb || e->water)
    return fail(CR_ERR_UNSUPPORTED, "umbrella windows are built for the analytic surfaces");
  if (e->xi_on || e->parent) return fail(CR_ERR_ARG, "an umbrella engine cannot be a parent or recrossing children");
  if (!(e->cfg.beta > 0.0) || !std::isfinite(e->cfg.beta)) return fail(CR_ERR_ARG, "umbrella sampling needs a temperature");
  if (nbins < 0 || (nbins > 0 && !(hi > lo))) return fail(CR_ERR_ARG, "bad histogram range");
  cr::XiDev x{};
  int rcode = make_xidev(e, rc, x);
  if (rcode) return rcode;
  const size_t T = (size_t)e->T, nh = T * (size_t)nbins;
  cudaFree(e->d_umb);
  e->d_umb = nullptr;
  CR_CUDA(cudaMalloc(&e->d_umb, (4 * T + nh + 1) * sizeof(double)));
  // [0] the sampling switch, [1] always 0 (the switch mdinit's bias reads)
  if (!e->d_umb_flag) CR_CUDA(cudaMalloc(&e->d_umb_flag, 2 * sizeof(int)));
  CR_CUDA(cudaMemcpy(e->d_umb, centers, T * 8, cudaMemcpyHostToDevice));
  CR_CUDA(cudaMemcpy(e->d_umb + T, kforce, T * 8, cudaMemcpyHostToDevice));
  CR_CUDA(cudaMemset(e->d_umb + 2 * T, 0, (2 * T + nh) * 8));
  CR_CUDA(cudaMemset(e->d_umb_flag, 0, 2 * sizeof(int)));
  e->umb_sampling = 0;
  cr::UmbrellaDev u{};
  u.center = e->d_umb;
  u.kforce = e->d_umb + T;
  u.beta = e->cfg.beta;
  u.sampling = e->d_umb_flag;
  u.xsum = e->d_umb + 2 * T;
  u.xsum2 = e->d_umb + 3 * T;
  u.nbins = nbins;
  u.lo = lo;
  u.hi = hi;
  u.hist = e->d_umb + 4 * T;
  e->split = true;
  e->sp.umbrella = 1;
  e->sp.umb = u;
  e->sp.xi = x;
  if (e->graph_exec) {
    cudaGraphExecDestroy(e->graph_exec);
    e->graph_exec = nullptr;
  }
  if (e->graph) {
    cudaGraphDestroy(e->graph);
    e->graph = nullptr;
  }
  return CR_OK;
}

int cr_engine_umbrella_sampling(cr_engine* e, int on) {
  if (!e || !e->d_umb_flag) return fail(CR_ERR_ARG, "no umbrella windows on this engine");
  const int v = on ? 1 : 0;
  CR_CUDA(cudaStreamSynchronize(e->stream));
  CR_CUDA(cudaMemcpy(e->d_umb_flag, &v, sizeof(int), cudaMemcpyHostToDevice));
  e->umb_sampling = v;
  return CR_OK;
}

// Drops the captured step graph (it holds the step parameters by value).
static void drop_graph(cr_engine* e) {
  if (e->graph_exec) {
    cudaGraphExecDestroy(e->graph_exec);
    e->graph_exec = nullptr;
  }
  if (e->graph) {
    cudaGraphDestroy(e->graph);
    e->graph = nullptr;
  }
}

int cr_engine_set_npt(cr_engine* e, double pressure_atm, const double* box_bohr) {
  if (!e) return fail(CR_ERR_ARG, "NULL engine");
  if (!e->ff || e->evb || !e->ff->dev.periodic)
    return fail(CR_ERR_UNSUPPORTED, "NpT is built for one periodic QMDFF force field (cr_qmdff_set_periodic)");
  if (e->parent || e->sp.umbrella) return fail(CR_ERR_UNSUPPORTED, "NpT with constrained parents or umbrella windows");
  if (!(pressure_atm >= 0.0)) return fail(CR_ERR_ARG, "Give a positive pressure!");
  const size_t T = (size_t)e->T;
  std::vector<double> box(3 * T);
  for (size_t t = 0; t < T; ++t)
    for (int k = 0; k < 3; ++k) {
      const double L = box_bohr ? box_bohr[3 * t + k] : e->ff->dev.box.len[k];
      if (!(L > 0.0) || !std::isfinite(L)) return fail(CR_ERR_ARG, "box edges must be positive");
      box[3 * t + k] = L;
    }
  CR_CUDA(cudaStreamSynchronize(e->stream));
  if (!e->d_box) {
    CR_CUDA(cudaMalloc(&e->d_box, 3 * T * sizeof(double)));
    CR_CUDA(cudaMalloc(&e->d_press, 2 * T * sizeof(double)));
    CR_CUDA(cudaMalloc(&e->d_vir, T * (size_t)e->P * sizeof(double)));
  }
  CR_CUDA(cudaMemcpy(e->d_box, box.data(), 3 * T * sizeof(double), cudaMemcpyHostToDevice));
  CR_CUDA(cudaMemset(e->d_press, 0, 2 * T * sizeof(double)));
  CR_CUDA(cudaMemset(e->d_vir, 0, T * (size_t)e->P * sizeof(double)));
  // mdinit's Berendsen constants (src/mdinit.f90:155-158) and the pressure
  // unit (src/general.f90:263, src/dynamic.f90:1331-1335)
  const double prescon = 290371576.61, taupres = 2.0, compress = 0.000046 * prescon / 1000.0;
  e->npt = true;
  e->npt_pressure = pressure_atm / prescon;
  e->npt_rate = e->cfg.dt * compress / taupres;
  drop_graph(e);
  return CR_OK;
}

int cr_engine_get_npt(cr_engine* e, double* box_bohr, double* pressure_au, double* pressure_sum_au, int reset_sum) {
  if (!e) return fail(CR_ERR_ARG, "NULL engine");
  if (!e->npt) return fail(CR_ERR_ARG, "NpT is not set (cr_engine_set_npt)");
  CR_CUDA(cudaStreamSynchronize(e->stream));
  const size_t T = (size_t)e->T;
  if (box_bohr) CR_CUDA(cudaMemcpy(box_bohr, e->d_box, 3 * T * sizeof(double), cudaMemcpyDeviceToHost));
  if (pressure_au || pressure_sum_au) {
    std::vector<double> h(2 * T);
    CR_CUDA(cudaMemcpy(h.data(), e->d_press, 2 * T * sizeof(double), cudaMemcpyDeviceToHost));
    for (size_t t = 0; t < T; ++t) {
      if (pressure_au) pressure_au[t] = h[2 * t];
      if (pressure_sum_au) pressure_sum_au[t] = h[2 * t + 1];
    }
  }
  if (reset_sum)  // the running sums only: every other word
    CR_CUDA(cudaMemset2D(e->d_press + 1, 2 * sizeof(double), 0, sizeof(double), T));
  return CR_OK;
}

int cr_engine_set_launch(cr_engine* e, int threads_per_block, int threads_per_bead) {
  if (!e) return fail(CR_ERR_ARG, "NULL engine");
  if (e->split) return fail(CR_ERR_UNSUPPORTED, "this engine steps through the graph path, which has no launch shape to set");
  CR_CUDA(cudaStreamSynchronize(e->stream));
  if (threads_per_block == 0) {
    choose_launch(e);
  } else if (!set_launch_shape(e, threads_per_block, threads_per_bead)) {
    return fail(CR_ERR_ARG, "threads_per_bead must be 1, 2 or 4 (as built for the surface: 4 for H3 and OH3, "
                            "1 for CH4H and CH4OH) and threads_per_block a multiple of threads_per_bead x the bead "
                            "group (next power of two of nbeads), at most 256, with the group scratch within 200 KB");
  }
  drop_graph(e);
  return CR_OK;
}

int cr_engine_get_launch(cr_engine* e, int* threads_per_block, int* blocks, int* threads_per_bead) {
  if (!e) return fail(CR_ERR_ARG, "NULL engine");
  if (threads_per_block) *threads_per_block = e->split ? 0 : e->block;
  if (blocks) *blocks = e->split ? 0 : e->grid;
  if (threads_per_bead) *threads_per_bead = e->split ? 0 : e->tpb;
  return CR_OK;
}

int cr_engine_autotune(cr_engine* e, int nsteps, int* threads_per_block, int* threads_per_bead, float* ms_per_step) {
  if (!e) return fail(CR_ERR_ARG, "NULL engine");
  if (e->split) return fail(CR_ERR_UNSUPPORTED, "this engine steps through the graph path, which has no launch shape to tune");
  if (nsteps < 1) return fail(CR_ERR_ARG, "nsteps must be >= 1");
  if (e->xi_on && e->istep + nsteps + 1 - e->side_step0 > e->side_cap)
    return fail(CR_ERR_ARG, "the trial runs exceed the recrossing step capacity set by cr_engine_set_recross");
  CR_CUDA(cudaStreamSynchronize(e->stream));
  // every trial starts from the same state: q, p, f, epot, status, the
  // chain velocities and the step counter are saved and put back after it
  const size_t nq = (size_t)e->T * e->P * e->NC, T = (size_t)e->T;
  const size_t nsave = 3 * nq + T + 4 * T;
  double* save = nullptr;
  int* save_st = nullptr;
  CR_CUDA(cudaMalloc(&save, nsave * sizeof(double)));
  if (cudaMalloc(&save_st, T * sizeof(int)) != cudaSuccess) {
    cudaFree(save);
    return fail(CR_ERR_CUDA, "cudaMalloc failed for the autotuner's state copy");
  }
  auto copy_state = [&](bool out) -> cudaError_t {
    double* dst[5] = {save, save + nq, save + 2 * nq, save + 3 * nq, save + 3 * nq + T};
    double* src[5] = {e->d_q, e->d_p, e->d_f, e->d_epot, e->d_vnh};
    const size_t n[5] = {nq, nq, nq, T, 4 * T};
    cudaError_t err = cudaSuccess;
    for (int k = 0; k < 5 && err == cudaSuccess; ++k)
      err = cudaMemcpyAsync(out ? dst[k] : src[k], out ? src[k] : dst[k], n[k] * 8, cudaMemcpyDeviceToDevice, e->stream);
    if (err == cudaSuccess)
      err = cudaMemcpyAsync(out ? save_st : e->d_status, out ? e->d_status : save_st, T * sizeof(int),
                            cudaMemcpyDeviceToDevice, e->stream);
    return err;
  };
  const int block0 = e->block, tpb0 = e->tpb, istep0 = e->istep;
  int best = block0, best_tpb = tpb0, rc = CR_OK;
  float best_ms = 0.f;
  cudaError_t err = copy_state(true);
  for (int tpb = 1; tpb <= 4 && rc == CR_OK && err == cudaSuccess; tpb *= 2) {
    const int cand[] = {e->G * tpb, 32, 64, 128, 256};
    for (int k = 0; k < 5 && rc == CR_OK && err == cudaSuccess; ++k) {
      const int b = cand[k];
      bool seen = false;
      for (int i = 0; i < k; ++i) seen |= cand[i] == b;
      if (seen || !set_launch_shape(e, b, tpb)) continue;
      // one untimed step (first launch of this shape), then the timed run
      for (int rep = 0; rep < 2 && rc == CR_OK; ++rep) {
        if ((rc = engine_run_async(e, rep == 0 ? 1 : nsteps))) break;
        err = cudaStreamSynchronize(e->stream);
        if (err != cudaSuccess) break;
        if (rep == 1) {
          float ms = 0.f;
          cudaEventElapsedTime(&ms, e->ev0, e->ev1);
          if (best_ms == 0.f || ms < best_ms) {
            best_ms = ms;
            best = b;
            best_tpb = tpb;
          }
        }
        e->istep = istep0;
        if ((err = copy_state(false)) != cudaSuccess) break;
      }
    }
  }
  cudaStreamSynchronize(e->stream);
  cudaFree(save);
  cudaFree(save_st);
  e->istep = istep0;
  if (rc) {
    set_launch_shape(e, block0, tpb0);
    return rc;
  }
  if (err != cudaSuccess) {
    set_launch_shape(e, block0, tpb0);
    return fail(CR_ERR_CUDA, cudaGetErrorString(err));
  }
  set_launch_shape(e, best, best_tpb);
  drop_graph(e);
  if (threads_per_block) *threads_per_block = best;
  if (threads_per_bead) *threads_per_bead = best_tpb;
  if (ms_per_step) *ms_per_step = best_ms / nsteps;
  return CR_OK;
}

int cr_engine_set_andersen_step(cr_engine* e, int andersen_step) {
  if (!e) return fail(CR_ERR_ARG, "NULL engine");
  if (andersen_step < 1) return fail(CR_ERR_ARG, "andersen_step must be >= 1");
  CR_CUDA(cudaStreamSynchronize(e->stream));
  e->cfg.andersen_step = andersen_step;
  e->prm.andersen_step = andersen_step;
  e->sp.andersen_step = andersen_step;
  drop_graph(e);
  return CR_OK;
}

int cr_engine_mdinit(cr_engine* e, unsigned draw) {
  if (!e) return fail(CR_ERR_ARG, "NULL engine");
  const bool umb = e->split && e->sp.umbrella;
  if (umb && e->umb_sampling) return fail(CR_ERR_ARG, "switch umbrella sampling off before mdinit");
  int rc = dispatch_forces(e);
  if (rc) return rc;
  if (umb) {  // src/mdinit.f90:96-100: umbrella(..., mode 0) on the initial forces
    cr::SplitParams s = e->sp;
    s.umb.sampling = e->d_umb_flag + 1;
    switch (e->N) {
      case 3: cr::split_umbrella_kernel<3><<<e->T, 64, 0, e->stream>>>(s); break;
      case 6: cr::split_umbrella_kernel<6><<<e->T, 64, 0, e->stream>>>(s); break;
      case 7: cr::split_umbrella_kernel<7><<<e->T, 64, 0, e->stream>>>(s); break;
      case 4: cr::split_umbrella_kernel<4><<<e->T, 64, 0, e->stream>>>(s); break;
      default: return fail(CR_ERR_UNSUPPORTED, "umbrella windows are built for the analytic surfaces");
    }
    CR_CUDA(cudaGetLastError());
  }
  // NVT: Andersen draw (src/mdinit.f90:118-121); NVE: zero momenta (:125)
  const int nve = e->cfg.thermostat == CR_THERMO_NONE;
  if ((rc = init_momenta_draw(e, nve, (uint32_t)draw))) return rc;
  CR_CUDA(cudaStreamSynchronize(e->stream));
  return CR_OK;
}

int cr_engine_umbrella_stats(cr_engine* e, double* xsum, double* xsum2, double* hist, int reset) {
  if (!e || !e->d_umb) return fail(CR_ERR_ARG, "no umbrella windows on this engine");
  const size_t T = (size_t)e->T, nh = T * (size_t)e->sp.umb.nbins;
  CR_CUDA(cudaStreamSynchronize(e->stream));
  if (xsum) CR_CUDA(cudaMemcpy(xsum, e->d_umb + 2 * T, T * 8, cudaMemcpyDeviceToHost));
  if (xsum2) CR_CUDA(cudaMemcpy(xsum2, e->d_umb + 3 * T, T * 8, cudaMemcpyDeviceToHost));
  if (hist && nh) CR_CUDA(cudaMemcpy(hist, e->d_umb + 4 * T, nh * 8, cudaMemcpyDeviceToHost));
  if (reset) CR_CUDA(cudaMemset(e->d_umb + 2 * T, 0, (2 * T + nh) * 8));
  return CR_OK;
}

int cr_engine_set_recross(cr_engine* e, const cr_recross* rc, int max_steps) {
  if (!e || !rc) return fail(CR_ERR_ARG, "NULL argument");
  if (max_steps < 1) return fail(CR_ERR_ARG, "max_steps must be >= 1");
  if (e->split) return fail(CR_ERR_UNSUPPORTED, "recrossing children are built for the analytic surfaces only");
  cr::XiDev x{};
  int rcode = make_xidev(e, rc, x);
  if (rcode) return rcode;

  cudaFree(e->d_side);
  cudaFree(e->d_w);
  cudaFree(e->d_kappa);
  cudaFree(e->d_wpos);
  e->d_side = nullptr;
  e->d_w = e->d_kappa = nullptr;
  e->d_wpos = nullptr;
  CR_CUDA(cudaMalloc(&e->d_side, (size_t)e->T * max_steps));
  CR_CUDA(cudaMalloc(&e->d_w, (size_t)e->T * sizeof(double)));
  CR_CUDA(cudaMalloc(&e->d_wpos, (size_t)e->T * sizeof(int)));
  CR_CUDA(cudaMalloc(&e->d_kappa, (size_t)(max_steps + 1) * sizeof(double)));
  CR_CUDA(cudaMemsetAsync(e->d_side, 0, (size_t)e->T * max_steps, e->stream));
  CR_CUDA(cudaMemsetAsync(e->d_w, 0, (size_t)e->T * sizeof(double), e->stream));
  CR_CUDA(cudaMemsetAsync(e->d_wpos, 0, (size_t)e->T * sizeof(int), e->stream));
  e->side_cap = max_steps;
  e->side_step0 = e->istep;
  e->xi_on = 1;
  e->prm.xi = x;
  e->prm.xi_on = 1;
  e->prm.side = e->d_side;
  e->prm.side_stride = max_steps;
  e->prm.side_step0 = e->istep;
  CR_CUDA(cudaStreamSynchronize(e->stream));
  return CR_OK;
}

int cr_engine_init_children(cr_engine* e, const double* q_parent) {
  if (!e || !q_parent) return fail(CR_ERR_ARG, "NULL argument");
  if (!e->xi_on) return fail(CR_ERR_ARG, "call cr_engine_set_recross first");
  if (e->split) return fail(CR_ERR_UNSUPPORTED, "recrossing children are built for the analytic surfaces only");
  if (!(e->cfg.beta > 0.0 && std::isfinite(e->cfg.beta))) return fail(CR_ERR_ARG, "children need a finite beta");
  const size_t bytes = (size_t)e->NC * e->P * sizeof(double);
  if (!e->d_qpar) CR_CUDA(cudaMalloc(&e->d_qpar, bytes));
  CR_CUDA(cudaMemcpyAsync(e->d_qpar, q_parent, bytes, cudaMemcpyHostToDevice, e->stream));
  const int nb = e->T * e->P;
  switch (e->cfg.pes) {
    case CR_PES_H3:
    case CR_PES_BRH2:
      cr::init_children_kernel<9><<<(nb + 127) / 128, 128, 0, e->stream>>>(
          e->T, e->P, e->cfg.seed, e->cfg.traj0, e->prm, e->d_qpar, e->d_q, e->d_p);
      break;
    case CR_PES_CH4H:
      cr::init_children_kernel<18><<<(nb + 127) / 128, 128, 0, e->stream>>>(
          e->T, e->P, e->cfg.seed, e->cfg.traj0, e->prm, e->d_qpar, e->d_q, e->d_p);
      break;
    case CR_PES_CH4OH:
    case CR_PES_GEH4OH:
      cr::init_children_kernel<21><<<(nb + 127) / 128, 128, 0, e->stream>>>(
          e->T, e->P, e->cfg.seed, e->cfg.traj0, e->prm, e->d_qpar, e->d_q, e->d_p);
      break;
    case CR_PES_OH3:
      cr::init_children_kernel<12><<<(nb + 127) / 128, 128, 0, e->stream>>>(
          e->T, e->P, e->cfg.seed, e->cfg.traj0, e->prm, e->d_qpar, e->d_q, e->d_p);
      break;
    default: return fail(CR_ERR_UNSUPPORTED, "PES not built");
  }
  CR_CUDA(cudaGetLastError());
  int rc = dispatch_forces(e);
  if (rc) return rc;
  const int tb = 128, gb = (e->T + tb - 1) / tb;
  switch (e->cfg.pes) {
    case CR_PES_H3:
    case CR_PES_BRH2:
      cr::child_flux_kernel<3><<<gb, tb, 0, e->stream>>>(e->T, e->P, e->prm, e->d_q, e->d_p, e->d_w, e->d_wpos);
      break;
    case CR_PES_CH4H:
      cr::child_flux_kernel<6><<<gb, tb, 0, e->stream>>>(e->T, e->P, e->prm, e->d_q, e->d_p, e->d_w, e->d_wpos);
      break;
    case CR_PES_CH4OH:
    case CR_PES_GEH4OH:
      cr::child_flux_kernel<7><<<gb, tb, 0, e->stream>>>(e->T, e->P, e->prm, e->d_q, e->d_p, e->d_w, e->d_wpos);
      break;
    case CR_PES_OH3:
      cr::child_flux_kernel<4><<<gb, tb, 0, e->stream>>>(e->T, e->P, e->prm, e->d_q, e->d_p, e->d_w, e->d_wpos);
      break;
    default: break;
  }
  CR_CUDA(cudaGetLastError());
  CR_CUDA(cudaMemsetAsync(e->d_side, 0, (size_t)e->T * e->side_cap, e->stream));
  CR_CUDA(cudaMemsetAsync(e->d_status, 0, (size_t)e->T * sizeof(int), e->stream));
  e->side_step0 = e->istep;
  e->prm.side_step0 = e->istep;
  CR_CUDA(cudaStreamSynchronize(e->stream));
  return CR_OK;
}

int cr_engine_kappa(cr_engine* e, double* num, double* denom, double* weights, int* nsteps) {
  if (!e || !num || !denom || !nsteps) return fail(CR_ERR_ARG, "NULL argument");
  if (!e->xi_on) return fail(CR_ERR_ARG, "no recrossing run in this engine");
  const int ns = e->istep - e->side_step0;
  *nsteps = ns;
  if (ns <= 0) {
    *denom = 0.0;
    return CR_OK;
  }
  cr::kappa_kernel<<<(ns + 1 + 127) / 128, 128, 0, e->stream>>>(e->T, ns, e->side_cap, e->d_side, e->d_w,
                                                                  e->d_wpos, e->d_kappa, e->d_kappa + ns);
  CR_CUDA(cudaGetLastError());
  CR_CUDA(cudaMemcpyAsync(num, e->d_kappa, (size_t)ns * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
  CR_CUDA(cudaMemcpyAsync(denom, e->d_kappa + ns, sizeof(double), cudaMemcpyDeviceToHost, e->stream));
  if (weights)
    CR_CUDA(cudaMemcpyAsync(weights, e->d_w, (size_t)e->T * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
  CR_CUDA(cudaStreamSynchronize(e->stream));
  return CR_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Batches: several engines (trajectory classes of different atom and bead
// counts, surfaces and precisions) stepped by one graph launch per chunk of
// steps.  Each engine's chunk is a branch of the graph on its own stream:
// a persistent analytic kernel (step index from the device counter) or the
// graph path's per-step kernels, so the classes fill the GPU together.
// ---------------------------------------------------------------------------
struct cr_batch {
  std::vector<cr_engine*> eng;
  int chunk = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t fork = nullptr, ev0 = nullptr, ev1 = nullptr;
  std::vector<cudaEvent_t> join;
  // timeline of a graph launch: t0 before the fork, each branch's first and
  // last node (timing events recorded inside the captured graph)
  cudaEvent_t t0 = nullptr;
  std::vector<cudaEvent_t> tb, te;
  struct Chunk {
    int len;
    int nodes;
    cudaGraph_t graph;
    cudaGraphExec_t exec;
  };
  std::vector<Chunk> graphs;
  long long launches = 0;  // kernels of the last cr_batch_run
  float last_ms = 0.f;
};

namespace {

int batch_prepare(cr_engine* e) {
  if (e->split) return split_prepare(e);
  return set_run_smem(e);
}

int batch_branch(cr_engine* e, int len) {
  if (e->split) {
    for (int n = 0; n < len; ++n) {
      int rc = split_step_launches(e);
      if (rc) return rc;
    }
    return CR_OK;
  }
  return launch_run(e, len, true);
}

cr_batch::Chunk* batch_graph(cr_batch* b, int len) {
  for (auto& c : b->graphs)
    if (c.len == len) return &c;
  if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    fail(CR_ERR_CUDA, "batch capture could not start");
    return nullptr;
  }
  // timing events as record nodes of the graph (External: recorded when the
  // graph runs, not turned into capture dependencies)
  int rc = (cudaEventRecordWithFlags(b->t0, b->stream, cudaEventRecordExternal) == cudaSuccess &&
            cudaEventRecord(b->fork, b->stream) == cudaSuccess)
               ? CR_OK
               : fail(CR_ERR_CUDA, "batch fork event failed");
  for (size_t i = 0; i < b->eng.size() && rc == CR_OK; ++i) {
    cr_engine* e = b->eng[i];
    if (cudaStreamWaitEvent(e->stream, b->fork, 0) != cudaSuccess ||
        cudaEventRecordWithFlags(b->tb[i], e->stream, cudaEventRecordExternal) != cudaSuccess) {
      rc = fail(CR_ERR_CUDA, "batch fork failed");
      break;
    }
    rc = batch_branch(e, len);
    if (rc == CR_OK && (cudaEventRecordWithFlags(b->te[i], e->stream, cudaEventRecordExternal) != cudaSuccess ||
                        cudaEventRecord(b->join[i], e->stream) != cudaSuccess ||
                        cudaStreamWaitEvent(b->stream, b->join[i], 0) != cudaSuccess))
      rc = fail(CR_ERR_CUDA, "batch join failed");
  }
  cudaGraph_t g = nullptr;
  cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
  if (rc != CR_OK || ce != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    if (rc == CR_OK) fail(CR_ERR_CUDA, std::string("batch capture: ") + cudaGetErrorString(ce));
    cudaGetLastError();
    return nullptr;
  }
  cr_batch::Chunk c{len, 0, g, nullptr};
  size_t nodes = 0;
  if (cudaGraphGetNodes(g, nullptr, &nodes) != cudaSuccess || cudaGraphInstantiate(&c.exec, g, 0) != cudaSuccess) {
    cudaGraphDestroy(g);
    fail(CR_ERR_CUDA, "batch graph instantiation failed");
    return nullptr;
  }
  // kernels only: the fork/join leave no nodes of their own; the timing
  // events are 1 + 2 per engine record nodes
  c.nodes = (int)nodes - (1 + 2 * (int)b->eng.size());
  b->graphs.push_back(c);
  return &b->graphs.back();
}

}  // namespace

extern "C" {

int cr_batch_create(cr_engine* const* engines, int nengines, int chunk_steps, cr_batch** out) {
  if (!out) return fail(CR_ERR_ARG, "NULL output handle");
  *out = nullptr;
  if (!engines || nengines < 1) return fail(CR_ERR_ARG, "a batch needs at least one engine");
  if (chunk_steps < 1) return fail(CR_ERR_ARG, "chunk_steps must be >= 1");
  for (int i = 0; i < nengines; ++i) {
    if (!engines[i]) return fail(CR_ERR_ARG, "NULL engine in the batch");
    for (int j = 0; j < i; ++j)
      if (engines[j] == engines[i]) return fail(CR_ERR_ARG, "an engine appears twice in the batch");
  }
  cr_batch* b = new cr_batch();
  b->eng.assign(engines, engines + nengines);
  b->chunk = chunk_steps;
  b->join.assign((size_t)nengines, nullptr);
  b->tb.assign((size_t)nengines, nullptr);
  b->te.assign((size_t)nengines, nullptr);
  bool ok = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) == cudaSuccess &&
            cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) == cudaSuccess &&
            cudaEventCreate(&b->ev0) == cudaSuccess && cudaEventCreate(&b->ev1) == cudaSuccess &&
            cudaEventCreate(&b->t0) == cudaSuccess;
  for (auto& ev : b->join) ok = ok && cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) == cudaSuccess;
  for (auto& ev : b->tb) ok = ok && cudaEventCreate(&ev) == cudaSuccess;
  for (auto& ev : b->te) ok = ok && cudaEventCreate(&ev) == cudaSuccess;
  if (!ok) {
    cr_batch_destroy(b);
    return fail(CR_ERR_CUDA, "batch stream or event creation failed");
  }
  *out = b;
  return CR_OK;
}

int cr_batch_destroy(cr_batch* b) {
  if (!b) return CR_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  for (auto& c : b->graphs) {
    if (c.exec) cudaGraphExecDestroy(c.exec);
    if (c.graph) cudaGraphDestroy(c.graph);
  }
  for (auto ev : b->join)
    if (ev) cudaEventDestroy(ev);
  for (auto ev : b->tb)
    if (ev) cudaEventDestroy(ev);
  for (auto ev : b->te)
    if (ev) cudaEventDestroy(ev);
  if (b->t0) cudaEventDestroy(b->t0);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return CR_OK;
}

int cr_batch_run(cr_batch* b, int nsteps) {
  if (!b) return fail(CR_ERR_ARG, "NULL batch");
  if (nsteps < 0) return fail(CR_ERR_ARG, "nsteps must be >= 0");
  for (cr_engine* e : b->eng)
    if (e->xi_on && e->istep + nsteps - e->side_step0 > e->side_cap)
      return fail(CR_ERR_ARG, "run exceeds the recrossing step capacity set by cr_engine_set_recross");
  if (nsteps == 0) return CR_OK;
  for (cr_engine* e : b->eng) {
    CR_CUDA(cudaStreamSynchronize(e->stream));  // work queued on the engine before the batch
    int rc = batch_prepare(e);
    if (rc) return rc;
    e->h_istep = e->istep;
    CR_CUDA(cudaMemcpyAsync(e->d_istep, &e->h_istep, sizeof(int), cudaMemcpyHostToDevice, b->stream));
  }
  const int full = nsteps / b->chunk, rem = nsteps % b->chunk;
  cr_batch::Chunk* cf = full ? batch_graph(b, b->chunk) : nullptr;
  if (full && !cf) return CR_ERR_CUDA;
  cr_batch::Chunk* cm = rem ? batch_graph(b, rem) : nullptr;
  if (rem && !cm) return CR_ERR_CUDA;
  CR_CUDA(cudaEventRecord(b->ev0, b->stream));
  for (int n = 0; n < full; ++n) CR_CUDA(cudaGraphLaunch(cf->exec, b->stream));
  if (rem) CR_CUDA(cudaGraphLaunch(cm->exec, b->stream));
  CR_CUDA(cudaEventRecord(b->ev1, b->stream));
  CR_CUDA(cudaStreamSynchronize(b->stream));
  CR_CUDA(cudaEventElapsedTime(&b->last_ms, b->ev0, b->ev1));
  b->launches = (long long)full * (cf ? cf->nodes : 0) + (cm ? cm->nodes : 0);
  int bad = 0;
  for (cr_engine* e : b->eng) {
    e->istep += nsteps;
    std::vector<int> st((size_t)e->T);
    CR_CUDA(cudaMemcpy(st.data(), e->d_status, st.size() * sizeof(int), cudaMemcpyDeviceToHost));
    for (int v : st) bad |= v;
  }
  if (bad) return fail(CR_ERR_TRAJECTORY, "a trajectory reported a non-finite coordinate or singular inertia");
  return CR_OK;
}

int cr_batch_timeline(const cr_batch* b, float* begin_ms, float* end_ms) {
  if (!b || !begin_ms || !end_ms) return fail(CR_ERR_ARG, "NULL argument");
  if (b->graphs.empty()) return fail(CR_ERR_ARG, "the batch has not run");
  for (size_t i = 0; i < b->eng.size(); ++i) {
    CR_CUDA(cudaEventElapsedTime(&begin_ms[i], b->t0, b->tb[i]));
    CR_CUDA(cudaEventElapsedTime(&end_ms[i], b->t0, b->te[i]));
  }
  return CR_OK;
}

int cr_batch_info(const cr_batch* b, long long* launches, int* graph_nodes, float* ms) {
  if (!b) return fail(CR_ERR_ARG, "NULL batch");
  if (launches) *launches = b->launches;
  if (graph_nodes) {
    *graph_nodes = 0;
    for (auto& c : b->graphs)
      if (c.len == b->chunk) *graph_nodes = c.nodes;
  }
  if (ms) *ms = b->last_ms;
  return CR_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Adjoint of the ring-polymer velocity-Verlet step (NVE, plain FP64, QMDFF):
// gradients of a loss L(q_K, p_K) at step K with respect to the force field's
// linear parameters and to the initial state, with checkpoints every `every`
// steps and the positions of one segment recomputed at a time.
//
// Forward step n:  p' = p_{n-1} - h g(q_{n-1});  (q_n, p'') = A (q_{n-1}, p');
//                  p_n = p'' - h g(q_n)          (h = dt/2, A the free ring
// polymer).  Reverse, from (lq, lp) = dL/d(q_K, p_K):
//   lq += -h H(q_K) lp                               (last half kick)
//   for n = K .. 1:  (lq, lp) <- A^T (lq, lp);
//                    lq += c H(q_{n-1}) lp,  c = -2h (n > 1: both half kicks
//                    at q_{n-1}), -h (n = 1)
// and the parameter gradient collects c d/dtheta (lp . g(q_m)) at each kick.
// A^T: K1, K2, K3 are symmetric, so A^T applied to (lq, lp) is A applied to
// (p := lq, q := lp) -- the forward drift kernel with swapped arrays and zero
// forces.
// ---------------------------------------------------------------------------
namespace cr {
__global__ void axpy_kernel(size_t n, double a, const double* x, double* y) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    y[i] = fma(a, x[i], y[i]);
}
}  // namespace cr

struct cr_adjoint {
  cr_engine* e = nullptr;
  int nsteps = 0, every = 0, nseg = 0, nlin = 0, scratch_beads = 0;
  size_t nall = 0;
  int istep0 = 0;
  bool forward_done = false;
  double* ck = nullptr;   // [nseg][3][nall]: q, p, f at the segment starts
  double* fin = nullptr;  // [3][nall]: the state after step K
  double* seg = nullptr;  // [every][nall]: positions of the current segment
  double *lq = nullptr, *lp = nullptr, *hw = nullptr, *zero = nullptr, *scratch = nullptr, *gacc = nullptr;
};

namespace {

int adj_copy_state(cr_engine* e, double* dst, bool to_engine) {
  const size_t b = (size_t)e->T * e->P * e->NC * sizeof(double);
  double* eng[3] = {e->d_q, e->d_p, e->d_f};
  for (int k = 0; k < 3; ++k) {
    double* x = dst + (size_t)k * (b / sizeof(double));
    CR_CUDA(cudaMemcpyAsync(to_engine ? eng[k] : x, to_engine ? x : eng[k], b, cudaMemcpyDeviceToDevice, e->stream));
  }
  return CR_OK;
}

int adj_axpy(cr_adjoint* a, double c, const double* x, double* y) {
  cr::axpy_kernel<<<1024, 256, 0, a->e->stream>>>(a->nall, c, x, y);
  CR_CUDA(cudaGetLastError());
  return CR_OK;
}

// lq += c H(q) lp;  gacc += c d/dtheta (lp . grad E(q))
int adj_kick(cr_adjoint* a, const double* q, double c) {
  cr_engine* e = a->e;
  const int nb = e->T * e->P;
  int rc = qmdff_hvp_launch(e->ff, q, a->lp, nb, nullptr, nullptr, a->hw, nullptr, e->stream);
  if (rc) return rc;
  if ((rc = adj_axpy(a, c, a->hw, a->lq))) return rc;
  return qmdff_vjp_launch(e->ff, q, a->lp, nb, nullptr, nullptr, c, a->scratch, a->scratch_beads, a->gacc, e->stream);
}

int adj_drift(cr_adjoint* a) {
  cr_engine* e = a->e;
  cr::SplitParams sp = e->sp;
  sp.p = a->lq;
  sp.q = a->lp;
  sp.f = a->zero;
  sp.thermostat = CR_THERMO_NONE;
  const int cw = cr::split_chunk(e->P);
  const dim3 grid((e->NC + cw - 1) / cw, e->T);
  cr::split_drift_kernel<<<grid, cr::kSplitBlock, e->smem_drift, e->stream>>>(sp);
  CR_CUDA(cudaGetLastError());
  return CR_OK;
}

}  // namespace

extern "C" {

int cr_adjoint_create(cr_engine* e, int nsteps, int every, cr_adjoint** out) {
  if (!out) return fail(CR_ERR_ARG, "NULL output handle");
  *out = nullptr;
  if (!e || nsteps < 1 || every < 1) return fail(CR_ERR_ARG, "adjoint needs an engine, nsteps >= 1, every >= 1");
  if (!e->ff || e->evb || !e->split) return fail(CR_ERR_UNSUPPORTED, "the adjoint is built for QMDFF engines");
  if (e->cfg.precision != CR_PREC_FP64) return fail(CR_ERR_UNSUPPORTED, "the adjoint runs the plain FP64 form");
  if (e->cfg.thermostat != CR_THERMO_NONE || e->cfg.transrot || e->parent || e->xi_on)
    return fail(CR_ERR_UNSUPPORTED, "the adjoint needs NVE steps without transrot, parent or recrossing");
  if (e->ff->nterm[4] > 0) return fail(CR_ERR_UNSUPPORTED, "second derivatives of H/halogen-bond terms are not built");
  cr_adjoint* a = new cr_adjoint();
  a->e = e;
  a->nsteps = nsteps;
  a->every = every;
  a->nseg = (nsteps + every - 1) / every;
  a->nlin = qmdff_nlin(e->ff);
  a->nall = (size_t)e->T * e->P * e->NC;
  a->scratch_beads = std::min(e->T * e->P, 4096);
  const size_t n = a->nall;
  bool ok = cudaMalloc(&a->ck, (size_t)a->nseg * 3 * n * 8) == cudaSuccess &&
            cudaMalloc(&a->fin, 3 * n * 8) == cudaSuccess && cudaMalloc(&a->seg, (size_t)every * n * 8) == cudaSuccess &&
            cudaMalloc(&a->lq, n * 8) == cudaSuccess && cudaMalloc(&a->lp, n * 8) == cudaSuccess &&
            cudaMalloc(&a->hw, n * 8) == cudaSuccess && cudaMalloc(&a->zero, n * 8) == cudaSuccess &&
            cudaMalloc(&a->scratch, (size_t)a->scratch_beads * std::max(a->nlin, 1) * 8) == cudaSuccess &&
            cudaMalloc(&a->gacc, (size_t)std::max(a->nlin, 1) * 8) == cudaSuccess &&
            cudaMemset(a->zero, 0, n * 8) == cudaSuccess;
  if (!ok) {
    cr_adjoint_destroy(a);
    return fail(CR_ERR_CUDA, "device allocation of the adjoint buffers failed");
  }
  *out = a;
  return CR_OK;
}

int cr_adjoint_destroy(cr_adjoint* a) {
  if (!a) return CR_OK;
  cudaFree(a->ck);
  cudaFree(a->fin);
  cudaFree(a->seg);
  cudaFree(a->lq);
  cudaFree(a->lp);
  cudaFree(a->hw);
  cudaFree(a->zero);
  cudaFree(a->scratch);
  cudaFree(a->gacc);
  delete a;
  return CR_OK;
}

int cr_adjoint_forward(cr_adjoint* a) {
  if (!a) return fail(CR_ERR_ARG, "NULL adjoint");
  cr_engine* e = a->e;
  a->istep0 = e->istep;
  for (int k = 0; k < a->nseg; ++k) {
    int rc = adj_copy_state(e, a->ck + (size_t)k * 3 * a->nall, false);
    if (rc) return rc;
    if ((rc = cr_engine_run(e, std::min(a->every, a->nsteps - k * a->every)))) return rc;
  }
  int rc = adj_copy_state(e, a->fin, false);
  if (rc) return rc;
  CR_CUDA(cudaStreamSynchronize(e->stream));
  a->forward_done = true;
  return CR_OK;
}

int cr_adjoint_backward(cr_adjoint* a, const double* dl_dq, const double* dl_dp, double* grad, double* dl_dq0,
                        double* dl_dp0) {
  if (!a || !dl_dq || !dl_dp || !grad) return fail(CR_ERR_ARG, "NULL argument");
  if (!a->forward_done) return fail(CR_ERR_ARG, "cr_adjoint_forward must run first");
  cr_engine* e = a->e;
  const size_t n = a->nall;
  const double h = 0.5 * e->cfg.dt;
  CR_CUDA(cudaMemcpyAsync(a->lq, dl_dq, n * 8, cudaMemcpyHostToDevice, e->stream));
  CR_CUDA(cudaMemcpyAsync(a->lp, dl_dp, n * 8, cudaMemcpyHostToDevice, e->stream));
  CR_CUDA(cudaMemsetAsync(a->gacc, 0, (size_t)std::max(a->nlin, 1) * 8, e->stream));
  int rc = adj_kick(a, a->fin, -h);  // the last half kick, at q_K
  if (rc) return rc;
  for (int k = a->nseg - 1; k >= 0; --k) {
    const int s0 = k * a->every, len = std::min(a->every, a->nsteps - s0);
    // recompute the segment's positions q_{s0} .. q_{s0+len-1}
    if ((rc = adj_copy_state(e, a->ck + (size_t)k * 3 * n, true))) return rc;
    e->istep = a->istep0 + s0;
    CR_CUDA(cudaMemcpyAsync(a->seg, e->d_q, n * 8, cudaMemcpyDeviceToDevice, e->stream));
    for (int i = 1; i < len; ++i) {
      if ((rc = cr_engine_run(e, 1))) return rc;
      CR_CUDA(cudaMemcpyAsync(a->seg + (size_t)i * n, e->d_q, n * 8, cudaMemcpyDeviceToDevice, e->stream));
    }
    for (int st = s0 + len; st > s0; --st) {
      if ((rc = adj_drift(a))) return rc;
      const int m = st - 1;
      if ((rc = adj_kick(a, a->seg + (size_t)(m - s0) * n, m > 0 ? -2.0 * h : -h))) return rc;
    }
  }
  // leave the engine in its state after step K
  if ((rc = adj_copy_state(e, a->fin, true))) return rc;
  e->istep = a->istep0 + a->nsteps;
  if (a->nlin) CR_CUDA(cudaMemcpyAsync(grad, a->gacc, (size_t)a->nlin * 8, cudaMemcpyDeviceToHost, e->stream));
  if (dl_dq0) CR_CUDA(cudaMemcpyAsync(dl_dq0, a->lq, n * 8, cudaMemcpyDeviceToHost, e->stream));
  if (dl_dp0) CR_CUDA(cudaMemcpyAsync(dl_dp0, a->lp, n * 8, cudaMemcpyDeviceToHost, e->stream));
  CR_CUDA(cudaStreamSynchronize(e->stream));
  return CR_OK;
}

}  // extern "C"

namespace cr {
const PesRuns* pes_runs(int pes) {
  switch (pes) {
    case CR_PES_H3: return &kRunsH3;
    case CR_PES_CH4H: return &kRunsCH4H;
    case CR_PES_CH4OH: return &kRunsCH4OH;
    case CR_PES_OH3: return &kRunsOH3;
    case CR_PES_GEH4OH: return &kRunsGeH4OH;
    case CR_PES_BRH2: return &kRunsBrH2;
    default: return nullptr;
  }
}
}  // namespace cr
