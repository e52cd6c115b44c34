// QMDFF force field: host set-up (parameter tables, the warp term schedule)
// and the per-bead energy/gradient kernel behind cr_qmdff_* (C-ABI).
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "host_util.h"
#include "qmdff_host.h"

namespace {

using cr::qmdff::kVAngl;
using cr::qmdff::kVPair;

// Term schedule of one kind: batches of 32 lanes; within a batch, terms of
// one colour touch disjoint atoms.  Greedy: each colour takes, in order, the
// remaining terms that do not touch an atom already used by that colour,
// until the batch holds 32 terms or has max_colours colours.  Every colour
// costs one scatter round of the warp while an unfilled lane wastes a whole
// term evaluation; on C20H42 the mixed form is fastest with at most 3
// colours for bonds, 4 for angles and 6 for torsions (2.99 -> 2.66 ms per
// 65 536 beads against 1 / 2 / 2: two colours left torsion batches half
// empty); pairs use schedule_pairs.
void schedule_kind(int nterm, int arity, int max_colours, const std::vector<int>& atoms,
                   const std::vector<int>& order, int natoms, std::vector<int>& slot,
                   std::vector<unsigned char>& color, std::vector<unsigned char>& ncol, int& nbatch,
                   int& colours) {
  std::vector<int> remaining = order;
  std::vector<int> stamp((size_t)natoms, -1);
  int stamp_id = 0;
  nbatch = 0;
  while (!remaining.empty()) {
    std::vector<int> bt, bc;
    int col = 0;
    while ((int)bt.size() < 32 && !remaining.empty() && col < max_colours) {
      ++stamp_id;
      std::vector<int> rest;
      rest.reserve(remaining.size());
      for (int t : remaining) {
        bool ok = (int)bt.size() < 32;
        for (int a = 0; ok && a < arity; ++a)
          if (stamp[(size_t)atoms[(size_t)t * arity + a]] == stamp_id) ok = false;
        if (!ok) {
          rest.push_back(t);
          continue;
        }
        for (int a = 0; a < arity; ++a) stamp[(size_t)atoms[(size_t)t * arity + a]] = stamp_id;
        bt.push_back(t);
        bc.push_back(col);
      }
      remaining.swap(rest);
      ++col;
    }
    for (int l = 0; l < 32; ++l) {
      slot.push_back(l < (int)bt.size() ? bt[(size_t)l] : -1);
      color.push_back((unsigned char)(l < (int)bc.size() ? bc[(size_t)l] : 0));
    }
    ncol.push_back((unsigned char)col);
    colours += col;
    ++nbatch;
  }
  (void)nterm;
}

// Pair terms: the circle method splits all atom pairs of n atoms (n even; a
// dummy atom for odd n) into n-1 perfect matchings; the pairs of one
// matching touch disjoint atoms, so each matching is one single-colour batch
// (split in 32-lane pieces when n > 64).
void schedule_pairs(int nterm, const std::vector<int>& atoms, int natoms, std::vector<int>& slot,
                    std::vector<unsigned char>& color, std::vector<unsigned char>& ncol, int& nbatch,
                    int& colours) {
  const int m = natoms + (natoms & 1);  // players, even
  std::vector<std::vector<int>> rounds((size_t)(m > 1 ? m - 1 : 1));
  for (int t = 0; t < nterm; ++t) {
    int i = atoms[(size_t)2 * t], j = atoms[(size_t)2 * t + 1];
    if (i > j) std::swap(i, j);
    // round r holds (r, m-1) and the pairs (r + k, r - k) mod (m-1), i.e. the
    // pairs with i + j = 2r (mod m-1); m/2 is the inverse of 2 modulo m-1
    const int r = (j == m - 1) ? i : (int)(((long long)(i + j) * (m / 2)) % (m - 1));
    rounds[(size_t)r].push_back(t);
  }
  nbatch = 0;
  for (const auto& rd : rounds) {
    for (size_t k0 = 0; k0 < rd.size(); k0 += 32) {
      for (int l = 0; l < 32; ++l) {
        const size_t k = k0 + (size_t)l;
        slot.push_back(k < rd.size() ? rd[k] : -1);
        color.push_back(0);
      }
      ncol.push_back(1);
      colours += 1;
      ++nbatch;
    }
  }
}

template <class T>
int upload(cr_qmdff* ff, const std::vector<T>& h, const T** d) {
  *d = nullptr;
  if (h.empty()) return CR_OK;
  void* p = nullptr;
  CR_TRY_CUDA(cudaMalloc(&p, h.size() * sizeof(T)));
  ff->allocs.push_back(p);
  CR_TRY_CUDA(cudaMemcpy(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
  *d = (const T*)p;
  return CR_OK;
}

template <class T>
std::vector<float> to_float(const std::vector<T>& v) {
  std::vector<float> o(v.size());
  for (size_t i = 0; i < v.size(); ++i) o[i] = (float)v[i];
  return o;
}

}  // namespace

namespace cr {

// MINB: blocks of kQmdffWarps warps kept resident per SM (the register cap
// follows: 65536 / (MINB * 128) per thread).  The FP64 form trades spills for
// occupancy differently from the mixed form; the autotuner below picks.
template <bool MIXED, int MINB, int MODE = qmdff::kFree>
__global__ void __launch_bounds__(kQmdffWarps * 32, MINB)
    qmdff_egrad_kernel(qmdff::Dev D, int nbeads, const double* q, double* e, double* g) {
  extern __shared__ double qsm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n3 = 3 * D.n;
  double* ws = qsm + (size_t)warp * (qmdff::warp_smem_bytes(D.n) / sizeof(double));
  for (int b = blockIdx.x * kQmdffWarps + warp; b < nbeads; b += gridDim.x * kQmdffWarps) {
    const double* qb = q + (size_t)b * n3;
    for (int a = lane; a < n3; a += 32) ws[a] = qb[a];
    __syncwarp();
    const double v = qmdff::warp_egrad<MIXED, MODE>(D, ws, g + (size_t)b * n3, 1.0, lane, b);
    if (lane == 0) e[b] = v;
    __syncwarp();
  }
}

// Energy, gradient and Hessian-vector product H w per bead (plain form, dual
// coordinates); dew[b] = w . grad E.
__global__ void __launch_bounds__(kQmdffWarps * 32)
    qmdff_hvp_kernel(qmdff::Dev D, int nbeads, const double* q, const double* w, double* e, double* g, double* hw,
                     double* dew) {
  extern __shared__ double qsm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n3 = 3 * D.n;
  double* ws = qsm + (size_t)warp * (qmdff::warp_hvp_smem_bytes(D.n) / sizeof(double));
  for (int b = blockIdx.x * kQmdffWarps + warp; b < nbeads; b += gridDim.x * kQmdffWarps) {
    const double* qb = q + (size_t)b * n3;
    const double* wb = w + (size_t)b * n3;
    for (int a = lane; a < n3; a += 32) {
      ws[a] = qb[a];
      ws[n3 + a] = wb[a];
    }
    __syncwarp();
    double de = 0.0;
    const double v = qmdff::warp_hvp(D, ws, g ? g + (size_t)b * n3 : nullptr, hw + (size_t)b * n3, de, lane);
    if (lane == 0) {
      if (e) e[b] = v;
      if (dew) dew[b] = de;
    }
    __syncwarp();
  }
}

// Per bead b and linear parameter t: out[b][t] = alpha_b (v_b . grad E_t|unit)
// + beta_b E_t|unit (alpha = 1, beta = 0 where the weights are NULL).
__global__ void __launch_bounds__(kQmdffWarps * 32)
    qmdff_vjp_kernel(qmdff::Dev D, qmdff::Tables<double> U, int nbeads, int nlin, const double* q, const double* v,
                     const double* alpha, const double* beta, double* out) {
  extern __shared__ double qsm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n3 = 3 * D.n;
  double* xs = qsm + (size_t)warp * 2 * n3;
  double* vs = xs + n3;
  for (int b = blockIdx.x * kQmdffWarps + warp; b < nbeads; b += gridDim.x * kQmdffWarps) {
    for (int a = lane; a < n3; a += 32) {
      xs[a] = q[(size_t)b * n3 + a];
      vs[a] = v[(size_t)b * n3 + a];
    }
    __syncwarp();
    qmdff::warp_param_vjp(D, U, xs, vs, alpha ? alpha[b] : 1.0, beta ? beta[b] : 0.0, out + (size_t)b * nlin, lane);
    __syncwarp();
  }
}

// acc[t] += scale * sum_b in[b][t], the beads summed in order (deterministic).
__global__ void sum_rows_kernel(int nrows, int ncols, const double* in, double scale, double* acc) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ncols) return;
  double s = 0.0;
  for (int r = 0; r < nrows; ++r) s += in[(size_t)r * ncols + t];
  acc[t] += scale * s;
}

}  // namespace cr

int qmdff_hvp_launch(const cr_qmdff* ff, const double* d_q, const double* d_w, int nbeads, double* d_e, double* d_g,
                     double* d_hw, double* d_dew, cudaStream_t s) {
  if (ff->nterm[4] > 0) return cr_set_error(CR_ERR_UNSUPPORTED, "second derivatives of H/halogen-bond terms are not built");
  const size_t smem = (size_t)kQmdffWarps * cr::qmdff::warp_hvp_smem_bytes(ff->n);
  CR_TRY_CUDA(cudaFuncSetAttribute(cr::qmdff_hvp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  if (nbeads == 0) return CR_OK;
  int grid = (nbeads + kQmdffWarps - 1) / kQmdffWarps;
  if (grid > 1 << 20) grid = 1 << 20;
  cr::qmdff_hvp_kernel<<<grid, kQmdffWarps * 32, smem, s>>>(ff->dev, nbeads, d_q, d_w, d_e, d_g, d_hw, d_dew);
  CR_TRY_CUDA(cudaGetLastError());
  return CR_OK;
}

int qmdff_nlin(const cr_qmdff* ff) { return ff->nterm[0] + ff->nterm[1] + ff->nterm[2] + ff->nterm[3]; }

int qmdff_vjp_launch(const cr_qmdff* ff, const double* d_q, const double* d_v, int nbeads, const double* d_alpha,
                     const double* d_beta, double scale, double* d_scratch, int scratch_beads, double* d_acc,
                     cudaStream_t s) {
  if (ff->nterm[4] > 0) return cr_set_error(CR_ERR_UNSUPPORTED, "parameter gradients of H/halogen-bond terms are not built");
  const int nlin = qmdff_nlin(ff);
  const size_t smem = (size_t)kQmdffWarps * 2 * 3 * ff->n * sizeof(double);
  CR_TRY_CUDA(cudaFuncSetAttribute(cr::qmdff_vjp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  if (nlin == 0) return CR_OK;
  const size_t n3 = (size_t)3 * ff->n;
  for (int b0 = 0; b0 < nbeads; b0 += scratch_beads) {
    const int nb = std::min(scratch_beads, nbeads - b0);
    const int grid = (nb + kQmdffWarps - 1) / kQmdffWarps;
    cr::qmdff_vjp_kernel<<<grid, kQmdffWarps * 32, smem, s>>>(ff->dev, ff->unit, nb, nlin, d_q + b0 * n3, d_v + b0 * n3,
                                                              d_alpha ? d_alpha + b0 : nullptr,
                                                              d_beta ? d_beta + b0 : nullptr, d_scratch);
    CR_TRY_CUDA(cudaGetLastError());
    cr::sum_rows_kernel<<<(nlin + 127) / 128, 128, 0, s>>>(nb, nlin, d_scratch, scale, d_acc);
    CR_TRY_CUDA(cudaGetLastError());
  }
  return CR_OK;
}

namespace {

using QmdffKernel = void (*)(cr::qmdff::Dev, int, const double*, double*, double*);
constexpr int kVariants = 3;
// [precision][variant]: blocks per SM 2 / 3 / 4 (FP64), 4 / 5 / 6 (mixed)
const QmdffKernel kKernels[2][kVariants] = {
    {cr::qmdff_egrad_kernel<false, 2>, cr::qmdff_egrad_kernel<false, 3>, cr::qmdff_egrad_kernel<false, 4>},
    {cr::qmdff_egrad_kernel<true, 4>, cr::qmdff_egrad_kernel<true, 5>, cr::qmdff_egrad_kernel<true, 6>}};
constexpr int kDefaultVariant = 1;
// the force field's periodic box, and NpT (per-trajectory boxes and the
// virial): one variant per form each
const QmdffKernel kBoxKernels[2] = {cr::qmdff_egrad_kernel<false, 3, cr::qmdff::kBox>,
                                    cr::qmdff_egrad_kernel<true, 5, cr::qmdff::kBox>};
const QmdffKernel kNptKernels[2] = {cr::qmdff_egrad_kernel<false, 3, cr::qmdff::kNpt>,
                                    cr::qmdff_egrad_kernel<true, 5, cr::qmdff::kNpt>};
constexpr int kTuneMinBeads = 2048;  // smaller batches keep the default

int launch_dev(const cr::qmdff::Dev& D, int prec, int v, const double* d_q, int nbeads, double* d_e, double* d_g,
               cudaStream_t s) {
  const size_t smem = (size_t)kQmdffWarps * cr::qmdff::warp_smem_bytes(D.n);
  int grid = (nbeads + kQmdffWarps - 1) / kQmdffWarps;
  if (grid > 1 << 20) grid = 1 << 20;
  const QmdffKernel k = D.periodic ? kBoxKernels[prec] : kKernels[prec][v];
  k<<<grid, kQmdffWarps * 32, smem, s>>>(D, nbeads, d_q, d_e, d_g);
  CR_TRY_CUDA(cudaGetLastError());
  return CR_OK;
}

int launch_variant(const cr_qmdff* ff, int prec, int v, const double* d_q, int nbeads, double* d_e, double* d_g,
                   cudaStream_t s) {
  return launch_dev(ff->dev, prec, v, d_q, nbeads, d_e, d_g, s);
}

// The NpT instantiation with the launch's boxes and virial array.
int launch_npt(const cr_qmdff* ff, int prec, const QmdffNpt& npt, const double* d_q, int nbeads, double* d_e,
               double* d_g, cudaStream_t s) {
  cr::qmdff::Dev D = ff->dev;
  D.tbox = npt.tbox;
  D.tbox_beads = npt.beads_per_box;
  D.vir = npt.vir;
  const size_t smem = (size_t)kQmdffWarps * cr::qmdff::warp_smem_bytes(D.n);
  if (smem > 48 * 1024)
    CR_TRY_CUDA(cudaFuncSetAttribute(kNptKernels[prec], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  if (nbeads <= 0) return CR_OK;
  int grid = (nbeads + kQmdffWarps - 1) / kQmdffWarps;
  if (grid > 1 << 20) grid = 1 << 20;
  kNptKernels[prec]<<<grid, kQmdffWarps * 32, smem, s>>>(D, nbeads, d_q, d_e, d_g);
  CR_TRY_CUDA(cudaGetLastError());
  return CR_OK;
}

// The force kernel over a subset of the term kinds (bit k of mask: kind k =
// bonds, angles, torsions, NCI pairs, H/halogen bonds), with or without
// E_zero: the pieces of Caracal's QMDFF call site (src/gradient.f90:341-358).
// The masked kinds' batch counts are set to zero in a copy of the schedule.
int qmdff_launch_kinds(const cr_qmdff* ff, unsigned mask, bool ezero, const double* d_q, int nbeads, double* d_e,
                       double* d_g, int precision, cudaStream_t s) {
  if (precision != CR_PREC_MIXED && precision != CR_PREC_FP64) return cr_set_error(CR_ERR_ARG, "unknown precision");
  const int prec = precision == CR_PREC_MIXED ? 1 : 0;
  const size_t smem = (size_t)kQmdffWarps * cr::qmdff::warp_smem_bytes(ff->n);
  if (smem > 48 * 1024) {
    for (int v = 0; v < kVariants; ++v)
      CR_TRY_CUDA(cudaFuncSetAttribute(kKernels[prec][v], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    CR_TRY_CUDA(cudaFuncSetAttribute(kBoxKernels[prec], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  }
  if (nbeads <= 0) return CR_OK;
  cr::qmdff::Dev D = ff->dev;
  for (int p = 0; p < 2; ++p)
    for (int k = 0; k < cr::qmdff::kKinds; ++k)
      if (!((mask >> k) & 1u)) D.sched[p].nb[k] = 0;
  if (!ezero) D.e_zero = 0.0;
  const int v = ff->variant[prec] >= 0 ? ff->variant[prec] : kDefaultVariant;
  return launch_dev(D, prec, v, d_q, nbeads, d_e, d_g, s);
}

// Host-array call of a kind subset: e, g overwritten, or accumulated into.
int qmdff_host_kinds(cr_qmdff* ff, unsigned mask, bool ezero, bool accumulate, const double* xyz, int nbeads,
                     double* e, double* g, int precision) {
  if (!ff) return cr_set_error(CR_ERR_ARG, "NULL force field");
  if (nbeads < 0 || (nbeads > 0 && (!xyz || !e || !g))) return cr_set_error(CR_ERR_ARG, "bad egrad arguments");
  if (nbeads == 0) return CR_OK;
  const size_t nq = (size_t)3 * ff->n * nbeads;
  double *d_q = nullptr, *d_e = nullptr, *d_g = nullptr;
  CR_TRY_CUDA(cudaMalloc(&d_q, nq * sizeof(double)));
  cudaError_t e1 = cudaMalloc(&d_e, (size_t)nbeads * sizeof(double));
  cudaError_t e2 = cudaMalloc(&d_g, nq * sizeof(double));
  std::vector<double> pe, pg;
  int rc = CR_OK;
  if (e1 != cudaSuccess || e2 != cudaSuccess) {
    rc = cr_set_error(CR_ERR_CUDA, "cudaMalloc failed in the QMDFF term call");
  } else if (cudaMemcpy(d_q, xyz, nq * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) {
    rc = cr_set_error(CR_ERR_CUDA, "copy of xyz failed");
  } else if ((rc = qmdff_launch_kinds(ff, mask, ezero, d_q, nbeads, d_e, d_g, precision, nullptr)) == CR_OK) {
    double* oe = e;
    double* og = g;
    if (accumulate) {
      pe.resize((size_t)nbeads);
      pg.resize(nq);
      oe = pe.data();
      og = pg.data();
    }
    if (cudaMemcpy(oe, d_e, (size_t)nbeads * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(og, d_g, nq * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) {
      rc = cr_set_error(CR_ERR_CUDA, "copy of results failed");
    } else if (accumulate) {
      for (int b = 0; b < nbeads; ++b) e[b] += pe[(size_t)b];
      for (size_t x = 0; x < nq; ++x) g[x] += pg[x];
    }
  }
  cudaFree(d_q);
  cudaFree(d_e);
  cudaFree(d_g);
  return rc;
}

}  // namespace

// Autotuner: the first launch with at least kTuneMinBeads beads outside a
// stream capture runs one untimed warm-up launch, then times every variant
// once on the caller's data (each writes the same outputs) and keeps the
// fastest for this force field and form.
int qmdff_launch(const cr_qmdff* ff_c, const double* d_q, int nbeads, double* d_e, double* d_g, int precision,
                 cudaStream_t s, const QmdffNpt* npt) {
  cr_qmdff* ff = const_cast<cr_qmdff*>(ff_c);
  if (precision != CR_PREC_MIXED && precision != CR_PREC_FP64) return cr_set_error(CR_ERR_ARG, "unknown precision");
  const int prec = precision == CR_PREC_MIXED ? 1 : 0;
  if (npt) return launch_npt(ff, prec, *npt, d_q, nbeads, d_e, d_g, s);
  const size_t smem = (size_t)kQmdffWarps * cr::qmdff::warp_smem_bytes(ff->n);
  // the attribute is set even for nbeads = 0, so a caller can prepare the
  // kernels before a stream capture
  if (smem > 48 * 1024) {
    for (int v = 0; v < kVariants; ++v)
      CR_TRY_CUDA(cudaFuncSetAttribute(kKernels[prec][v], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    CR_TRY_CUDA(cudaFuncSetAttribute(kBoxKernels[prec], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  }
  if (nbeads <= 0) return CR_OK;
  int choice = ff->variant[prec];
  if (choice < 0) {
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    CR_TRY_CUDA(cudaStreamIsCapturing(s, &cap));
    if (nbeads >= kTuneMinBeads && cap == cudaStreamCaptureStatusNone) {
      cudaEvent_t a, b;
      CR_TRY_CUDA(cudaEventCreate(&a));
      CR_TRY_CUDA(cudaEventCreate(&b));
      float best = 0.f;
      // one untimed launch first: the first launch of a kernel pays for
      // module load and cold caches, which would count against variant 0
      int rc0 = launch_variant(ff, prec, 0, d_q, nbeads, d_e, d_g, s);
      if (rc0) {
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        return rc0;
      }
      for (int v = 0; v < kVariants; ++v) {
        cudaEventRecord(a, s);
        int rc = launch_variant(ff, prec, v, d_q, nbeads, d_e, d_g, s);
        if (rc) {
          cudaEventDestroy(a);
          cudaEventDestroy(b);
          return rc;
        }
        cudaEventRecord(b, s);
        CR_TRY_CUDA(cudaEventSynchronize(b));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        ff->tune_ms[prec][v] = ms;
        if (v == 0 || ms < best) {
          best = ms;
          choice = v;
        }
      }
      cudaEventDestroy(a);
      cudaEventDestroy(b);
      ff->variant[prec] = choice;
      return CR_OK;  // the last variant's outputs equal the chosen one's
    }
    choice = kDefaultVariant;
  }
  return launch_variant(ff, prec, choice, d_q, nbeads, d_e, d_g, s);
}

extern "C" {

int cr_qmdff_destroy(cr_qmdff* ff) {
  if (!ff) return CR_OK;
  for (void* p : ff->allocs) cudaFree(p);
  delete ff;
  return CR_OK;
}

int cr_qmdff_create(const cr_qmdff_def* d, cr_qmdff** out) {
  if (!d || !out) return cr_set_error(CR_ERR_ARG, "NULL argument");
  *out = nullptr;
  const int n = d->natoms;
  if (n < 1 || n > cr::qmdff::kMaxAtoms) return cr_set_error(CR_ERR_ARG, "natoms must be 1..1024");
  if (d->nbond < 0 || d->nangl < 0 || d->ntors < 0 || d->nnci < 0)
    return cr_set_error(CR_ERR_ARG, "negative term count");
  if (!d->at || !d->q || !d->rad || (d->nbond && (!d->bond || !d->vbond)) || (d->nangl && (!d->angl || !d->vangl)) ||
      (d->ntors && (!d->tors || !d->vtors)) ||
      (d->nnci && (!d->nci || !d->r0ab || !d->zab || !d->r0094 || !d->sr42 || !d->c66ab)))
    return cr_set_error(CR_ERR_ARG, "missing force-field array");
  for (int i = 0; i < n; ++i)
    if (d->at[i] < 1 || d->at[i] > 94) return cr_set_error(CR_ERR_ARG, "element number out of 1..94");
  auto atom_ok = [&](int a) { return a >= 1 && a <= n; };
  for (int m = 0; m < 2 * d->nbond; ++m)
    if (!atom_ok(d->bond[m])) return cr_set_error(CR_ERR_ARG, "bond atom out of range");
  for (int m = 0; m < 3 * d->nangl; ++m)
    if (!atom_ok(d->angl[m])) return cr_set_error(CR_ERR_ARG, "angle atom out of range");
  for (int m = 0; m < d->ntors; ++m) {
    for (int a = 0; a < 4; ++a)
      if (!atom_ok(d->tors[6 * m + a])) return cr_set_error(CR_ERR_ARG, "torsion atom out of range");
    const int nt = d->tors[6 * m + 4];
    if (d->tors[6 * m + 5] != 2 && (nt < 0 || nt > 4)) return cr_set_error(CR_ERR_ARG, "torsion term count not 0..4");
  }
  for (int m = 0; m < d->nnci; ++m) {
    if (!atom_ok(d->nci[3 * m]) || !atom_ok(d->nci[3 * m + 1])) return cr_set_error(CR_ERR_ARG, "NCI atom out of range");
    if (d->nci[3 * m + 2] < 1 || d->nci[3 * m + 2] > 6) return cr_set_error(CR_ERR_ARG, "NCI category not 1..6");
  }
  if (d->nhb < 0 || (d->nhb > 0 && (!d->hb || !d->vhb))) return cr_set_error(CR_ERR_ARG, "missing H-bond arrays");
  for (int m = 0; m < 3 * d->nhb; ++m)
    if (!atom_ok(d->hb[m])) return cr_set_error(CR_ERR_ARG, "H-bond atom out of range");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return cr_set_error(CR_ERR_NO_DEVICE, "no CUDA device");

  const double pi = 3.1415926535897932384626433832795029;
  std::vector<double> rad((size_t)n), vbond(d->vbond, d->vbond + 3 * d->nbond), vtors(d->vtors, d->vtors + 14 * d->ntors);
  for (int i = 0; i < n; ++i) rad[(size_t)i] = d->rad[d->at[i] - 1];
  std::vector<double> vangl((size_t)kVAngl * d->nangl);
  for (int m = 0; m < d->nangl; ++m) {
    const double th0 = d->vangl[2 * m];
    vangl[(size_t)kVAngl * m] = th0;
    vangl[(size_t)kVAngl * m + 1] = d->vangl[2 * m + 1];
    vangl[(size_t)kVAngl * m + 2] = std::cos(th0);
    vangl[(size_t)kVAngl * m + 3] = (pi - th0 < 1e-6) ? 1.0 : 0.0;
  }
  std::vector<int> bond((size_t)2 * d->nbond), angl((size_t)3 * d->nangl), tors((size_t)6 * d->ntors),
      pair((size_t)2 * d->nnci);
  for (int m = 0; m < 2 * d->nbond; ++m) bond[(size_t)m] = d->bond[m] - 1;
  for (int m = 0; m < 3 * d->nangl; ++m) angl[(size_t)m] = d->angl[m] - 1;
  for (int m = 0; m < d->ntors; ++m) {
    for (int a = 0; a < 4; ++a) tors[(size_t)6 * m + a] = d->tors[6 * m + a] - 1;
    tors[(size_t)6 * m + 4] = d->tors[6 * m + 4];
    tors[(size_t)6 * m + 5] = d->tors[6 * m + 5];
  }
  std::vector<double> vpair((size_t)kVPair * d->nnci, 0.0);
  for (int m = 0; m < d->nnci; ++m) {
    const int i1 = d->nci[3 * m] - 1, i2 = d->nci[3 * m + 1] - 1, nk = d->nci[3 * m + 2];
    pair[(size_t)2 * m] = i1;
    pair[(size_t)2 * m + 1] = i2;
    const int z1 = d->at[i1] - 1, z2 = d->at[i2] - 1;
    const size_t e12 = (size_t)z1 + 94 * (size_t)z2;  // (iz1, iz2) column-major
    double* v = &vpair[(size_t)kVPair * m];
    v[0] = d->r0094[e12];
    v[1] = d->c66ab[(size_t)i2 + (size_t)n * i1];     // c66ab(i2, i1)
    v[2] = d->sr42[e12];
    v[3] = d->zab[e12];
    v[4] = d->r0ab[e12];
    v[5] = d->eps2[nk - 1];
    v[6] = d->zahn ? d->q[i1] * d->q[i2] : d->q[i1] * d->q[i2] * d->eps1[nk - 1];
  }

  // H/halogen bonds: A, B, H (0-based) and the kind (src/ff_hb.f90:71-78)
  std::vector<int> hb((size_t)4 * d->nhb);
  std::vector<double> vhb(d->vhb, d->vhb + 2 * d->nhb);
  for (int m = 0; m < d->nhb; ++m) {
    for (int a = 0; a < 3; ++a) hb[(size_t)4 * m + a] = d->hb[3 * m + a] - 1;
    hb[(size_t)4 * m + 3] = d->at[d->hb[3 * m + 2] - 1] == 1 ? 1 : 2;
  }

  cr_qmdff* ff = new cr_qmdff();
  ff->n = n;
  ff->nterm[0] = d->nbond;
  ff->nterm[1] = d->nangl;
  ff->nterm[2] = d->ntors;
  ff->nterm[3] = d->nnci;
  ff->nterm[4] = d->nhb;

  // schedules (plain, mixed): torsions grouped by (type, nt) so a batch runs
  // one code path
  std::vector<int> slot[2];
  std::vector<unsigned char> color[2], ncol[2];
  cr::qmdff::Dev& D = ff->dev;
  D.n = n;
  bool distinct = true;
  for (int form = 0; form < 2; ++form) {
    int boff = 0;
    for (int kind = 0; kind < cr::qmdff::kKinds; ++kind) {
      std::vector<int> order((size_t)ff->nterm[kind]);
      for (int m = 0; m < ff->nterm[kind]; ++m) order[(size_t)m] = m;
      std::vector<int> atoms;
      int arity = 2;
      if (kind == 0) atoms = bond;
      if (kind == 1) {
        arity = 3;
        atoms = angl;
      }
      if (kind == 2) {
        arity = 4;
        atoms.resize((size_t)4 * d->ntors);
        for (int m = 0; m < d->ntors; ++m)
          for (int a = 0; a < 4; ++a) atoms[(size_t)4 * m + a] = tors[(size_t)6 * m + a];
        std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
          const int kx = tors[(size_t)6 * x + 5] * 8 + tors[(size_t)6 * x + 4];
          const int ky = tors[(size_t)6 * y + 5] * 8 + tors[(size_t)6 * y + 4];
          return kx < ky;
        });
      }
      if (kind == 3) atoms = pair;
      if (kind == 4) {
        arity = 3;
        atoms.resize((size_t)3 * d->nhb);
        for (int m = 0; m < d->nhb; ++m)
          for (int a = 0; a < 3; ++a) atoms[(size_t)3 * m + a] = hb[(size_t)4 * m + a];
      }
      int nb = 0;
      int* colours = form == 1 ? &ff->ncolors : &ff->ncolors_fp64;
      if (form == 1 && kind == 3) {
        schedule_pairs(ff->nterm[kind], atoms, n, slot[form], color[form], ncol[form], nb, *colours);
      } else {
        const int max_colours = form == 0 ? 255 : (kind == 0 ? 3 : kind == 1 ? 4 : kind == 2 ? 6 : 2);
        schedule_kind(ff->nterm[kind], arity, max_colours, atoms, order, n, slot[form], color[form], ncol[form], nb,
                      *colours);
      }
      if (form == 0)
        for (int m = 0; m < ff->nterm[kind]; ++m)
          for (int x = 0; x < arity; ++x)
            for (int y = x + 1; y < arity; ++y)
              if (atoms[(size_t)m * arity + x] == atoms[(size_t)m * arity + y]) distinct = false;
      D.sched[form].nb[kind] = nb;
      D.sched[form].boff[kind] = boff;
      boff += nb;
    }
  }

  int rc = CR_OK;
  auto up = [&](auto& h, auto** dp) {
    if (rc == CR_OK) rc = upload(ff, h, dp);
  };
  for (int form = 0; form < 2; ++form) {
    up(slot[form], &D.sched[form].slot);
    up(color[form], &D.sched[form].color);
    up(ncol[form], &D.sched[form].ncol);
  }
  up(bond, &D.bond);
  up(angl, &D.angl);
  up(tors, &D.tors);
  up(pair, &D.pair);
  up(hb, &D.hb);
  up(vhb, &D.vhb);
  up(rad, &D.d.rad);
  up(vbond, &D.d.vbond);
  up(vangl, &D.d.vangl);
  up(vtors, &D.d.vtors);
  up(vpair, &D.d.vpair);
  std::vector<float> frad = to_float(rad), fvbond = to_float(vbond), fvangl = to_float(vangl),
                     fvtors = to_float(vtors), fvpair = to_float(vpair);
  up(frad, &D.f.rad);
  up(fvbond, &D.f.vbond);
  up(fvangl, &D.f.vangl);
  up(fvtors, &D.f.vtors);
  up(fvpair, &D.f.vpair);
  // mixed-form pair constants (pair_mixed)
  std::vector<float> fpair((size_t)kVPair * d->nnci);
  for (int m = 0; m < d->nnci; ++m) {
    const double* v = &vpair[(size_t)kVPair * m];
    float* o = &fpair[(size_t)kVPair * m];
    const double R02 = v[0] * v[0], R06 = R02 * R02 * R02;
    o[0] = (float)R06;
    o[1] = (float)(R06 * R02);
    o[2] = (float)(v[5] * v[1]);
    o[3] = (float)(v[5] * v[1] * v[2]);
    o[4] = (float)(v[5] * v[3]);
    o[5] = (float)(v[4] * 1.4426950408889634074);  // log2(e)
    o[6] = (float)v[6];
    o[7] = (float)v[4];
  }
  up(fpair, &D.fpair);
  if (rc != CR_OK) {
    cr_qmdff_destroy(ff);
    return rc;
  }
  D.coul_cut = d->coul_cut;
  D.zahn = d->zahn ? 1 : 0;
  D.zahn_a = d->zahn_a;
  D.zahn_par = d->zahn_par;
  D.fcoul_cut = (float)d->coul_cut;
  D.fzahn_a = (float)d->zahn_a;
  D.fzahn_par = (float)d->zahn_par;
  D.e_zero = d->e_zero;
  D.distinct = distinct ? 1 : 0;
  for (int k = 0; k < cr::qmdff::kKinds; ++k) D.nterm[k] = ff->nterm[k];
  // mixed form bond polynomial: a k u (1 - u) / r^2 = t H(t), t = r^2/r0^2 - 1,
  // H(t) = (a k / r0^2) [(1+t)^-(a/4+1) - (1+t)^-(a/2+1)] / t interpolated
  // at 48 Chebyshev nodes of |t| <= kBondSerMaxT, truncated to degree 23 and
  // written as a monomial in x = t / kBondSerMaxT; bonds with exponents
  // outside (0, 20] keep the FP32 formula
  {
    using cr::qmdff::kBondPoly;
    using cr::qmdff::kBondSer;
    const double T = cr::qmdff::kBondSerMaxT;
    const int nn = 48;
    std::vector<float2> bser((size_t)kBondSer * std::max(d->nbond, 1), make_float2(0.f, 0.f));
    auto split = [](double v) {
      const float hi = (float)v;
      return make_float2(hi, (float)(v - (double)hi));
    };
    for (int m = 0; m < d->nbond; ++m) {
      const double r0 = vbond[(size_t)3 * m], kk = vbond[(size_t)3 * m + 1], aa = vbond[(size_t)3 * m + 2];
      float2* row = &bser[(size_t)kBondSer * m];
      row[0] = split(1.0 / (r0 * r0));
      row[1] = split(r0 * r0);
      if (!(aa > 0.0) || aa > 20.0 || !(r0 > 0.0)) continue;
      const double p1 = aa / 4.0 + 1.0, p2 = aa / 2.0 + 1.0, scale = aa * kk / (r0 * r0);
      std::vector<double> hv((size_t)nn), cheb((size_t)kBondPoly, 0.0);
      for (int k = 0; k < nn; ++k) {
        const double xk = std::cos(pi * (k + 0.5) / nn), tk = T * xk;
        hv[(size_t)k] = (std::pow(1.0 + tk, -p1) - std::pow(1.0 + tk, -p2)) / tk;
      }
      for (int j = 0; j < kBondPoly; ++j) {
        double acc = 0.0;
        for (int k = 0; k < nn; ++k) acc += hv[(size_t)k] * std::cos(pi * j * (k + 0.5) / nn);
        cheb[(size_t)j] = (j == 0 ? 1.0 : 2.0) * acc / nn;
      }
      // Chebyshev -> monomial in x: T_0 = 1, T_1 = x, T_{j+1} = 2x T_j - T_{j-1}
      std::vector<double> tm1((size_t)kBondPoly, 0.0), t0((size_t)kBondPoly, 0.0), mono((size_t)kBondPoly, 0.0);
      tm1[0] = 1.0;
      if (kBondPoly > 1) t0[1] = 1.0;
      for (int j = 0; j < kBondPoly; ++j) {
        const std::vector<double>& tj = j == 0 ? tm1 : t0;
        for (int n = 0; n < kBondPoly; ++n) mono[(size_t)n] += cheb[(size_t)j] * tj[(size_t)n];
        if (j >= 1 && j + 1 < kBondPoly) {
          std::vector<double> tn((size_t)kBondPoly, 0.0);
          for (int n = 0; n + 1 < kBondPoly; ++n) tn[(size_t)n + 1] += 2.0 * t0[(size_t)n];
          for (int n = 0; n < kBondPoly; ++n) tn[(size_t)n] -= tm1[(size_t)n];
          tm1 = t0;
          t0 = tn;
        }
      }
      row[2] = make_float2(1.0f, 0.0f);
      for (int n = 0; n < kBondPoly; ++n) row[3 + n] = split(scale * mono[(size_t)n]);
    }
    up(bser, &D.bser);
  }
  // unit tables of the linear parameters (parameter gradients)
  std::vector<double> ubond = vbond, uangl = vangl, utors = vtors, upair = vpair;
  for (int m = 0; m < d->nbond; ++m) ubond[(size_t)3 * m + 1] = 1.0;
  for (int m = 0; m < d->nangl; ++m) uangl[(size_t)kVAngl * m + 1] = 1.0;
  for (int m = 0; m < d->ntors; ++m) utors[(size_t)14 * m + 1] = 1.0;
  for (int m = 0; m < d->nnci; ++m) {
    upair[(size_t)kVPair * m + 5] = 0.0;
    upair[(size_t)kVPair * m + 6] = 1.0;
  }
  ff->unit.rad = D.d.rad;
  up(ubond, &ff->unit.vbond);
  up(uangl, &ff->unit.vangl);
  up(utors, &ff->unit.vtors);
  up(upair, &ff->unit.vpair);
  if (rc != CR_OK) {
    cr_qmdff_destroy(ff);
    return rc;
  }
  *out = ff;
  return CR_OK;
}

int cr_qmdff_set_periodic(cr_qmdff* ff, const double* box_ang, double coul_cut_ang, double vdw_cut_ang,
                          double* cuts) {
  if (!ff) return cr_set_error(CR_ERR_ARG, "NULL force field");
  cr::qmdff::Dev& D = ff->dev;
  if (!box_ang) {
    D.periodic = 0;
    return CR_OK;
  }
  for (int k = 0; k < 3; ++k)
    if (!(box_ang[k] > 0.0)) return cr_set_error(CR_ERR_ARG, "box edges must be positive (Angstrom)");
  if (!(coul_cut_ang > 0.0) || !(vdw_cut_ang > 0.0)) return cr_set_error(CR_ERR_ARG, "cutoffs must be positive");
  // set_periodic (src/set_periodic.f90:67-113)
  const double bohr = 0.52917721092;
  double len[3];
  for (int k = 0; k < 3; ++k) len[k] = box_ang[k] / bohr;
  D.box = cr::qmdff::make_box(len);
  const double hmin = std::min(D.box.half[0], std::min(D.box.half[1], D.box.half[2]));
  double coul = coul_cut_ang / bohr;
  if (coul < 5.0) coul = hmin - 0.1;
  if (D.zahn) {
    const double spi = std::sqrt(3.14159265358979323846);
    D.zahn_a = 0.2 * bohr;
    coul = 10.0 / bohr;
    const double acut = D.zahn_a * coul;
    D.zahn_par = std::erfc(acut) / (coul * coul) + 2 * D.zahn_a / spi * std::exp(-acut * acut) / coul;
  }
  if (coul > hmin) coul = hmin - 0.1;
  D.coul_cut = coul;
  D.vdw_cut = vdw_cut_ang / bohr;
  D.fcoul_cut = (float)D.coul_cut;
  D.fvdw_cut = (float)D.vdw_cut;
  D.fzahn_a = (float)D.zahn_a;
  D.fzahn_par = (float)D.zahn_par;
  D.periodic = 1;
  if (cuts) {
    cuts[0] = D.coul_cut;
    cuts[1] = D.vdw_cut;
    cuts[2] = D.zahn_a;
    cuts[3] = D.zahn_par;
  }
  return CR_OK;
}

int cr_qmdff_schedule_info(const cr_qmdff* ff, int* batches, int* colors) {
  if (!ff) return cr_set_error(CR_ERR_ARG, "NULL force field");
  if (batches)
    for (int k = 0; k < cr::qmdff::kKinds; ++k) batches[k] = ff->dev.sched[1].nb[k];
  if (colors) *colors = ff->ncolors;
  return CR_OK;
}

int cr_qmdff_tuning(const cr_qmdff* ff, int precision, int* variant, float* ms) {
  if (!ff) return cr_set_error(CR_ERR_ARG, "NULL force field");
  if (precision != CR_PREC_MIXED && precision != CR_PREC_FP64) return cr_set_error(CR_ERR_ARG, "unknown precision");
  const int prec = precision == CR_PREC_MIXED ? 1 : 0;
  if (variant) *variant = ff->variant[prec];
  if (ms)
    for (int v = 0; v < kVariants; ++v) ms[v] = ff->tune_ms[prec][v];
  return CR_OK;
}

int cr_qmdff_egrad_device(cr_qmdff* ff, const double* d_xyz, int nbeads, double* d_e, double* d_g, int precision,
                          void* stream) {
  if (!ff) return cr_set_error(CR_ERR_ARG, "NULL force field");
  if (nbeads < 0 || (nbeads > 0 && (!d_xyz || !d_e || !d_g))) return cr_set_error(CR_ERR_ARG, "bad egrad arguments");
  return qmdff_launch(ff, d_xyz, nbeads, d_e, d_g, precision, (cudaStream_t)stream);
}

int cr_qmdff_egrad(cr_qmdff* ff, const double* xyz, int nbeads, double* e, double* g, int precision) {
  if (!ff) return cr_set_error(CR_ERR_ARG, "NULL force field");
  if (nbeads < 0 || (nbeads > 0 && (!xyz || !e || !g))) return cr_set_error(CR_ERR_ARG, "bad egrad arguments");
  if (nbeads == 0) return CR_OK;
  const size_t nq = (size_t)3 * ff->n * nbeads;
  double *d_q = nullptr, *d_e = nullptr, *d_g = nullptr;
  CR_TRY_CUDA(cudaMalloc(&d_q, nq * sizeof(double)));
  cudaError_t e1 = cudaMalloc(&d_e, (size_t)nbeads * sizeof(double));
  cudaError_t e2 = cudaMalloc(&d_g, nq * sizeof(double));
  int rc = CR_OK;
  if (e1 != cudaSuccess || e2 != cudaSuccess) {
    rc = cr_set_error(CR_ERR_CUDA, "cudaMalloc failed in cr_qmdff_egrad");
  } else if (cudaMemcpy(d_q, xyz, nq * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) {
    rc = cr_set_error(CR_ERR_CUDA, "copy of xyz failed");
  } else if ((rc = qmdff_launch(ff, d_q, nbeads, d_e, d_g, precision, nullptr)) == CR_OK) {
    if (cudaMemcpy(e, d_e, (size_t)nbeads * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(g, d_g, nq * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = cr_set_error(CR_ERR_CUDA, "copy of results failed");
  }
  cudaFree(d_q);
  cudaFree(d_e);
  cudaFree(d_g);
  return rc;
}

int cr_qmdff_egrad_virial(cr_qmdff* ff, const double* xyz, int nbeads, const double* box, double* e, double* g,
                          double* vir, int precision) {
  if (!ff) return cr_set_error(CR_ERR_ARG, "NULL force field");
  if (!ff->dev.periodic) return cr_set_error(CR_ERR_ARG, "the virial is formed for periodic force fields (NpT)");
  if (nbeads < 0 || (nbeads > 0 && (!xyz || !e || !g || !vir))) return cr_set_error(CR_ERR_ARG, "bad egrad arguments");
  if (precision != CR_PREC_MIXED && precision != CR_PREC_FP64) return cr_set_error(CR_ERR_ARG, "unknown precision");
  if (nbeads == 0) return CR_OK;
  const size_t nq = (size_t)3 * ff->n * nbeads, nb = (size_t)nbeads;
  std::vector<double> hb(3 * nb);
  for (size_t b = 0; b < nb; ++b)
    for (int k = 0; k < 3; ++k) hb[3 * b + k] = box ? box[3 * b + k] : ff->dev.box.len[k];
  double *d_q = nullptr, *d_e = nullptr, *d_g = nullptr, *d_b = nullptr, *d_w = nullptr;
  int rc = CR_OK;
  if (cudaMalloc(&d_q, nq * sizeof(double)) != cudaSuccess || cudaMalloc(&d_e, nb * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&d_g, nq * sizeof(double)) != cudaSuccess || cudaMalloc(&d_b, 3 * nb * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&d_w, nb * sizeof(double)) != cudaSuccess) {
    rc = cr_set_error(CR_ERR_CUDA, "cudaMalloc failed in cr_qmdff_egrad_virial");
  } else if (cudaMemcpy(d_q, xyz, nq * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
             cudaMemcpy(d_b, hb.data(), 3 * nb * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) {
    rc = cr_set_error(CR_ERR_CUDA, "copy of xyz failed");
  } else {
    const QmdffNpt np{d_b, 1, d_w};
    if ((rc = qmdff_launch(ff, d_q, nbeads, d_e, d_g, precision, nullptr, &np)) == CR_OK &&
        (cudaMemcpy(e, d_e, nb * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess ||
         cudaMemcpy(g, d_g, nq * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess ||
         cudaMemcpy(vir, d_w, nb * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess))
      rc = cr_set_error(CR_ERR_CUDA, "copy of results failed");
  }
  cudaFree(d_q);
  cudaFree(d_e);
  cudaFree(d_g);
  cudaFree(d_b);
  cudaFree(d_w);
  return rc;
}

int cr_qmdff_eg(cr_qmdff* ff, const double* xyz, int nbeads, double* e, double* g, int precision) {
  return qmdff_host_kinds(ff, 0x7u, false, false, xyz, nbeads, e, g, precision);
}

int cr_qmdff_nonb(cr_qmdff* ff, const double* xyz, int nbeads, double* e, double* g, int precision) {
  return qmdff_host_kinds(ff, 0x8u, false, true, xyz, nbeads, e, g, precision);
}

int cr_qmdff_hb(cr_qmdff* ff, const double* xyz, int nbeads, double* e, double* g, int precision) {
  return qmdff_host_kinds(ff, 0x10u, false, true, xyz, nbeads, e, g, precision);
}

int cr_qmdff_nparams(const cr_qmdff* ff, int* nlin) {
  if (!ff || !nlin) return cr_set_error(CR_ERR_ARG, "NULL argument");
  *nlin = qmdff_nlin(ff);
  return CR_OK;
}

int cr_qmdff_hvp(cr_qmdff* ff, const double* xyz, const double* w, int nbeads, double* e, double* g, double* hw) {
  if (!ff) return cr_set_error(CR_ERR_ARG, "NULL force field");
  if (nbeads < 0 || (nbeads > 0 && (!xyz || !w || !hw))) return cr_set_error(CR_ERR_ARG, "bad hvp arguments");
  if (ff->nterm[4] > 0) return cr_set_error(CR_ERR_UNSUPPORTED, "second derivatives of H/halogen-bond terms are not built");
  if (nbeads == 0) return CR_OK;
  const size_t nq = (size_t)3 * ff->n * nbeads;
  double* d = nullptr;
  CR_TRY_CUDA(cudaMalloc(&d, (4 * nq + nbeads) * sizeof(double)));
  double *dq = d, *dw = dq + nq, *dg = dw + nq, *dh = dg + nq, *de = dh + nq;
  int rc = CR_OK;
  if (cudaMemcpy(dq, xyz, nq * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(dw, w, nq * 8, cudaMemcpyHostToDevice) != cudaSuccess)
    rc = cr_set_error(CR_ERR_CUDA, "copy of the hvp inputs failed");
  else if ((rc = qmdff_hvp_launch(ff, dq, dw, nbeads, de, dg, dh, nullptr, nullptr)) == CR_OK &&
           (cudaMemcpy(hw, dh, nq * 8, cudaMemcpyDeviceToHost) != cudaSuccess ||
            (g && cudaMemcpy(g, dg, nq * 8, cudaMemcpyDeviceToHost) != cudaSuccess) ||
            (e && cudaMemcpy(e, de, (size_t)nbeads * 8, cudaMemcpyDeviceToHost) != cudaSuccess)))
    rc = cr_set_error(CR_ERR_CUDA, "copy of the hvp results failed");
  cudaFree(d);
  return rc;
}

int cr_qmdff_param_vjp(cr_qmdff* ff, const double* xyz, const double* v, int nbeads, double* grad) {
  if (!ff) return cr_set_error(CR_ERR_ARG, "NULL force field");
  if (nbeads < 0 || !grad || (nbeads > 0 && (!xyz || !v))) return cr_set_error(CR_ERR_ARG, "bad vjp arguments");
  if (ff->nterm[4] > 0) return cr_set_error(CR_ERR_UNSUPPORTED, "parameter gradients of H/halogen-bond terms are not built");
  const int nlin = qmdff_nlin(ff);
  for (int t = 0; t < nlin; ++t) grad[t] = 0.0;
  if (nbeads == 0 || nlin == 0) return CR_OK;
  const size_t nq = (size_t)3 * ff->n * nbeads;
  const int chunk = std::min(nbeads, 4096);
  double* d = nullptr;
  CR_TRY_CUDA(cudaMalloc(&d, (2 * nq + (size_t)chunk * nlin + nlin) * sizeof(double)));
  double *dq = d, *dv = dq + nq, *ds = dv + nq, *dacc = ds + (size_t)chunk * nlin;
  int rc = CR_OK;
  if (cudaMemcpy(dq, xyz, nq * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(dv, v, nq * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(dacc, 0, (size_t)nlin * 8) != cudaSuccess)
    rc = cr_set_error(CR_ERR_CUDA, "copy of the vjp inputs failed");
  else if ((rc = qmdff_vjp_launch(ff, dq, dv, nbeads, nullptr, nullptr, 1.0, ds, chunk, dacc, nullptr)) == CR_OK &&
           cudaMemcpy(grad, dacc, (size_t)nlin * 8, cudaMemcpyDeviceToHost) != cudaSuccess)
    rc = cr_set_error(CR_ERR_CUDA, "copy of the vjp result failed");
  cudaFree(d);
  return rc;
}

}  // extern "C"
