// Flexible SPC water box (csrc/water.cuh): the per-bead energy/gradient
// kernel, the host object behind cr_water_* (C-ABI) and its launch entry for
// the engine.
#include <algorithm>
#include <cmath>
#include <string>

#include "host_util.h"
#include "water_host.h"

namespace cr {

// One bead per CTA (grid-stride over beads), one thread per atom; shared
// memory: the bead's coordinates (3n doubles), the intramolecular gradient
// (3n doubles), the (hi, lo) split (3n float2, mixed form) and 32 doubles for
// the energy sum.
template <bool MIXED>
__global__ void __launch_bounds__(water::kMaxAtoms)
    water_egrad_kernel(water::Dev D, int nbeads, const double* q, double* e, double* g) {
  extern __shared__ double wsm[];
  const int n = D.n, n3 = 3 * n, tid = threadIdx.x;
  double* xs = wsm;
  double* gi = xs + n3;
  float2* hl = reinterpret_cast<float2*>(gi + n3);
  double* red = reinterpret_cast<double*>(hl + n3);
  for (int b = blockIdx.x; b < nbeads; b += gridDim.x) {
    const double* qb = q + (size_t)b * n3;
    for (int k = tid; k < n3; k += blockDim.x) {
      const double v = qb[k];
      xs[k] = v;
      gi[k] = 0.0;
      if (MIXED) {
        const float h = __double2float_rn(v);
        hl[k] = make_float2(h, __double2float_rn(v - (double)h));
      }
    }
    __syncthreads();
    double en = 0.0;
    if (tid < D.nwater) en = water::intra(D, xs, tid, gi);
    __syncthreads();
    if (tid < n) {
      double f[3] = {gi[3 * tid], gi[3 * tid + 1], gi[3 * tid + 2]};
      en += MIXED ? water::pairs_mixed(D, xs, hl, tid, f) : water::pairs_plain(D, xs, tid, f);
      double* gb = g + (size_t)b * n3 + 3 * tid;
      gb[0] = f[0];
      gb[1] = f[1];
      gb[2] = f[2];
    }
    // energy: warp shuffles, then the warps in order (deterministic)
    for (int o = 16; o >= 1; o >>= 1) en += __shfl_down_sync(0xffffffffu, en, o);
    if ((tid & 31) == 0) red[tid >> 5] = en;
    __syncthreads();
    if (tid == 0) {
      double s = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
      e[b] = s;
    }
    __syncthreads();
  }
}

}  // namespace cr

namespace {

size_t water_smem(int n) { return (size_t)3 * n * (8 + 8 + 8) + 32 * 8; }

}  // namespace

int water_launch(const cr_water* w, const double* d_q, int nbeads, double* d_e, double* d_g, int precision,
                 cudaStream_t s) {
  if (precision != CR_PREC_MIXED && precision != CR_PREC_FP64) return cr_set_error(CR_ERR_ARG, "unknown precision");
  const size_t smem = water_smem(w->dev.n);
  auto kern = precision == CR_PREC_MIXED ? cr::water_egrad_kernel<true> : cr::water_egrad_kernel<false>;
  if (smem > 48 * 1024) CR_TRY_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  if (nbeads <= 0) return CR_OK;
  const int threads = (w->dev.n + 31) / 32 * 32;
  const int grid = std::min(nbeads, 1 << 20);
  kern<<<grid, threads, smem, s>>>(w->dev, nbeads, d_q, d_e, d_g);
  CR_TRY_CUDA(cudaGetLastError());
  return CR_OK;
}

extern "C" {

int cr_water_create(const cr_water_def* d, cr_water** out) {
  if (!d || !out) return cr_set_error(CR_ERR_ARG, "NULL argument");
  *out = nullptr;
  if (d->nwater < 1 || 3 * d->nwater > cr::water::kMaxAtoms)
    return cr_set_error(CR_ERR_ARG, "nwater must be 1..341");
  if (d->periodic) {
    for (int k = 0; k < 3; ++k)
      if (!(d->box[k] > 0.0 && std::isfinite(d->box[k]))) return cr_set_error(CR_ERR_ARG, "box lengths must be > 0");
    if (!(d->coul_cut > 0.0)) return cr_set_error(CR_ERR_ARG, "a periodic box needs coul_cut > 0");
  }
  cr_water* w = new cr_water();
  cr::water::Dev& D = w->dev;
  // src/water_init.f90:74-103 (bohr, hartree of src/general.f90:256-257;
  // k_rr and epsilon_OO are REAL(4) literals there)
  const double bohr = 0.52917721092, hartree = 627.5094743;
  D.nwater = d->nwater;
  D.n = 3 * d->nwater;
  D.periodic = d->periodic ? 1 : 0;
  D.zahn = d->zahn ? 1 : 0;
  for (int k = 0; k < 3; ++k) {
    D.len[k] = d->periodic ? d->box[k] : 0.0;
    D.half[k] = D.len[k] * 0.5;
    D.flen[k] = (float)D.len[k];
    D.fhalf[k] = (float)D.half[k];
  }
  D.coul_cut = d->coul_cut;
  D.zahn_a = d->zahn_a;
  D.zahn_par = d->zahn_par;
  D.r0 = 1.0 / bohr;
  D.r0hh = 1.633 / bohr;
  D.de = 101.9188 / hartree;
  D.a = 2.567 * bohr;
  D.ktheta = 328.645606 / hartree * bohr * bohr;
  D.krtheta = -211.4672 / hartree * bohr * bohr;
  D.krr = (double)111.70765f / hartree * bohr * bohr;
  D.eh = 0.41;
  D.eo = -0.82;
  D.sigma = 3.166 / bohr;
  D.eps = (double)0.1554f / hartree;
  D.fcut = (float)D.coul_cut;
  D.fzahn_a = (float)D.zahn_a;
  D.fzahn_par = (float)D.zahn_par;
  D.feh = (float)D.eh;
  D.feo = (float)D.eo;
  D.fsigma = (float)D.sigma;
  D.feps = (float)D.eps;
  *out = w;
  return CR_OK;
}

int cr_water_destroy(cr_water* w) {
  delete w;
  return CR_OK;
}

int cr_water_egrad(const cr_water* w, const double* q, int nbeads, double* V, double* dVdq, int precision) {
  if (!w || !q || !V || !dVdq) return cr_set_error(CR_ERR_ARG, "NULL argument");
  if (nbeads < 0) return cr_set_error(CR_ERR_ARG, "nbeads must be >= 0");
  if (nbeads == 0) return CR_OK;
  const size_t n3 = (size_t)3 * w->dev.n, bytes = n3 * nbeads * sizeof(double);
  double *dq = nullptr, *dV = nullptr, *dg = nullptr;
  int rc = CR_OK;
  if (cudaMalloc(&dq, bytes) != cudaSuccess || cudaMalloc(&dV, (size_t)nbeads * 8) != cudaSuccess ||
      cudaMalloc(&dg, bytes) != cudaSuccess) {
    rc = cr_set_error(CR_ERR_CUDA, "device allocation failed");
  } else if (cudaMemcpy(dq, q, bytes, cudaMemcpyHostToDevice) != cudaSuccess) {
    rc = cr_set_error(CR_ERR_CUDA, "copy in failed");
  } else if ((rc = water_launch(w, dq, nbeads, dV, dg, precision, nullptr)) == CR_OK) {
    if (cudaMemcpy(V, dV, (size_t)nbeads * 8, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(dVdq, dg, bytes, cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = cr_set_error(CR_ERR_CUDA, "copy out failed");
  }
  cudaFree(dq);
  cudaFree(dV);
  cudaFree(dg);
  return rc;
}

int cr_water_natoms(const cr_water* w) { return w ? w->dev.n : -1; }

}  // extern "C"
