// dE-EVB of two QMDFFs: the cr_evb object and its C-ABI (cr_evb_*).
#include <cmath>
#include <string>
#include <vector>

#include "evb.cuh"
#include "host_util.h"
#include "qmdff_host.h"

struct cr_evb {
  cr_qmdff* ff1 = nullptr;
  cr_qmdff* ff2 = nullptr;
  cr::evb::Coupling C{};
};

// e, g <- EVB energy and gradient of nbeads beads; e2, g2 are scratch of the
// same sizes for the second force field.
int evb_launch(const cr_evb* evb, const double* d_q, int nbeads, double* d_e, double* d_g, double* d_e2,
               double* d_g2, int precision, cudaStream_t s) {
  int rc = qmdff_launch(evb->ff1, d_q, nbeads, d_e, d_g, precision, s);
  if (rc) return rc;
  rc = qmdff_launch(evb->ff2, d_q, nbeads, d_e2, d_g2, precision, s);
  if (rc) return rc;
  if (nbeads <= 0) return CR_OK;
  const int threads = 128;
  const long long nthreads = (long long)nbeads * 32;
  cr::evb::evb_combine_kernel<<<(unsigned)((nthreads + threads - 1) / threads), threads, 0, s>>>(
      evb->C, nbeads, 3 * evb->ff1->n, d_e, d_g, d_e2, d_g2);
  CR_TRY_CUDA(cudaGetLastError());
  return CR_OK;
}

cr_qmdff* evb_first(const cr_evb* evb) { return evb->ff1; }

namespace cr {
namespace evbfit {

// V12(dE) of a fit basis (src/lm_de_func.f90:57-177 parameter layout)
__device__ inline double fit_coupling(int basis, const double* x, double dE) {
  const double d2 = dE * dE;
  switch (basis) {
    case CR_FIT_1G: return x[0] * exp(-x[1] * d2);
    case CR_FIT_2G: return x[0] * exp(-x[1] * d2) + x[2] * exp(-x[3] * (dE + x[4]) * (dE + x[4]));
    case CR_FIT_3G:
      return x[0] * exp(-x[1] * d2) + x[2] * exp(-x[3] * (dE + x[6]) * (dE + x[6])) +
             x[4] * exp(-x[5] * (dE + x[7]) * (dE + x[7]));
    case CR_FIT_SP: return x[0] * exp(-x[1] * d2) + x[2] * dE * exp(-x[3] * d2);
    case CR_FIT_SD: return x[0] * exp(-x[1] * d2) + x[2] * d2 * exp(-x[3] * d2);
    case CR_FIT_SD2: return x[0] * exp(-x[1] * d2) + x[2] * d2 * exp(-x[3] * d2) + x[4] * d2 * exp(-x[5] * d2);
    case CR_FIT_SP2D:
      return x[0] * exp(-x[1] * d2) + x[2] * dE * exp(-x[3] * d2) + x[4] * dE * exp(-x[5] * d2) +
             x[6] * d2 * exp(-x[7] * d2);
    default:
      return x[0] * exp(-x[1] * d2) + x[2] * dE * exp(-x[3] * d2) + x[4] * dE * exp(-x[5] * d2) +
             x[6] * d2 * exp(-x[7] * d2) + x[8] * d2 * exp(-x[9] * d2) + x[10] * d2 * exp(-x[11] * d2);
  }
}

__device__ inline double fit_residual(int basis, const double* x, double e1, double e2, double eref) {
  const double dE = fabs(e1 - e2);
  const double v = fit_coupling(basis, x, dE);
  const double r = eref - 0.5 * (e1 + e2 - sqrt(dE * dE + 4.0 * v * v));
  return r * r;
}

// thread (i, j): j = 0 -> fvec[i]; j > 0 -> column j-1 of the forward
// differences with the parameter vector xp[j-1] (h[j-1] applied).
__global__ void fit_kernel(int basis, int npar, int m, const double* __restrict__ x, const double* __restrict__ xp,
                           const double* __restrict__ h, const double* __restrict__ e1, const double* __restrict__ e2,
                           const double* __restrict__ eref, double* fvec, double* fjac) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)m * (npar + 1)) return;
  const int i = (int)(idx % m), j = (int)(idx / m);
  const double f0 = fit_residual(basis, x, e1[i], e2[i], eref[i]);
  if (j == 0) {
    fvec[i] = f0;
    return;
  }
  const double w = fit_residual(basis, xp + (size_t)(j - 1) * npar, e1[i], e2[i], eref[i]);
  fjac[(size_t)(j - 1) * m + i] = (w - f0) / h[j - 1];
}

}  // namespace evbfit
}  // namespace cr

extern "C" {

int cr_evb_fit(int basis, const double* x, int npar, int m, const double* e1, const double* e2, const double* eref,
               double* fvec, double* fjac) {
  static const int kNpar[9] = {0, 2, 5, 8, 4, 4, 6, 8, 12};
  if (basis < CR_FIT_1G || basis > CR_FIT_SP2D3) return cr_set_error(CR_ERR_ARG, "unknown fit basis");
  if (npar != kNpar[basis]) return cr_set_error(CR_ERR_ARG, "parameter count does not match the basis");
  if (m < 0 || !x || (m > 0 && (!e1 || !e2 || !eref || !fvec))) return cr_set_error(CR_ERR_ARG, "bad fit arguments");
  if (m == 0) return CR_OK;
  // fdjac2 (src/lm_good.f:795-840): eps = sqrt(max(epsfcn = 0, epsmch))
  const double eps = std::sqrt(2.220446049250313e-16);
  std::vector<double> xp((size_t)npar * npar), h((size_t)npar);
  for (int j = 0; j < npar; ++j) {
    double hj = eps * std::fabs(x[j]);
    if (hj == 0.0) hj = eps;
    h[(size_t)j] = hj;
    for (int k = 0; k < npar; ++k) xp[(size_t)j * npar + k] = x[k];
    xp[(size_t)j * npar + j] = x[j] + hj;
  }
  const int cols = fjac ? npar : 0;
  double *d = nullptr;
  const size_t nx = (size_t)npar, nxp = xp.size(), nm = (size_t)m;
  const size_t total = nx + nxp + nx + 3 * nm + nm + (size_t)cols * nm;
  CR_TRY_CUDA(cudaMalloc(&d, total * sizeof(double)));
  double *dx = d, *dxp = dx + nx, *dh = dxp + nxp, *de1 = dh + nx, *de2 = de1 + nm, *der = de2 + nm,
         *dfv = der + nm, *dfj = dfv + nm;
  int rc = CR_OK;
  if (cudaMemcpy(dx, x, nx * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(dxp, xp.data(), nxp * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(dh, h.data(), nx * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(de1, e1, nm * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(de2, e2, nm * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(der, eref, nm * 8, cudaMemcpyHostToDevice) != cudaSuccess) {
    rc = cr_set_error(CR_ERR_CUDA, "upload of the fit data failed");
  } else {
    const long long n = (long long)m * (cols + 1);
    cr::evbfit::fit_kernel<<<(unsigned)((n + 127) / 128), 128>>>(basis, npar, m, dx, dxp, dh, de1, de2, der, dfv, dfj);
    if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess)
      rc = cr_set_error(CR_ERR_CUDA, "fit kernel failed");
    else if (cudaMemcpy(fvec, dfv, nm * 8, cudaMemcpyDeviceToHost) != cudaSuccess ||
             (fjac && cudaMemcpy(fjac, dfj, (size_t)cols * nm * 8, cudaMemcpyDeviceToHost) != cudaSuccess))
      rc = cr_set_error(CR_ERR_CUDA, "download of the fit results failed");
  }
  cudaFree(d);
  return rc;
}

int cr_evb_create(cr_qmdff* ff1, cr_qmdff* ff2, const cr_evb_def* def, cr_evb** out) {
  if (!ff1 || !ff2 || !def || !out) return cr_set_error(CR_ERR_ARG, "NULL argument");
  *out = nullptr;
  if (ff1->n != ff2->n) return cr_set_error(CR_ERR_ARG, "the two force fields need the same atoms");
  if (def->basis < CR_EVB_CONST || def->basis > CR_EVB_SP2D) return cr_set_error(CR_ERR_ARG, "unknown coupling basis");
  cr_evb* e = new cr_evb();
  e->ff1 = ff1;
  e->ff2 = ff2;
  e->C.basis = def->basis;
  e->C.a = def->a;
  e->C.b = def->b;
  e->C.c = def->c;
  e->C.d = def->d;
  e->C.e = def->e;
  e->C.f = def->f;
  e->C.g = def->g;
  e->C.h = def->h;
  e->C.m = def->m;
  e->C.n = def->n;
  *out = e;
  return CR_OK;
}

int cr_evb_destroy(cr_evb* evb) {
  delete evb;
  return CR_OK;
}

int cr_evb_egrad(cr_evb* evb, const double* xyz, int nbeads, double* e, double* g, int precision) {
  if (!evb) return cr_set_error(CR_ERR_ARG, "NULL EVB");
  if (nbeads < 0 || (nbeads > 0 && (!xyz || !e || !g))) return cr_set_error(CR_ERR_ARG, "bad egrad arguments");
  if (nbeads == 0) return CR_OK;
  const size_t nq = (size_t)3 * evb->ff1->n * nbeads;
  double *d_q = nullptr, *d_e = nullptr, *d_g = nullptr, *d_e2 = nullptr, *d_g2 = nullptr;
  int rc = CR_OK;
  if (cudaMalloc(&d_q, nq * 8) != cudaSuccess || cudaMalloc(&d_g, nq * 8) != cudaSuccess ||
      cudaMalloc(&d_g2, nq * 8) != cudaSuccess || cudaMalloc(&d_e, (size_t)nbeads * 8) != cudaSuccess ||
      cudaMalloc(&d_e2, (size_t)nbeads * 8) != cudaSuccess) {
    rc = cr_set_error(CR_ERR_CUDA, "cudaMalloc failed in cr_evb_egrad");
  } else if (cudaMemcpy(d_q, xyz, nq * 8, cudaMemcpyHostToDevice) != cudaSuccess) {
    rc = cr_set_error(CR_ERR_CUDA, "copy of xyz failed");
  } else if ((rc = evb_launch(evb, d_q, nbeads, d_e, d_g, d_e2, d_g2, precision, nullptr)) == CR_OK) {
    if (cudaMemcpy(e, d_e, (size_t)nbeads * 8, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(g, d_g, nq * 8, cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = cr_set_error(CR_ERR_CUDA, "copy of results failed");
  }
  cudaFree(d_q);
  cudaFree(d_e);
  cudaFree(d_g);
  cudaFree(d_e2);
  cudaFree(d_g2);
  return rc;
}

}  // extern "C"
