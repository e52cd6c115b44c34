// dE-EVB of two QMDFFs: the cr_evb object and its C-ABI (cr_evb_*).
#include <algorithm>
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

// V12(dE) of a fit basis (src/lm_de_func.f90:57-177 parameter layout); T is
// double or a dual number (analytic parameter gradients).
template <class T>
__device__ inline T fit_coupling(int basis, const T* x, double dE) {
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

template <class T>
__device__ inline T fit_residual(int basis, const T* x, double e1, double e2, double eref) {
  const double dE = fabs(e1 - e2);
  const T v = fit_coupling(basis, x, dE);
  const T r = eref - 0.5 * (e1 + e2 - sqrt(dE * dE + 4.0 * v * v));
  return r * r;
}

// Analytic gradient of sum_i fvec_i: thread i writes d fvec_i / d x_j for all
// j (dual numbers, one parameter seeded at a time) into out[i][npar].
__global__ void fit_grad_kernel(int basis, int npar, int m, const double* __restrict__ x,
                                const double* __restrict__ e1, const double* __restrict__ e2,
                                const double* __restrict__ eref, double* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  Dual xd[12];
  for (int j = 0; j < npar; ++j) {
    for (int k = 0; k < npar; ++k) xd[k] = Dual(x[k], k == j ? 1.0 : 0.0);
    out[(size_t)i * npar + j] = fit_residual<Dual>(basis, xd, e1[i], e2[i], eref[i]).d;
  }
}

// out[t] = sum_r in[r][t] in order (deterministic)
__global__ void column_sums_kernel(int nrows, int ncols, const double* in, double* out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ncols) return;
  double s = 0.0;
  for (int r = 0; r < nrows; ++r) s += in[(size_t)r * ncols + t];
  out[t] = s;
}

// thread (i, j): j = 0 -> fvec[i]; j > 0 -> column j-1 of the forward
// differences with the parameter vector xp[j-1] (h[j-1] applied).
__global__ void fit_kernel(int basis, int npar, int m, const double* __restrict__ x, const double* __restrict__ xp,
                           const double* __restrict__ h, const double* __restrict__ e1, const double* __restrict__ e2,
                           const double* __restrict__ eref, double* fvec, double* fjac) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)m * (npar + 1)) return;
  const int i = (int)(idx % m), j = (int)(idx / m);
  const double f0 = fit_residual<double>(basis, x, e1[i], e2[i], eref[i]);
  if (j == 0) {
    fvec[i] = f0;
    return;
  }
  const double w = fit_residual<double>(basis, xp + (size_t)(j - 1) * npar, e1[i], e2[i], eref[i]);
  fjac[(size_t)(j - 1) * m + i] = (w - f0) / h[j - 1];
}

// Per bead b: s1 = v . g1, s2 = v . g2 (one warp per bead), then the
// coupling-parameter derivatives of v . g_EVB, g_EVB = (g1 + g2 - Q (g1 - g2))/2,
// Q = K / sqrt(dE^2 + 4 V12^2): d(v . g)/dc_j = -(s1 - s2) dQ/dc_j / 2 into
// out[b][10] (c = a..h, m, n), and the weights of the first force field's
// parameter gradient: alpha = (1 - Q)/2 on v . dg1/dtheta, beta =
// -(s1 - s2) dQ/ddE / 2 on dE1/dtheta.
__global__ void evb_vjp_kernel(evb::Coupling C, int nbeads, int n3, const double* e1, const double* g1,
                               const double* e2, const double* g2, const double* v, double* out, double* alpha,
                               double* beta) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= nbeads) return;
  const double* a = g1 + (size_t)warp * n3;
  const double* b = g2 + (size_t)warp * n3;
  const double* w = v + (size_t)warp * n3;
  double s1 = 0.0, s2 = 0.0;
  for (int k = lane; k < n3; k += 32) {
    s1 += w[k] * a[k];
    s2 += w[k] * b[k];
  }
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
    s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    s2 += __shfl_xor_sync(0xffffffffu, s2, o);
  }
  if (lane != 0) return;
  const double ediff = e1[warp] - e2[warp], s12 = s1 - s2;
  const double c0[10] = {C.a, C.b, C.c, C.d, C.e, C.f, C.g, C.h, C.m, C.n};
  Dual c[10];
  for (int j = 0; j <= 10; ++j) {
    // j < 10: seed parameter j; j == 10: seed dE
    for (int k = 0; k < 10; ++k) c[k] = Dual(c0[k], k == j ? 1.0 : 0.0);
    const Dual de(ediff, j == 10 ? 1.0 : 0.0);
    Dual off, K;
    evb::coupling_t<Dual>(C.basis, c, de, off, K);
    const Dual Q = K / sqrt(de * de + 4.0 * off * off);
    if (j < 10) {
      out[(size_t)warp * 10 + j] = -0.5 * s12 * Q.d;
    } else {
      alpha[warp] = 0.5 * (1.0 - Q.v);
      beta[warp] = -0.5 * s12 * Q.d;
    }
  }
}

}  // namespace evbfit
}  // namespace cr

extern "C" {

int cr_evb_fit_grad(int basis, const double* x, int npar, int m, const double* e1, const double* e2,
                    const double* eref, double* grad) {
  static const int kNpar[9] = {0, 2, 5, 8, 4, 4, 6, 8, 12};
  if (basis < CR_FIT_1G || basis > CR_FIT_SP2D3) return cr_set_error(CR_ERR_ARG, "unknown fit basis");
  if (npar != kNpar[basis]) return cr_set_error(CR_ERR_ARG, "parameter count does not match the basis");
  if (m < 0 || !x || !grad || (m > 0 && (!e1 || !e2 || !eref))) return cr_set_error(CR_ERR_ARG, "bad fit arguments");
  for (int j = 0; j < npar; ++j) grad[j] = 0.0;
  if (m == 0) return CR_OK;
  const size_t nm = (size_t)m;
  double* d = nullptr;
  CR_TRY_CUDA(cudaMalloc(&d, ((size_t)npar + 3 * nm + nm * npar + npar) * sizeof(double)));
  double *dx = d, *de1 = dx + npar, *de2 = de1 + nm, *der = de2 + nm, *dout = der + nm, *dg = dout + nm * npar;
  int rc = CR_OK;
  if (cudaMemcpy(dx, x, (size_t)npar * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(de1, e1, nm * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(de2, e2, nm * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(der, eref, nm * 8, cudaMemcpyHostToDevice) != cudaSuccess) {
    rc = cr_set_error(CR_ERR_CUDA, "upload of the fit data failed");
  } else {
    cr::evbfit::fit_grad_kernel<<<(m + 127) / 128, 128>>>(basis, npar, m, dx, de1, de2, der, dout);
    cr::evbfit::column_sums_kernel<<<1, 32>>>(m, npar, dout, dg);
    if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess)
      rc = cr_set_error(CR_ERR_CUDA, "fit gradient kernel failed");
    else if (cudaMemcpy(grad, dg, (size_t)npar * 8, cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = cr_set_error(CR_ERR_CUDA, "download of the fit gradient failed");
  }
  cudaFree(d);
  return rc;
}

int cr_evb_param_vjp(cr_evb* evb, const double* xyz, const double* v, int nbeads, double* grad_coupling,
                     double* grad_ff1) {
  if (!evb || !grad_coupling || nbeads < 0 || (nbeads > 0 && (!xyz || !v)))
    return cr_set_error(CR_ERR_ARG, "bad EVB vjp arguments");
  cr_qmdff* f1 = evb->ff1;
  const int nlin = qmdff_nlin(f1);
  for (int j = 0; j < 10; ++j) grad_coupling[j] = 0.0;
  if (grad_ff1)
    for (int t = 0; t < nlin; ++t) grad_ff1[t] = 0.0;
  if (grad_ff1 && f1->nterm[4] > 0)
    return cr_set_error(CR_ERR_UNSUPPORTED, "parameter gradients of H/halogen-bond terms are not built");
  if (nbeads == 0) return CR_OK;
  const size_t n3 = (size_t)3 * f1->n, nq = n3 * nbeads, nb = (size_t)nbeads;
  const int chunk = std::min(nbeads, 4096);
  const size_t scratch = std::max((size_t)chunk * nlin, nb * 10);
  double* d = nullptr;
  CR_TRY_CUDA(cudaMalloc(&d, (4 * nq + 4 * nb + scratch + 10 + (size_t)nlin) * sizeof(double)));
  double *dq = d, *dv = dq + nq, *dg1 = dv + nq, *dg2 = dg1 + nq, *de1 = dg2 + nq, *de2 = de1 + nb, *da = de2 + nb,
         *db = da + nb, *ds = db + nb, *dc = ds + scratch, *dacc = dc + 10;
  int rc = CR_OK;
  if (cudaMemcpy(dq, xyz, nq * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(dv, v, nq * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(dacc, 0, (size_t)std::max(nlin, 1) * 8) != cudaSuccess) {
    rc = cr_set_error(CR_ERR_CUDA, "upload of the EVB vjp inputs failed");
  } else if ((rc = qmdff_launch(f1, dq, nbeads, de1, dg1, CR_PREC_FP64, nullptr)) == CR_OK &&
             (rc = qmdff_launch(evb->ff2, dq, nbeads, de2, dg2, CR_PREC_FP64, nullptr)) == CR_OK) {
    const long long nthreads = (long long)nbeads * 32;
    cr::evbfit::evb_vjp_kernel<<<(unsigned)((nthreads + 127) / 128), 128>>>(evb->C, nbeads, (int)n3, de1, dg1, de2,
                                                                            dg2, dv, ds, da, db);
    cr::evbfit::column_sums_kernel<<<1, 32>>>(nbeads, 10, ds, dc);
    if (cudaGetLastError() != cudaSuccess) rc = cr_set_error(CR_ERR_CUDA, "EVB vjp kernel failed");
    if (rc == CR_OK && grad_ff1)
      rc = qmdff_vjp_launch(f1, dq, dv, nbeads, da, db, 1.0, ds, chunk, dacc, nullptr);
    if (rc == CR_OK && (cudaDeviceSynchronize() != cudaSuccess ||
                        cudaMemcpy(grad_coupling, dc, 10 * 8, cudaMemcpyDeviceToHost) != cudaSuccess ||
                        (grad_ff1 && nlin && cudaMemcpy(grad_ff1, dacc, (size_t)nlin * 8, cudaMemcpyDeviceToHost) != cudaSuccess)))
      rc = cr_set_error(CR_ERR_CUDA, "download of the EVB vjp results failed");
  }
  cudaFree(d);
  return rc;
}

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
