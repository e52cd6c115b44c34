// dE-EVB of two QMDFFs: the cr_evb object and its C-ABI (cr_evb_*).
#include <string>

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

extern "C" {

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
