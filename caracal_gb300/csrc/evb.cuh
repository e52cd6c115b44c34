// dE-EVB of two QMDFFs on the device: the lower root of the 2x2 EVB matrix
// with Caracal's energy-difference couplings (src/gradient.f90:1228-1304).
// Both force fields are evaluated by the QMDFF kernel into separate buffers
// (each energy includes its E_zero); evb_combine_kernel then forms, per bead,
// dE = E1 - E2, V12(dE), E = (E1 + E2 - sqrt(dE^2 + 4 V12^2)) / 2 and
// g = (g1 + g2 - D / sqrt(dE^2 + 4 V12^2)) / 2 with Caracal's D per basis.
// FP64 throughout (a few operations per coordinate).
#pragma once
#include <cuda_runtime.h>

#include "dual.cuh"

namespace cr {
namespace evb {

enum Basis { CONST = 0, G1 = 1, G2 = 2, G3 = 3, SP = 4, SD = 5, SD2 = 6, SP2D = 7 };

struct Coupling {
  int basis;
  double a, b, c, d, e, f, g, h, m, n;  // offa..offh, offm, offn
};

// V12(dE) and the factor K such that Caracal's deldiscr = K * (g1 - g2).
// p = (a, b, c, d, e, f, g, h, m, n); T is double or a dual number
// (parameter gradients).
template <class T>
__host__ __device__ inline void coupling_t(int basis, const T* p, T ediff, T& offdiag, T& K) {
  const T e2 = ediff * ediff;
  const T &a = p[0], &b = p[1], &c = p[2], &d = p[3], &e = p[4], &f = p[5], &g = p[6], &h = p[7], &m = p[8], &n = p[9];
  switch (basis) {
    case CONST:
      offdiag = a;
      K = ediff;
      break;
    case G1:
      offdiag = a * exp(-b * e2);
      K = ediff * (1.0 - 2.0 * (4.0 * offdiag * offdiag) * b);
      break;
    case G2: {
      const T x1 = exp(-b * e2), x2 = exp(-d * (ediff + m) * (ediff + m));
      offdiag = a * x1 + c * x2;
      K = 1.0 * ediff + 4.0 * offdiag * (-2.0 * a * b * ediff * x1 - 2.0 * c * d * (m + ediff) * x2);
      break;
    }
    case G3: {
      const T x1 = exp(-b * e2), x2 = exp(-d * (ediff + m) * (ediff + m));
      const T x3 = exp(-f * (ediff + n) * (ediff + n));
      offdiag = a * x1 + c * x2 + e * x3;
      K = 1.0 * ediff + 4.0 * offdiag *
                            (-2.0 * a * b * ediff * x1 - 2.0 * c * d * (m + ediff) * x2 -
                             2.0 * e * f * (n + ediff) * x3);
      break;
    }
    case SP: {
      const T x1 = exp(-b * e2), x2 = exp(-d * e2);
      offdiag = a * x1 + c * ediff * x2;
      K = 1.0 * ediff + 4.0 * offdiag * (-2.0 * a * b * ediff * x1 + c * (1.0 - 2.0 * e2 * d) * x2);
      break;
    }
    case SD: {
      const T x1 = exp(-b * e2), x2 = exp(-d * e2);
      offdiag = a * x1 + c * e2 * x2;
      K = 1.0 * ediff + 4.0 * offdiag * (-2.0 * a * b * ediff * x1 + c * (2.0 * ediff - 2.0 * e2 * ediff * d) * x2);
      break;
    }
    case SD2: {
      const T x1 = exp(-b * e2), x2 = exp(-d * e2), x3 = exp(-f * e2);
      offdiag = a * x1 + c * e2 * x2 + e * e2 * x3;
      K = 1.0 * ediff + 4.0 * offdiag *
                            (-2.0 * a * b * ediff * x1 + c * (2.0 * ediff - 2.0 * e2 * ediff * d) * x2 +
                             e * (2.0 * ediff - 2.0 * e2 * ediff * f) * x3);
      break;
    }
    default: {  // SP2D
      const T x1 = exp(-b * e2), x2 = exp(-d * e2), x3 = exp(-f * e2), x4 = exp(-h * e2);
      offdiag = a * x1 + c * ediff * x2 + e * ediff * x3 + e2 * g * x4;
      K = 1.0 * ediff + 4.0 * offdiag *
                            (-2.0 * a * b * ediff * x1 + c * (1.0 - 2.0 * e2 * d) * x2 +
                             e * (1.0 - 2.0 * e2 * f) * x3 + g * (2.0 * ediff - 2.0 * e2 * ediff * h) * x4);
      break;
    }
  }
}

__host__ __device__ inline void coupling(const Coupling& C, double ediff, double& offdiag, double& K) {
  const double p[10] = {C.a, C.b, C.c, C.d, C.e, C.f, C.g, C.h, C.m, C.n};
  coupling_t<double>(C.basis, p, ediff, offdiag, K);
}

// One warp per bead: e[b] <- EVB energy, g[b] <- EVB gradient (g1 in place).
__global__ void evb_combine_kernel(Coupling C, int nbeads, int n3, double* e1, double* g1, const double* e2,
                                   const double* g2) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= nbeads) return;
  const double E1 = e1[warp], E2 = e2[warp];
  const double ediff = E1 - E2;
  double offdiag, K;
  coupling(C, ediff, offdiag, K);
  const double root2 = sqrt(ediff * ediff + 4.0 * offdiag * offdiag);
  double* ga = g1 + (size_t)warp * n3;
  const double* gb = g2 + (size_t)warp * n3;
  for (int k = lane; k < n3; k += 32) {
    const double a = ga[k], b = gb[k];
    ga[k] = 0.5 * (a + b - (K * (a - b)) / root2);
  }
  if (lane == 0) e1[warp] = 0.5 * (E1 + E2 - root2);
}

}  // namespace evb
}  // namespace cr
