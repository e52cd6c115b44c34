// Device-resident QMDFF force field (the object behind cr_qmdff) and its
// launch entry for the engine.
#pragma once
#include <vector>

#include <cuda_runtime.h>

#include "qmdff.cuh"

struct cr_qmdff {
  int n = 0;
  int nterm[cr::qmdff::kKinds] = {0, 0, 0, 0, 0};  // bonds, angles, torsions, NCI pairs, H/halogen bonds
  int ncolors = 0;              // colours summed over the mixed form's batches
  int ncolors_fp64 = 0;         // the same for the plain form's schedule
  cr::qmdff::Dev dev{};
  std::vector<void*> allocs;    // device buffers owned by the force field
  int variant[2] = {-1, -1};    // autotuned kernel variant per form (FP64, mixed); -1: not yet
  float tune_ms[2][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
};

// Warps per block of the QMDFF force kernel and its dynamic shared memory.
constexpr int kQmdffWarps = 4;

// e[b] (with E_zero) and g = dV/dq for nbeads beads of d_q(3, n, nbeads).
int qmdff_launch(const cr_qmdff* ff, const double* d_q, int nbeads, double* d_e, double* d_g, int precision,
                 cudaStream_t s);

// dE-EVB of two force fields (csrc/evb.cu): e, g <- EVB energy and gradient;
// e2, g2 are scratch of the same sizes for the second force field.
struct cr_evb;
int evb_launch(const cr_evb* evb, const double* d_q, int nbeads, double* d_e, double* d_g, double* d_e2,
               double* d_g2, int precision, cudaStream_t s);
cr_qmdff* evb_first(const cr_evb* evb);
