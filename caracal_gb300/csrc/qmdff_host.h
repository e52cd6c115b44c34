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
  cr::qmdff::Tables<double> unit{};  // linear parameters set to 1 (parameter gradients)
  float tune_ms[2][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
};

// Warps per block of the QMDFF force kernel and its dynamic shared memory.
constexpr int kQmdffWarps = 4;

// NpT arguments of one launch: each trajectory's box edges (tbox[3 t + k],
// bohr) for beads [t beads_per_box, (t + 1) beads_per_box), and the virial
// trace of each bead out (vir[b]).
struct QmdffNpt {
  const double* tbox;
  int beads_per_box;
  double* vir;
};

// e[b] (with E_zero) and g = dV/dq for nbeads beads of d_q(3, n, nbeads);
// npt: per-trajectory boxes and the virial (NULL: the force field's box).
int qmdff_launch(const cr_qmdff* ff, const double* d_q, int nbeads, double* d_e, double* d_g, int precision,
                 cudaStream_t s, const QmdffNpt* npt = nullptr);

// Plain-form derivatives for the adjoint (bonds, angles, torsions, NCI pairs):
// energy, gradient and H w per bead (d_e, d_g, d_dew may be NULL) ...
int qmdff_hvp_launch(const cr_qmdff* ff, const double* d_q, const double* d_w, int nbeads, double* d_e, double* d_g,
                     double* d_hw, double* d_dew, cudaStream_t s);
// ... and d_acc[t] += scale * sum_b (alpha_b v_b . grad E_t|unit + beta_b E_t|unit)
// over the linear parameters t (bond k, angle k, torsion V, pair qq; count
// qmdff_nlin); d_scratch holds scratch_beads * nlin doubles.
int qmdff_vjp_launch(const cr_qmdff* ff, const double* d_q, const double* d_v, int nbeads, const double* d_alpha,
                     const double* d_beta, double scale, double* d_scratch, int scratch_beads, double* d_acc,
                     cudaStream_t s);
int qmdff_nlin(const cr_qmdff* ff);

// dE-EVB of two force fields (csrc/evb.cu): e, g <- EVB energy and gradient;
// e2, g2 are scratch of the same sizes for the second force field.
struct cr_evb;
int evb_launch(const cr_evb* evb, const double* d_q, int nbeads, double* d_e, double* d_g, double* d_e2,
               double* d_g2, int precision, cudaStream_t s);
cr_qmdff* evb_first(const cr_evb* evb);
