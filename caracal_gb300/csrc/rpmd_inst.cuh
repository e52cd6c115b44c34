// The PesRuns table of one analytic surface: instantiates its persistent
// step kernel (both precision forms, threads per bead 1 .. MAXTPB) and its
// force kernel.  Included once per surface, by rpmd_<surface>.cu.
#pragma once
#include "pes_runs.h"
#include "rpmd_kernel.cuh"

namespace cr {

template <class PES, int MAXTPB>
struct RunsOf {
  template <bool MIXED, int TPB>
  static cudaError_t launch(const StepParams& prm, int grid, int block, size_t smem, cudaStream_t st, int istep,
                            int nsteps) {
    rpmd_run_kernel<PES, MIXED, TPB><<<grid, block, smem, st>>>(prm, istep, nsteps);
    return cudaGetLastError();
  }
  template <bool MIXED, int TPB>
  static cudaError_t smem_limit(size_t smem) {
    return cudaFuncSetAttribute(rpmd_run_kernel<PES, MIXED, TPB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem);
  }
  static cudaError_t run(const StepParams& prm, bool mixed, int tpb, int grid, int block, size_t smem,
                         cudaStream_t st, int istep, int nsteps) {
    if (tpb == 1) return mixed ? launch<true, 1>(prm, grid, block, smem, st, istep, nsteps)
                               : launch<false, 1>(prm, grid, block, smem, st, istep, nsteps);
    if constexpr (MAXTPB >= 2) {
      if (tpb == 2) return mixed ? launch<true, 2>(prm, grid, block, smem, st, istep, nsteps)
                                 : launch<false, 2>(prm, grid, block, smem, st, istep, nsteps);
    }
    if constexpr (MAXTPB >= 4) {
      if (tpb == 4) return mixed ? launch<true, 4>(prm, grid, block, smem, st, istep, nsteps)
                                 : launch<false, 4>(prm, grid, block, smem, st, istep, nsteps);
    }
    return cudaErrorInvalidValue;
  }
  static cudaError_t set_smem(bool mixed, int tpb, size_t smem) {
    if (tpb == 1) return mixed ? smem_limit<true, 1>(smem) : smem_limit<false, 1>(smem);
    if constexpr (MAXTPB >= 2) {
      if (tpb == 2) return mixed ? smem_limit<true, 2>(smem) : smem_limit<false, 2>(smem);
    }
    if constexpr (MAXTPB >= 4) {
      if (tpb == 4) return mixed ? smem_limit<true, 4>(smem) : smem_limit<false, 4>(smem);
    }
    return cudaErrorInvalidValue;
  }
  static cudaError_t egrad(bool mixed, int nbeads, const double* q, double* V, double* g, cudaStream_t st) {
    const int bs = 128, nb = (nbeads + bs - 1) / bs;
    if (nbeads <= 0) return cudaSuccess;
    if (mixed) egrad_kernel<PES, true><<<nb, bs, 0, st>>>(nbeads, q, V, g);
    else egrad_kernel<PES, false><<<nb, bs, 0, st>>>(nbeads, q, V, g);
    return cudaGetLastError();
  }
  static constexpr PesRuns table() { return PesRuns{MAXTPB, &run, &set_smem, &egrad}; }
};

}  // namespace cr
