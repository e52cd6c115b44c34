// Launch entry points of the analytic surfaces' kernels.  Each surface's
// persistent step kernel and one-thread-per-bead force kernel are compiled
// in their own translation unit (rpmd_h3.cu, rpmd_ch4h.cu, rpmd_ch4oh.cu,
// rpmd_oh3.cu, rpmd_geh4oh.cu, rpmd_brh2.cu), so the library builds them in parallel; the engine reaches
// them through this table.
#pragma once
#include <cstddef>

#include <cuda_runtime.h>

namespace cr {

struct StepParams;

struct PesRuns {
  int max_tpb;  // largest threads-per-bead variant of the step kernel built for the surface
  // rpmd_run_kernel<surface, mixed, tpb><<<grid, block, smem, st>>>(prm, istep, nsteps)
  cudaError_t (*run)(const StepParams& prm, bool mixed, int tpb, int grid, int block, size_t smem,
                     cudaStream_t st, int istep, int nsteps);
  // dynamic shared-memory limit of that kernel (set outside a stream capture)
  cudaError_t (*set_smem)(bool mixed, int tpb, size_t smem);
  // egrad_kernel<surface, mixed>: V and dV/dq of nbeads beads
  cudaError_t (*egrad)(bool mixed, int nbeads, const double* q, double* V, double* g, cudaStream_t st);
};

// The table of CR_PES_H3 / CH4H / CH4OH / OH3 / GEH4OH / BRH2; NULL for any other surface.
const PesRuns* pes_runs(int pes);

extern const PesRuns kRunsH3, kRunsCH4H, kRunsCH4OH, kRunsOH3, kRunsGeH4OH, kRunsBrH2;

}  // namespace cr
