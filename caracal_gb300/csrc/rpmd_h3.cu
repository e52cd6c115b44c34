// The H3 surface's persistent step kernel (threads per bead up to 4) and force kernel.
#include "pes_h3.cuh"
#include "rpmd_inst.cuh"

namespace cr {
const PesRuns kRunsH3 = RunsOf<PesH3, 4>::table();
}  // namespace cr
