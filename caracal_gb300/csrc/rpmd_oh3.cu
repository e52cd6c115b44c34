// The OH3 surface's persistent step kernel (threads per bead up to 4) and force kernel.
#include "pes_oh3.cuh"
#include "rpmd_inst.cuh"

namespace cr {
const PesRuns kRunsOH3 = RunsOf<PesOH3, 4>::table();
}  // namespace cr
