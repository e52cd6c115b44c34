// The BrH2 surface's persistent step kernel (threads per bead up to 1) and force kernel.
#include "pes_brh2.cuh"
#include "rpmd_inst.cuh"

namespace cr {
const PesRuns kRunsBrH2 = RunsOf<PesBrH2, 1>::table();
}  // namespace cr
