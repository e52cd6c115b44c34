// The GeH4OH surface's persistent step kernel (threads per bead up to 1) and force kernel.
#include "pes_ch4oh.cuh"
#include "rpmd_inst.cuh"

namespace cr {
const PesRuns kRunsGeH4OH = RunsOf<PesGeH4OH, 1>::table();
}  // namespace cr
