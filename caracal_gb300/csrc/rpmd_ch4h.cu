// The CH4H surface's persistent step kernel (threads per bead up to 1) and force kernel.
#include "pes_ch4h.cuh"
#include "rpmd_inst.cuh"

namespace cr {
const PesRuns kRunsCH4H = RunsOf<PesCH4H, 1>::table();
}  // namespace cr
