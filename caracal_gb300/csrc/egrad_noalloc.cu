// cr_egrad_h3_noalloc: the BKMP2 gradient of cr_egrad_h3 without any device
// memory allocation.
//
// cr_egrad_h3 stages the caller's host arrays through device buffers it
// allocates and frees on every call.  Some callers cannot allow that: a
// Fortran MD loop that calls the PES once per step cannot afford the
// device-wide synchronisation cudaMalloc/cudaFree imply on every step, and a
// host program whose device memory is owned by its own pre-sized pool may not
// create allocations outside it.  This variant stages through one
// file-scope device array instead, so a call allocates nothing.
//
// Limits and sharing:
//  * at most kNoAllocMaxBeads = 16384 beads (geometries) per call; larger
//    calls are rejected with CR_ERR_ARG.  The array takes 16384 * 19 doubles
//    = 2.49 MB on every device that loads this library, held until exit.
//  * every call on a device uses the same array and leaves the last call's
//    data in it; each call overwrites every element it reads back, so nothing
//    has to start at zero.  Calls that overlap on the GPU (from several host
//    threads, or with work on other streams touching the same device) race
//    on the array; callers must serialise them.
//  * the first call on a device resolves the array's device address with
//    cudaGetSymbolAddress (set-up, once per device, with that device
//    current); make that first call before any stream capture.
//  * the copies and the kernel run on the legacy default stream with
//    blocking cudaMemcpy, so a call waits for, and holds up, work on every
//    blocking stream of the device (streams created without
//    cudaStreamNonBlocking), and returns once the results are on the host.
//  * errors return a CR_ERR_* status and set the text of
//    cr_last_error_detail, as the other entry points do.
#include <mutex>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/caracal_gb300.h"
#include "host_util.h"
#include "pes_h3.cuh"

namespace {

constexpr int kNoAllocMaxBeads = 16384;
constexpr int kQ = 9;  // doubles per bead: q(3,3)
// layout: [q: 9*max][dVdq: 9*max][V: max]
constexpr size_t kScratchDoubles = (size_t)kNoAllocMaxBeads * (kQ + kQ + 1);

static __device__ __align__(256) double g_egrad_noalloc_scratch[kScratchDoubles];

std::mutex g_setup_mutex;
std::vector<double*> g_scratch_addr;  // per device, resolved once

__global__ void egrad_h3_noalloc_kernel(int nbeads, double* scratch) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nbeads) return;
  const double* q = scratch;
  double* g = scratch + (size_t)kNoAllocMaxBeads * kQ;
  double* V = scratch + (size_t)kNoAllocMaxBeads * 2 * kQ;
  double qq[kQ], gg[kQ], v;
#pragma unroll
  for (int c = 0; c < kQ; ++c) qq[c] = q[(size_t)b * kQ + c];
  cr::PesH3::egrad<double>(qq, v, gg);
  V[b] = v;
#pragma unroll
  for (int c = 0; c < kQ; ++c) g[(size_t)b * kQ + c] = gg[c];
}

// Address of the scratch array on the current device (set-up on first use).
int scratch_for_current_device(double** out) {
  int dev = 0;
  cudaError_t err = cudaGetDevice(&dev);
  if (err != cudaSuccess)
    return cr_set_error(CR_ERR_NO_DEVICE, std::string("cr_egrad_h3_noalloc: cudaGetDevice: ") + cudaGetErrorString(err));
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if ((int)g_scratch_addr.size() <= dev) g_scratch_addr.resize((size_t)dev + 1, nullptr);
  if (!g_scratch_addr[(size_t)dev]) {
    double* ptr = nullptr;
    err = cudaGetSymbolAddress((void**)&ptr, g_egrad_noalloc_scratch);
    if (err != cudaSuccess || !ptr)
      return cr_set_error(CR_ERR_CUDA, std::string("cr_egrad_h3_noalloc: cudaGetSymbolAddress: ") +
                                           cudaGetErrorString(err));
    g_scratch_addr[(size_t)dev] = ptr;
  }
  *out = g_scratch_addr[(size_t)dev];
  return CR_OK;
}

int cuda_fail(const char* what, cudaError_t err) {
  return cr_set_error(CR_ERR_CUDA, std::string("cr_egrad_h3_noalloc: ") + what + ": " + cudaGetErrorString(err));
}

}  // namespace

extern "C" int cr_egrad_h3_noalloc(const double* q, int natoms, int nbeads, double* V, double* dVdq,
                                   int* info) {
  if (info) *info = 0;
  if (natoms != 3) return cr_set_error(CR_ERR_ARG, "cr_egrad_h3_noalloc: natoms must be 3");
  if (nbeads < 0 || (nbeads > 0 && (!q || !V || !dVdq)))
    return cr_set_error(CR_ERR_ARG, "cr_egrad_h3_noalloc: negative bead count or NULL array");
  if (nbeads > kNoAllocMaxBeads)
    return cr_set_error(CR_ERR_ARG, "cr_egrad_h3_noalloc: " + std::to_string(nbeads) +
                                        " beads exceed the fixed maximum of " + std::to_string(kNoAllocMaxBeads) +
                                        " per call");
  if (nbeads == 0) return CR_OK;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return cr_set_error(CR_ERR_NO_DEVICE, "cr_egrad_h3_noalloc: no CUDA device");
  double* scratch = nullptr;
  int rc = scratch_for_current_device(&scratch);
  if (rc) return rc;
  double* d_q = scratch;
  double* d_g = scratch + (size_t)kNoAllocMaxBeads * kQ;
  double* d_V = scratch + (size_t)kNoAllocMaxBeads * 2 * kQ;
  const size_t nq = (size_t)kQ * nbeads;
  cudaError_t err = cudaMemcpy(d_q, q, nq * sizeof(double), cudaMemcpyHostToDevice);
  if (err != cudaSuccess) return cuda_fail("copy of q", err);
  const int bs = 128;
  egrad_h3_noalloc_kernel<<<(nbeads + bs - 1) / bs, bs>>>(nbeads, scratch);
  if ((err = cudaGetLastError()) != cudaSuccess) return cuda_fail("kernel launch", err);
  if ((err = cudaMemcpy(V, d_V, (size_t)nbeads * sizeof(double), cudaMemcpyDeviceToHost)) != cudaSuccess)
    return cuda_fail("copy of V", err);
  if ((err = cudaMemcpy(dVdq, d_g, nq * sizeof(double), cudaMemcpyDeviceToHost)) != cudaSuccess)
    return cuda_fail("copy of dVdq", err);
  return CR_OK;
}
