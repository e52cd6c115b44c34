// Host helpers shared by the engine's translation units: the per-thread
// error detail behind cr_last_error_detail and a CUDA status check.
#pragma once
#include <string>

#include <cuda_runtime.h>

#include "../../include/caracal_gb300.h"

// Records msg as this thread's last error detail and returns code.
int cr_set_error(int code, const std::string& msg);

#define CR_TRY_CUDA(call)                                                                     \
  do {                                                                                        \
    cudaError_t _e = (call);                                                                  \
    if (_e != cudaSuccess)                                                                    \
      return cr_set_error(CR_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e));   \
  } while (0)
