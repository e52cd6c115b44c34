// Device-side flexible SPC water box (the object behind cr_water) and its
// launch entry for the engine.
#pragma once
#include <cuda_runtime.h>

#include "../../include/caracal_gb300.h"
#include "water.cuh"

struct cr_water {
  cr::water::Dev dev{};
};

// e[b] and g = dV/dq for nbeads beads of d_q(3, n, nbeads).
int water_launch(const cr_water* w, const double* d_q, int nbeads, double* d_e, double* d_g, int precision,
                 cudaStream_t s);
