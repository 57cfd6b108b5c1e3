// Launchers of the step kernel instantiations (internal).
#pragma once
#include <cuda_runtime.h>

#include "device.cuh"
#include "internal.h"

namespace lbm {

struct Partials;

// FP64 store (step_f64.cu, built without FMA contraction).
lbm_status launch_step_f64(int Q, int mode, bool dry, const StepArgs& a, const Partials& p, int warps_per_block,
                           cudaStream_t st);
// FP32 / FP16-shifted / BF16-shifted stores (step_lp.cu).
lbm_status launch_step_lp(int Q, int store, int mode, bool dry, const StepArgs& a, const Partials& p,
                          int warps_per_block, cudaStream_t st);

}  // namespace lbm
