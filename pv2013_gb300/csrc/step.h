// Launchers of the step kernel instantiations (internal).  One translation
// unit per storage format so they compile in parallel; the FP64 one is built
// with -fmad=false.
#pragma once
#include <cuda_runtime.h>

#include "device.cuh"
#include "internal.h"

namespace lbm {

struct Partials;

lbm_status launch_step_f64(int Q, int mode, bool dry, int ra, const StepArgs& a, const Partials& p, int wpb,
                           cudaStream_t st);
lbm_status launch_step_f32(int Q, int mode, bool dry, int ra, const StepArgs& a, const Partials& p, int wpb,
                           cudaStream_t st);
lbm_status launch_step_f16s(int Q, int mode, bool dry, int ra, const StepArgs& a, const Partials& p, int wpb,
                            cudaStream_t st);
lbm_status launch_step_bf16s(int Q, int mode, bool dry, int ra, const StepArgs& a, const Partials& p, int wpb,
                             cudaStream_t st);

// TMA-staged pipeline (non-dry launches only); err receives 1 if a bounded wait gave up.
lbm_status launch_tma_f64(int Q, int mode, int ra, const StepArgs& a, int32_t* err, int wpb, cudaStream_t st);
lbm_status launch_tma_f32(int Q, int mode, int ra, const StepArgs& a, int32_t* err, int wpb, cudaStream_t st);
lbm_status launch_tma_f16s(int Q, int mode, int ra, const StepArgs& a, int32_t* err, int wpb, cudaStream_t st);
lbm_status launch_tma_bf16s(int Q, int mode, int ra, const StepArgs& a, int32_t* err, int wpb, cudaStream_t st);

// Paired kernel (two adjacent nodes per lane; non-dry launches, FP32 and
// 16-bit storage); a.chunks must be the paired chunk table.
lbm_status launch_pair_f32(int Q, int mode, int ra, const StepArgs& a, int wpb, cudaStream_t st);
lbm_status launch_pair_f16s(int Q, int mode, int ra, const StepArgs& a, int wpb, cudaStream_t st);
lbm_status launch_pair_bf16s(int Q, int mode, int ra, const StepArgs& a, int wpb, cudaStream_t st);

// Wall shear stress of every wall lane (one-node-per-lane chunk table):
// wss[out_pos] = |mu grad u| from the node velocities u (3 per output
// position); wall_flag[out_pos] = 1 when wall_flag is not null.
lbm_status launch_wss(int Q, int ra, const Chunk* chunks, int64_t nchunks, const uint32_t* mmask,
                      const int32_t* out_pos, const InstParam* insts, const double* u, double* wss,
                      uint8_t* wall_flag, cudaStream_t st);

}  // namespace lbm
