// Step kernel instantiations for storage ST_F32.
#include "step_launch.cuh"

namespace lbm {

lbm_status launch_step_f32(int Q, int mode, bool dry, int ra, const StepArgs& a, const Partials& p, int wpb,
                          cudaStream_t st) {
    return launch_store<ST_F32>(Q, mode, dry, ra, a, p, wpb, st);
}

lbm_status launch_tma_f32(int Q, int mode, int ra, const StepArgs& a, int32_t* err, int wpb, cudaStream_t st) {
    return launch_store_tma<ST_F32>(Q, mode, ra, a, err, wpb, st);
}

}  // namespace lbm
