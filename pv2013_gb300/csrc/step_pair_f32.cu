// Paired step kernel instantiations for storage ST_F32.
#include "step_pair.cuh"

namespace lbm {

lbm_status launch_pair_f32(int Q, int mode, int ra, const StepArgs& a, int wpb, cudaStream_t st) {
    return launch_pair_store<ST_F32>(Q, mode, ra, a, wpb, st);
}

}  // namespace lbm
