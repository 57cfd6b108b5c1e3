// Step kernel instantiations for storage ST_BF16S.
#include "step_launch.cuh"

namespace lbm {

lbm_status launch_step_bf16s(int Q, int mode, bool dry, int ra, const StepArgs& a, const Partials& p, int wpb,
                          cudaStream_t st) {
    return launch_store<ST_BF16S>(Q, mode, dry, ra, a, p, wpb, st);
}

lbm_status launch_tma_bf16s(int Q, int mode, int ra, const StepArgs& a, int32_t* err, int wpb, cudaStream_t st) {
    return launch_store_tma<ST_BF16S>(Q, mode, ra, a, err, wpb, st);
}

}  // namespace lbm
