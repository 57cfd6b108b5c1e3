// Step kernel instantiations for storage ST_BF16S.
#include "step_launch.cuh"

namespace lbm {

lbm_status launch_step_bf16s(int Q, int mode, bool dry, int ra, const StepArgs& a, const Partials& p, int wpb,
                          cudaStream_t st) {
    return launch_store<ST_BF16S>(Q, mode, dry, ra, a, p, wpb, st);
}

}  // namespace lbm
