// Paired step kernel instantiations for storage ST_F16S.
#include "step_pair.cuh"

namespace lbm {

lbm_status launch_pair_f16s(int Q, int mode, int ra, const StepArgs& a, int wpb, cudaStream_t st) {
    return launch_pair_store<ST_F16S>(Q, mode, ra, a, wpb, st);
}

}  // namespace lbm
