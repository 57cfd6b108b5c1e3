// Step kernel instantiations for storage ST_F64.  Built with -fmad=false so the
// collision and Zou-He arithmetic matches the reference bit for bit
// (Simulation.cpp:21-179, Boundary.cpp:87-148, Simulation.cpp:952-1348).
#include "step_launch.cuh"

namespace lbm {

lbm_status launch_step_f64(int Q, int mode, bool dry, int ra, const StepArgs& a, const Partials& p, int wpb,
                          cudaStream_t st) {
    return launch_store<ST_F64>(Q, mode, dry, ra, a, p, wpb, st);
}

lbm_status launch_tma_f64(int Q, int mode, int ra, const StepArgs& a, int32_t* err, int wpb, cudaStream_t st) {
    return launch_store_tma<ST_F64>(Q, mode, ra, a, err, wpb, st);
}

}  // namespace lbm
