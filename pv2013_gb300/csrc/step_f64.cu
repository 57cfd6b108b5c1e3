// FP64 instantiations of the fused step kernel.  Built with -fmad=false so
// the collision and Zou-He arithmetic matches the reference's FP64 results
// bit for bit (Simulation.cpp:21-179, Boundary.cpp:87-148,
// Simulation.cpp:952-1348).
#include "step.h"
#include "step_kernel.cuh"

namespace lbm {

template <int Q, int MODE, bool DRY>
static void launch(const StepArgs& a, const Partials& p, int wpb, cudaStream_t st) {
    const int64_t blocks = (a.nchunks + wpb - 1) / wpb;
    k_step<Q, ST_F64, MODE, DRY><<<(unsigned)(blocks > 0 ? blocks : 1), 32 * wpb, 0, st>>>(a, p);
}

template <int Q>
static void dispatch(int mode, bool dry, const StepArgs& a, const Partials& p, int wpb, cudaStream_t st) {
    if (dry) {
        if (mode == MODE_PULL) launch<Q, MODE_PULL, true>(a, p, wpb, st);
        else if (mode == MODE_AA_EVEN) launch<Q, MODE_AA_EVEN, true>(a, p, wpb, st);
        else launch<Q, MODE_AA_ODD, true>(a, p, wpb, st);
    } else {
        if (mode == MODE_PULL) launch<Q, MODE_PULL, false>(a, p, wpb, st);
        else if (mode == MODE_AA_EVEN) launch<Q, MODE_AA_EVEN, false>(a, p, wpb, st);
        else launch<Q, MODE_AA_ODD, false>(a, p, wpb, st);
    }
}

lbm_status launch_step_f64(int Q, int mode, bool dry, const StepArgs& a, const Partials& p, int wpb, cudaStream_t st) {
    if (Q == 19) dispatch<19>(mode, dry, a, p, wpb, st);
    else if (Q == 27) dispatch<27>(mode, dry, a, p, wpb, st);
    else return fail(LBM_ERR_ARG, "Q must be 19 or 27");
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(LBM_ERR_CUDA, "step launch: %s", cudaGetErrorString(e));
    return LBM_OK;
}

}  // namespace lbm
