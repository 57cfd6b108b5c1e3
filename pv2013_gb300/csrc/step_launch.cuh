// Launch dispatch for one storage format: Q x mode x dry x run axis.
#pragma once
#include "step.h"
#include "step_kernel.cuh"

namespace lbm {

template <int Q, int S, int MODE, bool DRY, int RA>
static void launch_one(const StepArgs& a, const Partials& p, int wpb, cudaStream_t st) {
    const int64_t blocks = (a.nchunks + wpb - 1) / wpb;
    k_step<Q, S, MODE, DRY, RA><<<(unsigned)(blocks > 0 ? blocks : 1), 32 * wpb, 0, st>>>(a, p);
}

template <int Q, int S, int RA>
static void launch_mode(int mode, bool dry, const StepArgs& a, const Partials& p, int wpb, cudaStream_t st) {
    if (dry) {
        if (mode == MODE_PULL) launch_one<Q, S, MODE_PULL, true, RA>(a, p, wpb, st);
        else if (mode == MODE_AA_EVEN) launch_one<Q, S, MODE_AA_EVEN, true, RA>(a, p, wpb, st);
        else launch_one<Q, S, MODE_AA_ODD, true, RA>(a, p, wpb, st);
    } else {
        if (mode == MODE_PULL) launch_one<Q, S, MODE_PULL, false, RA>(a, p, wpb, st);
        else if (mode == MODE_AA_EVEN) launch_one<Q, S, MODE_AA_EVEN, false, RA>(a, p, wpb, st);
        else launch_one<Q, S, MODE_AA_ODD, false, RA>(a, p, wpb, st);
    }
}

template <int S>
static lbm_status launch_store(int Q, int mode, bool dry, int ra, const StepArgs& a, const Partials& p, int wpb,
                               cudaStream_t st) {
    if (Q == 19) {
        if (ra == 1) launch_mode<19, S, 1>(mode, dry, a, p, wpb, st);
        else launch_mode<19, S, 2>(mode, dry, a, p, wpb, st);
    } else if (Q == 27) {
        if (ra == 1) launch_mode<27, S, 1>(mode, dry, a, p, wpb, st);
        else launch_mode<27, S, 2>(mode, dry, a, p, wpb, st);
    } else {
        return fail(LBM_ERR_ARG, "Q must be 19 or 27");
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(LBM_ERR_CUDA, "step launch: %s", cudaGetErrorString(e));
    return LBM_OK;
}

}  // namespace lbm
