// FP32-math instantiations of the fused step kernel: FP32 storage and the
// 16-bit shifted storages (FP16 scaled by 2^15, BF16).
#include "step.h"
#include "step_kernel.cuh"

namespace lbm {

template <int Q, int S, int MODE, bool DRY>
static void launch(const StepArgs& a, const Partials& p, int wpb, cudaStream_t st) {
    const int64_t blocks = (a.nchunks + wpb - 1) / wpb;
    k_step<Q, S, MODE, DRY><<<(unsigned)(blocks > 0 ? blocks : 1), 32 * wpb, 0, st>>>(a, p);
}

template <int Q, int S>
static void dispatch(int mode, bool dry, const StepArgs& a, const Partials& p, int wpb, cudaStream_t st) {
    if (dry) {
        if (mode == MODE_PULL) launch<Q, S, MODE_PULL, true>(a, p, wpb, st);
        else if (mode == MODE_AA_EVEN) launch<Q, S, MODE_AA_EVEN, true>(a, p, wpb, st);
        else launch<Q, S, MODE_AA_ODD, true>(a, p, wpb, st);
    } else {
        if (mode == MODE_PULL) launch<Q, S, MODE_PULL, false>(a, p, wpb, st);
        else if (mode == MODE_AA_EVEN) launch<Q, S, MODE_AA_EVEN, false>(a, p, wpb, st);
        else launch<Q, S, MODE_AA_ODD, false>(a, p, wpb, st);
    }
}

template <int Q>
static lbm_status dispatch_store(int store, int mode, bool dry, const StepArgs& a, const Partials& p, int wpb,
                                 cudaStream_t st) {
    switch (store) {
        case ST_F32: dispatch<Q, ST_F32>(mode, dry, a, p, wpb, st); break;
        case ST_F16S: dispatch<Q, ST_F16S>(mode, dry, a, p, wpb, st); break;
        case ST_BF16S: dispatch<Q, ST_BF16S>(mode, dry, a, p, wpb, st); break;
        default: return fail(LBM_ERR_ARG, "unknown storage format %d", store);
    }
    return LBM_OK;
}

lbm_status launch_step_lp(int Q, int store, int mode, bool dry, const StepArgs& a, const Partials& p, int wpb,
                          cudaStream_t st) {
    lbm_status s;
    if (Q == 19) s = dispatch_store<19>(store, mode, dry, a, p, wpb, st);
    else if (Q == 27) s = dispatch_store<27>(store, mode, dry, a, p, wpb, st);
    else return fail(LBM_ERR_ARG, "Q must be 19 or 27");
    if (s != LBM_OK) return s;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(LBM_ERR_CUDA, "step launch: %s", cudaGetErrorString(e));
    return LBM_OK;
}

}  // namespace lbm
