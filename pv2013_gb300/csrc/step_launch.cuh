// Launch dispatch for one storage format: Q x mode x dry x run axis.
#pragma once
#include <algorithm>

#include "step.h"
#include "step_kernel.cuh"
#include "step_tma.cuh"

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

template <int Q, int S, int MODE, int RA>
static lbm_status launch_tma_one(const StepArgs& a, int32_t* err, int wpb, cudaStream_t st) {
    // one launch configuration per instantiation and block size: the grid is
    // the number of co-resident blocks (each warp loops over its chunks)
    static int cached_wpb = 0, cached_blocks = 0;
    const size_t smem = (size_t)wpb * kStages * StageLayout<Q, S>::BYTES;
    if (cached_wpb != wpb) {
        cudaError_t e = cudaFuncSetAttribute(k_step_tma<Q, S, MODE, RA>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return fail(LBM_ERR_CUDA, "step kernel shared memory: %s", cudaGetErrorString(e));
        int per_sm = 0, dev = 0, sms = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_step_tma<Q, S, MODE, RA>, 32 * wpb, smem);
        if (e == cudaSuccess) e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return fail(LBM_ERR_CUDA, "occupancy query: %s", cudaGetErrorString(e));
        if (per_sm < 1) return fail(LBM_ERR_CUDA, "step kernel does not fit on an SM (%zu B shared)", smem);
        cached_blocks = per_sm * sms;
        cached_wpb = wpb;
    }
    const int64_t need = (a.nchunks + wpb - 1) / wpb;
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(cached_blocks, need));
    k_step_tma<Q, S, MODE, RA><<<blocks, 32 * wpb, smem, st>>>(a, err);
    return LBM_OK;
}

template <int Q, int S, int RA>
static lbm_status launch_tma_mode(int mode, const StepArgs& a, int32_t* err, int wpb, cudaStream_t st) {
    if (mode == MODE_PULL) return launch_tma_one<Q, S, MODE_PULL, RA>(a, err, wpb, st);
    if (mode == MODE_AA_EVEN) return launch_tma_one<Q, S, MODE_AA_EVEN, RA>(a, err, wpb, st);
    return launch_tma_one<Q, S, MODE_AA_ODD, RA>(a, err, wpb, st);
}

template <int S>
static lbm_status launch_store_tma(int Q, int mode, int ra, const StepArgs& a, int32_t* err, int wpb,
                                   cudaStream_t st) {
    lbm_status s;
    if (Q == 19) s = ra == 1 ? launch_tma_mode<19, S, 1>(mode, a, err, wpb, st) : launch_tma_mode<19, S, 2>(mode, a, err, wpb, st);
    else if (Q == 27) s = ra == 1 ? launch_tma_mode<27, S, 1>(mode, a, err, wpb, st) : launch_tma_mode<27, S, 2>(mode, a, err, wpb, st);
    else return fail(LBM_ERR_ARG, "Q must be 19 or 27");
    if (s != LBM_OK) return s;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(LBM_ERR_CUDA, "step launch: %s", cudaGetErrorString(e));
    return LBM_OK;
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
