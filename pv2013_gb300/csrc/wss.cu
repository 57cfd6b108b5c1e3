// Wall shear stress at the wall nodes (Simulation.cpp:1374-1421):
//   grad = mean over the existing neighbours x + c_q (q = 0..Q-1, the rest
//          direction included: the node is its own neighbour there) of
//          u(x + c_q) - u(x)                   ComputeVelocityGradientAtWall
//   wss  = |mu grad|, mu = 1/6 (2 tau - 1)    ComputeWallShearStress
// with u the velocities of the current populations (the values the
// reference's Collision stores in Node::velocity).  The sums run in the
// reference's direction order in FP64; this translation unit is built with
// -fmad=false so the results are the reference's bit for bit.
#include "step.h"
#include "step_kernel.cuh"

namespace lbm {

template <int Q, int RA>
__global__ void __launch_bounds__(128) k_wss(const Chunk* __restrict__ chunks, int64_t nchunks,
                                             const uint32_t* __restrict__ mmask, const int32_t* __restrict__ out_pos,
                                             const InstParam* __restrict__ insts, const double* __restrict__ u,
                                             double* __restrict__ wss, uint8_t* __restrict__ wall_flag) {
    using L = Lat<Q>;
    using X = Ax<Q, RA>;
    const int lane = threadIdx.x & 31;
    const int64_t ci = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (ci >= nchunks) return;
    const Chunk* cp = chunks + ci;
    const int len = (int)(__ldg(&cp->len_inst) & 63u);
    const uint32_t wmask = __ldg(&cp->wmask);
    if (lane >= len || !((wmask >> lane) & 1u)) return;
    const int32_t n0 = __ldg(&cp->n0);
    const uint32_t bmask = __ldg(&cp->bmask);
    int32_t K[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) K[c] = __ldg(&cp->K[c]);
    const uint32_t missing = __ldg(mmask + __ldg(&cp->mslot0) + __popc(bmask & ((1u << lane) - 1u)));
    const int32_t n = n0 + lane;
    const int64_t self = out_pos[n];
    const double ux = u[3 * self], uy = u[3 * self + 1], uz = u[3 * self + 2];
    double g0 = 0.0, g1 = 0.0, g2 = 0.0;
    int cnt = 0;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        if ((missing >> L::opp(q)) & 1u) continue;        // x + c_q is not a node of the reference
        const int32_t nb = q == L::REST ? n : nb_id(K, n0, lane, X::a(q), X::b(q), X::r(q));
        const int64_t p = out_pos[nb];
        g0 += (u[3 * p] - ux);
        g1 += (u[3 * p + 1] - uy);
        g2 += (u[3 * p + 2] - uz);
        ++cnt;
    }
    if (cnt > 0) {
        g0 /= cnt;
        g1 /= cnt;
        g2 /= cnt;
    }
    const double mu = 1.0 / 6.0 * (2.0 * insts[__ldg(&cp->len_inst) >> 8].tau - 1.0);
    const double s0 = mu * g0, s1 = mu * g1, s2 = mu * g2;
    wss[self] = sqrt(s0 * s0 + s1 * s1 + s2 * s2);
    if (wall_flag) wall_flag[self] = 1;
}

lbm_status launch_wss(int Q, int ra, const Chunk* chunks, int64_t nchunks, const uint32_t* mmask,
                      const int32_t* out_pos, const InstParam* insts, const double* u, double* wss,
                      uint8_t* wall_flag, cudaStream_t st) {
    const int wpb = 4;
    const unsigned blocks = (unsigned)std::max<int64_t>(1, (nchunks + wpb - 1) / wpb);
    if (Q == 19) {
        if (ra == 1) k_wss<19, 1><<<blocks, 32 * wpb, 0, st>>>(chunks, nchunks, mmask, out_pos, insts, u, wss, wall_flag);
        else k_wss<19, 2><<<blocks, 32 * wpb, 0, st>>>(chunks, nchunks, mmask, out_pos, insts, u, wss, wall_flag);
    } else {
        if (ra == 1) k_wss<27, 1><<<blocks, 32 * wpb, 0, st>>>(chunks, nchunks, mmask, out_pos, insts, u, wss, wall_flag);
        else k_wss<27, 2><<<blocks, 32 * wpb, 0, st>>>(chunks, nchunks, mmask, out_pos, insts, u, wss, wall_flag);
    }
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(LBM_ERR_CUDA, "wall shear stress launch: %s", cudaGetErrorString(e));
    return LBM_OK;
}

}  // namespace lbm
