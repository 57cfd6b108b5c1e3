// Device-side definitions shared by the CUDA translation units.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>

#include "lbm_gb300.h"

namespace lbm {

// ---------------------------------------------------------------------------
// Lattice tables (LatticeModel.cpp:51-151 for D3Q19 with the rest population
// at index 18; :208-334 for D3Q27 with the rest population at index 0).
template <int Q> struct Lat;

template <> struct Lat<19> {
    static constexpr int Q = 19;
    static constexpr int REST = 18;
    // direction index excluded from bounce-back (ApplyWallBc loops dir = 1..Q-1,
    // Simulation.cpp:1361): population opp(0) = 1 is never bounced back.
    static constexpr int NO_BB_POP = 1;
    __host__ __device__ static constexpr int cx(int q) {
        constexpr int v[19] = {1, -1, 0, 0, 0, 0, 1, 1, 1, 1, -1, -1, -1, -1, 0, 0, 0, 0, 0};
        return v[q];
    }
    __host__ __device__ static constexpr int cy(int q) {
        constexpr int v[19] = {0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0};
        return v[q];
    }
    __host__ __device__ static constexpr int cz(int q) {
        constexpr int v[19] = {0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 1, -1, 0};
        return v[q];
    }
    __host__ __device__ static constexpr int opp(int q) {
        constexpr int v[19] = {1, 0, 3, 2, 5, 4, 11, 10, 13, 12, 7, 6, 9, 8, 17, 16, 15, 14, 18};
        return v[q];
    }
    // weights exactly as the reference's double expressions 2/36, 1/36, 12/36
    __host__ __device__ static constexpr double w(int q) {
        return q < 6 ? 2.0 / 36.0 : (q < 18 ? 1.0 / 36.0 : 12.0 / 36.0);
    }
};

template <> struct Lat<27> {
    static constexpr int Q = 27;
    static constexpr int REST = 0;
    static constexpr int NO_BB_POP = -1;   // ApplyWallBc dir = 1..26 covers every moving direction
    __host__ __device__ static constexpr int cx(int q) {
        constexpr int v[27] = {0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, -1, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1};
        return v[q];
    }
    __host__ __device__ static constexpr int cy(int q) {
        constexpr int v[27] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, -1, 1, -1, -1, 1, -1, 1};
        return v[q];
    }
    __host__ __device__ static constexpr int cz(int q) {
        constexpr int v[27] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, -1, 1, -1, 1, -1, -1, 1, 1, -1, -1, 1};
        return v[q];
    }
    __host__ __device__ static constexpr int opp(int q) {
        constexpr int v[27] = {0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15, 20, 19, 22, 21, 24, 23, 26, 25};
        return v[q];
    }
    __host__ __device__ static constexpr double w(int q) {
        return q == 0 ? 8.0 / 27.0 : (q < 7 ? 2.0 / 27.0 : (q < 19 ? 1.0 / 54.0 : 1.0 / 216.0));
    }
};

// ---------------------------------------------------------------------------
// Ghost-padded run lattice.  Nodes are the fluid points plus a one-cell ghost
// layer (points that are not fluid but have a fluid point among their 26
// neighbours, on a grid padded by one cell so the layer is complete).  Nodes
// are numbered with the run axis fastest (z in the reference's x-major order,
// y when the vessels run along y); the two other axes (a, b) span the grid
// columns.  Each run of consecutive fluid points along the run axis is cut
// into chunks of at most 32 nodes, one warp per chunk, one lane per node.
//
// Because every 26-neighbour of a fluid point is a node, each neighbouring
// column holds nodes at every level r0-1 .. r0+len of a chunk, with
// consecutive ids; so the node id of a neighbour of lane t at column offset
// (da, db) and level offset o is K[col8(da, db)] + 1 + o + t (own column:
// n0 + o + t).  Ghost nodes are never updated; a boundary node carries a
// mask of the populations whose source is a ghost ("missing").
struct __align__(64) Chunk {
    int32_t n0;        // node id of lane 0 (every lane is a fluid node)
    uint32_t len_inst; // bits 0-5: nodes (1..32); bits 8-31: instance
    uint32_t wmask;    // lanes that are wall nodes (bounce-back)
    uint32_t zmask;    // lanes that carry a Zou-He boundary condition
    uint32_t bmask;    // lanes that are boundary nodes (may miss a source)
    int32_t zslot0;    // Zou-He slot of the first zmask lane
    int32_t mslot0;    // missing-mask slot of the first bmask lane
    int32_t K[8];      // neighbour columns: node id at level r0-1, index col8(da, db)
    uint32_t vmask;    // paired chunks: node slots that are fluid (the others are ghosts)
};
static_assert(sizeof(Chunk) == 64, "chunk descriptor is one 64-byte sector pair");

// (da, db) in {-1,0,1}^2 minus (0,0) -> 0..7
__host__ __device__ constexpr int col8(int da, int db) {
    return (da + 1) * 3 + (db + 1) - ((da + 1) * 3 + (db + 1) > 4 ? 1 : 0);
}

// Zou-He slot of one boundary node.
struct ZSlot {
    double profile;    // inlet profile factor (1 for outlets)
    int32_t list;      // global list index (instance lists concatenated)
    int32_t kind;      // lbm_bc_kind
};

// Per-list boundary parameters (device table).
struct ListParam {
    double rho;        // outlet density
    double dir[3];     // inlet direction
    int64_t amp_off;   // offset into the amplitude table array
    int64_t amp_len;   // period of the amplitude table (>= 1)
    int32_t kind;
    int32_t face;      // lbm_face of the LBM_BC_VELOCITY / LBM_BC_PRESSURE kinds
};

// Per-instance parameters.
struct InstParam {
    double omega;      // 1/tau
    float omega_f;
    float pad;
    double tau;
};

// Storage formats.  Shifted formats hold (f - w) scaled; FP64/FP32 hold f.
enum Store { ST_F64 = 0, ST_F32 = 1, ST_F16S = 2, ST_BF16S = 3 };
constexpr float kF16Scale = 32768.0f;    // 2^15 keeps small deviations out of FP16 subnormals

template <int S> struct StoreT;
template <> struct StoreT<ST_F64> { using T = double; static constexpr int bytes = 8; };
template <> struct StoreT<ST_F32> { using T = float; static constexpr int bytes = 4; };
template <> struct StoreT<ST_F16S> { using T = __half; static constexpr int bytes = 2; };
template <> struct StoreT<ST_BF16S> { using T = __nv_bfloat16; static constexpr int bytes = 2; };

// Arguments of one step launch.
struct StepArgs {
    const Chunk* chunks;
    int64_t nchunks;
    const uint32_t* mmask;    // missing-population masks of boundary lanes
    const void* src;          // populations read (pull) / the single lattice (AA)
    void* dst;                // populations written (pull) / same as src (AA)
    int64_t stride;           // elements between population planes (SoA)
    const ZSlot* zslots;
    const ListParam* lists;
    const InstParam* insts;
    const double* amp;        // concatenated amplitude tables
    int64_t step;             // reference iteration index of this step
    const int64_t* step_base; // when non-null, added to step (graph replays)
    // snapshot outputs (dry launch only): f (node-major, Q per node), rho, u (3 per node)
    double* out_f;
    double* out_rho;
    double* out_u;
    const int32_t* out_pos;   // output position of each node (x-major rank of the fluid point)
    int64_t n_nodes;
    uint32_t corr;            // lbm_sim_params.corrections (LBM_FIX_* bits)
    int32_t piece_lg;         // paired kernel: log2 of the lanes per chunk piece (2, 3 or 4)
    int64_t pf_ahead;         // paired kernel: L2 prefetch distance in chunk pieces (0 = none)
    const uint2* even_desc;   // paired kernel, AA even launch: per piece (n0, len_inst | 64 if a Zou-He lane)
    uint32_t spin_limit;      // TMA-staged kernel: polls of a stage's mbarrier before giving up (0 = default)
    int32_t stall_first;      // TMA-staged kernel, failure tests: each warp's first stage is never issued
};

}  // namespace lbm

// CUDA error check for host code returning lbm_status.
#define LBM_CUDA(call)                                                                          \
    do {                                                                                        \
        cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess)                                                                  \
            return ::lbm::fail(LBM_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                               __FILE__, __LINE__);                                             \
    } while (0)
