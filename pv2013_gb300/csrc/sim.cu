// Device lattice construction and the simulation handle (host orchestration +
// set-up kernels).  Replaces SubDomain (Subdomain.cpp:3-33, :375-651) and the
// Simulation driver (Simulation.cpp:3-13, :903-932) for one GPU.
//
// Lattice layout in HBM
//   nodes         the fluid points plus a one-cell ghost layer around them,
//                 on the grid padded by one cell on every side, numbered
//                 with the run axis (y or z) fastest (device.cuh)
//   populations   SoA planes, plane q holds population q of every node;
//                 plane stride = node count padded to 64 elements (128 B for
//                 16-bit storage); two plane sets for the pull pattern, one
//                 for AA
//   chunks        one 64-byte descriptor per <=32-node run piece (device.cuh):
//                 with the missing masks of boundary lanes, the only per-step
//                 index traffic (~2.5 B per fluid node on a vascular tree)
//   Zou-He slots  16 B per inlet/outlet node; list and instance tables
// Node typing follows CreateNodes (Subdomain.cpp:399-477): a boundary point
// takes the first predicate list that contains it (lowest list id, the
// reference's Inlet, Outlet1..6 order); boundary points in no list are wall
// nodes; other fluid points are interior nodes.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "device.cuh"
#include "internal.h"
#include "scan.cuh"
#include "nvtx.h"
#include "step.h"
#include "step_kernel.cuh"

namespace lbm {
// geometry accessors (geometry.cu)
const uint8_t* geometry_flags_dev(const lbm_geometry* g);
const int64_t* geometry_bidx_dev(const lbm_geometry* g);
const uint64_t* geometry_bmask_dev(const lbm_geometry* g);
int64_t geometry_nboundary(const lbm_geometry* g);
int64_t geometry_nfluid(const lbm_geometry* g);
void geometry_dims(const lbm_geometry* g, int dims[3]);
int geometry_device(const lbm_geometry* g);
}  // namespace lbm

using namespace lbm;

extern "C" void lbm_sim_destroy(lbm_sim* S);

namespace lbm {

// The pool keeps this much memory between frees and allocations (default
// pools of this process only; nothing outlives the process).
static constexpr uint64_t kPoolKeepBytes = 8ull << 30;

lbm_status dev_alloc(void** p, size_t bytes, void* stream, const char* what) {
    static std::mutex mu;
    static bool tuned[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess && dev >= 0 && dev < 64) {
        std::lock_guard<std::mutex> lock(mu);
        if (!tuned[dev]) {
            cudaMemPool_t pool;
            if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
                uint64_t keep = kPoolKeepBytes;
                cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
            }
            cudaGetLastError();
            tuned[dev] = true;
        }
    }
    *p = nullptr;
    const cudaError_t e = cudaMallocAsync(p, bytes, (cudaStream_t)stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return fail(LBM_ERR_NOMEM, "device allocation for %s (%zu bytes) failed: %s", what, bytes, cudaGetErrorString(e));
    }
    return LBM_OK;
}

void dev_free(void* p, void* stream) {
    if (p) cudaFreeAsync(p, (cudaStream_t)stream);
}

}  // namespace lbm

#define LBM_TRY(x)                      \
    do {                                \
        lbm_status s_ = (x);            \
        if (s_ != LBM_OK) return s_;    \
    } while (0)

namespace {

// Device buffer that frees itself, from the device's stream-ordered pool
// (dev_alloc): allocated and freed in the order of the stream that uses it.
template <class T>
struct DBuf {
    T* p = nullptr;
    cudaStream_t s = 0;
    DBuf() = default;
    DBuf(const DBuf&) = delete;
    ~DBuf() { if (p) dev_free(p, s); }
    lbm_status alloc(size_t n, const char* what, cudaStream_t st) {
        if (p) { dev_free(p, s); p = nullptr; }
        s = st;
        return dev_alloc(reinterpret_cast<void**>(&p), sizeof(T) * (n ? n : 1), st, what);
    }
    // takes ownership of pool memory allocated on stream st
    void adopt(T* q, cudaStream_t st) { p = q; s = st; }
    T* release() { T* q = p; p = nullptr; return q; }
};

int blocks_for(int64_t n, int threads) {
    int64_t b = (n + threads - 1) / threads;
    if (b > 152LL * 64) b = 152LL * 64;
    return (int)std::max<int64_t>(b, 1);
}

// --------------------------------------------------------------------------
// set-up kernels

__global__ void k_scatter_ids(const int64_t* __restrict__ node_grid, int64_t n, int32_t* __restrict__ node_of_point) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        node_of_point[node_grid[i]] = (int32_t)i;
}

// Grid permutation for the run axis.  Permuted layout: index (a*Nb + b)*Nr + r
// with r the run axis; for run axis z it is the x-major layout itself, for
// run axis y it is (x*Nz + z)*Ny + y.
struct Perm {
    int ra;             // 1 (y) or 2 (z)
    int Nx, Ny, Nz;
    __host__ __device__ int Na() const { return Nx; }
    __host__ __device__ int Nb() const { return ra == 2 ? Ny : Nz; }
    __host__ __device__ int Nr() const { return ra == 2 ? Nz : Ny; }
    __host__ __device__ int64_t to_perm(int64_t o) const {
        if (ra == 2) return o;
        const int64_t k = o % Nz, t = o / Nz, j = t % Ny, i = t / Ny;
        return (i * Nz + k) * Ny + j;
    }
    __host__ __device__ int64_t to_orig(int64_t p) const {
        if (ra == 2) return p;
        const int64_t j = p % Ny, t = p / Ny, k = t % Nz, i = t / Nz;
        return (i * Ny + j) * Nz + k;
    }
};

__global__ void k_permute_flags(const uint8_t* __restrict__ in, Perm P, uint8_t* __restrict__ out) {
    const int64_t n = (int64_t)P.Nx * P.Ny * P.Nz;
    for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < n; o += (int64_t)gridDim.x * blockDim.x)
        out[P.to_perm(o)] = in[o];
}

// Node types on the padded permuted grid (one extra cell on every side):
// 2 fluid, 1 ghost (not fluid, a fluid point among its 26 neighbours), 0 none.
struct Pad {
    int Na, Nb, Nr;                       // unpadded permuted dims
    __host__ __device__ int64_t Pa() const { return Na + 2; }
    __host__ __device__ int64_t Pb() const { return Nb + 2; }
    // padded run-axis length, rounded up to even (node ids keep the parity of
    // their level, which needs every column to end at an odd level)
    __host__ __device__ int64_t Pr() const { return (Nr + 3) & ~int64_t(1); }
    __host__ __device__ int64_t cells() const { return Pa() * Pb() * Pr(); }
    __host__ __device__ int64_t cell(int64_t a, int64_t b, int64_t r) const { return (a * Pb() + b) * Pr() + r; }
};

// Node types by separable dilation: the 3x3x3 neighbourhood test as three
// 3-point passes (run axis, b, a), one thread per cell with the coordinates
// taken from the launch grid.
__global__ void k_dil_r(const uint8_t* __restrict__ pflags, Pad D, uint8_t* __restrict__ t1) {
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t b = blockIdx.y, a = blockIdx.z;
    if (r >= D.Pr()) return;
    uint8_t v = 0;
    if (a >= 1 && a <= D.Na && b >= 1 && b <= D.Nb) {
        const uint8_t* col = pflags + ((a - 1) * D.Nb + (b - 1)) * (int64_t)D.Nr;
        for (int64_t rr = r - 1; rr <= r + 1; ++rr)
            if (rr >= 1 && rr <= D.Nr && col[rr - 1]) v = 1;
    }
    t1[D.cell(a, b, r)] = v;
}
__global__ void k_dil_b(const uint8_t* __restrict__ t1, Pad D, uint8_t* __restrict__ t2) {
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t b = blockIdx.y, a = blockIdx.z;
    if (r >= D.Pr()) return;
    uint8_t v = 0;
    for (int64_t bb = b - 1; bb <= b + 1; ++bb)
        if (bb >= 0 && bb < D.Pb()) v |= t1[D.cell(a, bb, r)];
    t2[D.cell(a, b, r)] = v;
}
__global__ void k_dil_a(const uint8_t* __restrict__ t2, const uint8_t* __restrict__ pflags, Pad D,
                        uint8_t* __restrict__ type) {
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t b = blockIdx.y, a = blockIdx.z;
    if (r >= D.Pr()) return;
    uint8_t v = 0;
    for (int64_t aa = a - 1; aa <= a + 1; ++aa)
        if (aa >= 0 && aa < D.Pa()) v |= t2[D.cell(aa, b, r)];
    const bool fluid = a >= 1 && a <= D.Na && b >= 1 && b <= D.Nb && r >= 1 && r <= D.Nr &&
                       pflags[((a - 1) * D.Nb + (b - 1)) * (int64_t)D.Nr + (r - 1)] != 0;
    type[D.cell(a, b, r)] = fluid ? 2 : (v ? 1 : 0);
}

// type of every padded cell (2 fluid, 1 ghost, 0 none); scratch: one more
// byte per cell
lbm_status compute_types(const uint8_t* pflags, const Pad& D, uint8_t* type, cudaStream_t st) {
    DBuf<uint8_t> tmp;
    LBM_TRY(tmp.alloc(D.cells(), "node type scratch", st));
    const dim3 grid((unsigned)((D.Pr() + 255) / 256), (unsigned)D.Pb(), (unsigned)D.Pa());
    k_dil_r<<<grid, 256, 0, st>>>(pflags, D, type);
    k_dil_b<<<grid, 256, 0, st>>>(type, D, tmp.p);
    k_dil_a<<<grid, 256, 0, st>>>(tmp.p, pflags, D, type);
    LBM_CUDA(cudaGetLastError());
    LBM_CUDA(cudaStreamSynchronize(st));   // the scratch is freed on return
    return LBM_OK;
}

// Extra ghost nodes so that every node id has the parity of its level: one
// below every segment of consecutive nodes that starts at an odd level and one
// above every segment that ends at an even level.  Then every segment starts
// at an even level and has even length, so ids (assigned in cell order) keep
// id = level (mod 2).  Changing a cell in place never changes another cell's
// test.
__global__ void k_parity_ghosts(Pad D, uint8_t* __restrict__ type) {
    const int64_t n = D.cells();
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
        if (type[c]) continue;
        const int64_t r = c % D.Pr();
        if ((r & 1) == 0 ? (r + 1 < D.Pr() && type[c + 1]) : (type[c - 1] != 0)) type[c] = 1;
    }
}

// out_pos of every node: x-major rank of its fluid point (ghosts: -1)
__global__ void k_out_pos(const int64_t* __restrict__ node_cell, int64_t n, const uint8_t* __restrict__ type, Pad D,
                          Perm P, const int32_t* __restrict__ rank_of_point, int64_t out_off, int32_t* __restrict__ pos) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = node_cell[i];
        if (type[c] != 2) { pos[i] = -1; continue; }
        const int64_t r = c % D.Pr(), t = c / D.Pr();
        const int64_t b = t % D.Pb(), a = t / D.Pb();
        const int64_t p = ((a - 1) * D.Nb + (b - 1)) * D.Nr + (r - 1);
        pos[i] = (int32_t)(out_off + rank_of_point[P.to_orig(p)]);
    }
}

// role per node: -1 ghost, 0 interior, 1 wall, 2+l first matching predicate list l
__global__ void k_roles_fluid(const int64_t* __restrict__ node_cell, int64_t n, const uint8_t* __restrict__ type,
                              int8_t* __restrict__ role) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        role[i] = type[node_cell[i]] == 2 ? 0 : -1;
}

__global__ void k_roles(const int64_t* __restrict__ bidx, const uint64_t* __restrict__ bmask, int64_t nb, Perm P, Pad D,
                        const int32_t* __restrict__ node_of_cell, int8_t* __restrict__ role) {
    for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < nb; b += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = P.to_perm(bidx[b]);
        const int64_t r = p % D.Nr, t = p / D.Nr;
        const int64_t bb = t % D.Nb, a = t / D.Nb;
        const int32_t n = node_of_cell[D.cell(a + 1, bb + 1, r + 1)];
        const uint64_t m = bmask[b];
        role[n] = m ? (int8_t)(2 + __ffsll((long long)m) - 1) : (int8_t)1;
    }
}

__global__ void k_zflag(const int8_t* __restrict__ role, int64_t n, uint64_t zlists, uint8_t* __restrict__ z) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int r = role[i];
        z[i] = (r >= 2 && ((zlists >> (r - 2)) & 1ull)) ? 1 : 0;
    }
}

__global__ void k_gather_role(const int64_t* __restrict__ ids, int64_t n, const int8_t* __restrict__ role,
                              const int32_t* __restrict__ pos, int8_t* __restrict__ out, int32_t* __restrict__ out_pos) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        out[i] = role[ids[i]];
        out_pos[i] = pos[ids[i]];
    }
}

// per padded column (a, b): chunks (runs of fluid cells, <= 32) and boundary lanes
__global__ void k_col_count(const uint8_t* __restrict__ type, const int32_t* __restrict__ node_of_cell,
                            const int8_t* __restrict__ role, Pad D, int32_t* __restrict__ nchunk,
                            int32_t* __restrict__ nbound) {
    const int64_t ncol = (int64_t)D.Na * D.Nb;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ncol; c += (int64_t)gridDim.x * blockDim.x) {
        const int64_t a = c / D.Nb + 1, b = c % D.Nb + 1;
        const int64_t base = D.cell(a, b, 0);
        int32_t nc = 0, nbd = 0;
        int run = 0;
        for (int64_t r = 0; r <= D.Pr(); ++r) {
            const bool fl = r < D.Pr() && type[base + r] == 2;
            if (fl) {
                ++run;
                if (role[node_of_cell[base + r]] >= 1) ++nbd;
            }
            if (!fl || run == 32) {
                if (run > 0) ++nc;
                run = 0;
            }
        }
        nchunk[c] = nc;
        nbound[c] = nbd;
    }
}

struct Vel {
    int8_t a[27], b[27], r[27];   // velocity components in (column a, column b, run) order
    int Q;
};

struct FillArgs {
    const uint8_t* type;
    const int32_t* node_of_cell;
    const int8_t* role;
    Pad D;
    Vel V;
    const int64_t* chunk_off;     // per column
    const int64_t* mslot_off;     // per column
    const int64_t* znodes;        // sorted local ids of Zou-He nodes
    int64_t nz;
    int64_t node_off, zslot_off, mslot_base;
    int32_t inst;
    int32_t piece;                // node slots per paired chunk piece (k_col_fill2)
    Chunk* chunks;
    uint32_t* mmask;
    int32_t* err;
};

__device__ int64_t lower_bound_i64(const int64_t* a, int64_t n, int64_t v) {
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        int64_t mid = (lo + hi) >> 1;
        if (a[mid] < v) lo = mid + 1; else hi = mid;
    }
    return lo;
}

__global__ void k_col_fill(FillArgs A) {
    const Pad& D = A.D;
    const int64_t ncol = (int64_t)D.Na * D.Nb;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ncol; c += (int64_t)gridDim.x * blockDim.x) {
        const int64_t a = c / D.Nb + 1, b = c % D.Nb + 1;
        const int64_t base = D.cell(a, b, 0);
        int64_t out = A.chunk_off[c];
        int64_t ms = A.mslot_off[c];
        int run = 0;
        int64_t r0 = 0;
        for (int64_t r = 0; r <= D.Pr(); ++r) {
            const bool fl = r < D.Pr() && A.type[base + r] == 2;
            if (fl) { if (run == 0) r0 = r; ++run; }
            if (!fl || run == 32) {
                if (run > 0) {
                    Chunk ch;
                    const int32_t n0 = A.node_of_cell[base + r0];
                    ch.n0 = (int32_t)(A.node_off + n0);
                    ch.len_inst = (uint32_t)run | ((uint32_t)A.inst << 8);
                    ch.wmask = ch.zmask = ch.bmask = 0;
                    ch.vmask = run == 32 ? 0xffffffffu : (1u << run) - 1u;
                    ch.mslot0 = (int32_t)(A.mslot_base + ms);
                    for (int t = 0; t < run; ++t) {
                        const int ro = A.role[n0 + t];
                        if (ro == 1) ch.wmask |= 1u << t;
                        if (ro >= 1) {
                            ch.bmask |= 1u << t;
                            uint32_t m = 0;
                            for (int q = 0; q < A.V.Q; ++q) {
                                const int64_t sc = D.cell(a - A.V.a[q], b - A.V.b[q], r0 + t - A.V.r[q]);
                                if (A.type[sc] != 2) m |= 1u << q;
                            }
                            A.mmask[ms++] = m;
                        }
                    }
                    const int64_t zfirst = lower_bound_i64(A.znodes, A.nz, n0);
                    ch.zslot0 = (int32_t)(A.zslot_off + zfirst);
                    for (int64_t zz = zfirst; zz < A.nz && A.znodes[zz] < n0 + run; ++zz)
                        ch.zmask |= 1u << (int)(A.znodes[zz] - n0);
                    for (int da = -1; da <= 1; ++da)
                        for (int db = -1; db <= 1; ++db) {
                            if (da == 0 && db == 0) continue;
                            const int32_t k = A.node_of_cell[D.cell(a + da, b + db, r0 - 1)];
                            // every level r0-1 .. r0+run of a neighbour column is a node
                            // with consecutive ids (ghost layer); checked at both ends
                            const int32_t k2 = A.node_of_cell[D.cell(a + da, b + db, r0 + run)];
                            if (k < 0 || k2 != k + run + 1) atomicOr(A.err, 1);
                            ch.K[col8(da, db)] = (int32_t)(A.node_off + (k < 0 ? 0 : k));
                        }
                    if (n0 < 1 || A.node_of_cell[base + r0 - 1] != n0 - 1 ||
                        A.node_of_cell[base + r0 + run] != n0 + run)
                        atomicOr(A.err, 1);
                    A.chunks[out++] = ch;
                }
                run = 0;
            }
        }
    }
}

// Paired chunks: each fluid run [rf, re] of a column widened to whole pairs
// [rf & ~1, re | 1] (the added slots are ghost nodes) and cut every `piece`
// slots (8, 16 or 32).
__global__ void k_col_count2(const uint8_t* __restrict__ type, Pad D, int piece, int32_t* __restrict__ nchunk) {
    const int64_t ncol = (int64_t)D.Na * D.Nb;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ncol; c += (int64_t)gridDim.x * blockDim.x) {
        const int64_t a = c / D.Nb + 1, b = c % D.Nb + 1;
        const int64_t base = D.cell(a, b, 0);
        int32_t nc = 0;
        int64_t rf = -1;
        for (int64_t r = 0; r <= D.Pr(); ++r) {
            const bool fl = r < D.Pr() && type[base + r] == 2;
            if (fl && rf < 0) rf = r;
            if (!fl && rf >= 0) {
                const int64_t r0 = rf & ~int64_t(1), r1 = (r - 1) | 1;
                nc += (int32_t)((r1 - r0 + 1 + piece - 1) / piece);
                rf = -1;
            }
        }
        nchunk[c] = nc;
    }
}

__global__ void k_col_fill2(FillArgs A) {
    const Pad& D = A.D;
    const int64_t ncol = (int64_t)D.Na * D.Nb;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ncol; c += (int64_t)gridDim.x * blockDim.x) {
        const int64_t a = c / D.Nb + 1, b = c % D.Nb + 1;
        const int64_t base = D.cell(a, b, 0);
        int64_t out = A.chunk_off[c];
        int64_t ms = A.mslot_off[c];
        int64_t rf = -1;
        for (int64_t r = 0; r <= D.Pr(); ++r) {
            const bool fl = r < D.Pr() && A.type[base + r] == 2;
            if (fl && rf < 0) rf = r;
            if (fl || rf < 0) continue;
            const int64_t re = r - 1;
            const int64_t r1 = re | 1;
            for (int64_t r0 = rf & ~int64_t(1); r0 <= r1; r0 += A.piece) {
                const int len = (int)std::min<int64_t>(A.piece, r1 - r0 + 1);
                const int64_t lf = std::max(r0, rf), ll = std::min(r0 + len - 1, re);   // fluid levels of the piece
                Chunk ch;
                const int32_t n0 = A.node_of_cell[base + r0];
                ch.n0 = (int32_t)(A.node_off + n0);
                ch.len_inst = (uint32_t)len | ((uint32_t)A.inst << 8);
                ch.vmask = ch.wmask = ch.zmask = ch.bmask = 0;
                ch.mslot0 = (int32_t)(A.mslot_base + ms);
                if ((n0 & 1) || (r0 & 1) || A.node_of_cell[base + r0 + len - 1] != n0 + len - 1 ||
                    A.node_of_cell[base + lf - 1] != n0 + (int32_t)(lf - 1 - r0) ||
                    A.node_of_cell[base + ll + 1] != n0 + (int32_t)(ll + 1 - r0))
                    atomicOr(A.err, 1);
                for (int64_t lv = lf; lv <= ll; ++lv) {
                    const int j = (int)(lv - r0);
                    ch.vmask |= 1u << j;
                    const int ro = A.role[n0 + j];
                    if (ro == 1) ch.wmask |= 1u << j;
                    if (ro >= 1) { ch.bmask |= 1u << j; ++ms; }
                }
                const int64_t zfirst = lower_bound_i64(A.znodes, A.nz, n0);
                ch.zslot0 = (int32_t)(A.zslot_off + zfirst);
                for (int64_t zz = zfirst; zz < A.nz && A.znodes[zz] < n0 + len; ++zz)
                    ch.zmask |= 1u << (int)(A.znodes[zz] - n0);
                for (int da = -1; da <= 1; ++da)
                    for (int db = -1; db <= 1; ++db) {
                        if (da == 0 && db == 0) continue;
                        // virtual id of level r0-1 such that K + 1 + (level - r0) is the id of
                        // every level of the fluid window lf-1 .. ll+1 (checked at both ends)
                        const int32_t kf = A.node_of_cell[D.cell(a + da, b + db, lf - 1)];
                        const int32_t kl = A.node_of_cell[D.cell(a + da, b + db, ll + 1)];
                        const int32_t k = kf - (int32_t)(lf - r0);
                        // (k + 1 is the id of level r0: even, like every id of an even level)
                        if (kf < 0 || kl != k + 1 + (int32_t)(ll + 1 - r0) || ((k + 1) & 1)) atomicOr(A.err, 1);
                        ch.K[col8(da, db)] = (int32_t)(A.node_off + (kf < 0 ? 0 : k));
                    }
                A.chunks[out++] = ch;
            }
            rf = -1;
        }
    }
}

// Paired pieces regrouped within windows of `win` consecutive pieces (at most
// 1024; 16 warps' worth by default): interior pieces (every slot a fluid
// node, no boundary node) first, then the others, each group in its original
// order.  The paired kernel's boundary work (missing-population fix-ups,
// per-half stores) is decided per warp, so warps made only of interior pieces
// skip it; the window keeps a warp's pieces within a few KB of each other in
// every plane.  Every piece carries its own ids and slots, so the order is free.
constexpr int kGroupMax = 1024;
constexpr int kGroupWarps = 16;         // window: this many warps' pieces (16 * 8 8-slot pieces <= kGroupMax)
__device__ __forceinline__ bool interior_piece(const Chunk& c) {
    const uint32_t len = c.len_inst & 63u;
    const uint32_t full = len >= 32 ? 0xffffffffu : (1u << len) - 1u;
    return c.bmask == 0u && c.zmask == 0u && c.vmask == full;
}
__global__ void __launch_bounds__(kGroupMax) k_group_pieces(const Chunk* __restrict__ in, Chunk* __restrict__ out,
                                                            int64_t n, int win) {
    __shared__ int cnt[kGroupMax / 32];
    const int i = threadIdx.x;
    for (int64_t w = blockIdx.x; w * win < n; w += gridDim.x) {
        const int64_t j = w * win + i;
        const bool have = i < win && j < n;
        Chunk c;
        bool inner = false;
        if (have) { c = in[j]; inner = interior_piece(c); }
        const uint32_t b = __ballot_sync(0xffffffffu, inner);
        if ((i & 31) == 0) cnt[i >> 5] = __popc(b);
        __syncthreads();
        int ninner = 0, before = __popc(b & ((1u << (i & 31)) - 1u));
        for (int k = 0; k < kGroupMax / 32; ++k) {
            ninner += cnt[k];
            if (k < (i >> 5)) before += cnt[k];
        }
        // the pieces of a window are items 0 .. m-1, so i items precede item i
        if (have) out[w * win + (inner ? before : ninner + (i - before))] = c;
        __syncthreads();
    }
}

// The AA even launch's 8-byte piece records: (n0, len_inst), bit 6 of
// len_inst set when the piece has a Zou-He lane (the launch then reads the
// descriptor's zmask); everything else of the 64-byte descriptor serves the
// neighbour launches only.
__global__ void k_even_desc(const Chunk* __restrict__ c, int64_t n, uint2* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const Chunk& ch = c[i];
        out[i] = make_uint2((uint32_t)ch.n0, (ch.len_inst & ~0xc0u) | (ch.zmask ? 64u : 0u));
    }
}

// NaN into every population slot of no fluid node (out_pos < 0, or beyond the
// N lattice nodes): lbm_sim_poison_ghosts.  eb = bytes per stored value.
__global__ void k_poison(void* a, int64_t stride, int Q, int eb, const int32_t* __restrict__ out_pos, int64_t N) {
    const int64_t n = stride * Q;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t id = i % stride;
        if (id < N && out_pos[id] >= 0) continue;
        if (eb == 8) reinterpret_cast<uint64_t*>(a)[i] = 0x7ff8000000000000ull;
        else if (eb == 4) reinterpret_cast<uint32_t*>(a)[i] = 0x7fc00000u;
        else reinterpret_cast<uint16_t*>(a)[i] = 0x7fc0u;        // a quiet NaN in FP16 and in BF16
    }
}

template <class T>
__global__ void k_init_pop(T* __restrict__ a, int64_t stride, int Q, const double* __restrict__ val) {
    const int64_t n = stride * Q;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int q = (int)(i / stride);
        a[i] = (T)val[q];
    }
}
__global__ void k_init_half(__half* a, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        a[i] = __float2half_rn(0.0f);
}
__global__ void k_init_bf16(__nv_bfloat16* a, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        a[i] = __float2bfloat16_rn(0.0f);
}

__global__ void k_add_step(int64_t* base, int64_t inc) { *base += inc; }

struct MonOut {
    double mass, inflow, outflow, maxu;
    int32_t bad;
};

__global__ void k_reduce_partials(Partials p, int64_t nblocks, MonOut* out) {
    // fixed-order reduction: thread t sums a contiguous range, then a
    // fixed tree over 256 threads (deterministic for a given block count)
    __shared__ double s[4][256];
    __shared__ int sb[256];
    const int t = threadIdx.x;
    const int64_t per = (nblocks + 255) / 256;
    const int64_t b = t * per, e = min(nblocks, b + per);
    double a0 = 0, a1 = 0, a2 = 0, a3 = 0;
    int bb = 0;
    for (int64_t i = b; i < e; ++i) {
        a0 += p.mass[i]; a1 += p.inflow[i]; a2 += p.outflow[i]; a3 = fmax(a3, p.maxu[i]); bb |= p.bad[i];
    }
    s[0][t] = a0; s[1][t] = a1; s[2][t] = a2; s[3][t] = a3; sb[t] = bb;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (t < o) {
            s[0][t] += s[0][t + o]; s[1][t] += s[1][t + o]; s[2][t] += s[2][t + o];
            s[3][t] = fmax(s[3][t], s[3][t + o]); sb[t] |= sb[t + o];
        }
        __syncthreads();
    }
    if (t == 0) { out->mass = s[0][0]; out->inflow = s[1][0]; out->outflow = s[2][0]; out->maxu = s[3][0]; out->bad = sb[0]; }
}

int store_of(int precision) {
    switch (precision) {
        case LBM_F64: return ST_F64;
        case LBM_F32: return ST_F32;
        case LBM_F16S: return ST_F16S;
        case LBM_BF16S: return ST_BF16S;
    }
    return -1;
}
int store_bytes(int s) { return s == ST_F64 ? 8 : (s == ST_F32 ? 4 : 2); }

}  // namespace

// ---------------------------------------------------------------------------

constexpr int64_t kLatticeSlack = 8;   // even: node ids keep the parity of their level
constexpr int kDryWarps = 4;           // warps per block of snapshot / monitor launches

struct lbm_sim {
    int dev = 0;
    int Q = 19, store = ST_F64, pattern = LBM_PULL, wpb = 4, ra = 2, staging = 0, npl = 1;
    int piece = 8;                 // node slots per paired chunk piece (8, 16 or 32)
    uint32_t corr = 0;             // LBM_FIX_* bits
    int32_t* err = nullptr;        // device flag: a bounded wait in the step kernel gave up
    int64_t N = 0, nchunks = 0, stride = 0, nz = 0;
    int64_t n_inst = 0;
    void* buf[2] = {nullptr, nullptr};
    int cur = 0;                   // pull: buffer holding the current state
    Chunk* chunks = nullptr;
    Chunk* chunks2 = nullptr;      // paired chunk table in use (nodes_per_lane = 2): chunks2s[piece]
    int64_t nchunks2 = 0;
    Chunk* chunks2s[3] = {nullptr, nullptr, nullptr};   // paired tables of 8-, 16- and 32-slot pieces
    Chunk* chunks2g = nullptr;     // the same pieces grouped (k_group_pieces): the AA odd launch's table
    Chunk* chunks2gs[3] = {nullptr, nullptr, nullptr};
    uint2* even2 = nullptr;        // the AA even launch's 8-byte records of chunks2 (k_even_desc)
    uint2* even2s[3] = {nullptr, nullptr, nullptr};
    int64_t nchunks2s[3] = {0, 0, 0};
    int aa_phase = 0;              // AA: launch n is an even (node-local) launch when n + aa_phase is even
    ZSlot* zslots = nullptr;
    ListParam* lists = nullptr;
    InstParam* insts = nullptr;
    double* amp = nullptr;
    int64_t NF = 0;                // fluid nodes (outputs); N counts fluid + ghost lattice nodes
    int64_t nmask = 0;
    uint32_t* mmask = nullptr;     // missing-population masks of boundary nodes
    int64_t* node_grid = nullptr;  // x-major grid index of each output node (per instance, x-major order)
    int32_t* out_pos = nullptr;    // output position (x-major rank) of each lattice node, -1 for ghosts
    std::vector<int64_t> inst_off; // output (fluid node) offsets, n_inst + 1
    int64_t steps_done = 0;
    // graph replay
    cudaGraphExec_t gexec = nullptr;
    cudaGraph_t graph = nullptr;
    int64_t glen = 0;
    int64_t* step_base = nullptr;
    // monitors
    double* part = nullptr;        // 4 * nblocks doubles
    int32_t* partbad = nullptr;
    MonOut* mon = nullptr;
    int64_t part_blocks = 0;
    double mass0 = 0.0;
    double div_tol = 1e-2;
    uint32_t spin_limit = 0;       // TMA-staged kernel's wait limit (0 = its default)
    int32_t stall_first = 0;       // failure tests: the TMA-staged kernel's first stages are not issued
    // wall nodes: output positions in wall-list order (built on first use)
    int64_t* wall_pos = nullptr;
    int64_t nwall = -1;
    std::vector<std::array<int, 3>> dims;   // grid of each instance
};

namespace {

struct InstBuild {
    int64_t N = 0;                 // nodes (fluid + ghost)
    int64_t NF = 0;                // fluid nodes
    DBuf<int64_t> node_grid;       // x-major grid indices of the fluid points, x-major order
    DBuf<int32_t> out_pos;         // output position of each node (-1 for ghosts)
    DBuf<Chunk> chunks;
    int64_t nchunks = 0;
    DBuf<Chunk> chunks2[3];        // paired pieces of 8, 16 and 32 slots
    int64_t nchunks2[3] = {0, 0, 0};
    DBuf<uint32_t> mmask;
    int64_t nmask = 0;
    std::vector<ZSlot> zslots;
};

Vel make_vel(int Q, int ra) {
    Vel v;
    v.Q = Q;
    for (int q = 0; q < Q; ++q) {
        int c[3];
        if (Q == 19) { c[0] = Lat<19>::cx(q); c[1] = Lat<19>::cy(q); c[2] = Lat<19>::cz(q); }
        else { c[0] = Lat<27>::cx(q); c[1] = Lat<27>::cy(q); c[2] = Lat<27>::cz(q); }
        v.a[q] = (int8_t)c[0];
        v.b[q] = (int8_t)(ra == 2 ? c[1] : c[2]);
        v.r[q] = (int8_t)(ra == 2 ? c[2] : c[1]);
    }
    return v;
}

// Chunk count of a run axis straight from the x-major fluid flags (no
// permutation, no node typing): the fluid runs along the axis, each cut into
// pieces of `piece` slots, widened to whole pairs of padded levels when
// `pairs` (the paired kernel's pieces, k_col_count2); summed into *total.
__global__ void k_count_runs(const uint8_t* __restrict__ flags, int Nx, int Ny, int Nz, int ra, int piece, int pairs,
                             unsigned long long* __restrict__ total) {
    const int64_t nb = ra == 2 ? Ny : Nz, len = ra == 2 ? Nz : Ny, stride = ra == 2 ? 1 : Nz;
    const int64_t ncol = (int64_t)Nx * nb;
    unsigned long long cnt = 0;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ncol; c += (int64_t)gridDim.x * blockDim.x) {
        const int64_t x = c / nb, b = c % nb;
        const int64_t base = ra == 2 ? (x * Ny + b) * Nz : x * (int64_t)Ny * Nz + b;
        int64_t rf = -1;
        for (int64_t r = 0; r <= len; ++r) {
            const bool fl = r < len && flags[base + r * stride] != 0;
            if (fl && rf < 0) rf = r;
            if (!fl && rf >= 0) {
                int64_t lo = rf + 1, hi = r;                 // padded levels of the run
                if (pairs) { lo &= ~int64_t(1); hi |= 1; }
                cnt += (unsigned long long)((hi - lo + piece) / piece);
                rf = -1;
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(total, cnt);
}

// Number of chunks of the step kernel in use (paired pieces of `piece`
// slots, or one-node chunks of at most 32 nodes) for a run axis.
lbm_status count_chunks(const lbm_geometry* g, int ra, int piece, bool pairs, cudaStream_t st, int64_t* n) {
    int dims[3];
    geometry_dims(g, dims);
    DBuf<unsigned long long> tot;
    LBM_TRY(tot.alloc(1, "chunk count", st));
    LBM_CUDA(cudaMemsetAsync(tot.p, 0, sizeof(unsigned long long), st));
    const int64_t ncol = (int64_t)dims[0] * (ra == 2 ? dims[1] : dims[2]);
    k_count_runs<<<blocks_for(ncol, 128), 128, 0, st>>>(geometry_flags_dev(g), dims[0], dims[1], dims[2], ra, piece,
                                                          pairs ? 1 : 0, tot.p);
    LBM_CUDA(cudaGetLastError());
    unsigned long long h = 0;
    LBM_CUDA(cudaMemcpyAsync(&h, tot.p, sizeof h, cudaMemcpyDeviceToHost, st));
    LBM_CUDA(cudaStreamSynchronize(st));
    *n = (int64_t)h;
    return LBM_OK;
}

lbm_status build_instance(const lbm_geometry* g, const lbm_sim_params* p, int Q, int32_t inst, int ra, int npl,
                          int piece, int64_t node_off, int64_t out_off, int64_t zslot_off, int64_t mslot_off, int32_t* d_err,
                          cudaStream_t st, InstBuild& out) {
    int dims[3];
    geometry_dims(g, dims);
    const Perm P{ra, dims[0], dims[1], dims[2]};
    const int64_t npts = (int64_t)dims[0] * dims[1] * dims[2];
    const uint8_t* flags = geometry_flags_dev(g);
    DBuf<uint8_t> fperm;
    const uint8_t* pflags = flags;
    if (ra != 2) {
        LBM_TRY(fperm.alloc(npts, "permuted flags", st));
        k_permute_flags<<<blocks_for(npts, 256), 256, 0, st>>>(flags, P, fperm.p);
        pflags = fperm.p;
    }
    // 1. fluid + ghost nodes on the padded grid, numbered in permuted order
    const Pad D{P.Na(), P.Nb(), P.Nr()};
    DBuf<uint8_t> type;
    LBM_TRY(type.alloc(D.cells(), "node types", st));
    LBM_TRY(compute_types(pflags, D, type.p, st));
    k_parity_ghosts<<<blocks_for(D.cells(), 256), 256, 0, st>>>(D, type.p);
    int64_t* nc = nullptr;
    LBM_TRY(scan::compact(type.p, D.cells(), &nc, &out.N, st));
    DBuf<int64_t> node_cell; node_cell.adopt(nc, st);
    if (node_off + out.N >= INT32_MAX) return fail(LBM_ERR_ARG, "more than 2^31 lattice nodes");
    DBuf<int32_t> noc;
    LBM_TRY(noc.alloc(D.cells(), "node map", st));
    LBM_CUDA(cudaMemsetAsync(noc.p, 0xff, sizeof(int32_t) * D.cells(), st));
    k_scatter_ids<<<blocks_for(out.N, 256), 256, 0, st>>>(nc, out.N, noc.p);
    // 2. outputs in x-major order (the reference's node order, Subdomain.cpp:638-651)
    {
        int64_t* xg = nullptr;
        LBM_TRY(scan::compact(flags, npts, &xg, &out.NF, st));
        out.node_grid.adopt(xg, st);
        if (out.NF == 0) return fail(LBM_ERR_ARG, "instance %d has no fluid node", inst);
        DBuf<int32_t> rank;
        LBM_TRY(rank.alloc(npts, "rank map", st));
        k_scatter_ids<<<blocks_for(out.NF, 256), 256, 0, st>>>(xg, out.NF, rank.p);
        LBM_TRY(out.out_pos.alloc(out.N, "output positions", st));
        k_out_pos<<<blocks_for(out.N, 256), 256, 0, st>>>(nc, out.N, type.p, D, P, rank.p, out_off, out.out_pos.p);
    }
    // 3. roles
    DBuf<int8_t> role;
    LBM_TRY(role.alloc(out.N, "node roles", st));
    k_roles_fluid<<<blocks_for(out.N, 256), 256, 0, st>>>(nc, out.N, type.p, role.p);
    const int64_t nb = geometry_nboundary(g);
    if (nb)
        k_roles<<<blocks_for(nb, 256), 256, 0, st>>>(geometry_bidx_dev(g), geometry_bmask_dev(g), nb, P, D, noc.p, role.p);
    // 4. Zou-He nodes: role list with a boundary-condition kind
    int kind[64] = {0};
    const lbm_list_bc* lbc[64] = {nullptr};
    for (size_t b = 0; b < p->nbcs; ++b) {
        const lbm_list_bc& L = p->bcs[b];
        if (L.list_id < 0 || L.list_id > 63) return fail(LBM_ERR_ARG, "bc %zu: list id %d", b, L.list_id);
        kind[L.list_id] = L.kind;
        lbc[L.list_id] = &L;
    }
    uint64_t zl = 0;
    for (int l = 0; l < 64; ++l) if (kind[l] != LBM_BC_NONE) zl |= 1ull << l;
    DBuf<uint8_t> zf;
    LBM_TRY(zf.alloc(out.N, "zou-he flags", st));
    k_zflag<<<blocks_for(out.N, 256), 256, 0, st>>>(role.p, out.N, zl, zf.p);
    int64_t* zn = nullptr;
    int64_t nzn = 0;
    LBM_TRY(scan::compact(zf.p, out.N, &zn, &nzn, st));
    DBuf<int64_t> znodes; znodes.adopt(zn, st);
    {
        // profile values follow the list's x-major order (the reference's
        // InletBoundaryNode_ order); slots follow the internal node order
        DBuf<int8_t> zr;
        DBuf<int32_t> zp;
        LBM_TRY(zr.alloc(nzn, "zou-he roles", st));
        LBM_TRY(zp.alloc(nzn, "zou-he output positions", st));
        if (nzn)
            k_gather_role<<<blocks_for(nzn, 256), 256, 0, st>>>(zn, nzn, role.p, out.out_pos.p, zr.p, zp.p);
        std::vector<int8_t> hr(nzn);
        std::vector<int64_t> hid(nzn);
        if (nzn) {
            std::vector<int32_t> pos(nzn);
            LBM_CUDA(cudaMemcpyAsync(hr.data(), zr.p, nzn, cudaMemcpyDeviceToHost, st));
            LBM_CUDA(cudaMemcpyAsync(pos.data(), zp.p, sizeof(int32_t) * nzn, cudaMemcpyDeviceToHost, st));
            LBM_CUDA(cudaStreamSynchronize(st));
            for (int64_t s = 0; s < nzn; ++s) hid[s] = pos[s];
        }
        std::vector<int64_t> order(nzn);
        for (int64_t s = 0; s < nzn; ++s) order[s] = s;
        std::sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return hid[a] < hid[b]; });
        std::vector<int64_t> rank(64, 0), slot_rank(nzn);
        for (int64_t s : order) slot_rank[s] = rank[hr[s] - 2]++;
        out.zslots.resize(nzn);
        for (int64_t s = 0; s < nzn; ++s) {
            const int l = hr[s] - 2;
            const lbm_list_bc* L = lbc[l];
            ZSlot z;
            z.list = inst * 64 + l;
            z.kind = kind[l];
            const int64_t r = slot_rank[s];
            z.profile = 1.0;
            if (L && L->profile) {
                if ((size_t)r >= L->profile_len)
                    return fail(LBM_ERR_ARG, "list %d: profile has %zu entries, fewer than the list's nodes", l,
                                L->profile_len);
                z.profile = L->profile[r];
            }
            out.zslots[s] = z;
        }
        for (int l = 0; l < 64; ++l) {
            const lbm_list_bc* L = lbc[l];
            if (L && L->profile && L->profile_len != (size_t)rank[l])
                return fail(LBM_ERR_ARG, "list %d: profile has %zu entries, list has %lld nodes", l, L->profile_len,
                            (long long)rank[l]);
        }
    }
    // 5. chunks and missing masks
    const int64_t ncol = (int64_t)D.Na * D.Nb;
    DBuf<int32_t> ccount, bcount;
    DBuf<int64_t> coff, moff;
    LBM_TRY(ccount.alloc(ncol, "chunk counts", st));
    LBM_TRY(bcount.alloc(ncol, "boundary counts", st));
    LBM_TRY(coff.alloc(ncol, "chunk offsets", st));
    LBM_TRY(moff.alloc(ncol, "mask offsets", st));
    k_col_count<<<blocks_for(ncol, 128), 128, 0, st>>>(type.p, noc.p, role.p, D, ccount.p, bcount.p);
    LBM_TRY(scan::exclusive_scan(ccount.p, ncol, coff.p, &out.nchunks, st));
    LBM_TRY(scan::exclusive_scan(bcount.p, ncol, moff.p, &out.nmask, st));
    LBM_TRY(out.chunks.alloc(out.nchunks, "chunks", st));
    LBM_TRY(out.mmask.alloc(out.nmask, "missing masks", st));
    FillArgs fa;
    fa.type = type.p; fa.node_of_cell = noc.p; fa.role = role.p; fa.D = D; fa.V = make_vel(Q, ra);
    fa.chunk_off = coff.p; fa.mslot_off = moff.p;
    fa.znodes = zn; fa.nz = nzn; fa.node_off = node_off; fa.zslot_off = zslot_off; fa.mslot_base = mslot_off;
    fa.inst = inst; fa.chunks = out.chunks.p; fa.mmask = out.mmask.p; fa.err = d_err;
    k_col_fill<<<blocks_for(ncol, 128), 128, 0, st>>>(fa);
    LBM_CUDA(cudaGetLastError());
    if (npl == 2) {
        // paired chunks of every piece size (the autotuner may switch sizes);
        // they share the missing masks (same boundary-node order)
        for (int k = 0; k < 3; ++k) {
            const int pc = 8 << k;
            DBuf<int64_t> coff2;
            LBM_TRY(coff2.alloc(ncol, "paired chunk offsets", st));
            k_col_count2<<<blocks_for(ncol, 128), 128, 0, st>>>(type.p, D, pc, ccount.p);
            LBM_TRY(scan::exclusive_scan(ccount.p, ncol, coff2.p, &out.nchunks2[k], st));
            LBM_TRY(out.chunks2[k].alloc(out.nchunks2[k], "paired chunks", st));
            FillArgs f2 = fa;
            f2.chunk_off = coff2.p;
            f2.chunks = out.chunks2[k].p;
            f2.mmask = nullptr;
            f2.piece = pc;
            k_col_fill2<<<blocks_for(ncol, 128), 128, 0, st>>>(f2);
            LBM_CUDA(cudaGetLastError());
            LBM_CUDA(cudaStreamSynchronize(st));   // coff2 is freed on return
        }
    }
    int32_t herr = 0;
    LBM_CUDA(cudaMemcpyAsync(&herr, d_err, sizeof herr, cudaMemcpyDeviceToHost, st));
    LBM_CUDA(cudaStreamSynchronize(st));
    if (herr) return fail(LBM_ERR_STATE, "lattice construction: a neighbour column window is not fully populated");
    return LBM_OK;
}

lbm_status sim_launch(lbm_sim* S, int mode, bool dry, void* src, void* dst, int64_t step, const int64_t* step_base,
                      const Partials& part, double* of, double* orho, double* ou, cudaStream_t st) {
    StepArgs a{};
    a.chunks = S->chunks; a.nchunks = S->nchunks;
    a.src = src; a.dst = dst; a.stride = S->stride;
    a.zslots = S->zslots; a.lists = S->lists; a.insts = S->insts; a.amp = S->amp;
    a.step = step; a.step_base = step_base;
    a.out_f = of; a.out_rho = orho; a.out_u = ou; a.out_pos = S->out_pos; a.n_nodes = S->NF;
    a.mmask = S->mmask;
    a.corr = S->corr;
    a.spin_limit = S->spin_limit;
    a.stall_first = S->stall_first;
    a.piece_lg = S->piece == 8 ? 2 : (S->piece == 16 ? 3 : 4);
    if (!dry && S->npl == 2) {
        a.chunks = mode == MODE_AA_ODD ? S->chunks2g : S->chunks2;
        a.nchunks = S->nchunks2;
        a.even_desc = S->even2;
        switch (S->store) {
            case ST_F32: return launch_pair_f32(S->Q, mode, S->ra, a, S->wpb, st);
            case ST_F16S: return launch_pair_f16s(S->Q, mode, S->ra, a, S->wpb, st);
            default: return launch_pair_bf16s(S->Q, mode, S->ra, a, S->wpb, st);
        }
    }
    if (!dry && S->staging == 0) {
        switch (S->store) {
            case ST_F64: return launch_tma_f64(S->Q, mode, S->ra, a, S->err, S->wpb, st);
            case ST_F32: return launch_tma_f32(S->Q, mode, S->ra, a, S->err, S->wpb, st);
            case ST_F16S: return launch_tma_f16s(S->Q, mode, S->ra, a, S->err, S->wpb, st);
            default: return launch_tma_bf16s(S->Q, mode, S->ra, a, S->err, S->wpb, st);
        }
    }
    // snapshot / monitor launches use a fixed block (their partial sums are
    // sized for it); steps use the tuned one
    const int wpb = dry ? kDryWarps : S->wpb;
    switch (S->store) {
        case ST_F64: return launch_step_f64(S->Q, mode, dry, S->ra, a, part, wpb, st);
        case ST_F32: return launch_step_f32(S->Q, mode, dry, S->ra, a, part, wpb, st);
        case ST_F16S: return launch_step_f16s(S->Q, mode, dry, S->ra, a, part, wpb, st);
        default: return launch_step_bf16s(S->Q, mode, dry, S->ra, a, part, wpb, st);
    }
}

// The paired kernels' first launch, outside any stream capture and over an
// empty piece list: loads their module and caches the occupancy their
// launcher sizes the L2 prefetch distance with (graph capture may follow).
static lbm_status pair_first_launch(lbm_sim* S, cudaStream_t st) {
    const int save_npl = S->npl;
    const int64_t save_n = S->nchunks2;
    S->npl = 2;
    S->nchunks2 = 0;
    Partials np = {nullptr, nullptr, nullptr, nullptr, nullptr};
    lbm_status s = LBM_OK;
    if (S->pattern == LBM_PULL)
        s = sim_launch(S, MODE_PULL, false, S->buf[0], S->buf[1], 0, nullptr, np, nullptr, nullptr, nullptr, st);
    for (int mode = MODE_AA_EVEN; S->pattern != LBM_PULL && mode <= MODE_AA_ODD && s == LBM_OK; ++mode)
        s = sim_launch(S, mode, false, S->buf[0], S->buf[0], 0, nullptr, np, nullptr, nullptr, nullptr, st);
    S->npl = save_npl;
    S->nchunks2 = save_n;
    if (s != LBM_OK) return s;
    LBM_CUDA(cudaGetLastError());
    return LBM_OK;
}

// The paired piece table of `piece` slots (8, 16 or 32) becomes the one in use.
void select_piece(lbm_sim* S, int piece) {
    const int k = piece == 8 ? 0 : (piece == 16 ? 1 : 2);
    S->piece = piece;
    S->chunks2 = S->chunks2s[k];
    S->chunks2g = S->chunks2gs[k];
    S->even2 = S->even2s[k];
    S->nchunks2 = S->nchunks2s[k];
}

// AA pattern: the launch at the current state is the even (node-local) one
// when steps_done + aa_phase is even (aa_phase changes when a pull state
// becomes an AA state, lbm_sim_set_pattern).
int aa_mode(const lbm_sim* S) { return ((S->steps_done + S->aa_phase) & 1) == 0 ? MODE_AA_EVEN : MODE_AA_ODD; }

// Launches one step at the current state; advances cur/steps_done.
lbm_status sim_one_step(lbm_sim* S, int64_t step_arg, const int64_t* step_base, cudaStream_t st, bool advance_count) {
    Partials np = {nullptr, nullptr, nullptr, nullptr, nullptr};
    lbm_status s;
    if (S->pattern == LBM_PULL) {
        s = sim_launch(S, MODE_PULL, false, S->buf[S->cur], S->buf[1 - S->cur], step_arg, step_base, np, nullptr,
                       nullptr, nullptr, st);
        S->cur = 1 - S->cur;
    } else {
        s = sim_launch(S, aa_mode(S), false, S->buf[0], S->buf[0], step_arg, step_base, np, nullptr, nullptr, nullptr,
                       st);
    }
    if (advance_count) S->steps_done++;
    return s;
}

// Dry launch at the current state (fields and/or monitor partials).
lbm_status sim_dry(lbm_sim* S, double* of, double* orho, double* ou, bool partials, cudaStream_t st) {
    Partials p = {nullptr, nullptr, nullptr, nullptr, nullptr};
    if (partials) {
        p.mass = S->part;
        p.inflow = S->part + S->part_blocks;
        p.outflow = S->part + 2 * S->part_blocks;
        p.maxu = S->part + 3 * S->part_blocks;
        p.bad = S->partbad;
    }
    int mode;
    void* src;
    if (S->pattern == LBM_PULL) { mode = MODE_PULL; src = S->buf[S->cur]; }
    else { mode = aa_mode(S); src = S->buf[0]; }
    LBM_TRY(sim_launch(S, mode, true, src, src, S->steps_done, nullptr, p, of, orho, ou, st));
    if (partials) k_reduce_partials<<<1, 256, 0, st>>>(p, S->part_blocks, S->mon);
    LBM_CUDA(cudaGetLastError());
    return LBM_OK;
}

// Reads the step kernel's error flag (synchronises the stream) and clears it:
// a timeout is reported once.
lbm_status check_timeout(lbm_sim* S, cudaStream_t st) {
    int32_t e = 0;
    LBM_CUDA(cudaMemcpyAsync(&e, S->err, sizeof e, cudaMemcpyDeviceToHost, st));
    LBM_CUDA(cudaStreamSynchronize(st));
    if (e) {
        LBM_CUDA(cudaMemsetAsync(S->err, 0, sizeof(int32_t), st));
        LBM_CUDA(cudaStreamSynchronize(st));
        return fail(LBM_ERR_TIMEOUT, "a bounded wait in the step kernel gave up (staged copies did not arrive)%s; "
                    "the populations are incomplete", (e & 2) ? ", and draining its copies in flight gave up too" : "");
    }
    return LBM_OK;
}

lbm_status sim_monitors(lbm_sim* S, lbm_monitors* out, cudaStream_t st) {
    LBM_TRY(check_timeout(S, st));
    LBM_TRY(sim_dry(S, nullptr, nullptr, nullptr, true, st));
    MonOut h;
    LBM_CUDA(cudaMemcpyAsync(&h, S->mon, sizeof h, cudaMemcpyDeviceToHost, st));
    LBM_CUDA(cudaStreamSynchronize(st));
    out->step = S->steps_done;
    out->mass = h.mass;
    out->inlet_flux = h.inflow;
    out->outlet_flux = h.outflow;
    out->max_speed = h.maxu;
    out->nonfinite = h.bad;
    return LBM_OK;
}

void free_graph(lbm_sim* S) {
    if (S->gexec) cudaGraphExecDestroy(S->gexec);
    if (S->graph) cudaGraphDestroy(S->graph);
    S->gexec = nullptr;
    S->graph = nullptr;
    S->glen = 0;
}

lbm_status sim_create(const lbm_geometry* const* g, const lbm_sim_params* p, size_t n, cudaStream_t st, lbm_sim** out) {
    std::unique_ptr<lbm_sim, void (*)(lbm_sim*)> S(new lbm_sim(), lbm_sim_destroy);
    cudaGetDevice(&S->dev);
    const lbm_sim_params& p0 = p[0];
    if (p0.Q != 19 && p0.Q != 27) return fail(LBM_ERR_ARG, "Q must be 19 or 27 (got %d)", p0.Q);
    S->Q = p0.Q;
    S->store = store_of(p0.precision);
    if (S->store < 0) return fail(LBM_ERR_ARG, "unknown precision %d", p0.precision);
    S->pattern = p0.pattern == LBM_AUTO ? LBM_AA : p0.pattern;
    if (S->pattern != LBM_PULL && S->pattern != LBM_AA) return fail(LBM_ERR_ARG, "unknown pattern %d", p0.pattern);
    // default block: 4 warps for the one-node-per-lane kernels, 1 warp (its
    // chunk pieces) for the paired kernel (measured on the vascular tree)
    S->wpb = p0.warps_per_block > 0 ? p0.warps_per_block : 0;
    if (S->wpb > 8) return fail(LBM_ERR_ARG, "warps_per_block must be <= 8");
    if (p0.run_axis != 0 && p0.run_axis != 1 && p0.run_axis != 2) return fail(LBM_ERR_ARG, "run_axis must be 0, 1 or 2");
    if (p0.staging != 0 && p0.staging != 1) return fail(LBM_ERR_ARG, "staging must be 0 or 1");
    S->staging = p0.staging;
    if (p0.nodes_per_lane < 0 || p0.nodes_per_lane > 2) return fail(LBM_ERR_ARG, "nodes_per_lane must be 0, 1 or 2");
    S->npl = p0.nodes_per_lane != 0 ? p0.nodes_per_lane : (S->store == ST_F64 ? 1 : 2);
    if (S->npl == 2 && S->store == ST_F64)
        return fail(LBM_ERR_ARG, "nodes_per_lane = 2 needs FP32 or 16-bit storage (FP64 runs one node per lane)");
    if (S->wpb == 0) S->wpb = S->npl == 2 ? 1 : 4;
    if (p0.piece_slots != 0 && p0.piece_slots != 8 && p0.piece_slots != 16 && p0.piece_slots != 32)
        return fail(LBM_ERR_ARG, "piece_slots must be 0, 8, 16 or 32 (got %d)", p0.piece_slots);
    // 8 slots (4 lanes) per piece: on the vascular tree 95 % of the slots
    // hold fluid nodes (90 % with 16, 83 % with 32), on the 64-vessel
    // ensemble 93 % (86 %, 76 %); the kernel is issue-bound, so the emptier
    // pieces cost more than the 8 descriptor bytes per node of short ones
    S->piece = p0.piece_slots != 0 ? p0.piece_slots : 8;
    if (p0.corrections & ~(LBM_FIX_BB_ALL_DIRS | LBM_FIX_LIST_NODES))
        return fail(LBM_ERR_ARG, "unknown corrections bits 0x%x", (unsigned)p0.corrections);
    S->corr = (uint32_t)p0.corrections;
    for (size_t i = 0; i < n; ++i) {
        if (p[i].Q != p0.Q || p[i].precision != p0.precision || p[i].pattern != p0.pattern)
            return fail(LBM_ERR_ARG, "batch members must share Q, precision and pattern");
        if (!(p[i].tau > 0.5)) return fail(LBM_ERR_ARG, "instance %zu: tau must be > 0.5 (got %g)", i, p[i].tau);
        if (geometry_device(g[i]) != S->dev) return fail(LBM_ERR_ARG, "geometry %zu lives on another device", i);
    }
    S->n_inst = (int64_t)n;
    for (size_t i = 0; i < n; ++i) {
        int d[3];
        geometry_dims(g[i], d);
        S->dims.push_back({d[0], d[1], d[2]});
    }
    if (p0.run_axis != 0) {
        S->ra = p0.run_axis;
    } else {
        int64_t cy = 0, cz = 0;
        for (size_t i = 0; i < n; ++i) {
            int64_t a = 0, b = 0;
            const bool pairs = S->npl == 2;
            LBM_TRY(count_chunks(g[i], 1, pairs ? S->piece : 32, pairs, st, &a));
            LBM_TRY(count_chunks(g[i], 2, pairs ? S->piece : 32, pairs, st, &b));
            cy += a;
            cz += b;
        }
        S->ra = cy < cz ? 1 : 2;
    }
    LBM_CUDA(cudaMalloc(&S->err, sizeof(int32_t)));
    LBM_CUDA(cudaMemsetAsync(S->err, 0, sizeof(int32_t), st));
    std::vector<std::unique_ptr<InstBuild>> builds;
    std::vector<ZSlot> zall;
    // node ids start at kLatticeSlack and the arrays end kLatticeSlack ids
    // after the last node: the paired kernel reads up to three ids beyond a
    // chunk's window for node slots it discards
    int64_t node_off = kLatticeSlack, out_off = 0, nch = 0, nch2[3] = {0, 0, 0}, nmask = 0;
    std::vector<int64_t> lat_off(1, node_off), chunk_off(1, 0), mask_off(1, 0);
    std::vector<int64_t> chunk2_off[3] = {{0}, {0}, {0}};
    S->inst_off.push_back(0);
    for (size_t i = 0; i < n; ++i) {
        builds.emplace_back(new InstBuild());
        LBM_TRY(build_instance(g[i], &p[i], S->Q, (int32_t)i, S->ra, S->store == ST_F64 ? 1 : 2, S->piece, node_off,
                               out_off, (int64_t)zall.size(), nmask, S->err, st, *builds.back()));
        const InstBuild& B = *builds.back();
        node_off += B.N;
        out_off += B.NF;
        nch += B.nchunks;
        for (int k = 0; k < 3; ++k) nch2[k] += B.nchunks2[k];
        nmask += B.nmask;
        zall.insert(zall.end(), B.zslots.begin(), B.zslots.end());
        S->inst_off.push_back(out_off);
        lat_off.push_back(node_off);
        chunk_off.push_back(nch);
        for (int k = 0; k < 3; ++k) chunk2_off[k].push_back(nch2[k]);
        mask_off.push_back(nmask);
    }
    S->N = node_off + kLatticeSlack;
    S->NF = out_off;
    S->nchunks = nch;
    for (int k = 0; k < 3; ++k) S->nchunks2s[k] = nch2[k];
    S->nmask = nmask;
    S->nz = (int64_t)zall.size();
    // concatenate per-instance arrays
    LBM_CUDA(cudaMalloc(&S->chunks, sizeof(Chunk) * std::max<int64_t>(nch, 1)));
    if (S->store != ST_F64)
        for (int k = 0; k < 3; ++k)
            LBM_CUDA(cudaMalloc(&S->chunks2s[k], sizeof(Chunk) * std::max<int64_t>(nch2[k], 1)));
    LBM_CUDA(cudaMalloc(&S->mmask, sizeof(uint32_t) * std::max<int64_t>(nmask, 1)));
    LBM_CUDA(cudaMalloc(&S->node_grid, sizeof(int64_t) * S->NF));
    LBM_CUDA(cudaMalloc(&S->out_pos, sizeof(int32_t) * S->N));
    LBM_CUDA(cudaMemsetAsync(S->out_pos, 0xff, sizeof(int32_t) * S->N, st));
    for (size_t i = 0; i < n; ++i) {
        const InstBuild& B = *builds[i];
        LBM_CUDA(cudaMemcpyAsync(S->chunks + chunk_off[i], B.chunks.p, sizeof(Chunk) * B.nchunks,
                                 cudaMemcpyDeviceToDevice, st));
        for (int k = 0; k < 3 && S->store != ST_F64; ++k)
            if (B.nchunks2[k])
                LBM_CUDA(cudaMemcpyAsync(S->chunks2s[k] + chunk2_off[k][i], B.chunks2[k].p,
                                         sizeof(Chunk) * B.nchunks2[k], cudaMemcpyDeviceToDevice, st));
        if (B.nmask)
            LBM_CUDA(cudaMemcpyAsync(S->mmask + mask_off[i], B.mmask.p, sizeof(uint32_t) * B.nmask,
                                     cudaMemcpyDeviceToDevice, st));
        LBM_CUDA(cudaMemcpyAsync(S->node_grid + S->inst_off[i], B.node_grid.p, sizeof(int64_t) * B.NF,
                                 cudaMemcpyDeviceToDevice, st));
        LBM_CUDA(cudaMemcpyAsync(S->out_pos + lat_off[i], B.out_pos.p, sizeof(int32_t) * B.N, cudaMemcpyDeviceToDevice,
                                 st));
    }
    // the AA odd launch's tables: interior pieces ahead of boundary pieces
    // within windows of kGroupWarps warps (the node-local launches keep the
    // memory order, which measured faster for them)
    for (int k = 0; k < 3 && S->store != ST_F64; ++k) {
        LBM_CUDA(cudaMalloc(&S->chunks2gs[k], sizeof(Chunk) * std::max<int64_t>(nch2[k], 1)));
        if (nch2[k] == 0) continue;
        const int win = kGroupWarps * (8 >> k);   // 8, 4, 2 pieces per warp for 8-, 16-, 32-slot pieces
        const int64_t nwin = (nch2[k] + win - 1) / win;
        k_group_pieces<<<(unsigned)std::min<int64_t>(nwin, 152 * 8), kGroupMax, 0, st>>>(S->chunks2s[k],
                                                                                          S->chunks2gs[k], nch2[k], win);
        LBM_CUDA(cudaGetLastError());
    }
    for (int k = 0; k < 3 && S->store != ST_F64; ++k) {
        LBM_CUDA(cudaMalloc(&S->even2s[k], sizeof(uint2) * std::max<int64_t>(nch2[k], 1)));
        if (nch2[k] == 0) continue;
        k_even_desc<<<blocks_for(nch2[k], 256), 256, 0, st>>>(S->chunks2s[k], nch2[k], S->even2s[k]);
        LBM_CUDA(cudaGetLastError());
    }
    select_piece(S.get(), S->piece);       // after the piece tables exist
    LBM_CUDA(cudaMalloc(&S->zslots, sizeof(ZSlot) * std::max<size_t>(zall.size(), 1)));
    if (!zall.empty())
        LBM_CUDA(cudaMemcpyAsync(S->zslots, zall.data(), sizeof(ZSlot) * zall.size(), cudaMemcpyHostToDevice, st));
    // list, amplitude and instance tables
    std::vector<ListParam> lists(64 * n);
    std::vector<double> amp;
    std::vector<InstParam> insts(n);
    for (size_t i = 0; i < n; ++i) {
        insts[i].omega = 1.0 / p[i].tau;
        insts[i].omega_f = (float)insts[i].omega;
        insts[i].pad = 0.f;
        insts[i].tau = p[i].tau;
        for (int l = 0; l < 64; ++l) {
            ListParam& L = lists[64 * i + l];
            std::memset(&L, 0, sizeof L);
            L.rho = 1.0;
            L.amp_off = 0;
            L.amp_len = 1;
        }
        for (size_t b = 0; b < p[i].nbcs; ++b) {
            const lbm_list_bc& B = p[i].bcs[b];
            ListParam& L = lists[64 * i + B.list_id];
            L.kind = B.kind;
            L.rho = B.rho;
            for (int a = 0; a < 3; ++a) L.dir[a] = B.dir[a];
            L.amp_off = (int64_t)amp.size() + 1;   // entry 0 of the table is the constant 1
            if (B.amp_len > 0x7fffffffull) return fail(LBM_ERR_ARG, "bc %zu: amplitude table longer than 2^31", b);
            if (B.amp && B.amp_len) {
                L.amp_len = (int64_t)B.amp_len;
                amp.insert(amp.end(), B.amp, B.amp + B.amp_len);
            } else {
                L.amp_len = 1;
                amp.push_back(1.0);
            }
            L.face = B.face;
            if (B.kind < LBM_BC_NONE || B.kind > LBM_BC_PRESSURE) return fail(LBM_ERR_ARG, "bc %zu: unknown kind %d", b, B.kind);
            if ((B.kind == LBM_BC_VELOCITY || B.kind == LBM_BC_PRESSURE) && (B.face < 0 || B.face > 5))
                return fail(LBM_ERR_ARG, "bc %zu: face must be 0..5 (lbm_face)", b);
            if (p0.Q == 19 && B.kind == LBM_BC_VEL_POSX) return fail(LBM_ERR_ARG, "LBM_BC_VEL_POSX needs Q=27");
            if (p0.Q == 27 && B.kind >= LBM_BC_VEL_NEGY && B.kind <= LBM_BC_PRESS_POSZ)
                return fail(LBM_ERR_ARG, "bc %zu: the reference's D3Q19 routine %d needs Q=19 (use LBM_BC_VELOCITY / "
                                         "LBM_BC_PRESSURE with a face)", b, B.kind);
        }
    }
    amp.insert(amp.begin(), 1.0);
    LBM_CUDA(cudaMalloc(&S->lists, sizeof(ListParam) * lists.size()));
    LBM_CUDA(cudaMemcpyAsync(S->lists, lists.data(), sizeof(ListParam) * lists.size(), cudaMemcpyHostToDevice, st));
    LBM_CUDA(cudaMalloc(&S->amp, sizeof(double) * amp.size()));
    LBM_CUDA(cudaMemcpyAsync(S->amp, amp.data(), sizeof(double) * amp.size(), cudaMemcpyHostToDevice, st));
    LBM_CUDA(cudaMalloc(&S->insts, sizeof(InstParam) * n));
    LBM_CUDA(cudaMemcpyAsync(S->insts, insts.data(), sizeof(InstParam) * n, cudaMemcpyHostToDevice, st));
    // populations, initial f = w (Node.cpp:30-37): stored w for F64/F32, 0 for shifted
    S->stride = (S->N + 63) / 64 * 64;
    // the step kernels address populations with 32-bit element offsets
    if ((uint64_t)S->stride * (uint64_t)S->Q > 0xffffffffull)
        return fail(LBM_ERR_ARG, "lattice of %lld nodes x %d populations exceeds 2^32 values", (long long)S->N, S->Q);
    const int nb = S->pattern == LBM_PULL ? 2 : 1;
    const size_t bytes = (size_t)S->stride * S->Q * store_bytes(S->store);
    std::vector<double> wv(S->Q);
    for (int q = 0; q < S->Q; ++q) wv[q] = S->Q == 19 ? Lat<19>::w(q) : Lat<27>::w(q);
    DBuf<double> dw;
    LBM_TRY(dw.alloc(S->Q, "weights", st));
    LBM_CUDA(cudaMemcpyAsync(dw.p, wv.data(), sizeof(double) * S->Q, cudaMemcpyHostToDevice, st));
    for (int b = 0; b < nb; ++b) {
        if (cudaMalloc(&S->buf[b], bytes) != cudaSuccess)
            return fail(LBM_ERR_NOMEM, "cudaMalloc of %zu bytes of populations failed", bytes);
        const int64_t tot = S->stride * S->Q;
        if (S->store == ST_F64) k_init_pop<double><<<blocks_for(tot, 256), 256, 0, st>>>((double*)S->buf[b], S->stride, S->Q, dw.p);
        else if (S->store == ST_F32) k_init_pop<float><<<blocks_for(tot, 256), 256, 0, st>>>((float*)S->buf[b], S->stride, S->Q, dw.p);
        else if (S->store == ST_F16S) k_init_half<<<blocks_for(tot, 256), 256, 0, st>>>((__half*)S->buf[b], tot);
        else k_init_bf16<<<blocks_for(tot, 256), 256, 0, st>>>((__nv_bfloat16*)S->buf[b], tot);
    }
    // monitor buffers (one partial per block of the dry launch)
    S->part_blocks = std::max<int64_t>((S->nchunks + kDryWarps - 1) / kDryWarps, 1);
    LBM_CUDA(cudaMalloc(&S->part, sizeof(double) * 4 * S->part_blocks));
    LBM_CUDA(cudaMalloc(&S->partbad, sizeof(int32_t) * S->part_blocks));
    LBM_CUDA(cudaMalloc(&S->mon, sizeof(MonOut)));
    LBM_CUDA(cudaMalloc(&S->step_base, sizeof(int64_t)));
    LBM_CUDA(cudaGetLastError());
    LBM_CUDA(cudaStreamSynchronize(st));
    if (S->store != ST_F64) LBM_TRY(pair_first_launch(S.get(), st));
    lbm_monitors m;
    LBM_TRY(sim_monitors(S.get(), &m, st));
    S->mass0 = m.mass;
    *out = S.release();
    return LBM_OK;
}

__global__ void k_gather_f64(const double* __restrict__ src, const int64_t* __restrict__ idx, int64_t n,
                             double* __restrict__ dst) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = src[idx[i]];
}

// Output positions of the wall nodes in wall-list order (the x-major order of
// the outputs), found once from the chunk masks.
lbm_status sim_wall_positions(lbm_sim* S, const double* d_u, double* d_wss_pos, cudaStream_t st) {
    if (S->nwall >= 0) return LBM_OK;
    DBuf<uint8_t> flag;
    LBM_TRY(flag.alloc(S->NF, "wall flags", st));
    LBM_CUDA(cudaMemsetAsync(flag.p, 0, S->NF, st));
    LBM_TRY(launch_wss(S->Q, S->ra, S->chunks, S->nchunks, S->mmask, S->out_pos, S->insts, d_u, d_wss_pos, flag.p, st));
    int64_t* idx = nullptr;
    int64_t cnt = 0;
    LBM_TRY(scan::compact(flag.p, S->NF, &idx, &cnt, st));
    S->wall_pos = idx;
    S->nwall = cnt;
    return LBM_OK;
}

// rho, u of the current state into d_rho / d_u (either may be null), and the
// wall shear stress in wall-list order into d_wss (needs d_u and an NF-sized
// scratch d_wss_pos).
lbm_status sim_outputs(lbm_sim* S, double* d_rho, double* d_u, double* d_wss_pos, double* d_wss, cudaStream_t st) {
    LBM_TRY(sim_dry(S, nullptr, d_rho, d_u, false, st));
    if (d_wss) {
        LBM_TRY(sim_wall_positions(S, d_u, d_wss_pos, st));
        LBM_TRY(launch_wss(S->Q, S->ra, S->chunks, S->nchunks, S->mmask, S->out_pos, S->insts, d_u, d_wss_pos,
                           nullptr, st));
        if (S->nwall > 0)
            k_gather_f64<<<blocks_for(S->nwall, 256), 256, 0, st>>>(d_wss_pos, S->wall_pos, S->nwall, d_wss);
        LBM_CUDA(cudaGetLastError());
    }
    return LBM_OK;
}

}  // namespace

struct lbm_snapshot {
    lbm_sim* S = nullptr;
    uint32_t what = 0;
    double *d_rho = nullptr, *d_u = nullptr, *d_wss_pos = nullptr, *d_wss = nullptr;
    double *h_rho = nullptr, *h_u = nullptr, *h_wss = nullptr;
    int64_t n = 0, nwall = 0, step = -1;
    cudaStream_t copy = nullptr;
    cudaEvent_t computed = nullptr, ready = nullptr;
    bool pending = false;
    std::vector<int64_t> grid, inst_off;        // output grid indices, instance offsets
    std::vector<int64_t> wall_inst_off;         // wall nodes per instance (offsets)
    std::vector<int64_t> wall_grid_pos_;        // output position of each wall node
};

namespace {

void snapshot_free(lbm_snapshot* P) {
    if (P->pending && P->ready) cudaEventSynchronize(P->ready);
    for (double* d : {P->d_rho, P->d_u, P->d_wss_pos, P->d_wss}) if (d) cudaFree(d);
    for (double* h : {P->h_rho, P->h_u, P->h_wss}) if (h) cudaFreeHost(h);
    if (P->computed) cudaEventDestroy(P->computed);
    if (P->ready) cudaEventDestroy(P->ready);
    if (P->copy) cudaStreamDestroy(P->copy);
    delete P;
}

lbm_status snapshot_wait(lbm_snapshot* P) {
    if (P->pending) {
        LBM_CUDA(cudaEventSynchronize(P->ready));
        P->pending = false;
    }
    if (P->step < 0) return fail(LBM_ERR_STATE, "snapshot: nothing captured yet");
    return LBM_OK;
}

}  // namespace

extern "C" {

lbm_status lbm_sim_create(const lbm_geometry* g, const lbm_sim_params* p, void* stream, lbm_sim** out) {
    const NvtxRange nvtx_range("lbm_sim_create");
    if (!g || !p || !out) return fail(LBM_ERR_ARG, "lbm_sim_create: null argument");
    clear_error();
    *out = nullptr;
    lbm_sim* S = nullptr;
    lbm_status s = guarded("lbm_sim_create", [&] { return sim_create(&g, p, 1, (cudaStream_t)stream, &S); });
    if (s != LBM_OK) return s;
    *out = S;
    return LBM_OK;
}

lbm_status lbm_batch_create(const lbm_geometry* const* g, const lbm_sim_params* p, size_t n, void* stream,
                            lbm_sim** out) {
    const NvtxRange nvtx_range("lbm_batch_create");
    if (!g || !p || !out || n == 0) return fail(LBM_ERR_ARG, "lbm_batch_create: bad argument");
    if (n >= (1u << 24)) return fail(LBM_ERR_ARG, "lbm_batch_create: too many instances");
    clear_error();
    *out = nullptr;
    lbm_sim* S = nullptr;
    lbm_status s = guarded("lbm_batch_create", [&] { return sim_create(g, p, n, (cudaStream_t)stream, &S); });
    if (s != LBM_OK) return s;
    *out = S;
    return LBM_OK;
}

}  // extern "C"

namespace {

// The CUDA graph of G launches (G even) from an aligned state (pull: the
// first buffer is the source; AA: an even, node-local launch first), plus the
// step-counter update; captured once per length.  The simulation's state is
// untouched: the graph's launches take their step numbers from step_base.
lbm_status ensure_graph(lbm_sim* S, int64_t G) {
    if (S->glen == G) return LBM_OK;
    free_graph(S);
    cudaStream_t cs;
    LBM_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    const int cur0 = S->cur;
    const int64_t sd0 = S->steps_done;
    // aligned state for the capture (restored below)
    S->cur = 0;
    S->steps_done = sd0 + ((sd0 + S->aa_phase) & 1);
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    lbm_status ls = LBM_OK;
    for (int64_t s = 0; s < G && ls == LBM_OK && e == cudaSuccess; ++s) {
        ls = sim_one_step(S, s, S->step_base, cs, false);
        S->steps_done++;   // parity for AA within the capture
    }
    if (e == cudaSuccess) {
        k_add_step<<<1, 1, 0, cs>>>(S->step_base, G);
        e = cudaStreamEndCapture(cs, &S->graph);
    }
    S->cur = cur0;
    S->steps_done = sd0;
    cudaStreamDestroy(cs);
    if (ls != LBM_OK) return ls;
    if (e != cudaSuccess) return fail(LBM_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
    LBM_CUDA(cudaGraphInstantiate(&S->gexec, S->graph, 0));
    S->glen = G;
    return LBM_OK;
}

// graph length lbm_sim_step uses for nsteps from the current state (0: none)
int64_t graph_length(const lbm_sim* S, int64_t nsteps) {
    if (nsteps < 4) return 0;
    const bool misaligned = S->pattern == LBM_PULL ? S->cur != 0 : aa_mode(S) != MODE_AA_EVEN;
    const int64_t G = std::min<int64_t>(64, (nsteps - (misaligned ? 1 : 0)) & ~1LL);
    return G >= 2 ? G : 0;
}

}  // namespace

extern "C" {

lbm_status lbm_sim_prepare_graph(lbm_sim* S, int64_t nsteps, void* stream) {
    if (!S || nsteps < 0) return fail(LBM_ERR_ARG, "lbm_sim_prepare_graph: bad argument");
    clear_error();
    (void)stream;
    const int64_t G = graph_length(S, nsteps);
    return G ? ensure_graph(S, G) : LBM_OK;
}

lbm_status lbm_sim_step(lbm_sim* S, int64_t nsteps, uint32_t flags, void* stream) {
    const NvtxRange nvtx_range("lbm_sim_step");
    if (!S || nsteps < 0) return fail(LBM_ERR_ARG, "lbm_sim_step: bad argument");
    // the kernels take the inlet waveform phase from a 32-bit step count
    if (S->steps_done + nsteps > (int64_t)0xffffffffLL)
        return fail(LBM_ERR_ARG, "lbm_sim_step: a simulation is limited to 2^32 - 1 steps");
    clear_error();
    cudaStream_t st = (cudaStream_t)stream;
    int64_t left = nsteps;
    const int64_t G = (flags & LBM_STEP_GRAPH) ? graph_length(S, nsteps) : 0;
    if (G) {
        // state parity must match the captured graph: pull buffer index and
        // AA step parity both return to their start after an even step count
        if (S->pattern == LBM_PULL ? S->cur != 0 : aa_mode(S) != MODE_AA_EVEN) {
            LBM_TRY(sim_one_step(S, S->steps_done, nullptr, st, true));
            --left;
        }
        LBM_TRY(ensure_graph(S, G));
        int64_t sd = S->steps_done;
        LBM_CUDA(cudaMemcpyAsync(S->step_base, &sd, sizeof sd, cudaMemcpyHostToDevice, st));
        while (left >= G) {
            LBM_CUDA(cudaGraphLaunch(S->gexec, st));
            S->steps_done += G;
            left -= G;
        }
    }
    for (; left > 0; --left) LBM_TRY(sim_one_step(S, S->steps_done, nullptr, st, true));
    LBM_CUDA(cudaGetLastError());
    if (flags & LBM_STEP_MONITOR) {
        lbm_monitors m;
        LBM_TRY(sim_monitors(S, &m, st));
        if (m.nonfinite || !(std::fabs(m.mass / S->mass0 - 1.0) <= S->div_tol))
            return fail(LBM_ERR_DIVERGED, "diverged at step %lld: mass %.17g (initial %.17g), non-finite=%d",
                        (long long)S->steps_done, m.mass, S->mass0, m.nonfinite);
    }
    return LBM_OK;
}

// Pattern conversion.  After an AA even launch slot opp(q) of node x holds
// f*_q(x), the post-collision population the pull pattern keeps in slot q of
// its source lattice (and the bounced values of boundary nodes sit where each
// pattern's next launch reads them); so the two states differ by a
// permutation of the population planes.  AA -> pull needs that state (the
// next AA launch odd); pull -> AA always works and sets aa_phase so that the
// next AA launch is the odd one.
static lbm_status convert_pattern(lbm_sim* S, int pattern, cudaStream_t st) {
    if (pattern == S->pattern) return LBM_OK;
    const size_t es = store_bytes(S->store), plane = (size_t)S->stride * es;
    const size_t bytes = plane * S->Q;
    auto swap_planes = [&](void* dst, const void* src) -> lbm_status {
        for (int q = 0; q < S->Q; ++q) {
            const int o = S->Q == 19 ? Lat<19>::opp(q) : Lat<27>::opp(q);
            LBM_CUDA(cudaMemcpyAsync((char*)dst + (size_t)q * plane, (const char*)src + (size_t)o * plane, plane,
                                     cudaMemcpyDeviceToDevice, st));
        }
        return LBM_OK;
    };
    if (pattern == LBM_PULL) {
        if (aa_mode(S) != MODE_AA_ODD)
            return fail(LBM_ERR_STATE, "AA -> pull needs the state after an even (node-local) launch; step once more");
        if (!S->buf[1] && cudaMalloc(&S->buf[1], bytes) != cudaSuccess) {
            cudaGetLastError();
            S->buf[1] = nullptr;
            return fail(LBM_ERR_NOMEM, "no room for the pull pattern's second lattice (%zu bytes)", bytes);
        }
        LBM_TRY(swap_planes(S->buf[1], S->buf[0]));
        S->cur = 1;
    } else {
        void* src = S->buf[S->cur];
        void* dst = S->buf[1 - S->cur];
        LBM_TRY(swap_planes(dst, src));
        LBM_CUDA(cudaStreamSynchronize(st));
        cudaFree(src);                     // the AA pattern keeps one lattice
        S->buf[0] = dst;
        S->buf[1] = nullptr;
        S->cur = 0;
        S->aa_phase = (int)((S->steps_done + 1) & 1);     // the next launch is an odd one
    }
    LBM_CUDA(cudaStreamSynchronize(st));
    S->pattern = pattern;
    free_graph(S);
    return LBM_OK;
}

lbm_status lbm_sim_set_pattern(lbm_sim* S, int32_t pattern, void* stream) {
    const NvtxRange nvtx_range("lbm_sim_set_pattern");
    if (!S || (pattern != LBM_PULL && pattern != LBM_AA)) return fail(LBM_ERR_ARG, "lbm_sim_set_pattern: bad argument");
    clear_error();
    LBM_TRY(check_timeout(S, (cudaStream_t)stream));
    return convert_pattern(S, pattern, (cudaStream_t)stream);
}

lbm_status lbm_sim_autotune(lbm_sim* S, int32_t launches, void* stream, lbm_tune_entry* entries, size_t cap,
                            size_t* n) {
    const NvtxRange nvtx_range("lbm_sim_autotune");
    if (!S || launches < 2) return fail(LBM_ERR_ARG, "lbm_sim_autotune: null handle or fewer than 2 launches");
    clear_error();
    cudaStream_t st = (cudaStream_t)stream;
    LBM_TRY(check_timeout(S, st));
    // scratch copies of the state: the candidates run on them, the simulation is untouched
    const size_t bytes = (size_t)S->stride * S->Q * store_bytes(S->store);
    // patterns: the current one; the other one where the state converts now
    // (AA -> pull after an even launch; pull -> AA always) and its memory fits
    std::vector<int> patterns = {S->pattern};
    if (S->pattern == LBM_PULL || aa_mode(S) == MODE_AA_ODD)
        patterns.push_back(S->pattern == LBM_PULL ? LBM_AA : LBM_PULL);
    void* scratch[2] = {nullptr, nullptr};
    const bool need2 = std::find(patterns.begin(), patterns.end(), (int)LBM_PULL) != patterns.end();
    for (int b = 0; b < (need2 ? 2 : 1); ++b)
        if (cudaMalloc(&scratch[b], bytes) != cudaSuccess) {
            cudaGetLastError();
            scratch[b] = nullptr;
            if (b == 0) return fail(LBM_ERR_NOMEM, "lbm_sim_autotune: no room for a scratch copy of the state (%zu bytes)", bytes);
            patterns = {S->pattern};        // no room for pull's second lattice: keep the pattern
            if (S->pattern == LBM_PULL) {
                cudaFree(scratch[0]);
                return fail(LBM_ERR_NOMEM, "lbm_sim_autotune: no room for two scratch lattices (%zu bytes)", bytes);
            }
        }
    struct Cand { int pattern, npl, staging, wpb, piece; float ms; };
    std::vector<Cand> cands;
    const int wpbs[4] = {1, 2, 4, 8};
    for (int pat : patterns) {
        for (int w : wpbs) cands.push_back({pat, 1, 1, w, S->piece, 0.f});
        for (int w : wpbs) cands.push_back({pat, 1, 0, w, S->piece, 0.f});
        if (S->store != ST_F64)
            for (int pc : {8, 16, 32})
                for (int w : wpbs) cands.push_back({pat, 2, 1, w, pc, 0.f});
    }
    const int save_pattern = S->pattern, save_npl = S->npl, save_staging = S->staging, save_wpb = S->wpb,
              save_piece = S->piece;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    lbm_status res = LBM_OK;
    auto run = [&](int count) -> lbm_status {
        for (int i = 0; i < count; ++i) {
            Partials np = {nullptr, nullptr, nullptr, nullptr, nullptr};
            lbm_status s;
            if (S->pattern == LBM_PULL)
                s = sim_launch(S, MODE_PULL, false, scratch[i & 1], scratch[1 - (i & 1)], S->steps_done + i, nullptr,
                               np, nullptr, nullptr, nullptr, st);
            else
                s = sim_launch(S, ((S->steps_done + S->aa_phase + i) & 1) ? MODE_AA_ODD : MODE_AA_EVEN, false,
                               scratch[0], scratch[0], S->steps_done + i, nullptr, np, nullptr, nullptr, nullptr, st);
            if (s != LBM_OK) return s;
        }
        return LBM_OK;
    };
    do {
        if (cudaMemcpyAsync(scratch[0], S->buf[S->pattern == LBM_PULL ? S->cur : 0], bytes, cudaMemcpyDeviceToDevice,
                            st) != cudaSuccess ||
            cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
            res = fail(LBM_ERR_CUDA, "lbm_sim_autotune: set-up failed");
            break;
        }
        for (Cand& c : cands) {
            S->pattern = c.pattern; S->npl = c.npl; S->staging = c.staging; S->wpb = c.wpb;
            if (c.npl == 2) select_piece(S, c.piece);
            if ((res = run(2)) != LBM_OK) break;      // warm-up (even count keeps the AA parity)
            cudaEventRecord(e0, st);
            if ((res = run(launches & ~1)) != LBM_OK) break;
            cudaEventRecord(e1, st);
            if (cudaEventSynchronize(e1) != cudaSuccess) { res = fail(LBM_ERR_CUDA, "lbm_sim_autotune: timing"); break; }
            cudaEventElapsedTime(&c.ms, e0, e1);
            c.ms /= (float)(launches & ~1);
        }
    } while (false);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    for (void* b : scratch) if (b) cudaFree(b);
    S->pattern = save_pattern; S->npl = save_npl; S->staging = save_staging; S->wpb = save_wpb;
    select_piece(S, save_piece);
    if (res != LBM_OK) return res;
    LBM_TRY(check_timeout(S, st));
    const Cand* best = &cands[0];
    for (const Cand& c : cands) if (c.ms < best->ms) best = &c;
    if (best->pattern != S->pattern) LBM_TRY(convert_pattern(S, best->pattern, st));
    S->npl = best->npl; S->staging = best->staging; S->wpb = best->wpb;
    if (S->npl == 2) select_piece(S, best->piece);
    free_graph(S);                         // the captured launches used the old shape
    if (n) *n = cands.size();
    if (entries)
        for (size_t i = 0; i < cands.size() && i < cap; ++i) {
            entries[i].nodes_per_lane = cands[i].npl;
            entries[i].staging = cands[i].staging;
            entries[i].warps_per_block = cands[i].wpb;
            entries[i].chosen = &cands[i] == best ? 1 : 0;
            entries[i].pattern = cands[i].pattern;
            entries[i].piece_slots = cands[i].npl == 2 ? cands[i].piece : 0;
            entries[i].ms_per_launch = cands[i].ms;
        }
    return LBM_OK;
}

lbm_status lbm_sim_info_get(const lbm_sim* S, lbm_sim_info* info) {
    if (!S || !info) return fail(LBM_ERR_ARG, "lbm_sim_info_get: null argument");
    std::memset(info, 0, sizeof *info);
    info->n_nodes = S->NF;
    info->n_instances = S->n_inst;
    info->steps_done = S->steps_done;
    info->n_chunks = S->npl == 2 ? S->nchunks2 : S->nchunks;
    info->n_lattice_nodes = S->N;
    info->nodes_per_lane = S->npl;
    info->piece_slots = S->npl == 2 ? S->piece : 0;
    info->Q = S->Q;
    info->precision = S->store;
    info->pattern = S->pattern;
    info->warps_per_block = S->wpb;
    info->run_axis = S->ra;
    info->state_bytes = (int64_t)S->stride * S->Q * store_bytes(S->store) * (S->pattern == LBM_PULL ? 2 : 1);
    info->algorithmic_bytes_per_update = 2.0 * S->Q * store_bytes(S->store);
    return LBM_OK;
}

lbm_status lbm_sim_fields(lbm_sim* S, double* rho, double* u, double* f, size_t n_nodes, void* stream) {
    const NvtxRange nvtx_range("lbm_sim_fields");
    if (!S) return fail(LBM_ERR_ARG, "lbm_sim_fields: null handle");
    if (n_nodes < (size_t)S->NF) return fail(LBM_ERR_ARG, "lbm_sim_fields: capacity %zu < %lld nodes", n_nodes, (long long)S->NF);
    clear_error();
    cudaStream_t st = (cudaStream_t)stream;
    DBuf<double> df, dr, du;
    if (f) LBM_TRY(df.alloc((size_t)S->NF * S->Q, "field f", st));
    if (rho) LBM_TRY(dr.alloc(S->NF, "field rho", st));
    if (u) LBM_TRY(du.alloc((size_t)S->NF * 3, "field u", st));
    LBM_TRY(check_timeout(S, st));
    LBM_TRY(sim_dry(S, df.p, dr.p, du.p, false, st));
    if (f) LBM_CUDA(cudaMemcpyAsync(f, df.p, sizeof(double) * S->NF * S->Q, cudaMemcpyDeviceToHost, st));
    if (rho) LBM_CUDA(cudaMemcpyAsync(rho, dr.p, sizeof(double) * S->NF, cudaMemcpyDeviceToHost, st));
    if (u) LBM_CUDA(cudaMemcpyAsync(u, du.p, sizeof(double) * S->NF * 3, cudaMemcpyDeviceToHost, st));
    LBM_CUDA(cudaStreamSynchronize(st));
    return LBM_OK;
}

// ---------------------------------------------------------------------------
// Fields without device allocation (lbm_sim_fields_noalloc).
//
// lbm_sim_fields takes its FP64 output buffers from the device's memory pool:
// a call may grow the pool (a driver allocation, which can wait for the
// device) and leaves that memory reserved for later calls.  Callers that
// sample rho and u while other work keeps the GPU busy -- a time loop or
// another simulation running on other streams, a lattice sized to fill the
// device memory, a process whose memory belongs to another allocator --
// cannot afford that wait or that allocation.  This variant runs
// the same snapshot launch of the step kernel into one fixed device array
// that is part of the library image, so a call allocates nothing.
//
// Limits: at most kStaticFieldNodes nodes (rho and u in FP64: 32 B per node,
// 16 MiB in all); larger lattices are rejected with LBM_ERR_ARG.  Every call,
// from any handle, uses the same array, and the array keeps what the last
// call wrote: calls whose GPU work overlaps (other threads, other streams)
// race on it.  Each call writes every value it copies out (one rho and one u
// per fluid node), so nothing has to be cleared between calls.
// Each call looks up the array's device address with the handle's device
// current (cudaGetSymbolAddress: a table lookup once the module is loaded; the
// first call on a device may load it).  The address is not cached, so a call
// after a device reset or a new primary context uses the module's new address.
static constexpr int64_t kStaticFieldNodes = int64_t(1) << 19;
static __device__ __align__(256) double g_field_scratch[4 * kStaticFieldNodes];

namespace {
// device address of g_field_scratch on the current device
lbm_status field_scratch(double** out) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_field_scratch);
    if (e != cudaSuccess || !p)
        return fail(LBM_ERR_CUDA, "cudaGetSymbolAddress(field scratch): %s", cudaGetErrorString(e));
    *out = (double*)p;
    return LBM_OK;
}
}  // namespace

lbm_status lbm_sim_fields_noalloc(lbm_sim* S, double* rho, double* u, size_t n_nodes, void* stream) {
    if (!S || !rho || !u) return fail(LBM_ERR_ARG, "lbm_sim_fields_noalloc: null argument");
    if (S->NF > kStaticFieldNodes)
        return fail(LBM_ERR_ARG, "lbm_sim_fields_noalloc: %lld nodes exceed the fixed scratch of %lld nodes",
                    (long long)S->NF, (long long)kStaticFieldNodes);
    if (n_nodes < (size_t)S->NF)
        return fail(LBM_ERR_ARG, "lbm_sim_fields_noalloc: capacity %zu < %lld nodes", n_nodes, (long long)S->NF);
    clear_error();
    int dev = -1;
    LBM_CUDA(cudaGetDevice(&dev));
    if (dev != S->dev)
        return fail(LBM_ERR_STATE, "lbm_sim_fields_noalloc: device %d is current, the handle lives on %d", dev, S->dev);
    double* scratch = nullptr;
    LBM_TRY(field_scratch(&scratch));
    cudaStream_t st = (cudaStream_t)stream;
    double* drho = scratch;
    double* du = scratch + kStaticFieldNodes;
    LBM_TRY(check_timeout(S, st));
    LBM_TRY(sim_dry(S, nullptr, drho, du, false, st));
    LBM_CUDA(cudaMemcpyAsync(rho, drho, sizeof(double) * S->NF, cudaMemcpyDeviceToHost, st));
    LBM_CUDA(cudaMemcpyAsync(u, du, sizeof(double) * 3 * S->NF, cudaMemcpyDeviceToHost, st));
    LBM_CUDA(cudaStreamSynchronize(st));
    return LBM_OK;
}

lbm_status lbm_sim_nodes(const lbm_sim* S, int64_t* grid_index, size_t cap) {
    if (!S || !grid_index) return fail(LBM_ERR_ARG, "lbm_sim_nodes: null argument");
    if (cap < (size_t)S->NF) return fail(LBM_ERR_ARG, "lbm_sim_nodes: capacity %zu < %lld", cap, (long long)S->NF);
    LBM_CUDA(cudaMemcpy(grid_index, S->node_grid, sizeof(int64_t) * S->NF, cudaMemcpyDeviceToHost));
    return LBM_OK;
}

lbm_status lbm_sim_instance_offsets(const lbm_sim* S, int64_t* off, size_t cap) {
    if (!S || !off) return fail(LBM_ERR_ARG, "lbm_sim_instance_offsets: null argument");
    if (cap < S->inst_off.size()) return fail(LBM_ERR_ARG, "lbm_sim_instance_offsets: capacity too small");
    std::memcpy(off, S->inst_off.data(), sizeof(int64_t) * S->inst_off.size());
    return LBM_OK;
}

lbm_status lbm_sim_monitors(lbm_sim* S, lbm_monitors* out, void* stream) {
    const NvtxRange nvtx_range("lbm_sim_monitors");
    if (!S || !out) return fail(LBM_ERR_ARG, "lbm_sim_monitors: null argument");
    clear_error();
    return sim_monitors(S, out, (cudaStream_t)stream);
}

lbm_status lbm_sim_set_wait_limit(lbm_sim* S, uint32_t polls) {
    if (!S) return fail(LBM_ERR_ARG, "lbm_sim_set_wait_limit: null handle");
    S->spin_limit = polls;
    free_graph(S);                         // captured launches carry the old limit
    return LBM_OK;
}

lbm_status lbm_sim_test_stall(lbm_sim* S, int32_t enable) {
    if (!S) return fail(LBM_ERR_ARG, "lbm_sim_test_stall: null handle");
    S->stall_first = enable ? 1 : 0;
    free_graph(S);
    return LBM_OK;
}

lbm_status lbm_sim_poison_ghosts(lbm_sim* S, void* stream) {
    if (!S) return fail(LBM_ERR_ARG, "lbm_sim_poison_ghosts: null handle");
    clear_error();
    cudaStream_t st = (cudaStream_t)stream;
    const int eb = store_bytes(S->store);
    for (void* b : S->buf)
        if (b)
            k_poison<<<blocks_for(S->stride * S->Q, 256), 256, 0, st>>>(b, S->stride, S->Q, eb, S->out_pos, S->N);
    LBM_CUDA(cudaGetLastError());
    LBM_CUDA(cudaStreamSynchronize(st));
    return LBM_OK;
}

lbm_status lbm_sim_set_divergence_tolerance(lbm_sim* S, double rel_tol) {
    if (!S || !(rel_tol > 0)) return fail(LBM_ERR_ARG, "lbm_sim_set_divergence_tolerance: bad argument");
    S->div_tol = rel_tol;
    return LBM_OK;
}

lbm_status lbm_sim_wall_shear_stress(lbm_sim* S, double* wss, size_t cap, size_t* n, void* stream) {
    const NvtxRange nvtx_range("lbm_sim_wall_shear_stress");
    if (!S) return fail(LBM_ERR_ARG, "lbm_sim_wall_shear_stress: null handle");
    clear_error();
    cudaStream_t st = (cudaStream_t)stream;
    DBuf<double> du, dpos, dw;
    LBM_TRY(du.alloc((size_t)S->NF * 3, "velocity", st));
    LBM_TRY(dpos.alloc(S->NF, "wall shear stress", st));
    LBM_TRY(check_timeout(S, st));
    LBM_TRY(sim_dry(S, nullptr, nullptr, du.p, false, st));
    LBM_TRY(sim_wall_positions(S, du.p, dpos.p, st));
    if (n) *n = (size_t)S->nwall;
    if (!wss) {
        LBM_CUDA(cudaStreamSynchronize(st));
        return LBM_OK;
    }
    if (cap < (size_t)S->nwall) return fail(LBM_ERR_ARG, "lbm_sim_wall_shear_stress: capacity %zu < %lld wall nodes", cap,
                                            (long long)S->nwall);
    LBM_TRY(dw.alloc(S->nwall, "wall shear stress", st));
    LBM_TRY(sim_outputs(S, nullptr, du.p, dpos.p, dw.p, st));
    if (S->nwall) LBM_CUDA(cudaMemcpyAsync(wss, dw.p, sizeof(double) * S->nwall, cudaMemcpyDeviceToHost, st));
    LBM_CUDA(cudaStreamSynchronize(st));
    return LBM_OK;
}

lbm_status lbm_snapshot_create(lbm_sim* S, uint32_t what, lbm_snapshot** out) {
    if (!S || !out || !what || (what & ~(uint32_t)(LBM_SNAP_FIELDS | LBM_SNAP_WSS)))
        return fail(LBM_ERR_ARG, "lbm_snapshot_create: bad argument");
    clear_error();
    *out = nullptr;
    std::unique_ptr<lbm_snapshot, void (*)(lbm_snapshot*)> P(new lbm_snapshot(), snapshot_free);
    P->S = S;
    P->what = what;
    P->n = S->NF;
    const size_t n = (size_t)S->NF;
    auto dmal = [&](double** p, size_t cnt, const char* what_) -> lbm_status {
        if (cudaMalloc(p, sizeof(double) * (cnt ? cnt : 1)) != cudaSuccess)
            return fail(LBM_ERR_NOMEM, "snapshot: cudaMalloc for %s failed", what_);
        return LBM_OK;
    };
    auto hmal = [&](double** p, size_t cnt, const char* what_) -> lbm_status {
        if (cudaHostAlloc(p, sizeof(double) * (cnt ? cnt : 1), cudaHostAllocDefault) != cudaSuccess)
            return fail(LBM_ERR_NOMEM, "snapshot: pinned host allocation for %s failed", what_);
        return LBM_OK;
    };
    LBM_TRY(dmal(&P->d_u, 3 * n, "velocity"));
    if (what & LBM_SNAP_FIELDS) {
        LBM_TRY(dmal(&P->d_rho, n, "density"));
        LBM_TRY(hmal(&P->h_rho, n, "density"));
        LBM_TRY(hmal(&P->h_u, 3 * n, "velocity"));
    }
    if (what & LBM_SNAP_WSS) {
        LBM_TRY(dmal(&P->d_wss_pos, n, "wall shear stress"));
        LBM_TRY(sim_outputs(S, nullptr, P->d_u, nullptr, nullptr, nullptr));   // velocities for the wall search
        LBM_TRY(sim_wall_positions(S, P->d_u, P->d_wss_pos, nullptr));
        P->nwall = S->nwall;
        LBM_TRY(dmal(&P->d_wss, P->nwall, "wall shear stress"));
        LBM_TRY(hmal(&P->h_wss, P->nwall, "wall shear stress"));
    }
    LBM_CUDA(cudaStreamCreateWithFlags(&P->copy, cudaStreamNonBlocking));
    LBM_CUDA(cudaEventCreateWithFlags(&P->computed, cudaEventDisableTiming));
    LBM_CUDA(cudaEventCreateWithFlags(&P->ready, cudaEventDisableTiming));
    // node and wall coordinates per instance (host copies)
    P->grid.resize(n);
    LBM_CUDA(cudaMemcpy(P->grid.data(), S->node_grid, sizeof(int64_t) * n, cudaMemcpyDeviceToHost));
    P->inst_off = S->inst_off;
    if (what & LBM_SNAP_WSS) {
        std::vector<int64_t> wp((size_t)P->nwall);
        if (P->nwall) LBM_CUDA(cudaMemcpy(wp.data(), S->wall_pos, sizeof(int64_t) * P->nwall, cudaMemcpyDeviceToHost));
        P->wall_inst_off.assign(1, 0);
        size_t w = 0;
        for (size_t i = 0; i + 1 < P->inst_off.size(); ++i) {
            while (w < wp.size() && wp[w] < P->inst_off[i + 1]) ++w;
            P->wall_inst_off.push_back((int64_t)w);
        }
        P->wall_grid_pos_ = std::move(wp);
    }
    *out = P.release();
    return LBM_OK;
}

lbm_status lbm_snapshot_capture(lbm_snapshot* P, void* stream) {
    if (!P) return fail(LBM_ERR_ARG, "lbm_snapshot_capture: null handle");
    clear_error();
    if (P->pending) LBM_CUDA(cudaEventSynchronize(P->ready));   // one capture in flight
    cudaStream_t st = (cudaStream_t)stream;
    lbm_sim* S = P->S;
    LBM_TRY(check_timeout(S, st));
    LBM_TRY(sim_outputs(S, P->d_rho, P->d_u, P->d_wss_pos, P->d_wss, st));
    LBM_CUDA(cudaEventRecord(P->computed, st));
    LBM_CUDA(cudaStreamWaitEvent(P->copy, P->computed, 0));
    const size_t n = (size_t)P->n;
    if (P->what & LBM_SNAP_FIELDS) {
        LBM_CUDA(cudaMemcpyAsync(P->h_rho, P->d_rho, sizeof(double) * n, cudaMemcpyDeviceToHost, P->copy));
        LBM_CUDA(cudaMemcpyAsync(P->h_u, P->d_u, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, P->copy));
    }
    if ((P->what & LBM_SNAP_WSS) && P->nwall)
        LBM_CUDA(cudaMemcpyAsync(P->h_wss, P->d_wss, sizeof(double) * P->nwall, cudaMemcpyDeviceToHost, P->copy));
    LBM_CUDA(cudaEventRecord(P->ready, P->copy));
    P->pending = true;
    P->step = S->steps_done;
    return LBM_OK;
}

lbm_status lbm_snapshot_wait(lbm_snapshot* P) {
    if (!P) return fail(LBM_ERR_ARG, "lbm_snapshot_wait: null handle");
    clear_error();
    return snapshot_wait(P);
}

lbm_status lbm_snapshot_data(lbm_snapshot* P, const double** rho, const double** u, const double** wss, size_t* n_nodes,
                             size_t* n_wall, int64_t* step) {
    if (!P) return fail(LBM_ERR_ARG, "lbm_snapshot_data: null handle");
    clear_error();
    LBM_TRY(snapshot_wait(P));
    if (rho) *rho = P->h_rho;
    if (u) *u = P->h_u;
    if (wss) *wss = P->h_wss;
    if (n_nodes) *n_nodes = (size_t)P->n;
    if (n_wall) *n_wall = (size_t)P->nwall;
    if (step) *step = P->step;
    return LBM_OK;
}

lbm_status lbm_snapshot_write_fields_vtu(lbm_snapshot* P, const char* path, int32_t instance) {
    if (!P || !path) return fail(LBM_ERR_ARG, "lbm_snapshot_write_fields_vtu: null argument");
    if (!(P->what & LBM_SNAP_FIELDS)) return fail(LBM_ERR_STATE, "snapshot was created without LBM_SNAP_FIELDS");
    if (instance < 0 || instance >= (int32_t)P->S->n_inst) return fail(LBM_ERR_ARG, "instance %d out of range", instance);
    clear_error();
    LBM_TRY(snapshot_wait(P));
    const std::array<int, 3>& d = P->S->dims[instance];
    const int64_t b = P->inst_off[instance], e = P->inst_off[instance + 1], m = e - b;
    // the reference's loop order: z outermost, x fastest (OutputFile.cpp:43-45)
    std::vector<int64_t> order((size_t)m);
    for (int64_t i = 0; i < m; ++i) order[(size_t)i] = b + i;
    auto key = [&](int64_t o) {
        const int64_t g = P->grid[(size_t)o];
        const int64_t i = g / ((int64_t)d[1] * d[2]), j = (g / d[2]) % d[1], k = g % d[2];
        return (k * d[1] + j) * (int64_t)d[0] + i;
    };
    std::sort(order.begin(), order.end(), [&](int64_t x, int64_t y) { return key(x) < key(y); });
    std::vector<float> xyz(3 * (size_t)m);
    std::vector<double> vel(3 * (size_t)m), pres((size_t)m), mag((size_t)m), rho((size_t)m);
    for (int64_t t = 0; t < m; ++t) {
        const int64_t o = order[(size_t)t], g = P->grid[(size_t)o];
        xyz[3 * t] = (float)(g / ((int64_t)d[1] * d[2]));
        xyz[3 * t + 1] = (float)((g / d[2]) % d[1]);
        xyz[3 * t + 2] = (float)(g % d[2]);
        const double ux = P->h_u[3 * o], uy = P->h_u[3 * o + 1], uz = P->h_u[3 * o + 2];
        vel[3 * t] = ux; vel[3 * t + 1] = uy; vel[3 * t + 2] = uz;
        rho[t] = P->h_rho[o];
        pres[t] = (1.0 / 3.0) * P->h_rho[o];     // Node::Pressure: c_s^2 rho (Node.cpp:112-118)
        mag[t] = std::sqrt(ux * ux + uy * uy + uz * uz);
    }
    const lbm_vtu_array arr[4] = {{"Velocity", 3, 0, vel.data()}, {"Pressure", 1, 0, pres.data()},
                                  {"VelocityMagnitude", 1, 0, mag.data()}, {"Density", 1, 0, rho.data()}};
    return lbm_vtu_write(path, (size_t)m, xyz.data(), 4, arr);
}

lbm_status lbm_snapshot_write_wss_vtu(lbm_snapshot* P, const char* path, int32_t instance) {
    if (!P || !path) return fail(LBM_ERR_ARG, "lbm_snapshot_write_wss_vtu: null argument");
    if (!(P->what & LBM_SNAP_WSS)) return fail(LBM_ERR_STATE, "snapshot was created without LBM_SNAP_WSS");
    if (instance < 0 || instance >= (int32_t)P->S->n_inst) return fail(LBM_ERR_ARG, "instance %d out of range", instance);
    clear_error();
    LBM_TRY(snapshot_wait(P));
    const std::array<int, 3>& d = P->S->dims[instance];
    const int64_t b = P->wall_inst_off[instance], e = P->wall_inst_off[instance + 1], m = e - b;
    std::vector<float> xyz(3 * (size_t)m);
    for (int64_t t = 0; t < m; ++t) {
        const int64_t g = P->grid[(size_t)P->wall_grid_pos_[(size_t)(b + t)]];
        xyz[3 * t] = (float)(g / ((int64_t)d[1] * d[2]));
        xyz[3 * t + 1] = (float)((g / d[2]) % d[1]);
        xyz[3 * t + 2] = (float)(g % d[2]);
    }
    const lbm_vtu_array arr[1] = {{"WallShearStress", 1, 0, P->h_wss + b}};
    return lbm_vtu_write(path, (size_t)m, xyz.data(), 1, arr);
}

void lbm_snapshot_destroy(lbm_snapshot* P) {
    if (P) snapshot_free(P);
}

// Checkpoint file: a fixed header, then the populations of the current state
// (the plane-major device array, stride * Q values of the storage type).
namespace {
struct CkptHeader {
    char magic[8];            // "LBMCKPT2"
    int32_t Q, store, pattern, n_inst;
    int32_t aa_phase, pad;
    int64_t N, NF, stride, nchunks, steps_done;
    uint64_t grid_hash;       // FNV-1a of the output nodes' grid indices
    uint64_t bytes;
};
uint64_t fnv1a(const void* p, size_t n, uint64_t h = 1469598103934665603ull) {
    const unsigned char* c = (const unsigned char*)p;
    for (size_t i = 0; i < n; ++i) { h ^= c[i]; h *= 1099511628211ull; }
    return h;
}
lbm_status ckpt_header(lbm_sim* S, CkptHeader& h) {
    std::memset(&h, 0, sizeof h);
    std::memcpy(h.magic, "LBMCKPT2", 8);
    h.Q = S->Q; h.store = S->store; h.pattern = S->pattern; h.n_inst = (int32_t)S->n_inst;
    h.aa_phase = S->aa_phase;
    h.N = S->N; h.NF = S->NF; h.stride = S->stride; h.nchunks = S->nchunks; h.steps_done = S->steps_done;
    std::vector<int64_t> g((size_t)S->NF);
    LBM_CUDA(cudaMemcpy(g.data(), S->node_grid, sizeof(int64_t) * S->NF, cudaMemcpyDeviceToHost));
    h.grid_hash = fnv1a(g.data(), g.size() * sizeof(int64_t));
    h.bytes = (uint64_t)S->stride * S->Q * store_bytes(S->store);
    return LBM_OK;
}
constexpr size_t kCkptBlock = size_t(64) << 20;
}  // namespace

lbm_status lbm_sim_checkpoint(lbm_sim* S, const char* path, void* stream) {
    const NvtxRange nvtx_range("lbm_sim_checkpoint");
    if (!S || !path) return fail(LBM_ERR_ARG, "lbm_sim_checkpoint: null argument");
    clear_error();
    cudaStream_t st = (cudaStream_t)stream;
    LBM_TRY(check_timeout(S, st));         // also orders the state after the caller's work
    CkptHeader h;
    LBM_TRY(ckpt_header(S, h));
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(LBM_ERR_IO, "cannot open %s for writing", path);
    bool ok = std::fwrite(&h, sizeof h, 1, f) == 1;
    const char* src = (const char*)S->buf[S->pattern == LBM_PULL ? S->cur : 0];
    std::vector<char> blk(std::min<size_t>(kCkptBlock, (size_t)h.bytes));
    for (uint64_t off = 0; ok && off < h.bytes; off += blk.size()) {
        const size_t n = (size_t)std::min<uint64_t>(blk.size(), h.bytes - off);
        if (cudaMemcpy(blk.data(), src + off, n, cudaMemcpyDeviceToHost) != cudaSuccess) {
            std::fclose(f);
            return fail(LBM_ERR_CUDA, "checkpoint: device copy failed");
        }
        ok = std::fwrite(blk.data(), 1, n, f) == n;
    }
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) return fail(LBM_ERR_IO, "writing %s failed", path);
    return LBM_OK;
}

lbm_status lbm_sim_restart(lbm_sim* S, const char* path, void* stream) {
    const NvtxRange nvtx_range("lbm_sim_restart");
    if (!S || !path) return fail(LBM_ERR_ARG, "lbm_sim_restart: null argument");
    clear_error();
    cudaStream_t st = (cudaStream_t)stream;
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(LBM_ERR_IO, "cannot open %s", path);
    CkptHeader h, mine;
    const bool got = std::fread(&h, sizeof h, 1, f) == 1;
    lbm_status hs = ckpt_header(S, mine);
    if (hs != LBM_OK) { std::fclose(f); return hs; }
    if (!got || std::memcmp(h.magic, "LBMCKPT2", 8) != 0) {
        std::fclose(f);
        return fail(LBM_ERR_PARSE, "%s is not a checkpoint of this engine", path);
    }
    if (h.Q != mine.Q || h.store != mine.store || h.pattern != mine.pattern || h.n_inst != mine.n_inst ||
        h.N != mine.N || h.NF != mine.NF || h.stride != mine.stride || h.nchunks != mine.nchunks ||
        h.grid_hash != mine.grid_hash || h.bytes != mine.bytes) {
        std::fclose(f);
        return fail(LBM_ERR_ARG, "%s was written for another lattice or storage (Q %d/%d, precision %d/%d, pattern "
                                 "%d/%d, nodes %lld/%lld)", path, h.Q, mine.Q, h.store, mine.store, h.pattern,
                    mine.pattern, (long long)h.N, (long long)mine.N);
    }
    LBM_CUDA(cudaStreamSynchronize(st));
    char* dst = (char*)S->buf[0];
    std::vector<char> blk(std::min<size_t>(kCkptBlock, (size_t)h.bytes));
    for (uint64_t off = 0; off < h.bytes; off += blk.size()) {
        const size_t n = (size_t)std::min<uint64_t>(blk.size(), h.bytes - off);
        if (std::fread(blk.data(), 1, n, f) != n) {
            std::fclose(f);
            return fail(LBM_ERR_PARSE, "%s is truncated", path);
        }
        if (cudaMemcpy(dst + off, blk.data(), n, cudaMemcpyHostToDevice) != cudaSuccess) {
            std::fclose(f);
            return fail(LBM_ERR_CUDA, "restart: device copy failed");
        }
    }
    std::fclose(f);
    S->cur = 0;
    S->steps_done = h.steps_done;
    S->aa_phase = h.aa_phase;
    free_graph(S);
    return LBM_OK;
}

void lbm_sim_destroy(lbm_sim* S) {
    if (!S) return;
    cudaDeviceSynchronize();               // pool memory (wall_pos) is freed without an implicit wait
    free_graph(S);
    for (void* b : S->buf) if (b) cudaFree(b);
    if (S->chunks) cudaFree(S->chunks);
    for (Chunk* c : S->chunks2s) if (c) cudaFree(c);
    for (Chunk* c : S->chunks2gs) if (c) cudaFree(c);
    for (uint2* c : S->even2s) if (c) cudaFree(c);
    if (S->wall_pos) cudaFree(S->wall_pos);
    if (S->zslots) cudaFree(S->zslots);
    if (S->lists) cudaFree(S->lists);
    if (S->insts) cudaFree(S->insts);
    if (S->amp) cudaFree(S->amp);
    if (S->node_grid) cudaFree(S->node_grid);
    if (S->out_pos) cudaFree(S->out_pos);
    if (S->mmask) cudaFree(S->mmask);
    if (S->part) cudaFree(S->part);
    if (S->partbad) cudaFree(S->partbad);
    if (S->mon) cudaFree(S->mon);
    if (S->step_base) cudaFree(S->step_base);
    if (S->err) cudaFree(S->err);
    delete S;
}

}  // extern "C"
