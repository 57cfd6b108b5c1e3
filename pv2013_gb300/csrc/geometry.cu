// GPU voxelization and boundary classification (sm_103a).  Compiled with
// -fmad=false: every FP64 expression below is evaluated operation by
// operation like the reference's C++ (no fused multiply-add), which is what
// makes the node-type field bit-exact.
//
// Reference semantics restated here:
//   grid points        x = min_x + i*spacing        ComplexGeometry.cpp:199-201
//   ray                +z from the point, end z = (z + L) + 0.1, L = max_z-min_z,
//                      x/y nudged 0.01 inward on bbox faces  :334-357, :438-492
//   crossing test      t = ((q-p).n)/((e-s).n) with the file normal,
//                      t in [-1e-7, 1+1e-7], then the inclusive xy inside test
//                      at (p + t(e-s))                          :284-330, :264-281
//   label              odd count -> Fluid                       :495-502
//   boundary points    Fluid with a NotFluid 26-neighbour or on a bbox face,
//                      x-major order                            :509-556
//   lists              plane predicates, then wall = the rest   :559-638
//
// Work decomposition (GB300-first, not the reference's point x triangle loop):
//   1. one thread per triangle enumerates the grid columns (i,j) whose ray can
//      pass its xy-projection (padded box; for needle-thin projections also a
//      band along the supporting line, where rounding can make the inclusive
//      test succeed beyond the segment) and keeps those passing the exact xy
//      test.  Count pass, scan, fill pass -> per-column candidate lists.
//   2. one warp per column stages the candidates' plane terms in shared memory
//      and evaluates the exact crossing test for every z of the column, lanes
//      strided over z; parity is written as one byte per point (coalesced).
// Because the ray is vertical, the xy inside test is independent of z, so
// the split is exact.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "device.cuh"
#include "internal.h"
#include "scan.cuh"
#include "nvtx.h"

namespace lbm {

struct VoxGrid {
    double bb[6];      // min_x,max_x,min_y,max_y,min_z,max_z
    double spacing;
    int32_t Nx, Ny, Nz;
};

// ---------------------------------------------------------------------------
// exact helpers (no contraction in this TU)

__device__ __forceinline__ bool inside2d(double x, double y, const double* T) {
    const double x1 = T[0], y1 = T[1], x2 = T[3], y2 = T[4], x3 = T[6], y3 = T[7];
    const double d1 = ((x - x2) * (y1 - y2) - (y - y2) * (x1 - x2));
    const double d2 = ((x - x3) * (y2 - y3) - (y - y3) * (x2 - x3));
    const double d3 = ((x - x1) * (y3 - y1) - (y - y1) * (x3 - x1));
    const bool neg = (d1 < 0) || (d2 < 0) || (d3 < 0);
    const bool pos = (d1 > 0) || (d2 > 0) || (d3 > 0);
    return !(neg && pos);
}

// Ray start x,y of column (i,j) after adjustLineCoordinates case 0.
__device__ __forceinline__ void column_xy(const VoxGrid& g, int i, int j, double& sx, double& sy) {
    sx = g.bb[0] + (double)i * g.spacing;
    sy = g.bb[2] + (double)j * g.spacing;
    const double off = 0.01;
    if (sx == g.bb[0]) sx += off;
    if (sx == g.bb[1]) sx -= off;
    if (sy == g.bb[2]) sy += off;
    if (sy == g.bb[3]) sy -= off;
}

// Candidate columns of triangle T, in two parts.  enum_box calls fn(col) for
// the columns of the projection's bounding box that pass the exact xy test
// and returns kPointLike when the projection is degenerate to a point (such
// a triangle is tested by every column instead), kNeedle when it is so thin
// that the xy test can also pass on its supporting line outside the box, and
// kBoxOnly otherwise.  enum_band covers the needle case: a band around the
// supporting line of the longest edge across the whole grid, the columns
// lane, lane + nl, ... of it (a warp shares one triangle's band).
constexpr int kPointLike = 0, kBoxOnly = 1, kNeedle = 2;

struct BoxRange {
    long i0, i1, j0, j1;
};

template <class F>
__device__ int enum_box(const VoxGrid& g, const double* T, BoxRange& r, F fn) {
    const double s = g.spacing;
    const double xmn = fmin(T[0], fmin(T[3], T[6])), xmx = fmax(T[0], fmax(T[3], T[6]));
    const double ymn = fmin(T[1], fmin(T[4], T[7])), ymx = fmax(T[1], fmax(T[4], T[7]));
    // columns whose ray (min + i*s, nudged by at most 0.01 at the grid faces)
    // lies within 0.01 of the projection's bounding box: a non-degenerate
    // triangle contains no point outside its box, and the margin covers the
    // face nudge; the bounds are found with the same expression column_xy uses
    auto lower = [&](double v, double base, int n) -> long {   // first i with base + i*s >= v
        long i = max((long)floor((v - base) / s) - 1, 0L);
        while (i < n && base + (double)i * s < v) ++i;
        return i;
    };
    auto upper = [&](double v, double base, int n) -> long {   // last i with base + i*s <= v
        long i = min((long)ceil((v - base) / s) + 1, (long)n - 1);
        while (i >= 0 && base + (double)i * s > v) --i;
        return i;
    };
    r.i0 = lower(xmn - 0.01, g.bb[0], g.Nx);
    r.i1 = upper(xmx + 0.01, g.bb[0], g.Nx);
    r.j0 = lower(ymn - 0.01, g.bb[2], g.Ny);
    r.j1 = upper(ymx + 0.01, g.bb[2], g.Ny);
    double ex[3] = {T[3] - T[0], T[6] - T[3], T[0] - T[6]};
    double ey[3] = {T[4] - T[1], T[7] - T[4], T[1] - T[7]};
    double best = -1.0;
    for (int m = 0; m < 3; ++m) {
        double l = fabs(ex[m]) + fabs(ey[m]);
        if (l > best) best = l;
    }
    const double scale = 1.0 + fmax(fmax(fabs(xmn), fabs(xmx)), fmax(fabs(ymn), fabs(ymx)));
    if (!(best > 1e-9 * scale)) return kPointLike;    // point-like projection: every column tests it
    for (long i = r.i0; i <= r.i1; ++i)
        for (long j = r.j0; j <= r.j1; ++j) {
            double sx, sy;
            column_xy(g, (int)i, (int)j, sx, sy);
            if (inside2d(sx, sy, T)) fn(i * (long)g.Ny + j);
        }
    // needle-thin projection: the band below is needed as well
    const double area2 = fabs((T[3] - T[0]) * (T[7] - T[1]) - (T[4] - T[1]) * (T[6] - T[0]));
    return area2 > 1e-9 * best * scale ? kBoxOnly : kNeedle;   // height above 1e-9 relative: box is enough
}

template <class F>
__device__ void enum_band(const VoxGrid& g, const double* T, const BoxRange& r, int lane, int nl, F fn) {
    const double s = g.spacing;
    const int bp = 2 + (int)ceil(0.01 / s);
    double ex[3] = {T[3] - T[0], T[6] - T[3], T[0] - T[6]};
    double ey[3] = {T[4] - T[1], T[7] - T[4], T[1] - T[7]};
    int e = 0;
    double best = -1.0;
    for (int m = 0; m < 3; ++m) {
        double l = fabs(ex[m]) + fabs(ey[m]);
        if (l > best) { best = l; e = m; }
    }
    const double ox = T[3 * e], oy = T[3 * e + 1];
    const double dx = ex[e], dy = ey[e];
    if (fabs(dx) >= fabs(dy)) {
        for (long i = lane; i < g.Nx; i += nl) {
            if (i >= r.i0 && i <= r.i1) continue;
            double sx, sy;
            column_xy(g, (int)i, 0, sx, sy);
            double y = oy + (sx - ox) * (dy / dx);
            long jc = (long)floor((y - g.bb[2]) / s);
            for (long j = max(0L, jc - bp); j <= min((long)g.Ny - 1, jc + 1 + bp); ++j) {
                column_xy(g, (int)i, (int)j, sx, sy);
                if (inside2d(sx, sy, T)) fn(i * (long)g.Ny + j);
            }
        }
    } else {
        for (long j = lane; j < g.Ny; j += nl) {
            if (j >= r.j0 && j <= r.j1) continue;
            double sx, sy;
            column_xy(g, 0, (int)j, sx, sy);
            double x = ox + (sy - oy) * (dx / dy);
            long ic = (long)floor((x - g.bb[0]) / s);
            for (long i = max(0L, ic - bp); i <= min((long)g.Nx - 1, ic + 1 + bp); ++i) {
                column_xy(g, (int)i, (int)j, sx, sy);
                if (inside2d(sx, sy, T)) fn(i * (long)g.Ny + j);
            }
        }
    }
}

// One thread per triangle for the box; the warp's needle triangles then
// take turns, each band scanned by all 32 lanes.  Threads past the end
// stay for the warp-wide vote.
template <class FMake>
__device__ void enumerate_warp(const VoxGrid& g, const double* tris, int64_t t, int64_t ntris, FMake make_fn,
                               int32_t* global_list, int32_t* nglobal) {
    const int lane = threadIdx.x & 31;
    const bool valid = t < ntris;
    int kind = kBoxOnly;
    BoxRange r = {0, -1, 0, -1};
    if (valid) {
        kind = enum_box(g, tris + 12 * t, r, make_fn(t));
        if (kind == kPointLike && global_list) {
            const int slot = atomicAdd(nglobal, 1);
            global_list[slot] = (int32_t)t;
        }
    }
    unsigned m = __ballot_sync(0xffffffffu, valid && kind == kNeedle);
    while (m) {
        const int src = __ffs(m) - 1;
        m &= m - 1;
        const long long ts = __shfl_sync(0xffffffffu, (long long)t, src);
        BoxRange rs;
        rs.i0 = __shfl_sync(0xffffffffu, (long long)r.i0, src);
        rs.i1 = __shfl_sync(0xffffffffu, (long long)r.i1, src);
        rs.j0 = __shfl_sync(0xffffffffu, (long long)r.j0, src);
        rs.j1 = __shfl_sync(0xffffffffu, (long long)r.j1, src);
        enum_band(g, tris + 12 * ts, rs, lane, 32, make_fn((int64_t)ts));
    }
}

__global__ void k_tri_count(VoxGrid g, const double* __restrict__ tris, int64_t ntris, int32_t* __restrict__ colcount,
                            int32_t* __restrict__ global_list, int32_t* __restrict__ nglobal) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    enumerate_warp(g, tris, t, ntris, [&](int64_t) { return [colcount](long col) { atomicAdd(&colcount[col], 1); }; },
                   global_list, nglobal);
}

__global__ void k_tri_fill(VoxGrid g, const double* __restrict__ tris, int64_t ntris, const int64_t* __restrict__ colstart,
                           int32_t* __restrict__ cursor, int32_t* __restrict__ pairs) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    enumerate_warp(g, tris, t, ntris, [&](int64_t tt) {
        return [=](long col) {
            int slot = atomicAdd(&cursor[col], 1);
            pairs[colstart[col] + slot] = (int32_t)tt;
        };
    }, nullptr, nullptr);
}

// Per-candidate plane terms staged in shared memory.
struct Cand {
    double c;     // (qx - sx)*nx + (qy - sy)*ny
    double qz;
    double nz;
    double d0;    // (ex - sx)*nx + (ey - sy)*ny  (ex == sx, ey == sy)
};

constexpr int kVoxWarps = 8;
constexpr int kCandPerWarp = 64;

// One warp per column.  Lanes first filter candidates with the exact xy test
// and stage survivors; then each lane walks its z values and counts crossings.
__global__ void __launch_bounds__(kVoxWarps * 32)
k_columns(VoxGrid g, const double* __restrict__ tris, const int64_t* __restrict__ colstart,
          const int32_t* __restrict__ pairs, const int32_t* __restrict__ global_list, int32_t nglobal,
          uint8_t* __restrict__ flags) {
    __shared__ Cand cand[kVoxWarps][kCandPerWarp];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t col = blockIdx.x * (int64_t)kVoxWarps + w;
    const int64_t ncol = (int64_t)g.Nx * g.Ny;
    if (col >= ncol) return;
    const int i = (int)(col / g.Ny), j = (int)(col % g.Ny);
    double sx, sy;
    column_xy(g, i, j, sx, sy);
    const double L = g.bb[5] - g.bb[4];
    const int64_t c0 = colstart[col], c1 = colstart[col + 1];
    const int64_t total = (c1 - c0) + nglobal;
    uint8_t* out = flags + col * (int64_t)g.Nz;
    // parity per z kept in registers: lane owns z = lane + 32*m
    constexpr int kMaxM = 64;   // Nz <= 2048 handled in one sweep of registers-by-bits
    uint64_t par_bits = 0;      // bit m <-> z = lane + 32*m, m < 64
    const int nm = (g.Nz + 31) / 32;
    for (int64_t cb = 0; cb < total; cb += kCandPerWarp) {
        // stage up to kCandPerWarp survivors from candidates [cb, cb+kCandPerWarp)
        int nsurv = 0;
        for (int64_t k = cb; k < min(total, cb + (int64_t)kCandPerWarp); k += 32) {
            int64_t idx = k + lane;
            bool keep = false;
            Cand cd;
            if (idx < min(total, cb + (int64_t)kCandPerWarp)) {
                int32_t t = idx < (c1 - c0) ? pairs[c0 + idx] : global_list[idx - (c1 - c0)];
                const double* T = tris + 12 * (int64_t)t;
                if (inside2d(sx, sy, T)) {
                    keep = true;
                    const double dxv = sx - sx, dyv = sy - sy;
                    cd.c = (T[0] - sx) * T[9] + (T[1] - sy) * T[10];
                    cd.qz = T[2];
                    cd.nz = T[11];
                    cd.d0 = dxv * T[9] + dyv * T[10];
                }
            }
            unsigned bal = __ballot_sync(0xffffffffu, keep);
            if (keep) cand[w][nsurv + __popc(bal & ((1u << lane) - 1))] = cd;
            nsurv += __popc(bal);
        }
        __syncwarp();
        for (int m = 0; m < nm; ++m) {
            const int z = lane + 32 * m;
            if (z >= g.Nz) break;
            const double pz = g.bb[4] + (double)z * g.spacing;
            double ez = pz + L;
            ez = ez + 0.1;
            const double dzv = ez - pz;
            int cnt = 0;
            for (int s = 0; s < nsurv; ++s) {
                const Cand cd = cand[w][s];
                const double num = cd.c + (cd.qz - pz) * cd.nz;
                const double den = cd.d0 + dzv * cd.nz;
                const double t = num / den;
                cnt += (t >= -1e-7 && t <= 1 + 1e-7) ? 1 : 0;
            }
            if (cnt & 1) par_bits ^= (1ull << m);
        }
        __syncwarp();
    }
    for (int m = 0; m < nm && m < kMaxM; ++m) {
        const int z = lane + 32 * m;
        if (z < g.Nz) out[z] = (uint8_t)((par_bits >> m) & 1);
    }
}

// Boundary points: ComplexGeometry.cpp:509-556.
__global__ void k_boundary(VoxGrid g, const uint8_t* __restrict__ flags, uint8_t* __restrict__ isb) {
    const int64_t n = (int64_t)g.Nx * g.Ny * g.Nz;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
        uint8_t r = 0;
        if (flags[p]) {
            const int k = (int)(p % g.Nz);
            const int64_t ij = p / g.Nz;
            const int j = (int)(ij % g.Ny), i = (int)(ij / g.Ny);
            bool b = (i == 0 || i == g.Nx - 1 || j == 0 || j == g.Ny - 1 || k == 0 || k == g.Nz - 1);
            for (int dx = -1; dx <= 1 && !b; ++dx)
                for (int dy = -1; dy <= 1 && !b; ++dy)
                    for (int dz = -1; dz <= 1 && !b; ++dz) {
                        const int a = i + dx, c = j + dy, e = k + dz;
                        if (a >= 0 && a < g.Nx && c >= 0 && c < g.Ny && e >= 0 && e < g.Nz &&
                            !flags[((int64_t)a * g.Ny + c) * g.Nz + e])
                            b = true;
                    }
            r = b ? 1 : 0;
        }
        isb[p] = r;
    }
}

struct DevPred {
    int32_t list_id, axis;
    double plane_hi, plane_lo, tol;
    double lo[3], hi[3];
};

// getInOutBP predicates, |p - plane| <= tol with plane = hi + lo (double-double).
__global__ void k_predicates(VoxGrid g, const int64_t* __restrict__ bidx, int64_t nb, const DevPred* __restrict__ preds,
                             int np, uint64_t* __restrict__ mask) {
    for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < nb; b += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = bidx[b];
        const int k = (int)(p % g.Nz);
        const int64_t ij = p / g.Nz;
        const int j = (int)(ij % g.Ny), i = (int)(ij / g.Ny);
        const double c[3] = {g.bb[0] + (double)i * g.spacing, g.bb[2] + (double)j * g.spacing,
                             g.bb[4] + (double)k * g.spacing};
        uint64_t m = 0;
        for (int q = 0; q < np; ++q) {
            const DevPred& P = preds[q];
            const double d = (c[P.axis] - P.plane_hi) - P.plane_lo;
            bool ok = fabs(d) <= P.tol;
            for (int a = 0; a < 3 && ok; ++a) {
                if (a == P.axis) continue;
                if (!isnan(P.lo[a]) && !(P.lo[a] < c[a])) ok = false;
                if (!isnan(P.hi[a]) && !(c[a] < P.hi[a])) ok = false;
            }
            if (ok) m |= 1ull << P.list_id;
        }
        mask[b] = m;
    }
}

__global__ void k_list_flag(const uint64_t* __restrict__ mask, int64_t nb, int list, uint8_t* __restrict__ fl) {
    for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < nb; b += (int64_t)gridDim.x * blockDim.x)
        fl[b] = list >= 0 ? (uint8_t)((mask[b] >> list) & 1) : (uint8_t)(mask[b] == 0);
}

__global__ void k_gather_i64(const int64_t* __restrict__ src, const int64_t* __restrict__ idx, int64_t n,
                             int64_t* __restrict__ out) {
    for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < n; b += (int64_t)gridDim.x * blockDim.x)
        out[b] = src[idx[b]];
}

}  // namespace lbm

// ---------------------------------------------------------------------------
// host side

struct lbm_geometry {
    lbm::VoxGrid grid;
    int dev = 0;
    uint8_t* d_flags = nullptr;        // Nx*Ny*Nz
    int64_t* d_bidx = nullptr;         // boundary point grid indices
    uint64_t* d_bmask = nullptr;       // predicate mask per boundary point
    int64_t n_fluid = 0, n_boundary = 0;
    std::vector<int64_t> list_sizes;   // per list id (64)
    int64_t n_wall = 0;
    int32_t n_lists = 0;
    double vox_ms = 0, cls_ms = 0;
};

namespace lbm {

static int g_blocks_for(int64_t n, int threads) {
    int64_t b = (n + threads - 1) / threads;
    if (b > 152LL * 64) b = 152LL * 64;
    if (b < 1) b = 1;
    return (int)b;
}

// Device buffer that frees itself, from the device's stream-ordered pool
// (dev_alloc): allocated and freed in the order of the stream that uses it.
template <class T>
struct DBuf {
    T* p = nullptr;
    cudaStream_t s = 0;
    ~DBuf() { if (p) dev_free(p, s); }
    lbm_status alloc(size_t n, const char* what, cudaStream_t st) {
        s = st;
        return dev_alloc(reinterpret_cast<void**>(&p), sizeof(T) * (n ? n : 1), st, what);
    }
    void adopt(T* q, cudaStream_t st) { p = q; s = st; }
    T* release() { T* q = p; p = nullptr; return q; }
};

}  // namespace lbm

using namespace lbm;

#define LBM_TRY(x)                      \
    do {                                \
        lbm_status s_ = (x);            \
        if (s_ != LBM_OK) return s_;    \
    } while (0)

static lbm_status geometry_build(lbm_geometry* G, const lbm_tri* tris, size_t ntris, double spacing,
                                 const lbm_grid* grid, const lbm_bc_predicate* preds, size_t npreds, cudaStream_t st) {
    VoxGrid& g = G->grid;
    g.spacing = spacing;
    if (grid) {
        for (int a = 0; a < 3; ++a) {
            if (grid->dims[a] < 1) return fail(LBM_ERR_ARG, "grid dims must be >= 1");
            g.bb[2 * a] = grid->min[a];
            g.bb[2 * a + 1] = grid->min[a] + (grid->dims[a] - 1) * spacing;
        }
        g.Nx = grid->dims[0]; g.Ny = grid->dims[1]; g.Nz = grid->dims[2];
    } else {
        if (ntris == 0) return fail(LBM_ERR_ARG, "tight grid needs at least one triangle");
        double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (size_t t = 0; t < ntris; ++t) {
            const double* T = &tris[t].x1;
            for (int a = 0; a < 3; ++a) {
                mn[a] = std::min(mn[a], std::min(T[a], std::min(T[3 + a], T[6 + a])));
                mx[a] = std::max(mx[a], std::max(T[a], std::max(T[3 + a], T[6 + a])));
            }
        }
        int d[3];
        for (int a = 0; a < 3; ++a) {
            g.bb[2 * a] = mn[a]; g.bb[2 * a + 1] = mx[a];
            double n = std::ceil((mx[a] - mn[a]) / spacing);
            if (!(n >= 0 && n < 1e6)) return fail(LBM_ERR_ARG, "grid extent on axis %d is not finite or too large", a);
            d[a] = (int)n + 1;
        }
        g.Nx = d[0]; g.Ny = d[1]; g.Nz = d[2];
    }
    if (g.Nz > 2048) return fail(LBM_ERR_ARG, "Nz = %d exceeds the voxelizer's 2048-point column limit", g.Nz);
    const int64_t npts = (int64_t)g.Nx * g.Ny * g.Nz;
    const int64_t ncol = (int64_t)g.Nx * g.Ny;
    for (size_t p = 0; p < npreds; ++p) {
        if (preds[p].list_id < 0 || preds[p].list_id > 63 || preds[p].axis < 0 || preds[p].axis > 2)
            return fail(LBM_ERR_ARG, "predicate %zu: list id must be 0..63 and axis 0..2", p);
    }
    if (ntris >= (size_t)INT32_MAX) return fail(LBM_ERR_ARG, "too many triangles");

    cudaEvent_t e0, e1, e2;
    LBM_CUDA(cudaEventCreate(&e0));
    LBM_CUDA(cudaEventCreate(&e1));
    LBM_CUDA(cudaEventCreate(&e2));

    DBuf<double> d_tris;
    LBM_TRY(d_tris.alloc(ntris * 12, "triangles", st));
    if (ntris) LBM_CUDA(cudaMemcpyAsync(d_tris.p, tris, sizeof(double) * 12 * ntris, cudaMemcpyHostToDevice, st));
    DBuf<int32_t> colcount, cursor, glist, nglob;
    DBuf<int64_t> colstart;
    DBuf<uint8_t> flags;
    LBM_TRY(colcount.alloc(ncol, "column counts", st));
    LBM_TRY(cursor.alloc(ncol, "column cursors", st));
    LBM_TRY(colstart.alloc(ncol + 1, "column offsets", st));
    LBM_TRY(glist.alloc(ntris, "global triangle list", st));
    LBM_TRY(nglob.alloc(1, "global count", st));
    LBM_TRY(flags.alloc(npts, "node-type field", st));
    LBM_CUDA(cudaEventRecord(e0, st));
    LBM_CUDA(cudaMemsetAsync(colcount.p, 0, sizeof(int32_t) * ncol, st));
    LBM_CUDA(cudaMemsetAsync(cursor.p, 0, sizeof(int32_t) * ncol, st));
    LBM_CUDA(cudaMemsetAsync(nglob.p, 0, sizeof(int32_t), st));
    const int TB = 128;
    if (ntris) k_tri_count<<<(unsigned)((ntris + TB - 1) / TB), TB, 0, st>>>(g, d_tris.p, (int64_t)ntris, colcount.p, glist.p, nglob.p);
    int64_t npairs = 0;
    LBM_TRY(scan::exclusive_scan(colcount.p, ncol, colstart.p, &npairs, st));
    LBM_CUDA(cudaMemcpyAsync(colstart.p + ncol, &npairs, sizeof(int64_t), cudaMemcpyHostToDevice, st));
    int32_t nglobal = 0;
    LBM_CUDA(cudaMemcpyAsync(&nglobal, nglob.p, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    DBuf<int32_t> pairs;
    LBM_TRY(pairs.alloc(npairs, "column candidate lists", st));
    if (ntris) k_tri_fill<<<(unsigned)((ntris + TB - 1) / TB), TB, 0, st>>>(g, d_tris.p, (int64_t)ntris, colstart.p, cursor.p, pairs.p);
    LBM_CUDA(cudaStreamSynchronize(st));
    k_columns<<<(unsigned)((ncol + kVoxWarps - 1) / kVoxWarps), kVoxWarps * 32, 0, st>>>(
        g, d_tris.p, colstart.p, pairs.p, glist.p, nglobal, flags.p);
    LBM_CUDA(cudaGetLastError());
    LBM_CUDA(cudaEventRecord(e1, st));

    // boundary points and predicate lists
    DBuf<uint8_t> isb;
    LBM_TRY(isb.alloc(npts, "boundary flags", st));
    k_boundary<<<g_blocks_for(npts, 256), 256, 0, st>>>(g, flags.p, isb.p);
    LBM_TRY(scan::count_nonzero(flags.p, npts, &G->n_fluid, st));
    int64_t* bidx = nullptr;
    LBM_TRY(scan::compact(isb.p, npts, &bidx, &G->n_boundary, st));
    G->d_bidx = bidx;
    DBuf<uint64_t> bmask;
    LBM_TRY(bmask.alloc(G->n_boundary, "boundary masks", st));
    std::vector<DevPred> hp(npreds);
    int32_t nl = 0;
    for (size_t p = 0; p < npreds; ++p) {
        hp[p] = {preds[p].list_id, preds[p].axis, preds[p].plane_hi, preds[p].plane_lo, preds[p].tol,
                 {preds[p].lo[0], preds[p].lo[1], preds[p].lo[2]}, {preds[p].hi[0], preds[p].hi[1], preds[p].hi[2]}};
        nl = std::max(nl, preds[p].list_id + 1);
    }
    DBuf<DevPred> dpred;
    LBM_TRY(dpred.alloc(npreds, "predicates", st));
    if (npreds) LBM_CUDA(cudaMemcpyAsync(dpred.p, hp.data(), sizeof(DevPred) * npreds, cudaMemcpyHostToDevice, st));
    if (G->n_boundary)
        k_predicates<<<g_blocks_for(G->n_boundary, 256), 256, 0, st>>>(g, bidx, G->n_boundary, dpred.p, (int)npreds, bmask.p);
    LBM_CUDA(cudaGetLastError());
    LBM_CUDA(cudaEventRecord(e2, st));
    G->d_bmask = bmask.release();
    G->d_flags = flags.release();
    G->n_lists = nl;
    G->list_sizes.assign(64, 0);
    {
        DBuf<uint8_t> fl;
        LBM_TRY(fl.alloc(G->n_boundary, "list flags", st));
        for (int l = -1; l < nl; ++l) {
            k_list_flag<<<g_blocks_for(G->n_boundary, 256), 256, 0, st>>>(G->d_bmask, G->n_boundary, l, fl.p);
            int64_t c = 0;
            LBM_TRY(scan::count_nonzero(fl.p, G->n_boundary, &c, st));
            if (l < 0) G->n_wall = c; else G->list_sizes[l] = c;
        }
    }
    LBM_CUDA(cudaStreamSynchronize(st));
    float ms1 = 0, ms2 = 0;
    cudaEventElapsedTime(&ms1, e0, e1);
    cudaEventElapsedTime(&ms2, e1, e2);
    G->vox_ms = ms1;
    G->cls_ms = ms2;
    cudaEventDestroy(e0); cudaEventDestroy(e1); cudaEventDestroy(e2);
    return LBM_OK;
}

extern "C" {

lbm_status lbm_geometry_create(const lbm_tri* tris, size_t ntris, double spacing, const lbm_grid* grid,
                               const lbm_bc_predicate* preds, size_t npreds, void* stream, lbm_geometry** out) {
    const NvtxRange nvtx_range("lbm_geometry_create");
    if (!out || (!tris && ntris) || (!preds && npreds) || !(spacing > 0))
        return fail(LBM_ERR_ARG, "lbm_geometry_create: bad argument");
    clear_error();
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(LBM_ERR_NODEV, "no CUDA device");
    lbm_geometry* G = new lbm_geometry();
    cudaGetDevice(&G->dev);
    lbm_status s = guarded("lbm_geometry_create",
                           [&] { return geometry_build(G, tris, ntris, spacing, grid, preds, npreds, (cudaStream_t)stream); });
    if (s != LBM_OK) { lbm_geometry_destroy(G); return s; }
    *out = G;
    return LBM_OK;
}

lbm_status lbm_predicates_pv2013(lbm_bc_predicate* out, size_t cap, size_t* n) {
    // ComplexGeometry.cpp:587-633; plane constants are long double literals,
    // represented here as double-double (hi + lo).
    struct P { int list, axis; long double plane; double lo[3], hi[3]; };
    const double N = NAN;
    const P tab[7] = {
        {0, 1, -175.275L, {-9.9, N, -129.979}, {-3.3, N, -124.799}},
        {1, 1, -164.075L, {N, N, N}, {N, N, N}},
        {2, 1, -174.475L, {-5.4, N, -101.379}, {-5, N, -100.979}},
        {3, 0, -28.3L, {N, -179.975, -97.2794}, {N, -178.875, -96.2794}},
        {4, 0, -25.5L, {N, -180.675, -100.779}, {N, -179.875, -100.379}},
        {5, 0, -37.0L, {N, N, N}, {N, N, N}},
        {6, 2, -108.379L, {-29.7, -196.375, N}, {-28.1, -194.575, N}},
    };
    if (!n) return fail(LBM_ERR_ARG, "lbm_predicates_pv2013: null n");
    *n = 7;
    if (!out) return LBM_OK;
    if (cap < 7) return fail(LBM_ERR_ARG, "lbm_predicates_pv2013: capacity %zu < 7", cap);
    for (int i = 0; i < 7; ++i) {
        lbm_bc_predicate& p = out[i];
        p.list_id = tab[i].list;
        p.axis = tab[i].axis;
        p.plane_hi = (double)tab[i].plane;
        p.plane_lo = (double)(tab[i].plane - (long double)p.plane_hi);
        p.tol = 1e-2;
        for (int a = 0; a < 3; ++a) { p.lo[a] = tab[i].lo[a]; p.hi[a] = tab[i].hi[a]; }
    }
    return LBM_OK;
}

lbm_status lbm_geometry_info_get(const lbm_geometry* G, lbm_geometry_info* info) {
    if (!G || !info) return fail(LBM_ERR_ARG, "lbm_geometry_info_get: null argument");
    std::memset(info, 0, sizeof *info);
    info->dims[0] = G->grid.Nx; info->dims[1] = G->grid.Ny; info->dims[2] = G->grid.Nz;
    for (int a = 0; a < 6; ++a) info->bbox[a] = G->grid.bb[a];
    info->spacing = G->grid.spacing;
    info->n_points = (int64_t)G->grid.Nx * G->grid.Ny * G->grid.Nz;
    info->n_fluid = G->n_fluid;
    info->n_boundary = G->n_boundary;
    info->n_wall = G->n_wall;
    for (int l = 0; l < 64; ++l) info->list_size[l] = G->list_sizes.empty() ? 0 : G->list_sizes[l];
    info->n_lists = G->n_lists;
    info->voxelize_ms = G->vox_ms;
    info->classify_ms = G->cls_ms;
    return LBM_OK;
}

lbm_status lbm_geometry_flags(const lbm_geometry* G, uint8_t* host_out, size_t cap) {
    if (!G || !host_out) return fail(LBM_ERR_ARG, "lbm_geometry_flags: null argument");
    size_t n = (size_t)G->grid.Nx * G->grid.Ny * G->grid.Nz;
    if (cap < n) return fail(LBM_ERR_ARG, "lbm_geometry_flags: capacity %zu < %zu", cap, n);
    LBM_CUDA(cudaMemcpy(host_out, G->d_flags, n, cudaMemcpyDeviceToHost));
    return LBM_OK;
}

lbm_status lbm_geometry_list(const lbm_geometry* G, int32_t list, int64_t* host_out, size_t cap, size_t* n) {
    if (!G || !n || list < -2 || list > 63) return fail(LBM_ERR_ARG, "lbm_geometry_list: bad argument");
    clear_error();
    int64_t cnt = list == LBM_LIST_BOUNDARY ? G->n_boundary : (list == LBM_LIST_WALL ? G->n_wall : G->list_sizes[list]);
    *n = (size_t)cnt;
    if (!host_out) return LBM_OK;
    if (cap < (size_t)cnt) return fail(LBM_ERR_ARG, "lbm_geometry_list: capacity %zu < %lld", cap, (long long)cnt);
    if (cnt == 0) return LBM_OK;
    if (list == LBM_LIST_BOUNDARY) {
        LBM_CUDA(cudaMemcpy(host_out, G->d_bidx, sizeof(int64_t) * cnt, cudaMemcpyDeviceToHost));
        return LBM_OK;
    }
    cudaStream_t st = 0;
    DBuf<uint8_t> fl;
    LBM_TRY(fl.alloc(G->n_boundary, "list flags", st));
    k_list_flag<<<g_blocks_for(G->n_boundary, 256), 256, 0, st>>>(G->d_bmask, G->n_boundary,
                                                                  list == LBM_LIST_WALL ? -1 : list, fl.p);
    int64_t* pos = nullptr;
    int64_t c = 0;
    LBM_TRY(scan::compact(fl.p, G->n_boundary, &pos, &c, st));
    DBuf<int64_t> posb; posb.adopt(pos, st);
    DBuf<int64_t> vals;
    LBM_TRY(vals.alloc(c, "list values", st));
    k_gather_i64<<<g_blocks_for(c, 256), 256, 0, st>>>(G->d_bidx, pos, c, vals.p);
    LBM_CUDA(cudaMemcpy(host_out, vals.p, sizeof(int64_t) * c, cudaMemcpyDeviceToHost));
    return LBM_OK;
}

void lbm_geometry_destroy(lbm_geometry* G) {
    if (!G) return;
    cudaDeviceSynchronize();               // pool memory is freed without an implicit wait
    if (G->d_flags) cudaFree(G->d_flags);
    if (G->d_bidx) cudaFree(G->d_bidx);
    if (G->d_bmask) cudaFree(G->d_bmask);
    delete G;
}

}  // extern "C"

// accessors for the lattice builder (sim.cu)
namespace lbm {
const uint8_t* geometry_flags_dev(const lbm_geometry* g) { return g->d_flags; }
const int64_t* geometry_bidx_dev(const lbm_geometry* g) { return g->d_bidx; }
const uint64_t* geometry_bmask_dev(const lbm_geometry* g) { return g->d_bmask; }
int64_t geometry_nboundary(const lbm_geometry* g) { return g->n_boundary; }
int64_t geometry_nfluid(const lbm_geometry* g) { return g->n_fluid; }
void geometry_dims(const lbm_geometry* g, int dims[3]) { dims[0] = g->grid.Nx; dims[1] = g->grid.Ny; dims[2] = g->grid.Nz; }
int geometry_device(const lbm_geometry* g) { return g->dev; }
const std::vector<int64_t>& geometry_list_sizes(const lbm_geometry* g) { return g->list_sizes; }
}  // namespace lbm
