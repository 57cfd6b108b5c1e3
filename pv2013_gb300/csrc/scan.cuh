// Order-preserving prefix sums and stream compaction (hand-written, three
// passes: per-tile totals, a single-block scan of the totals, per-tile
// rescan and write).  Used by the set-up kernels: boundary-point lists,
// node numbering, run-table construction.  Tiles are 256 threads x 16 items.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "internal.h"

namespace lbm {
namespace scan {

constexpr int kThreads = 256;
constexpr int kItems = 16;
constexpr int64_t kTile = (int64_t)kThreads * kItems;

__device__ __forceinline__ int64_t warp_incl_scan(int64_t v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int64_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// Exclusive block scan of one value per thread; returns the exclusive prefix
// and writes the block total to *total (all threads).
__device__ __forceinline__ int64_t block_excl_scan(int64_t v, int64_t* total) {
    __shared__ int64_t warp_sums[kThreads / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int64_t inc = warp_incl_scan(v);
    if (lane == 31) warp_sums[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        int64_t s = lane < kThreads / 32 ? warp_sums[lane] : 0;
        s = warp_incl_scan(s);
        if (lane < kThreads / 32) warp_sums[lane] = s;
    }
    __syncthreads();
    int64_t before = wid > 0 ? warp_sums[wid - 1] : 0;
    *total = warp_sums[kThreads / 32 - 1];
    __syncthreads();
    return before + inc - v;
}

template <class T>
__global__ void tile_totals(const T* __restrict__ in, int64_t n, int64_t* __restrict__ tile_sum, bool nonzero) {
    int64_t base = blockIdx.x * kTile + (int64_t)threadIdx.x * kItems;
    int64_t s = 0;
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
        int64_t idx = base + i;
        if (idx < n) s += nonzero ? (in[idx] != 0 ? 1 : 0) : (int64_t)in[idx];
    }
    int64_t tot;
    block_excl_scan(s, &tot);
    if (threadIdx.x == 0) tile_sum[blockIdx.x] = tot;
}

// Single block: exclusive scan of ntiles totals in place; grand total to *total.
static __global__ void scan_totals(int64_t* __restrict__ tile_sum, int64_t ntiles, int64_t* __restrict__ total) {
    int64_t per = (ntiles + kThreads - 1) / kThreads;
    int64_t b = threadIdx.x * per, e = min(ntiles, b + per);
    int64_t s = 0;
    for (int64_t i = b; i < e; ++i) s += tile_sum[i];
    int64_t tot;
    int64_t off = block_excl_scan(s, &tot);
    for (int64_t i = b; i < e; ++i) {
        int64_t v = tile_sum[i];
        tile_sum[i] = off;
        off += v;
    }
    if (threadIdx.x == 0) *total = tot;
}

// Exclusive scan of counts into out (int64).
template <class T>
__global__ void tile_scan_write(const T* __restrict__ in, int64_t n, const int64_t* __restrict__ tile_off,
                                int64_t* __restrict__ out) {
    int64_t base = blockIdx.x * kTile + (int64_t)threadIdx.x * kItems;
    int64_t v[kItems];
    int64_t s = 0;
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
        int64_t idx = base + i;
        v[i] = idx < n ? (int64_t)in[idx] : 0;
        s += v[i];
    }
    int64_t tot;
    int64_t off = block_excl_scan(s, &tot) + tile_off[blockIdx.x];
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
        int64_t idx = base + i;
        if (idx < n) out[idx] = off;
        off += v[i];
    }
}

// Writes the indices of nonzero entries, in order.
template <class T>
__global__ void tile_compact_write(const T* __restrict__ in, int64_t n, const int64_t* __restrict__ tile_off,
                                   int64_t* __restrict__ out) {
    int64_t base = blockIdx.x * kTile + (int64_t)threadIdx.x * kItems;
    uint32_t bits = 0;
    int64_t s = 0;
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
        int64_t idx = base + i;
        bool nz = idx < n && in[idx] != 0;
        bits |= (nz ? 1u : 0u) << i;
        s += nz ? 1 : 0;
    }
    int64_t tot;
    int64_t off = block_excl_scan(s, &tot) + tile_off[blockIdx.x];
#pragma unroll
    for (int i = 0; i < kItems; ++i)
        if (bits & (1u << i)) out[off++] = base + i;
}

// Workspace for one scan of n elements.
struct Workspace {
    int64_t* tiles = nullptr;
    int64_t* total = nullptr;
    int64_t ntiles = 0;
    cudaStream_t st = 0;
};

#define LBM_SCAN_TRY(x)                 \
    do {                                \
        lbm_status s_ = (x);            \
        if (s_ != LBM_OK) return s_;    \
    } while (0)

inline lbm_status ws_alloc(Workspace& w, int64_t n, cudaStream_t st) {
    w.ntiles = (n + kTile - 1) / kTile;
    if (w.ntiles < 1) w.ntiles = 1;
    LBM_SCAN_TRY(dev_alloc(reinterpret_cast<void**>(&w.tiles), sizeof(int64_t) * (w.ntiles + 1), st, "scan workspace"));
    w.total = w.tiles + w.ntiles;
    w.st = st;
    return LBM_OK;
}
inline void ws_free(Workspace& w) {
    if (w.tiles) dev_free(w.tiles, w.st);
    w.tiles = nullptr;
}

// Exclusive scan of n counts; *h_total receives the sum (synchronises stream).
template <class T>
lbm_status exclusive_scan(const T* d_in, int64_t n, int64_t* d_out, int64_t* h_total, cudaStream_t st) {
    Workspace w;
    lbm_status s = ws_alloc(w, n, st);
    if (s != LBM_OK) return s;
    tile_totals<T><<<(unsigned)w.ntiles, kThreads, 0, st>>>(d_in, n, w.tiles, false);
    scan_totals<<<1, kThreads, 0, st>>>(w.tiles, w.ntiles, w.total);
    tile_scan_write<T><<<(unsigned)w.ntiles, kThreads, 0, st>>>(d_in, n, w.tiles, d_out);
    cudaError_t e = cudaMemcpyAsync(h_total, w.total, sizeof(int64_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    ws_free(w);
    if (e != cudaSuccess) return fail(LBM_ERR_CUDA, "exclusive_scan: %s", cudaGetErrorString(e));
    return LBM_OK;
}

// Counts nonzero entries (synchronises).
template <class T>
lbm_status count_nonzero(const T* d_in, int64_t n, int64_t* h_count, cudaStream_t st) {
    Workspace w;
    lbm_status s = ws_alloc(w, n, st);
    if (s != LBM_OK) return s;
    tile_totals<T><<<(unsigned)w.ntiles, kThreads, 0, st>>>(d_in, n, w.tiles, true);
    scan_totals<<<1, kThreads, 0, st>>>(w.tiles, w.ntiles, w.total);
    cudaError_t e = cudaMemcpyAsync(h_count, w.total, sizeof(int64_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    ws_free(w);
    if (e != cudaSuccess) return fail(LBM_ERR_CUDA, "count_nonzero: %s", cudaGetErrorString(e));
    return LBM_OK;
}

// Ordered indices of nonzero entries into *d_out (allocated here from the
// stream-ordered pool on st, count in *h_count).
template <class T>
lbm_status compact(const T* d_in, int64_t n, int64_t** d_out, int64_t* h_count, cudaStream_t st) {
    Workspace w;
    lbm_status s = ws_alloc(w, n, st);
    if (s != LBM_OK) return s;
    tile_totals<T><<<(unsigned)w.ntiles, kThreads, 0, st>>>(d_in, n, w.tiles, true);
    scan_totals<<<1, kThreads, 0, st>>>(w.tiles, w.ntiles, w.total);
    cudaError_t e = cudaMemcpyAsync(h_count, w.total, sizeof(int64_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) { ws_free(w); return fail(LBM_ERR_CUDA, "compact: %s", cudaGetErrorString(e)); }
    s = dev_alloc(reinterpret_cast<void**>(d_out), sizeof(int64_t) * (*h_count > 0 ? *h_count : 1), st, "compacted indices");
    if (s != LBM_OK) { ws_free(w); return s; }
    tile_compact_write<T><<<(unsigned)w.ntiles, kThreads, 0, st>>>(d_in, n, w.tiles, *d_out);
    e = cudaStreamSynchronize(st);
    ws_free(w);
    if (e != cudaSuccess) return fail(LBM_ERR_CUDA, "compact: %s", cudaGetErrorString(e));
    return LBM_OK;
}

}  // namespace scan
}  // namespace lbm
