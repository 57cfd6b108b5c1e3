// Pipelined step kernel: TMA bulk copies stage each chunk's populations in
// shared memory several chunks ahead of the warp that processes them.
//
// Why: the direct-load kernel (step_kernel.cuh) is latency bound -- a warp can
// only keep its 19 (27) population loads in flight while it holds the values
// in registers, so HBM sees too few bytes in flight.  Here every warp owns an
// S-stage ring in shared memory; for chunk k+S-1 it issues one
// cp.async.bulk per population plane (the chunk's source range in that plane
// is contiguous: a run of node ids in one grid column) while it computes
// chunk k, so S-1 chunks of data are in flight per warp without registers.
//
// Per chunk and plane, the copied range is the column window's node range
// rounded out to 16-byte boundaries (TMA alignment); lanes index into it.
// Writes stay per-lane global stores (coalesced per plane): their ranges are
// not 16-byte aligned and neighbouring chunks write the bytes around them.
//
// Arithmetic, boundary handling and the streaming patterns are those of
// k_step (shared device functions); only the source of the gathered values
// changes.  Waits on an mbarrier are bounded: after kSpinLimit polls the warp
// records an error (read back by the host as LBM_ERR_TIMEOUT) and stops.
#pragma once
#include "step_kernel.cuh"

namespace lbm {

constexpr int kStages = 4;
constexpr uint32_t kSpinLimit = 1u << 22;

template <int S> struct Slot;          // bytes per staged plane range and elements per 16 B
template <> struct Slot<ST_F64> { static constexpr int EB = 8, EPG = 2, BYTES = 288; };
template <> struct Slot<ST_F32> { static constexpr int EB = 4, EPG = 4, BYTES = 160; };
template <> struct Slot<ST_F16S> { static constexpr int EB = 2, EPG = 8, BYTES = 96; };
template <> struct Slot<ST_BF16S> { static constexpr int EB = 2, EPG = 8, BYTES = 96; };

template <int Q, int S>
struct StageLayout {
    static constexpr int DESC = 0;          // 128 B chunk descriptor
    static constexpr int BAR = 128;         // 8 B mbarrier
    static constexpr int DATA = 144;        // Q slots
    static constexpr int BYTES = (DATA + Q * Slot<S>::BYTES + 15) / 16 * 16;
};

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile(
        "{\n\t.reg .b64 st;\n\t"
        "mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(bar),
        "r"(bytes)
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
        "l"(src), "r"(bytes), "r"(bar)
        : "memory");
}

// Column (0..7 = col8, 8 = own column) and plane read for population q.
template <int Q, int RA, int MODE>
__host__ __device__ constexpr int src_col(int q) {
    using X = Ax<Q, RA>;
    return (X::a(q) == 0 && X::b(q) == 0) || MODE == MODE_AA_EVEN ? 8 : col8(-X::a(q), -X::b(q));
}
template <int Q, int MODE>
__host__ __device__ constexpr int src_plane(int q) {
    return MODE == MODE_AA_ODD ? Lat<Q>::opp(q) : q;
}
// 4-bit (column) and 5-bit (plane) tables packed in 64-bit words, indexed by lane
template <int Q, int RA, int MODE>
__host__ __device__ constexpr uint64_t col_table(int half) {
    uint64_t t = 0;
    for (int q = 16 * half; q < Q && q < 16 * half + 16; ++q) t |= (uint64_t)src_col<Q, RA, MODE>(q) << (4 * (q - 16 * half));
    return t;
}
template <int Q, int MODE>
__host__ __device__ constexpr uint64_t plane_table(int part) {
    uint64_t t = 0;
    for (int q = 12 * part; q < Q && q < 12 * part + 12; ++q) t |= (uint64_t)src_plane<Q, MODE>(q) << (5 * (q - 12 * part));
    return t;
}

template <int Q, int S, int MODE, int RA>
__global__ void __launch_bounds__(256) k_step_tma(StepArgs a, int32_t* err) {
    using L = Lat<Q>;
    using X = Ax<Q, RA>;
    using T = typename Work<S>::T;
    using SL = Slot<S>;
    using LY = StageLayout<Q, S>;
    extern __shared__ __align__(128) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, W = blockDim.x >> 5;
    unsigned char* ring = smem + (size_t)warp * kStages * LY::BYTES;
    const int64_t G = (int64_t)gridDim.x * W;
    const int64_t gw = (int64_t)blockIdx.x * W + warp;
    const uint32_t* words = (const uint32_t*)a.chunks;
    const char* gsrc = (const char*)a.src;

    if (lane == 0) {
        for (int s = 0; s < kStages; ++s) mbar_init(smem_addr(ring + s * LY::BYTES + LY::BAR), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();

    constexpr uint64_t CT0 = col_table<Q, RA, MODE>(0), CT1 = col_table<Q, RA, MODE>(1);
    constexpr uint64_t PT0 = plane_table<Q, MODE>(0), PT1 = plane_table<Q, MODE>(1), PT2 = plane_table<Q, MODE>(2);
    const int my_col = lane < Q ? (int)(((lane < 16 ? CT0 : CT1) >> (4 * (lane & 15))) & 15u) : 8;
    const int my_plane = lane < Q ? (int)(((lane < 12 ? PT0 : (lane < 24 ? PT1 : PT2)) >> (5 * (lane % 12))) & 31u) : 0;

    // Stage chunk c (descriptor word of this lane in dw) into stage s.
    auto issue = [&](int s, uint32_t dw) {
        unsigned char* stg = ring + s * LY::BYTES;
        ((uint32_t*)(stg + LY::DESC))[lane] = dw;
        const uint32_t n0 = __shfl_sync(0xffffffffu, dw, 0);
        const uint32_t li = __shfl_sync(0xffffffffu, dw, 1);
        const int c = lane & 7;
        const uint32_t b = __shfl_sync(0xffffffffu, dw, 6 + c);
        const uint32_t mlo = __shfl_sync(0xffffffffu, dw, 14 + 2 * c);
        const uint32_t mhi = __shfl_sync(0xffffffffu, dw, 15 + 2 * c);
        int32_t start, cnt;
        if (lane == 8) {
            const int e0 = (li >> 6) & 1, e1 = (li >> 7) & 1;
            start = (int32_t)n0 - e0;
            cnt = (int32_t)(li & 63u) + e0 + e1;
        } else {
            start = (int32_t)b;
            cnt = __popc(mlo) + __popc(mhi);
        }
        const int32_t as = start & ~(SL::EPG - 1);
        const int32_t ae = (start + cnt + SL::EPG - 1) & ~(SL::EPG - 1);
        const uint32_t bytes = cnt > 0 ? (uint32_t)(ae - as) * SL::EB : 0u;
        const int32_t q_as = __shfl_sync(0xffffffffu, as, my_col);
        const uint32_t q_bytes = __shfl_sync(0xffffffffu, bytes, my_col);
        const uint32_t mine = lane < Q ? q_bytes : 0u;
        const uint32_t total = __reduce_add_sync(0xffffffffu, mine);
        const uint32_t bar = smem_addr(stg + LY::BAR);
        if (lane == 0) mbar_expect_tx(bar, total);
        __syncwarp();
        if (mine) {
            bulk_g2s(smem_addr(stg + LY::DATA + lane * SL::BYTES),
                     gsrc + ((int64_t)my_plane * a.stride + q_as) * SL::EB, mine, bar);
        }
    };
    auto chunk_of = [&](int64_t k) { return gw + k * G; };
    auto load_desc = [&](int64_t k) -> uint32_t {
        const int64_t c = chunk_of(k);
        return c < a.nchunks ? __ldg(words + c * 32 + lane) : 0u;
    };

    uint32_t dw = load_desc(0);
    for (int k = 0; k < kStages - 1; ++k) {
        if (chunk_of(k) < a.nchunks) issue(k, dw);
        dw = load_desc(k + 1);
    }
    uint32_t parity = 0;   // bit s: phase parity of stage s
    const int64_t step = a.step + (a.step_base ? *a.step_base : 0);
    for (int64_t k = 0; chunk_of(k) < a.nchunks; ++k) {
        const int s = (int)(k % kStages);
        if (chunk_of(k + kStages - 1) < a.nchunks) issue((int)((k + kStages - 1) % kStages), dw);
        const uint32_t dw_next = load_desc(k + kStages);
        unsigned char* stg = ring + s * LY::BYTES;
        {
            const uint32_t bar = smem_addr(stg + LY::BAR);
            const uint32_t ph = (parity >> s) & 1u;
            uint32_t spins = 0;
            bool ok = true;
            while (!mbar_try_wait(bar, ph)) {
                if (++spins > kSpinLimit) { ok = false; break; }
            }
            if (!ok) {
                // record the failure, then drain (bounded) every stage still in flight
                if (lane == 0) atomicOr(err, 1);
                for (int64_t j = k; j < k + kStages && chunk_of(j) < a.nchunks; ++j) {
                    const int sj = (int)(j % kStages);
                    const uint32_t bj = smem_addr(ring + sj * LY::BYTES + LY::BAR);
                    for (uint32_t t = 0; t < kSpinLimit && !mbar_try_wait(bj, (parity >> sj) & 1u); ++t) {
                    }
                    parity ^= 1u << sj;
                }
                return;
            }
            parity ^= 1u << s;
        }
        const uint32_t* dsc = (const uint32_t*)(stg + LY::DESC);
        const Chunk* cp = (const Chunk*)dsc;
        const int32_t n0 = cp->n0;
        const uint32_t li = cp->len_inst;
        const int len = (int)(li & 63u);
        if (lane < len) {
            const uint32_t wmask = cp->wmask, zmask = cp->zmask, bmask = cp->bmask;
            const int inst = (int)(li >> 8);
            const int32_t n = n0 + lane;
            const bool isb = (bmask >> lane) & 1u;
            const uint32_t e0 = (li >> 6) & 1u;
            // per-lane table relative to each staged range
            int32_t pb[8], rb[8];
            uint32_t bits[8];
            const uint64_t lm = (2ull << lane) - 1ull;
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                const uint64_t m = cp->mask[c];
                const int32_t b = cp->base[c];
                bits[c] = (uint32_t)(m >> lane) & 7u;
                pb[c] = b + __popcll(m & lm);
                rb[c] = pb[c] - (b & ~(SL::EPG - 1));
            }
            const int32_t own_as = ((int32_t)n0 - (int32_t)e0) & ~(SL::EPG - 1);
            const uint32_t own = ((lane > 0 || e0) ? 1u : 0u) | 2u | ((lane < len - 1 || ((li >> 7) & 1u)) ? 4u : 0u);
            const unsigned char* data = stg + LY::DATA;
            T f[Q];
            uint32_t missing = 0;
#pragma unroll
            for (int q = 0; q < Q; ++q) {
                const int da = MODE == MODE_AA_EVEN ? 0 : -X::a(q), db = MODE == MODE_AA_EVEN ? 0 : -X::b(q);
                const int o = MODE == MODE_AA_EVEN ? 0 : -X::r(q);
                bool has;
                int32_t g, r;
                if (da == 0 && db == 0) {
                    has = (own >> (1 + o)) & 1u;
                    g = n + o;
                    r = g - own_as;
                } else {
                    nbr(pb, bits, own, n, da, db, o, has, g);
                    r = rb[col8(da, db)] + (g - pb[col8(da, db)]);
                }
                if (MODE == MODE_AA_EVEN && isb) {   // a missing source still matters for the fix-ups
                    bool h2;
                    int32_t g2;
                    nbr(pb, bits, own, n, -X::a(q), -X::b(q), -X::r(q), h2, g2);
                    if (!h2) missing |= 1u << q;
                } else if (!has) {
                    missing |= 1u << q;
                }
                T v = T(0);
                if (has) {
                    const unsigned char* slot = data + q * SL::BYTES;
                    if constexpr (S == ST_F64) v = ((const double*)slot)[r];
                    else if constexpr (S == ST_F32) v = ((const float*)slot)[r] - (float)L::w(q);
                    else if constexpr (S == ST_F16S) v = __half2float(((const __half*)slot)[r]);
                    else v = __bfloat162float(((const __nv_bfloat16*)slot)[r]);
                }
                f[q] = v;
            }
            const void* A = a.src;
            if (missing) {
                const bool wall = (wmask >> lane) & 1u;
#pragma unroll
                for (int q = 0; q < Q; ++q) {
                    if (!((missing >> q) & 1u)) continue;
                    if (wall && q != L::NO_BB_POP) {
                        if constexpr (MODE == MODE_PULL) f[q] = ld<S, Q, true>(A, a.stride, L::opp(q), n);
                        else if constexpr (MODE == MODE_AA_ODD) f[q] = ld<S, Q>(A, a.stride, q, n);
                    } else {
                        f[q] = S == ST_F64 ? T(L::w(q)) : T(0);
                    }
                }
            }
            if (((zmask >> lane) & 1u) && step > 0) {
                const int slot = cp->zslot0 + __popc(zmask & ((1u << lane) - 1u));
                const ZSlot z = a.zslots[slot];
                const ListParam lp = a.lists[z.list];
                T p[Q];
#pragma unroll
                for (int q = 0; q < Q; ++q) p[q] = plain<S, Q>(f[q], q);
                if (z.kind == LBM_BC_VEL_NEGY || z.kind == LBM_BC_VEL_POSX) {
                    const double amp = a.amp[lp.amp_off + (step - 1) % lp.amp_len];
                    const double sc = amp * z.profile;
                    const T v[3] = {T(sc * lp.dir[0]), T(sc * lp.dir[1]), T(sc * lp.dir[2])};
                    if constexpr (Q == 19) {
                        if (z.kind == LBM_BC_VEL_NEGY) zh_vel_negy<T>(p, v);
                    } else {
                        if (z.kind == LBM_BC_VEL_POSX) zh_vel_posx_q27<T>(p, v);
                    }
                } else {
                    if constexpr (Q == 19) zh_press<T>(p, z.kind, T(lp.rho));
                }
#pragma unroll
                for (int q = 0; q < Q; ++q) f[q] = unplain<S, Q>(p[q], q);
            }
            collide<Q, S>(f, a.insts[inst]);
            void* D = a.dst;
#pragma unroll
            for (int q = 0; q < Q; ++q) {
                if constexpr (MODE == MODE_PULL) {
                    st<S, Q>(D, a.stride, q, n, f[q]);
                } else if constexpr (MODE == MODE_AA_EVEN) {
                    st<S, Q>(D, a.stride, L::opp(q), n, f[q]);
                } else {
                    bool has;
                    int32_t d;
                    nbr(pb, bits, own, n, X::a(q), X::b(q), X::r(q), has, d);
                    if (has) st<S, Q>(D, a.stride, q, d, f[q]);
                    else st<S, Q>(D, a.stride, L::opp(q), n, f[q]);
                }
            }
        }
        // order this stage's generic reads before the async-proxy writes that refill it
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncwarp();
        dw = dw_next;
    }
}

}  // namespace lbm
