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
// changes.  Waits on an mbarrier are bounded: after kSpinLimit polls (or
// a.spin_limit non-blocking tests, when set) the warp records an error (bit 0 of *err, read back by
// the host as LBM_ERR_TIMEOUT), drains the stages still in flight with waits
// bounded by kSpinLimit each, and stops.  A drain that gives up too sets bit 1:
// that only follows a stall of the copy hardware itself, and the warp may then
// exit with bulk copies still writing into its shared memory.  For failure
// tests (a.stall_first) each warp leaves its first stage unissued -- no copy,
// no arrival -- so that stage's wait cannot complete: the warp gives up, and
// its drain skips that stage (nothing is in flight there).
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
    static constexpr int DESC = 0;          // 64 B chunk descriptor
    static constexpr int BAR = 64;          // 8 B mbarrier
    static constexpr int DATA = 80;         // Q slots
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

// non-blocking test of a phase (try_wait may suspend the thread for a while)
__device__ __forceinline__ bool mbar_test_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
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

// Source of population q: column (0..7 = col8, 8 = own), level offset + 1
// (0..2) and the plane read.  Packed per lane: bits 0-3 column, 4-5 offset,
// 6-10 plane.
template <int Q, int RA, int MODE>
__host__ __device__ constexpr uint32_t src_code(int q) {
    using X = Ax<Q, RA>;
    if (MODE == MODE_AA_EVEN) return 8u | (1u << 4) | ((uint32_t)q << 6);
    const int col = (X::a(q) == 0 && X::b(q) == 0) ? 8 : col8(-X::a(q), -X::b(q));
    const int plane = MODE == MODE_AA_ODD ? Lat<Q>::opp(q) : q;
    return (uint32_t)col | ((uint32_t)(1 - X::r(q)) << 4) | ((uint32_t)plane << 6);
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

    uint32_t code = 0;
#pragma unroll
    for (int q = 0; q < Q; ++q)
        if (lane == q) code = src_code<Q, RA, MODE>(q);
    const int my_col = (int)(code & 15u), my_o = (int)((code >> 4) & 3u) - 1, my_plane = (int)(code >> 6);

    // Stage chunk (descriptor word `dw` of this lane, lanes 0..15) into stage s.
    auto issue = [&](int s, uint32_t dw) {
        unsigned char* stg = ring + s * LY::BYTES;
        if (lane < 16) ((uint32_t*)(stg + LY::DESC))[lane] = dw;
        const int32_t n0 = (int32_t)__shfl_sync(0xffffffffu, dw, 0);
        const int len = (int)(__shfl_sync(0xffffffffu, dw, 1) & 63u);
        const int32_t kc = (int32_t)__shfl_sync(0xffffffffu, dw, 7 + (my_col & 7));
        const int32_t start = (my_col == 8 ? n0 - 1 : kc) + 1 + my_o;
        const int32_t as = start & ~(SL::EPG - 1);
        const int32_t ae = (start + len + SL::EPG - 1) & ~(SL::EPG - 1);
        const uint32_t mine = lane < Q ? (uint32_t)(ae - as) * SL::EB : 0u;
        const uint32_t total = __reduce_add_sync(0xffffffffu, mine);
        const uint32_t bar = smem_addr(stg + LY::BAR);
        if (lane == 0) mbar_expect_tx(bar, total);
        __syncwarp();
        if (mine)
            bulk_g2s(smem_addr(stg + LY::DATA + lane * SL::BYTES), gsrc + ((int64_t)my_plane * a.stride + as) * SL::EB,
                     mine, bar);
    };
    auto chunk_of = [&](int64_t k) { return gw + k * G; };
    auto load_desc = [&](int64_t k) -> uint32_t {
        const int64_t c = chunk_of(k);
        return (c < a.nchunks && lane < 16) ? __ldg(words + c * 16 + lane) : 0u;
    };

    uint32_t dw = load_desc(0);
    for (int k = 0; k < kStages - 1; ++k) {
        if (chunk_of(k) < a.nchunks && !(k == 0 && a.stall_first)) issue(k, dw);
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
            if (a.spin_limit) {
                while (!mbar_test_wait(bar, ph))
                    if (++spins >= a.spin_limit) { ok = false; break; }
            } else {
                while (!mbar_try_wait(bar, ph))
                    if (++spins >= kSpinLimit) { ok = false; break; }
            }
            if (!ok) {
                // record the failure, then drain (bounded) every stage still in flight
                bool drained = true;
                for (int64_t j = k; j < k + kStages && chunk_of(j) < a.nchunks; ++j) {
                    if (j == 0 && a.stall_first) continue;      // never issued
                    const int sj = (int)(j % kStages);
                    const uint32_t bj = smem_addr(ring + sj * LY::BYTES + LY::BAR);
                    uint32_t t = 0;
                    while (!mbar_try_wait(bj, (parity >> sj) & 1u))
                        if (++t >= kSpinLimit) { drained = false; break; }
                    parity ^= 1u << sj;
                }
                if (lane == 0) atomicOr(err, drained ? 1 : 3);
                return;
            }
            parity ^= 1u << s;
        }
        const Chunk* cp = (const Chunk*)(stg + LY::DESC);
        const int32_t n0 = cp->n0;
        const uint32_t li = cp->len_inst;
        const int len = (int)(li & 63u);
        if (lane < len) {
            const uint32_t wmask = cp->wmask, zmask = cp->zmask, bmask = cp->bmask;
            int32_t K[8];
#pragma unroll
            for (int c = 0; c < 8; ++c) K[c] = cp->K[c];
            const int32_t n = n0 + lane;
            const uint32_t missing =
                ((bmask >> lane) & 1u) ? __ldg(a.mmask + cp->mslot0 + __popc(bmask & ((1u << lane) - 1u))) : 0u;
            const unsigned char* data = stg + LY::DATA;
            T f[Q];
#pragma unroll
            for (int q = 0; q < Q; ++q) {
                const bool ev = MODE == MODE_AA_EVEN;
                const int32_t st0 = ev ? n0 : nb_id(K, n0, 0, -X::a(q), -X::b(q), -X::r(q));
                const int r = (st0 & (SL::EPG - 1)) + lane;
                T v = T(0);
                if (ev || !((missing >> q) & 1u)) {
                    const unsigned char* slot = data + q * SL::BYTES;
                    if constexpr (S == ST_F64) v = ((const double*)slot)[r];
                    else if constexpr (S == ST_F32) v = ((const float*)slot)[r] - (float)L::w(q);
                    else if constexpr (S == ST_F16S) v = __half2float(((const __half*)slot)[r]);
                    else v = __bfloat162float(((const __nv_bfloat16*)slot)[r]);
                }
                f[q] = v;
            }
            double mon[5];
            node_update<Q, S, MODE, false>(a, cp->zslot0, f, missing, wmask, zmask, lane, n, (int)(li >> 8), step, mon);
            void* D = a.dst;
            if constexpr (MODE == MODE_AA_ODD) {
                // re-read the bases rather than hold them across the update
#pragma unroll
                for (int c = 0; c < 8; ++c) K[c] = ((const volatile int32_t*)cp->K)[c];
            }
#pragma unroll
            for (int q = 0; q < Q; ++q) {
                if constexpr (MODE == MODE_PULL) {
                    st<S, Q>(D, a.stride, q, n, f[q]);
                } else if constexpr (MODE == MODE_AA_EVEN) {
                    st<S, Q>(D, a.stride, L::opp(q), n, f[q]);
                } else {
                    const bool back = (missing >> L::opp(q)) & 1u;
                    const bool keep = !back || bounce_back_pop<Q>(L::opp(q), (wmask >> lane) & 1u, a.corr);
                    st_sel<S, Q>(D, (uint32_t)a.stride, q, nb_id(K, n0, lane, X::a(q), X::b(q), X::r(q)), back, n,
                                 keep ? f[q] : init_work<S, Q>(q));
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
