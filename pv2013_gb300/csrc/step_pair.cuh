// Paired step kernel: two adjacent nodes per lane, 4, 8 or 16 lanes per chunk
// piece.
//
// Same operations and streaming patterns as k_step (step_kernel.cuh), for the
// FP32 and 16-bit storages; what changes is how a lane covers its nodes:
//   * lane t of a piece's lane group owns the nodes at levels r0+2t and
//     r0+2t+1 of its chunk (a pair).  The lattice numbers every node so that
//     its id has the parity of its level (sim.cu), so a pair is one aligned
//     32-bit (16-bit storage) or 64-bit (FP32 storage) word in each
//     population plane;
//   * a neighbour pair one level up or down straddles two aligned words: the
//     lane loads both and takes the high half of one and the low half of the
//     other (a byte permute, no shuffle);
//   * the collision runs on packed FP32 pairs (add/sub/mul/fma.rn.f32x2), one
//     instruction for both nodes;
//   * boundary fix-ups and Zou-He run per node, only in warps that have them.
//     The AA even launch has no fix-ups: the odd launch before it left the
//     bounced or initial values in the node's own slots (step_kernel.cuh).
//     The AA odd launch's bounce-back source is the node's own word: boundary
//     lanes copy their own words into shared memory (cp.async) while the
//     gathers are in flight, so the fix-up waits on no further load; the
//     fix-up widens each population's two node flags to half-word masks
//     with one byte permute.  The AA odd launch runs on a piece table in
//     which interior pieces come first within every 16-warp window
//     (k_group_pieces, sim.cu), so most warps take no boundary branch.
//   * descriptors: the AA even launch reads an 8-byte record per piece
//     (n0, length and instance, a Zou-He flag; k_even_desc, sim.cu) and L2-
//     prefetches the population windows of the piece half a wave ahead; the
//     other launches read the 64-byte descriptor, the AA odd launch
//     prefetching only the descriptor one wave ahead.
// Chunk pieces start at even levels and hold up to 8, 16 or 32 node slots
// (lbm_sim_params.piece_slots: shorter pieces leave fewer idle lanes where a
// run ends, for more descriptor bytes per node); a slot at either end may be a
// ghost node (not in the piece's vmask): its values are computed and
// discarded, and in the AA odd pattern it stores nothing.
#pragma once
#include "step.h"
#include "step_kernel.cuh"

namespace lbm {

// ---------------------------------------------------------------------------
// packed FP32 pair: node of the lower level in .lo, upper level in .hi
struct F2 {
    unsigned long long v;
};
__device__ __forceinline__ F2 f2(float lo, float hi) {
    F2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ F2 f2s(float a) { return f2(a, a); }
__device__ __forceinline__ void f2split(F2 a, float& lo, float& hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(a.v));
}
__device__ __forceinline__ F2 operator+(F2 a, F2 b) {
    F2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
__device__ __forceinline__ F2 operator-(F2 a, F2 b) {
    F2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
__device__ __forceinline__ F2 operator*(F2 a, F2 b) {
    F2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
__device__ __forceinline__ F2 fma2(F2 a, F2 b, F2 c) {
    F2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.v) : "l"(a.v), "l"(b.v), "l"(c.v));
    return r;
}

// ---------------------------------------------------------------------------
// storage word of a pair and its conversion to / from working values
template <int S> struct PairWord;
template <> struct PairWord<ST_F32> { using W = uint2; };
template <> struct PairWord<ST_F16S> { using W = uint32_t; };
template <> struct PairWord<ST_BF16S> { using W = uint32_t; };

template <int S> constexpr int elem_bytes() { return S == ST_F32 ? 4 : 2; }

// pair word wo of the population array: elements 2 wo and 2 wo + 1.  Plane
// strides and pair ids are even, so word offsets (plane * stride/2 + id/2)
// are formed directly in 32-bit registers from one base pointer
template <int S>
__device__ __forceinline__ typename PairWord<S>::W ldw(const void* base, uint32_t wo) {
    return reinterpret_cast<const typename PairWord<S>::W*>(base)[wo];
}
// high element of word a, low element of word b (a pair one level out of phase)
template <int S>
__device__ __forceinline__ typename PairWord<S>::W straddle(typename PairWord<S>::W a, typename PairWord<S>::W b) {
    if constexpr (S == ST_F32) return make_uint2(a.y, b.x);
    else return __byte_perm(a, b, 0x5432);
}
template <int S, int Q>
__device__ __forceinline__ F2 unpack(typename PairWord<S>::W w, int q) {
    if constexpr (S == ST_F32) {
        const float wq = (float)Lat<Q>::w(q);
        return f2(__uint_as_float(w.x), __uint_as_float(w.y)) - f2s(wq);
    } else if constexpr (S == ST_F16S) {
        const float2 v = __half22float2(*reinterpret_cast<const __half2*>(&w));
        return f2(v.x, v.y);
    } else {
        return f2(__uint_as_float(w << 16), __uint_as_float(w & 0xffff0000u));
    }
}
template <int S, int Q>
__device__ __forceinline__ typename PairWord<S>::W pack(F2 v, int q) {
    if constexpr (S == ST_F32) {
        float lo, hi;
        f2split(v + f2s((float)Lat<Q>::w(q)), lo, hi);
        return make_uint2(__float_as_uint(lo), __float_as_uint(hi));
    } else if constexpr (S == ST_F16S) {
        float lo, hi;
        f2split(v, lo, hi);
        const __half2 h = __floats2half2_rn(lo, hi);
        return *reinterpret_cast<const uint32_t*>(&h);
    } else {
        float lo, hi;
        f2split(v, lo, hi);
        const __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
        return *reinterpret_cast<const uint32_t*>(&h);
    }
}
template <int S>
__device__ __forceinline__ void stw(void* base, uint32_t wo, typename PairWord<S>::W w) {
    reinterpret_cast<typename PairWord<S>::W*>(base)[wo] = w;
}
// one element (one node) of a plane
template <int S, int Q>
__device__ __forceinline__ void st_one(void* base, uint32_t off, float v, int q) {
    if constexpr (S == ST_F32) reinterpret_cast<float*>(base)[off] = v + (float)Lat<Q>::w(q);
    else if constexpr (S == ST_F16S) reinterpret_cast<__half*>(base)[off] = __float2half_rn(v);
    else reinterpret_cast<__nv_bfloat16*>(base)[off] = __float2bfloat16_rn(v);
}

// ---------------------------------------------------------------------------
// one node (half) of a storage word
template <int S>
__device__ __forceinline__ typename PairWord<S>::W take_half(typename PairWord<S>::W w, bool hi,
                                                           typename PairWord<S>::W src) {
    if constexpr (S == ST_F32) {
        if (hi) w.y = src.y; else w.x = src.x;
        return w;
    } else {
        const uint32_t m = hi ? 0xffff0000u : 0x0000ffffu;
        return (w & ~m) | (src & m);
    }
}
// the value a population keeps when the reference never writes it: w_q
// (stored unshifted for FP32, as 0 for the shifted formats)
template <int S, int Q>
__device__ __forceinline__ typename PairWord<S>::W init_half(typename PairWord<S>::W w, bool hi, int q) {
    if constexpr (S == ST_F32) {
        const uint32_t b = __float_as_uint((float)Lat<Q>::w(q));
        if (hi) w.y = b; else w.x = b;
        return w;
    } else {
        return w & (hi ? 0x0000ffffu : 0xffff0000u);
    }
}
template <int S, int Q>
__device__ __forceinline__ float half_plain(typename PairWord<S>::W w, bool hi, int q) {
    float l, h;
    f2split(unpack<S, Q>(w, q), l, h);
    return plain<S, Q>(hi ? h : l, q);
}
template <int S, int Q>
__device__ __forceinline__ typename PairWord<S>::W set_half_plain(typename PairWord<S>::W w, bool hi, float p, int q) {
    const float v = unplain<S, Q>(p, q);
    if constexpr (S == ST_F32) {
        const uint32_t b = __float_as_uint(v + (float)Lat<Q>::w(q));
        if (hi) w.y = b; else w.x = b;
        return w;
    } else {
        uint32_t b;
        if constexpr (S == ST_F16S) b = __half_as_ushort(__float2half_rn(v));
        else b = __bfloat16_as_ushort(__float2bfloat16_rn(v));
        return hi ? ((w & 0x0000ffffu) | (b << 16)) : ((w & 0xffff0000u) | b);
    }
}

// Zou-He on one node (half) of the pair words, in FP32 on plain populations;
// the results are rounded to the storage format before the collision.
// raw[q * 32] holds population q's word (a warp's words interleaved in
// shared memory, so the rest of the pair's words need no registers here)
template <int Q, int S>
__device__ __forceinline__ void zou_he_half(const StepArgs& a, int slot, typename PairWord<S>::W* raw, bool hi,
                                            int64_t step) {
    using T = float;
    const ZSlot z = a.zslots[slot];
    const ListParam lp = a.lists[z.list];
    T p[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) p[q] = half_plain<S, Q>(raw[q * 32], hi, q);
    T v[3] = {T(0), T(0), T(0)};
    if (is_velocity_kind(z.kind)) {
        // 32-bit phase: the step count stays below 2^32 (lbm_sim_step checks)
        const double amp = a.amp[lp.amp_off + (uint32_t)(step - 1) % (uint32_t)lp.amp_len];
        const double sc = amp * z.profile;
        v[0] = T(sc * lp.dir[0]); v[1] = T(sc * lp.dir[1]); v[2] = T(sc * lp.dir[2]);
    }
    zou_he_apply<Q, T>(p, z.kind, lp.face, v, T(lp.rho));
#pragma unroll
    for (int q = 0; q < Q; ++q) raw[q * 32] = set_half_plain<S, Q>(raw[q * 32], hi, p[q], q);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// 0x0000ffff where bit 15 of f is set, | 0xffff0000 where bit 31 is set:
// prmt with the sign-replicate selector bit (bytes 0-1 from the sign of byte
// 1, bytes 2-3 from the sign of byte 3)
__device__ __forceinline__ uint32_t half_masks(uint32_t f) {
    uint32_t r;
    asm("prmt.b32 %0, %1, 0, 0xBB99;" : "=r"(r) : "r"(f));
    return r;
}

// identity the compiler cannot see through: the relaxation unpacks the words
// again instead of keeping the first unpacked values alive
__device__ __forceinline__ uint32_t opaque(uint32_t x) {
    asm volatile("mov.b32 %0, %0;" : "+r"(x));
    return x;
}
__device__ __forceinline__ uint2 opaque(uint2 x) {
    asm volatile("mov.b32 %0, %0;" : "+r"(x.x));
    asm volatile("mov.b32 %0, %0;" : "+r"(x.y));
    return x;
}

// ---------------------------------------------------------------------------
// BGK collision on packed pairs (the FP32 branch of collide(), each operation
// on both nodes at once).  The populations stay in storage words and are
// unpacked twice -- for the moments, then for the relaxation -- so that only
// one word per population is live; emit(q, value) stores each result.
template <int Q, int S, class Emit>
__device__ __forceinline__ void collide2(const typename PairWord<S>::W* raw, float om_f, Emit emit) {
    using L = Lat<Q>;
    constexpr float K = Work<S>::K;
    F2 drho, px, nx, py, ny, pz, nz;
    bool hpx = false, hnx = false, hpy = false, hny = false, hpz = false, hnz = false;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const F2 v = unpack<S, Q>(raw[q], q);
        drho = q == 0 ? v : drho + v;
        if (L::cx(q) > 0) { px = hpx ? px + v : v; hpx = true; }
        if (L::cx(q) < 0) { nx = hnx ? nx + v : v; hnx = true; }
        if (L::cy(q) > 0) { py = hpy ? py + v : v; hpy = true; }
        if (L::cy(q) < 0) { ny = hny ? ny + v : v; hny = true; }
        if (L::cz(q) > 0) { pz = hpz ? pz + v : v; hpz = true; }
        if (L::cz(q) < 0) { nz = hnz ? nz + v : v; hnz = true; }
    }
    const F2 Krho = drho + f2s(K);
    float k0, k1;
    f2split(Krho, k0, k1);
    const F2 inv = f2(__fdividef(1.0f, k0), __fdividef(1.0f, k1));
    const F2 ux = (px - nx) * inv, uy = (py - ny) * inv, uz = (pz - nz) * inv;
    const F2 usq = fma2(uz, uz, fma2(uy, uy, ux * ux));
    const F2 base = fma2(Krho, usq * f2s(-1.5f), drho);   // K (rho - 1) - 1.5 K rho u^2
    const F2 Krho45 = Krho * f2s(4.5f);
    const F2 om = f2s(om_f);
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const int o = L::opp(q);
        const float w = (float)L::w(q);
        if (o == q) {
            const F2 v = unpack<S, Q>(opaque(raw[q]), q);
            emit(q, fma2(om, base * f2s(w) - v, v));
        } else if (q < o) {
            F2 cu;
            bool have = false;
            if (L::cx(q)) { cu = L::cx(q) > 0 ? ux : f2s(0.f) - ux; have = true; }
            if (L::cy(q)) { cu = have ? (L::cy(q) > 0 ? cu + uy : cu - uy) : (L::cy(q) > 0 ? uy : f2s(0.f) - uy); have = true; }
            if (L::cz(q)) { cu = have ? (L::cz(q) > 0 ? cu + uz : cu - uz) : (L::cz(q) > 0 ? uz : f2s(0.f) - uz); have = true; }
            const F2 sym = fma2(Krho45, cu * cu, base) * f2s(w);
            const F2 anti = (Krho * f2s(3.0f * w)) * cu;
            const F2 vq = unpack<S, Q>(opaque(raw[q]), q), vo = unpack<S, Q>(opaque(raw[o]), o);
            emit(q, fma2(om, (sym + anti) - vq, vq));
            emit(o, fma2(om, (sym - anti) - vo, vo));
        }
    }
}

// register budget per thread: D3Q19 with 16-bit storage holds one 32-bit
// word per population; 64 registers for the node-local and pull patterns, 72
// for the AA odd pattern (its scatter needs a few more; 72 keeps 28 warps per
// SM); FP32 storage (two registers per word) and D3Q27 get 128.
template <int Q, int S, int MODE> struct PairMaxReg {
    static constexpr int value = (Q == 19 && S != ST_F32) ? (MODE == MODE_AA_ODD ? 72 : 64) : 128;
};

template <int Q, int S, int MODE, int RA>
__global__ void __launch_bounds__(256) __maxnreg__((PairMaxReg<Q, S, MODE>::value)) k_step2(StepArgs a) {
    using L = Lat<Q>;
    using X = Ax<Q, RA>;
    using W = typename PairWord<S>::W;
    const int lane = threadIdx.x & 31;
    // a chunk piece is served by 2^lg lanes (4, 8 or 16): 32 >> lg pieces per warp
    const int lg = a.piece_lg;
    const int t = lane & ((1 << lg) - 1);         // pair index within the chunk
    const int pw = lane >> lg;                    // piece of this lane within the warp
    const int64_t ci = (((int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) << (5 - lg)) + pw;
    const bool have_chunk = ci < a.nchunks;
    // chunk descriptor words 0-7 (n0, len_inst, wmask, zmask, bmask, zslot0, mslot0, K0);
    // the AA even launch reads the 8-byte record (n0, len_inst) instead and
    // the descriptor's zmask only for pieces with a Zou-He lane
    const uint4* cw = reinterpret_cast<const uint4*>(a.chunks + (have_chunk ? ci : 0));
    uint4 d0;
    if constexpr (MODE == MODE_AA_EVEN) {
        const uint2 de = have_chunk ? __ldg(a.even_desc + ci) : make_uint2(0u, 0u);
        d0 = make_uint4(de.x, de.y, 0u, 0u);
    } else {
        d0 = have_chunk ? __ldg(cw) : make_uint4(0u, 0u, 0u, 0u);
    }
    // start id of the piece half a wave of resident warps ahead: its
    // population windows are prefetched into L2 below (the load is in flight
    // with d0)
    const int64_t cfp = ci + a.pf_ahead;
    const bool hfp = MODE != MODE_AA_ODD && a.pf_ahead > 0 && cfp < a.nchunks;   // (the odd launch: none)
    uint32_t nfp = 0;
    if (hfp) {
        if constexpr (MODE == MODE_AA_EVEN)
            asm volatile("ld.global.nc.u32 %0, [%1];" : "=r"(nfp) : "l"(&a.even_desc[cfp].x));
        else
            asm volatile("ld.global.nc.u32 %0, [%1];" : "=r"(nfp) : "l"(&a.chunks[cfp].n0));
    }
    const uint4 d1 = have_chunk && MODE != MODE_AA_EVEN ? __ldg(cw + 1) : make_uint4(0u, 0u, 0u, 0u);
    const int32_t n0 = (int32_t)d0.x;
    const uint32_t li = d0.y;
    const bool act = have_chunk && 2 * t < (int)(li & 63u);
    // node slots 2t (lo) and 2t+1 (hi) of the chunk
    const uint32_t bm_all = act ? d1.x : 0u;
    uint32_t zm_all = act ? d0.w : 0u;
    if (MODE == MODE_AA_EVEN && act && (li & 64u))
        asm volatile("ld.global.nc.u32 %0, [%1];" : "=r"(zm_all) : "l"(&cw[0].w));   // zmask
    uint32_t m_lo = 0u, m_hi = 0u;
    if (MODE != MODE_AA_EVEN && ((bm_all >> (2 * t)) & 3u)) {
        const int32_t ms = (int32_t)d1.z + __popc(bm_all & ((1u << (2 * t)) - 1u));
        if ((bm_all >> (2 * t)) & 1u) m_lo = __ldg(a.mmask + ms);
        if ((bm_all >> (2 * t + 1)) & 1u) m_hi = __ldg(a.mmask + ms + ((bm_all >> (2 * t)) & 1u));
    }
    const uint32_t e = (uint32_t)(n0 + 2 * t);     // id of the lo node (even)
    const uint32_t st = (uint32_t)a.stride;
    const uint32_t sw = st >> 1, ew = (uint32_t)(n0 >> 1) + (uint32_t)t;   // word offsets: plane stride, the pair's word
    const int64_t step = a.step + (a.step_base ? *a.step_base : 0);
    const void* A = a.src;

    // column bases (virtual id of level r0-1) of the eight neighbour columns
    auto load_K = [&](int32_t* K, bool fresh) {
        uint4 k1, k2;
        uint32_t k0;
        if (fresh) {
            asm volatile("ld.global.nc.u32 %0, [%1];" : "=r"(k0) : "l"(&cw[1].w));
            asm volatile("ld.global.nc.v4.u32 {%0, %1, %2, %3}, [%4];"
                         : "=r"(k1.x), "=r"(k1.y), "=r"(k1.z), "=r"(k1.w) : "l"(cw + 2));
            asm volatile("ld.global.nc.v4.u32 {%0, %1, %2, %3}, [%4];"
                         : "=r"(k2.x), "=r"(k2.y), "=r"(k2.z), "=r"(k2.w) : "l"(cw + 3));
        } else {
            k0 = d1.w;
            k1 = __ldg(cw + 2);
            k2 = __ldg(cw + 3);
        }
        K[0] = (int32_t)k0; K[1] = (int32_t)k1.x; K[2] = (int32_t)k1.y; K[3] = (int32_t)k1.z;
        K[4] = (int32_t)k1.w; K[5] = (int32_t)k2.x; K[6] = (int32_t)k2.y; K[7] = (int32_t)k2.z;
    };

    W raw[Q];
    // dynamic shared memory: per warp one word per population and lane (the
    // AA odd launch's bounce-back sources, then the Zou-He path's staging);
    // after all warps' words, the AA odd launch's column bases (8 per piece,
    // at most 8 pieces per warp)
    extern __shared__ __align__(16) unsigned char zsm[];
    W* buf = (W*)zsm + (threadIdx.x >> 5) * (Q * 32) + lane;
    int32_t* ksm = reinterpret_cast<int32_t*>((W*)zsm + (blockDim.x >> 5) * (Q * 32)) + (threadIdx.x >> 5) * 64;
    if (act) {
        int32_t K[8];
        if constexpr (MODE != MODE_AA_EVEN) load_K(K, false);
        if constexpr (MODE == MODE_AA_ODD) {
            if (t == 0) {
#pragma unroll
                for (int c = 0; c < 8; ++c) ksm[pw * 8 + c] = K[c];
            }
            // boundary lanes: own words (slot q holds f*_opp(q) of the even
            // launch, the bounce-back value of population q), in flight with
            // the gathers
            if ((bm_all >> (2 * t)) & 3u) {
#pragma unroll
                for (int q = 0; q < Q; ++q)
                    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(smem_u32(buf + q * 32)),
                                 "l"(reinterpret_cast<const W*>(A) + ((uint32_t)q * sw + ew)), "n"(sizeof(W))
                                 : "memory");
                asm volatile("cp.async.commit_group;" ::: "memory");
            }
        }
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            if constexpr (MODE == MODE_AA_EVEN) {
                raw[q] = ldw<S>(A, (uint32_t)q * sw + ew);
            } else {
                const int da = -X::a(q), db = -X::b(q), o = -X::r(q);
                // word of the neighbour column's pair at the same levels (K + 1 is even)
                const uint32_t pb = (uint32_t)(MODE == MODE_AA_ODD ? L::opp(q) : q) * sw;
                const uint32_t s = (da == 0 && db == 0) ? ew : ((uint32_t)(K[col8(da, db)] + 1) >> 1) + (uint32_t)t;
                if (o == 0) raw[q] = ldw<S>(A, pb + s);
                else if (o > 0) raw[q] = straddle<S>(ldw<S>(A, pb + s), ldw<S>(A, pb + s + 1));
                else raw[q] = straddle<S>(ldw<S>(A, pb + s - 1), ldw<S>(A, pb + s));
            }
        }
    }

    // L2 prefetch of that piece's window in every plane: lane t of the piece's
    // lane group takes planes t, t + 2^lg, ..., one prefetch at the window's
    // first word (an 8-slot window is 16 B; a second prefetch at its end
    // measured 2 % slower).  Neighbour columns' windows are the windows of
    // nearby pieces, prefetched by them.  Ids stay in [8, N - 8), so the word
    // lies inside the population array.
    if (hfp) {
        const uint32_t wf = nfp >> 1;
        const char* Ab = reinterpret_cast<const char*>(A);
        for (int q = t; q < Q; q += 1 << lg)
            asm volatile("prefetch.global.L2 [%0];" ::"l"(Ab + (size_t)((uint32_t)q * sw + wf) * sizeof(W)));
    }
    // the AA odd launch prefetches only the descriptor of the piece a wave
    // ahead (its population windows: see the launcher)
    if (MODE == MODE_AA_ODD && t == 0 && a.pf_ahead > 0 && cfp < a.nchunks)
        asm volatile("prefetch.global.L2 [%0];" ::"l"(a.chunks + cfp));
    // the odd pattern's column bases go through shared memory (lane 0 of
    // each chunk wrote them): fewer registers held across the collision
    if constexpr (MODE == MODE_AA_ODD) __syncwarp();
    // populations missing at some node of the warp (warp-uniform)
    const uint32_t umiss = MODE == MODE_AA_ODD ? __reduce_or_sync(0xffffffffu, m_lo | m_hi) : 0u;
    // AA odd: missing populations (boundary nodes) take the bounced value from
    // the node's own word or the initial value (bounce_back_pop); only the
    // populations missing somewhere in the warp are visited (a per-lane loop
    // over the missing bits through shared memory measured 6 % slower)
    if constexpr (MODE == MODE_AA_ODD) {
        // every lane that issued own-word copies waits for them here, before
        // the buffer is read or reused (a boundary node may miss no population)
        if (__any_sync(0xffffffffu, ((bm_all >> (2 * t)) & 3u) != 0u)) {
            asm volatile("cp.async.wait_all;" ::: "memory");
            __syncwarp();
        }
        if (umiss) {
            uint32_t wm = 0u;
            if (act) asm volatile("ld.global.nc.u32 %0, [%1];" : "=r"(wm) : "l"(&cw[0].z));   // wmask, read late
            wm = (wm >> (2 * t)) & 3u;
            // populations each node bounces back (the others take the initial value)
            uint32_t keep = ~0u;
            if (L::NO_BB_POP >= 0 && !(a.corr & LBM_FIX_BB_ALL_DIRS)) keep = ~(1u << (L::NO_BB_POP & 31));
            const bool fix_list = a.corr & LBM_FIX_LIST_NODES;
            const uint32_t b_lo = ((wm & 1u) || fix_list) ? (m_lo & keep) : 0u;
            const uint32_t b_hi = ((wm & 2u) || fix_list) ? (m_hi & keep) : 0u;
            if constexpr (S == ST_F32) {
#pragma unroll
                for (int q = 0; q < Q; ++q) {
                    if (!((umiss >> q) & 1u)) continue;
                    const bool bl = (b_lo >> q) & 1u, bh = (b_hi >> q) & 1u;
                    const bool il = ((m_lo & ~b_lo) >> q) & 1u, ih = ((m_hi & ~b_hi) >> q) & 1u;
                    if (bl || bh) {
                        const W own = buf[q * 32];
                        if (bl) raw[q] = take_half<S>(raw[q], false, own);
                        if (bh) raw[q] = take_half<S>(raw[q], true, own);
                    }
                    if (il) raw[q] = init_half<S, Q>(raw[q], false, q);
                    if (ih) raw[q] = init_half<S, Q>(raw[q], true, q);
                }
            } else {
                // 16-bit halves: the flags of population q for both nodes
                // (lo node in bits 0-15, hi node in bits 16-31 of a flag word
                // per 16 populations) shifted to bits 15 and 31, widened to
                // half masks by a sign-replicating byte permute
                const uint32_t i_lo = m_lo & ~b_lo, i_hi = m_hi & ~b_hi;
                const uint32_t fb0 = (b_lo & 0xffffu) | (b_hi << 16), fb1 = (b_lo >> 16) | (b_hi & 0xffff0000u);
                const uint32_t fi0 = (i_lo & 0xffffu) | (i_hi << 16), fi1 = (i_lo >> 16) | (i_hi & 0xffff0000u);
#pragma unroll
                for (int q = 0; q < Q; ++q) {
                    if (!((umiss >> q) & 1u)) continue;
                    const uint32_t mb = half_masks(q < 16 ? fb0 << (15 - q) : fb1 << (31 - q));
                    const uint32_t mi = half_masks(q < 16 ? fi0 << (15 - q) : fi1 << (31 - q));
                    // bounced halves from the node's own word; initial-value halves 0
                    raw[q] = ((raw[q] & ~mb) | (buf[q * 32] & mb)) & ~mi;
                }
            }
            __syncwarp();
        }
    }
    // pull: missing populations (boundary nodes) bounce back from slot opp(q)
    // of the source lattice or take the initial value
    if (MODE == MODE_PULL && __any_sync(0xffffffffu, (m_lo | m_hi) != 0u)) {
        uint32_t wm = 0u;
        if (act) asm volatile("ld.global.nc.u32 %0, [%1];" : "=r"(wm) : "l"(&cw[0].z));   // wmask, read late
        wm = (wm >> (2 * t)) & 3u;
        if (a.corr & LBM_FIX_LIST_NODES) wm = 3u;       // every boundary node bounces back
        const bool all_dirs = a.corr & LBM_FIX_BB_ALL_DIRS;
        const bool w_lo = wm & 1u, w_hi = (wm >> 1) & 1u;
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const bool ml = (m_lo >> q) & 1u, mh = (m_hi >> q) & 1u;
            if (ml || mh) {
                const bool dir_ok = q != L::NO_BB_POP || all_dirs;
                const bool bl = ml && w_lo && dir_ok, bh = mh && w_hi && dir_ok;
                // bounce-back source: own node, slot opp(q) of the source lattice;
                // a predicated load and selects instead of branches
                W own = raw[q];
                if (bl || bh) own = ldw<S>(A, (uint32_t)L::opp(q) * sw + ew);
                raw[q] = take_half<S>(raw[q], false, bl ? own : raw[q]);
                raw[q] = take_half<S>(raw[q], true, bh ? own : raw[q]);
                if (ml && !bl) raw[q] = init_half<S, Q>(raw[q], false, q);
                if (mh && !bh) raw[q] = init_half<S, Q>(raw[q], true, q);
            }
        }
    }
    // Zou-He: launch n applies the boundary conditions of iteration n-1
    const uint32_t zm = (zm_all >> (2 * t)) & 3u;
    if (__any_sync(0xffffffffu, zm != 0u && step > 0)) {
        // the warp's words go through shared memory around the per-node update
#pragma unroll
        for (int q = 0; q < Q; ++q) buf[q * 32] = raw[q];
        if (step > 0 && zm) {
            int32_t zs;
            asm volatile("ld.global.nc.u32 %0, [%1];" : "=r"(zs) : "l"(&cw[1].y));     // zslot0, read late
            const int z0 = zs + __popc(zm_all & ((1u << (2 * t)) - 1u));
            if (zm & 1u) zou_he_half<Q, S>(a, z0, buf, false, step);
            if (zm & 2u) zou_he_half<Q, S>(a, z0 + (int)(zm & 1u), buf, true, step);
        }
#pragma unroll
        for (int q = 0; q < Q; ++q) raw[q] = buf[q * 32];
    }
    if (!act) return;
    const float om = a.insts[li >> 8].omega_f;
    void* D = a.dst;
    if constexpr (MODE == MODE_PULL) {
        collide2<Q, S>(raw, om, [&](int q, F2 v) { stw<S>(D, (uint32_t)q * sw + ew, pack<S, Q>(v, q)); });
    } else if constexpr (MODE == MODE_AA_EVEN) {
        collide2<Q, S>(raw, om, [&](int q, F2 v) { stw<S>(D, (uint32_t)L::opp(q) * sw + ew, pack<S, Q>(v, q)); });
    } else {
        // AA odd: f*_q to slot q of x + c_q, or (absent destination) to slot
        // opp(q) of x, there f*_q or the initial value (bounce_back_pop);
        // ghost slots of the pair store nothing
        uint32_t vm, wm = 0u;
        asm volatile("ld.global.nc.u32 %0, [%1];" : "=r"(vm) : "l"(&cw[3].w));
        if (umiss) asm volatile("ld.global.nc.u32 %0, [%1];" : "=r"(wm) : "l"(&cw[0].z));   // wmask
        vm = (vm >> (2 * t)) & 3u;
        wm = (wm >> (2 * t)) & 3u;
        const volatile int32_t* ks = ksm + pw * 8;
        // whole-word stores of the directions without a run-axis component
        // when every lane of the warp holds two fluid nodes (a warp-uniform
        // branch; per lane it diverged, measured 1.5 % slower)
        const bool wword = __all_sync(__activemask(), vm == 3u);
        collide2<Q, S>(raw, om, [&](int q, F2 v) {
            const int da = X::a(q), db = X::b(q), o = X::r(q);
            const uint32_t s = (uint32_t)((da == 0 && db == 0 ? n0 - 1 : ks[col8(da, db)]) + 1 + 2 * t);
            const uint32_t pq = (uint32_t)q * st;
            if (umiss == 0u) {
                // no node of the warp misses a population: every destination
                // x + c_q exists (a warp-uniform test)
                if (o == 0 && wword) {
                    stw<S>(D, (uint32_t)q * sw + (s >> 1), pack<S, Q>(v, q));
                } else {
                    float l, h;
                    f2split(v, l, h);
                    if (vm & 1u) st_one<S, Q>(D, pq + s + o, l, q);
                    if (vm & 2u) st_one<S, Q>(D, pq + s + 1 + o, h, q);
                }
            } else {
                const bool bl = (m_lo >> L::opp(q)) & 1u, bh = (m_hi >> L::opp(q)) & 1u;
                const uint32_t po = (uint32_t)L::opp(q) * st;
                float l, h;
                f2split(v, l, h);
                if (bl && !bounce_back_pop<Q>(L::opp(q), wm & 1u, a.corr)) l = 0.f;
                if (bh && !bounce_back_pop<Q>(L::opp(q), (wm >> 1) & 1u, a.corr)) h = 0.f;
                if (vm & 1u) st_one<S, Q>(D, bl ? po + e : pq + s + o, l, q);
                if (vm & 2u) st_one<S, Q>(D, bh ? po + e + 1 : pq + s + 1 + o, h, q);
            }
        });
    }
}

// ---------------------------------------------------------------------------
// launch: 32 / 2^piece_lg chunk pieces per warp, wpb warps per block
template <int Q, int S, int MODE, int RA>
static lbm_status launch_pair_one(const StepArgs& a, int wpb, cudaStream_t st) {
    // dynamic shared memory: one word per population and lane of each warp
    // (the Zou-He path); above 48 KB it needs the opt-in attribute
    // per-device caches (written with the same value by any thread that
    // fills them): the shared-memory opt-in and the blocks resident at once
    constexpr int kDevs = 16;
    static int opted[kDevs] = {0};
    static int resident[kDevs][9] = {{0}};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kDevs)
        return fail(LBM_ERR_CUDA, "paired step kernel: device %d not supported", dev);
    const size_t smem = (size_t)wpb * (Q * 32 * sizeof(typename PairWord<S>::W) + (MODE == MODE_AA_ODD ? 256 : 0));
    if (smem > 48 * 1024 && opted[dev] < (int)smem) {
        const cudaError_t e = cudaFuncSetAttribute(k_step2<Q, S, MODE, RA>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return fail(LBM_ERR_CUDA, "paired step kernel shared memory: %s", cudaGetErrorString(e));
        opted[dev] = (int)smem;
    }
    const int64_t per_block = (int64_t)wpb << (5 - a.piece_lg);
    const int64_t blocks = (a.nchunks + per_block - 1) / per_block;
    // prefetch distance: in pieces, from the blocks resident at once
    if (resident[dev][wpb] == 0) {
        int sms = 0, nb = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_step2<Q, S, MODE, RA>, 32 * wpb, smem) != cudaSuccess)
            return fail(LBM_ERR_CUDA, "paired step kernel occupancy: %s", cudaGetErrorString(cudaGetLastError()));
        resident[dev][wpb] = sms * (nb > 0 ? nb : 1);
    }
    // half a wave ahead: measured 0.4 % faster than one wave, 1.5 % faster
    // than 1.5 waves.  The AA odd launch prefetches no population window: on
    // its grouped piece table that cost more than it saved (without it the
    // tree's step measured 2.7 % faster; one or two waves ahead: no gain);
    // it prefetches the descriptor one wave ahead (+1 %; half a wave and two
    // waves measured the same within 0.3 %)
    StepArgs b = a;
    b.pf_ahead = (int64_t)resident[dev][wpb] * per_block / (MODE == MODE_AA_ODD ? 1 : 2);
    k_step2<Q, S, MODE, RA><<<(unsigned)(blocks > 0 ? blocks : 1), 32 * wpb, smem, st>>>(b);
    return LBM_OK;
}

template <int Q, int S, int RA>
static lbm_status launch_pair_mode(int mode, const StepArgs& a, int wpb, cudaStream_t st) {
    if (mode == MODE_PULL) return launch_pair_one<Q, S, MODE_PULL, RA>(a, wpb, st);
    if (mode == MODE_AA_EVEN) return launch_pair_one<Q, S, MODE_AA_EVEN, RA>(a, wpb, st);
    return launch_pair_one<Q, S, MODE_AA_ODD, RA>(a, wpb, st);
}

template <int S>
static lbm_status launch_pair_store(int Q, int mode, int ra, const StepArgs& a, int wpb, cudaStream_t st) {
    lbm_status s;
    if (Q == 19) s = ra == 1 ? launch_pair_mode<19, S, 1>(mode, a, wpb, st) : launch_pair_mode<19, S, 2>(mode, a, wpb, st);
    else if (Q == 27) s = ra == 1 ? launch_pair_mode<27, S, 1>(mode, a, wpb, st) : launch_pair_mode<27, S, 2>(mode, a, wpb, st);
    else return fail(LBM_ERR_ARG, "Q must be 19 or 27");
    if (s != LBM_OK) return s;
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(LBM_ERR_CUDA, "paired step launch: %s", cudaGetErrorString(e));
    return LBM_OK;
}

}  // namespace lbm
