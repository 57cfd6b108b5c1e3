// Fused lattice Boltzmann step: gather (streaming) + boundary conditions +
// BGK collision + store, one warp per run-table chunk, one lane per node.
//
// One launch performs one Iterate() body of the reference
// (Simulation.cpp:909-915) with the state kept in the populations array:
//   gather      f_q(x) = f*_q(x - c_q)                     Streaming :184-198
//   missing     source node absent (NotFluid or outside the grid):
//                 wall node, q != the population the reference never bounces
//                 back (opp of dir 0 for D3Q19)  -> f*_{opp q}(x)   ApplyWallBc :1353-1370
//                 otherwise the population is never written by the reference
//                 and keeps its initial value w_q (Node.cpp:30-37)
//   Zou-He      velocity / pressure formulas on the node's own populations
//                 (Boundary.cpp:87-148, Simulation.cpp:952-1348)
//   collision   rho, u, f_eq, f* = omega f_eq + (1-omega) f  (Simulation.cpp:21-179)
// The reference applies its boundary conditions after streaming and before
// the next collision; here they run at the start of the next launch, which
// is the same sequence of operations on every node.
//
// Streaming patterns:
//   PULL     two lattices: read f*(step n-1) from src, write f*(step n) to dst
//   AA_EVEN  one lattice, node-local: read slot q, write f*_q to slot opp(q)
//   AA_ODD   one lattice, neighbour: read slot opp(q) of x - c_q, write f*_q
//            to slot q of x + c_q (to slot opp(q) of x when x + c_q is absent)
// DRY launches run the gather and boundary part only and write f_n, rho_n,
// u_n in FP64 (snapshots and monitors); they never modify the state.
//
// Missing populations in the AA pattern (source node x - c_q absent): the
// AA odd launch stores, for an absent x + c_q, f*_q (bounced) or the initial
// value (where the reference never writes the population: direction 0 of its
// wall loop, inlet/outlet nodes; see bounce_back_pop) in slot opp(q) of x,
// which is where the next AA even launch reads population opp(q): that
// launch needs no fix-up.  The AA odd launch takes a missing population from
// the node's own slot q (the even launch left f*_opp(q) there) or resets it.
//
// Neighbour addressing: on the ghost-padded run lattice (device.cuh) the
// source of population q of lane t is K[column] + const + t, one integer add;
// boundary lanes read a precomputed mask of their missing populations.
//
// Arithmetic: Store ST_F64 follows the reference's FP64 expressions operation
// by operation (its TU is built with -fmad=false), so FP64 runs are bit-exact
// with the reference.  The other stores compute in FP32 on shifted populations
// f - w, scaled by 2^15 for FP16 (the scale is folded into the equilibrium,
// never applied per population), with the equilibrium evaluated for
// opposite pairs from a symmetric and an antisymmetric part.
#pragma once
#include "device.cuh"

namespace lbm {

enum StepMode { MODE_PULL = 0, MODE_AA_EVEN = 1, MODE_AA_ODD = 2 };

template <int S> struct Work { using T = float; static constexpr float K = 1.0f; };
template <> struct Work<ST_F64> { using T = double; static constexpr double K = 1.0; };
template <> struct Work<ST_F16S> { using T = float; static constexpr float K = kF16Scale; };

// Velocity components in (a, b, run) order for a run axis.
template <int Q, int RA> struct Ax;
template <int Q> struct Ax<Q, 2> {   // run axis z: columns (x, y)
    __host__ __device__ static constexpr int a(int q) { return Lat<Q>::cx(q); }
    __host__ __device__ static constexpr int b(int q) { return Lat<Q>::cy(q); }
    __host__ __device__ static constexpr int r(int q) { return Lat<Q>::cz(q); }
};
template <int Q> struct Ax<Q, 1> {   // run axis y: columns (x, z)
    __host__ __device__ static constexpr int a(int q) { return Lat<Q>::cx(q); }
    __host__ __device__ static constexpr int b(int q) { return Lat<Q>::cz(q); }
    __host__ __device__ static constexpr int r(int q) { return Lat<Q>::cy(q); }
};

// storage -> working value (F64: f; F32/BF16: f - w; F16: (f - w) * 2^15)
// (the read-only path is used for the pull pattern only: in the AA patterns
// the kernel writes the array it reads)
template <int S, int Q, bool RO = false>
__device__ __forceinline__ typename Work<S>::T ld(const void* base, int64_t stride, int q, uint32_t i) {
    // 32-bit element offset (the lattice holds < 2^32 values)
    const uint32_t off = (uint32_t)q * (uint32_t)stride + i;
    if constexpr (S == ST_F64) {
        const double* p = (const double*)base + off;
        return RO ? __ldg(p) : *p;
    } else if constexpr (S == ST_F32) {
        const float* p = (const float*)base + off;
        return (RO ? __ldg(p) : *p) - (float)Lat<Q>::w(q);
    } else if constexpr (S == ST_F16S) {
        const __half* p = (const __half*)base + off;
        return __half2float(RO ? __ldg(p) : *p);
    } else {
        const __nv_bfloat16* p = (const __nv_bfloat16*)base + off;
        return __bfloat162float(RO ? __ldg(p) : *p);
    }
}

template <int S, int Q>
__device__ __forceinline__ void st(void* base, int64_t stride, int q, uint32_t i, typename Work<S>::T v) {
    const uint32_t off = (uint32_t)q * (uint32_t)stride + i;
    if constexpr (S == ST_F64) {
        ((double*)base)[off] = v;
    } else if constexpr (S == ST_F32) {
        ((float*)base)[off] = v + (float)Lat<Q>::w(q);
    } else if constexpr (S == ST_F16S) {
        ((__half*)base)[off] = __float2half_rn(v);
    } else {
        ((__nv_bfloat16*)base)[off] = __float2bfloat16_rn(v);
    }
}

// store to slot q of node i, or (back) to slot opp(q) of node n: a select
// between two 32-bit element offsets (the lattice holds < 2^32 values)
template <int S, int Q>
__device__ __forceinline__ void st_sel(void* base, uint32_t stride, int q, uint32_t i, bool back, uint32_t n,
                                       typename Work<S>::T v) {
    const uint32_t off = back ? (uint32_t)Lat<Q>::opp(q) * stride + n : (uint32_t)q * stride + i;
    if constexpr (S == ST_F64) {
        ((double*)base)[off] = v;
    } else if constexpr (S == ST_F32) {
        ((float*)base)[off] = v + (float)Lat<Q>::w(q);
    } else if constexpr (S == ST_F16S) {
        ((__half*)base)[off] = __float2half_rn(v);
    } else {
        ((__nv_bfloat16*)base)[off] = __float2bfloat16_rn(v);
    }
}

// working value <-> plain population
template <int S, int Q>
__device__ __forceinline__ typename Work<S>::T plain(typename Work<S>::T v, int q) {
    if constexpr (S == ST_F64) return v;
    else if constexpr (S == ST_F16S) return (float)Lat<Q>::w(q) + v * (1.0f / kF16Scale);
    else return v + (float)Lat<Q>::w(q);
}
template <int S, int Q>
__device__ __forceinline__ typename Work<S>::T unplain(typename Work<S>::T v, int q) {
    if constexpr (S == ST_F64) return v;
    else if constexpr (S == ST_F16S) return (v - (float)Lat<Q>::w(q)) * kF16Scale;
    else return v - (float)Lat<Q>::w(q);
}

// ---------------------------------------------------------------------------
// Zou-He boundary formulas on plain populations, written in the reference's
// operation order.  T = double reproduces the reference bit for bit.

template <class T>
__device__ __forceinline__ void zh_vel_negy(T* f, const T* v) {
    // Boundary::ApplyBc, D3Q19 (Boundary.cpp:129-148)
    T rhoN = (f[0] + f[1] + f[4] + f[5] + f[8] + f[9] + f[12] + f[13] + f[18] +
              T(2.0) * (f[2] + f[6] + f[10] + f[14] + f[15])) / (T(1) + v[1]);
    T Nx = T(0.5) * (f[0] + f[8] + f[9] - (f[1] + f[12] + f[13])) - (T(1.0) / T(3.0)) * rhoN * v[0];
    T Nz = T(0.5) * (f[4] + f[8] + f[12] - (f[5] + f[9] + f[13])) - (T(1.0) / T(3.0)) * rhoN * v[2];
    f[3] = f[2] - (T(1.0) / T(3.0)) * rhoN * v[1];
    f[11] = f[6] + (T(1.0) / T(6.0)) * rhoN * (-v[1] - v[0]) + Nx;
    f[7] = f[10] + (T(1.0) / T(6.0)) * rhoN * (-v[1] + v[0]) - Nx;
    f[17] = f[14] + (T(1.0) / T(6.0)) * rhoN * (-v[1] - v[2]) + Nz;
    f[16] = f[15] + (T(1.0) / T(6.0)) * rhoN * (-v[1] + v[2]) - Nz;
}

template <class T>
__device__ __forceinline__ void zh_vel_posx_q27(T* f, const T* v) {
    // Boundary::ApplyBc, D3Q27 (Boundary.cpp:87-123)
    T rho = ((f[0] + f[3] + f[4] + f[5] + f[6] + f[15] + f[16] + f[17] + f[18]) +
             T(2) * (f[2] + f[9] + f[10] + f[12] + f[14] + f[20] + f[22] + f[24] + f[26])) / (T(1) - v[0]);
    T Ny = (T(1.0) / T(6)) * (f[3] + f[15] + f[16] - f[4] - f[17] - f[18]) - (T(1.0) / T(9)) * (rho * v[1]);
    T Nz = (T(1.0) / T(6)) * (f[5] + f[15] + f[17] - f[6] - f[16] - f[18]) - (T(1.0) / T(9)) * (rho * v[2]);
    f[1] = f[2] + (T(4) / T(9.0)) * rho * v[0];
    f[7] = f[10] + (T(1) / T(9.0)) * rho * (v[0] + v[1]) - Ny;
    f[8] = f[9] + (T(1) / T(9.0)) * rho * (v[0] - v[1]) + Ny;
    f[11] = f[14] + (T(1) / T(9.0)) * rho * (v[0] + v[2]) - Nz;
    f[13] = f[12] + (T(1) / T(9.0)) * rho * (v[0] - v[2]) + Nz;
    f[19] = f[20] + (T(1) / T(36.0)) * rho * (v[0] + v[1] + v[2]) - Ny - Nz;
    f[21] = f[22] + (T(1) / T(36.0)) * rho * (v[0] + v[1] - v[2]) - Ny + Nz;
    f[23] = f[24] + (T(1) / T(36.0)) * rho * (v[0] - v[1] + v[2]) + Ny - Nz;
    f[25] = f[26] + (T(1) / T(36.0)) * rho * (v[0] - v[1] - v[2]) + Ny + Nz;
}

// ApplyOutletBc bodies (Simulation.cpp:952-1348); transverse velocities are 0.
template <class T>
__device__ __forceinline__ void zh_press(T* f, int kind, T rho) {
    const T vx = T(0.0), vz = T(0.0), vy0 = T(0.0);
    if (kind == LBM_BC_PRESS_NEGY) {
        T vy = T(-1) + (T(1.0) / rho) * (f[0] + f[1] + f[4] + f[5] + f[8] + f[9] + f[12] + f[13] + f[18] +
                                         T(2.0) * (f[2] + f[6] + f[10] + f[14] + f[15]));
        T Nyx = T(0.5) * (f[0] + f[8] + f[9] - (f[1] + f[12] + f[13])) - (T(1.0) / T(3.0)) * rho * vx;
        T Nyz = T(0.5) * (f[4] + f[8] + f[12] - (f[5] + f[9] + f[13])) - (T(1.0) / T(3.0)) * rho * vz;
        f[3] = f[2] - (T(1.0) / T(3.0)) * rho * vy;
        f[11] = f[6] + (T(1.0) / T(6.0)) * rho * (-vx - vy) + Nyx;
        f[7] = f[10] + (T(1.0) / T(6.0)) * rho * (vx - vy) - Nyx;
        f[17] = f[14] + (T(1.0) / T(6.0)) * rho * (-vy - vz) + Nyz;
        f[16] = f[15] + (T(1.0) / T(6.0)) * rho * (-vy + vz) - Nyz;
    } else if (kind == LBM_BC_PRESS_POSY) {
        T vy = T(1) - (T(1.0) / rho) * (f[0] + f[1] + f[4] + f[5] + f[8] + f[9] + f[12] + f[13] + f[18] +
                                        T(2.0) * (f[3] + f[7] + f[11] + f[16] + f[17]));
        T Nyx = T(0.5) * (f[0] + f[8] + f[9] - (f[1] + f[12] + f[13])) - (T(1.0) / T(3.0)) * rho * vx;
        T Nyz = T(0.5) * (f[4] + f[8] + f[12] - (f[5] + f[9] + f[13])) - (T(1.0) / T(3.0)) * rho * vz;
        f[2] = f[3] + (T(1.0) / T(3.0)) * rho * vy;
        f[6] = f[11] + (T(1.0) / T(6.0)) * rho * (vx + vy) - Nyx;
        f[10] = f[7] + (T(1.0) / T(6.0)) * rho * (-vx + vy) + Nyx;
        f[14] = f[17] + (T(1.0) / T(6.0)) * rho * (vy + vz) - Nyz;
        f[15] = f[16] + (T(1.0) / T(6.0)) * rho * (vy - vz) + Nyz;
    } else if (kind == LBM_BC_PRESS_POSX) {
        const T vy = vy0;
        T ux = T(1) - (T(1.0) / rho) * (f[2] + f[3] + f[4] + f[5] + f[14] + f[15] + f[16] + f[17] + f[18] +
                                        T(2.0) * (f[1] + f[10] + f[11] + f[12] + f[13]));
        T Nxy = T(0.5) * (f[2] + f[14] + f[15] - (f[3] + f[16] + f[17])) - (T(1.0) / T(3.0)) * rho * vy;
        T Nxz = T(0.5) * (f[4] + f[10] + f[14] - (f[5] + f[15] + f[17])) - (T(1.0) / T(3.0)) * rho * vz;
        f[0] = f[1] + (T(1.0) / T(3.0)) * rho * ux;
        f[7] = f[10] + (T(1.0) / T(6.0)) * rho * (ux - vy) + Nxy;
        f[6] = f[11] + (T(1.0) / T(6.0)) * rho * (ux + vy) - Nxy;
        f[8] = f[13] + (T(1.0) / T(6.0)) * rho * (ux + vz) - Nxz;
        f[9] = f[12] + (T(1.0) / T(6.0)) * rho * (ux - vz) + Nxz;
    } else if (kind == LBM_BC_PRESS_POSZ) {
        const T vy = vy0;
        T uz = T(1) - (T(1.0) / rho) * (f[0] + f[1] + f[2] + f[3] + f[6] + f[7] + f[10] + f[11] + f[18] +
                                        T(2.0) * (f[5] + f[9] + f[13] + f[15] + f[17]));
        T Nzx = T(0.5) * (f[0] + f[6] + f[7] - (f[1] + f[10] + f[11])) - (T(1.0) / T(3.0)) * rho * vx;
        T Nzy = T(0.5) * (f[2] + f[6] + f[10] - (f[3] + f[7] + f[11])) - (T(1.0) / T(3.0)) * rho * vy;
        f[4] = f[5] + (T(1.0) / T(3.0)) * rho * uz;
        f[8] = f[13] + (T(1.0) / T(6.0)) * rho * (uz + vx) - Nzx;
        f[12] = f[9] + (T(1.0) / T(6.0)) * rho * (uz - vx) + Nzx;
        f[14] = f[17] + (T(1.0) / T(6.0)) * rho * (uz + vy) - Nzy;
        f[16] = f[15] + (T(1.0) / T(6.0)) * rho * (uz - vy) + Nzy;
    }
}

// Zou-He on an axis-aligned face of any orientation.  The reference writes
// one routine per orientation (the functions above); they share one form,
// written here over the lattice tables for unknowns sg along axis A
// (face = 2A + (sg < 0)):
//   S0 = sum of f over c_A = 0, Sk = sum of f over c_A = -sg
//   velocity: rho = (S0 + 2 Sk) / (1 - sg u_A)
//   pressure: u_A = sg (1 - (S0 + 2 Sk) / rho), transverse u = 0
//   N_T = a sum_{c_A = 0} c_T f - b rho u_T  (a, b = 1/2, 1/3 for D3Q19 and
//         1/6, 1/9 for D3Q27, the reference's coefficients)
//   unknown f_q (c_A(q) = sg) = f_opp(q) + 6 w_q rho (c_q . u) - sum_T c_T(q) N_T
template <int Q>
__host__ __device__ constexpr int lat_c(int q, int ax) {
    return ax == 0 ? Lat<Q>::cx(q) : (ax == 1 ? Lat<Q>::cy(q) : Lat<Q>::cz(q));
}

template <int Q, class T>
__device__ __forceinline__ void zh_face(T* f, int face, bool vel, const T* v, T rho_in) {
    using L = Lat<Q>;
    const int A = face >> 1, sg = (face & 1) ? -1 : 1;
    T S0 = T(0), Sk = T(0);
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const int ca = lat_c<Q>(q, A);
        if (ca == 0) S0 += f[q];
        else if (ca == -sg) Sk += f[q];
    }
    T u[3] = {T(0), T(0), T(0)};
    T rho;
    if (vel) {
        u[0] = v[0]; u[1] = v[1]; u[2] = v[2];
        rho = (S0 + T(2) * Sk) / (T(1) - T(sg) * u[A]);
    } else {
        rho = rho_in;
        u[A] = T(sg) * (T(1) - (S0 + T(2) * Sk) / rho);
    }
    const T ka = Q == 19 ? T(0.5) : T(1.0) / T(6.0), kb = Q == 19 ? T(1.0) / T(3.0) : T(1.0) / T(9.0);
    T N[3] = {T(0), T(0), T(0)};
#pragma unroll
    for (int t = 0; t < 3; ++t) {
        if (t == A) continue;
        T m = T(0);
#pragma unroll
        for (int q = 0; q < Q; ++q)
            if (lat_c<Q>(q, A) == 0 && lat_c<Q>(q, t) != 0) m += lat_c<Q>(q, t) > 0 ? f[q] : -f[q];
        N[t] = ka * m - kb * rho * u[t];
    }
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        if (lat_c<Q>(q, A) != sg) continue;
        const T cu = T(L::cx(q)) * u[0] + T(L::cy(q)) * u[1] + T(L::cz(q)) * u[2];
        T val = f[L::opp(q)] + T(6.0 * L::w(q)) * rho * cu;
#pragma unroll
        for (int t = 0; t < 3; ++t)
            if (t != A && lat_c<Q>(q, t) != 0) val -= T(lat_c<Q>(q, t)) * N[t];
        f[q] = val;
    }
}

// Any Zou-He kind on plain populations p (velocity v for the velocity kinds).
template <int Q, class T>
__device__ __forceinline__ void zou_he_apply(T* p, int kind, int face, const T* v, T rho) {
    if (kind == LBM_BC_VELOCITY) {
        zh_face<Q, T>(p, face, true, v, rho);
    } else if (kind == LBM_BC_PRESSURE) {
        zh_face<Q, T>(p, face, false, v, rho);
    } else if constexpr (Q == 19) {
        if (kind == LBM_BC_VEL_NEGY) zh_vel_negy<T>(p, v);
        else zh_press<T>(p, kind, rho);
    } else {
        if (kind == LBM_BC_VEL_POSX) zh_vel_posx_q27<T>(p, v);
    }
}

// Whether boundary node population p (its source absent) takes the bounced
// value f*_opp(p) or keeps the initial value: wall nodes bounce back every
// population but opp(0) of D3Q19 (ApplyWallBc loops dir = 1..Q-1,
// Simulation.cpp:1361); inlet/outlet nodes keep the initial value (their
// Zou-He routine rewrites the unknowns); LBM_FIX_* widen both.
template <int Q>
__device__ __forceinline__ bool bounce_back_pop(int p, bool wall, uint32_t corr) {
    return (wall || (corr & LBM_FIX_LIST_NODES)) && (p != Lat<Q>::NO_BB_POP || (corr & LBM_FIX_BB_ALL_DIRS));
}
// initial value of population q as a working value (node_update's reset)
template <int S, int Q>
__device__ __forceinline__ typename Work<S>::T init_work(int q) {
    return S == ST_F64 ? typename Work<S>::T(Lat<Q>::w(q)) : typename Work<S>::T(0);
}

__host__ __device__ constexpr bool is_velocity_kind(int kind) {
    return kind == LBM_BC_VEL_NEGY || kind == LBM_BC_VEL_POSX || kind == LBM_BC_VELOCITY;
}

// rho and u from plain populations with the reference's grouped sums
// (Simulation.cpp:32-79 for D3Q19, :82-148 for D3Q27).
template <int Q, class T>
__device__ __forceinline__ void macro_ref(const T* f, T& rho, T& ux, T& uy, T& uz) {
    rho = T(0.0);
#pragma unroll
    for (int q = 0; q < Q; ++q) rho += f[q];
    if constexpr (Q == 19) {
        ux = ((f[0] + f[6] + f[7] + f[8] + f[9]) - (f[1] + f[10] + f[11] + f[12] + f[13])) / rho;
        uy = ((f[2] + f[6] + f[10] + f[14] + f[15]) - (f[3] + f[7] + f[11] + f[16] + f[17])) / rho;
        uz = ((f[4] + f[8] + f[12] + f[14] + f[16]) - (f[5] + f[9] + f[13] + f[15] + f[17])) / rho;
    } else {
        ux = ((f[1] + f[7] + f[8] + f[11] + f[13] + f[19] + f[21] + f[23] + f[25]) -
              (f[2] + f[9] + f[10] + f[12] + f[14] + f[20] + f[22] + f[24] + f[26])) / rho;
        uy = ((f[3] + f[7] + f[9] + f[15] + f[16] + f[19] + f[21] + f[24] + f[26]) -
              (f[4] + f[8] + f[10] + f[17] + f[18] + f[20] + f[22] + f[23] + f[25])) / rho;
        uz = ((f[5] + f[11] + f[12] + f[15] + f[17] + f[19] + f[22] + f[23] + f[26]) -
              (f[6] + f[13] + f[14] + f[16] + f[18] + f[20] + f[21] + f[24] + f[25])) / rho;
    }
}

// BGK collision.  F64: the reference's expressions.  FP32: shifted (and for
// FP16 scaled) form with pairwise equilibrium.
template <int Q, int S>
__device__ __forceinline__ void collide(typename Work<S>::T* f, const InstParam& ip) {
    using L = Lat<Q>;
    if constexpr (S == ST_F64) {
        double rho, ux, uy, uz;
        macro_ref<Q, double>(f, rho, ux, uy, uz);
        const double om = ip.omega;
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const double du = ux * (double)L::cx(q) + uy * (double)L::cy(q) + uz * (double)L::cz(q);
            const double usq = ux * ux + uy * uy + uz * uz;
            const double feq = L::w(q) * rho * (1.0 + 3.0 * du + 9.0 / 2.0 * du * du - 3.0 / 2.0 * usq);
            f[q] = om * feq + (1.0 - om) * f[q];
        }
    } else {
        constexpr float K = Work<S>::K;
        float drho = 0.f, jx = 0.f, jy = 0.f, jz = 0.f;
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            drho += f[q];
            if (L::cx(q)) jx += L::cx(q) > 0 ? f[q] : -f[q];
            if (L::cy(q)) jy += L::cy(q) > 0 ? f[q] : -f[q];
            if (L::cz(q)) jz += L::cz(q) > 0 ? f[q] : -f[q];
        }
        const float Krho = K + drho;            // K * rho
        const float inv = __fdividef(1.0f, Krho);   // Krho > 0 (rho near 1)
        const float ux = jx * inv, uy = jy * inv, uz = jz * inv;
        const float usq15 = 1.5f * (ux * ux + uy * uy + uz * uz);
        const float om = ip.omega_f;
        const float base = drho - Krho * usq15;    // K (rho - 1) + K rho (-1.5 u^2)
        const float Krho45 = 4.5f * Krho;
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const int o = L::opp(q);
            if (o == q) {
                f[q] += om * ((float)L::w(q) * base - f[q]);
            } else if (q < o) {
                float cu = 0.f;
                if (L::cx(q)) cu += L::cx(q) > 0 ? ux : -ux;
                if (L::cy(q)) cu += L::cy(q) > 0 ? uy : -uy;
                if (L::cz(q)) cu += L::cz(q) > 0 ? uz : -uz;
                const float w = (float)L::w(q);
                const float sym = w * (base + Krho45 * cu * cu);
                const float anti = (3.0f * w) * Krho * cu;
                f[q] += om * ((sym + anti) - f[q]);
                f[o] += om * ((sym - anti) - f[o]);
            }
        }
    }
}

// load that the compiler may not merge with an earlier load of the same
// address, so a value is re-read instead of held in a register across a
// long stretch of code
__device__ __forceinline__ int32_t ld_fresh(const int32_t* p) {
    int32_t v;
    asm volatile("ld.global.nc.b32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}

struct Partials {
    double* mass;      // per block
    double* inflow;
    double* outflow;
    double* maxu;
    int32_t* bad;
};

// Node id of the neighbour of lane `lane` at column offset (da, db) and level
// offset o (see Chunk): all compile-time except the chunk's bases.
__device__ __forceinline__ int32_t nb_id(const int32_t* K, int32_t n0, int lane, int da, int db, int o) {
    return (da == 0 && db == 0 ? n0 - 1 : K[col8(da, db)]) + 1 + o + lane;
}

// Missing-population mask of a lane (0 for interior lanes).
__device__ __forceinline__ uint32_t lane_missing(const StepArgs& a, const Chunk* cp, uint32_t bmask, int lane) {
    if (!((bmask >> lane) & 1u)) return 0u;
    return __ldg(a.mmask + __ldg(&cp->mslot0) + __popc(bmask & ((1u << lane) - 1u)));
}

// Fix-ups of missing populations (bounce-back from the node's own post-
// collision value, or the initial value for populations the reference never
// rewrites), Zou-He, then collision or snapshot.  Shared by both kernels.
template <int Q, int S, int MODE, bool DRY>
__device__ __forceinline__ void node_update(const StepArgs& a, int32_t zslot0, typename Work<S>::T* f, uint32_t missing,
                                            uint32_t wmask, uint32_t zmask, int lane, int32_t n, int inst, int64_t step,
                                            double* mon) {
    using L = Lat<Q>;
    using T = typename Work<S>::T;
    const void* A = a.src;
    if (__any_sync(__activemask(), missing != 0u)) {
        // predicated per population, so lanes of a warp do not diverge
        // wall nodes bounce back (inlet/outlet nodes too with LBM_FIX_LIST_NODES);
        // the reference never bounces back population opp(0) of D3Q19
        const bool wall = ((wmask >> lane) & 1u) || (a.corr & LBM_FIX_LIST_NODES);
        const bool all_dirs = a.corr & LBM_FIX_BB_ALL_DIRS;
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const bool miss = (missing >> q) & 1u;
            const bool bb = miss && wall && (q != L::NO_BB_POP || all_dirs);
            if constexpr (MODE == MODE_PULL) {
                if (bb) f[q] = ld<S, Q, true>(A, a.stride, L::opp(q), n);
            } else if constexpr (MODE == MODE_AA_ODD) {
                if (bb) f[q] = ld<S, Q>(A, a.stride, q, n);
            }
            // AA_EVEN: slot q of x already holds f*_{opp q}(x)
            if (miss && !bb) f[q] = S == ST_F64 ? T(L::w(q)) : T(0);
        }
    }
    // launch n turns f*(n-1) into f_n: its boundary conditions are those of
    // reference iteration n-1 (Simulation.cpp:913-915); f_0 is the initial
    // state, which the reference collides before any boundary condition
    const bool zl = ((zmask >> lane) & 1u) && step > 0;
    double zdir = 0.0;
    if (zl) {
        const int slot = zslot0 + __popc(zmask & ((1u << lane) - 1u));
        const ZSlot z = a.zslots[slot];
        const ListParam lp = a.lists[z.list];
        T p[Q];
#pragma unroll
        for (int q = 0; q < Q; ++q) p[q] = plain<S, Q>(f[q], q);
        T v[3] = {T(0), T(0), T(0)};
        if (is_velocity_kind(z.kind)) {
            // 32-bit phase: the step count stays below 2^32 (lbm_sim_step checks)
            const double amp = a.amp[lp.amp_off + (uint32_t)(step - 1) % (uint32_t)lp.amp_len];
            const double sc = amp * z.profile;
            v[0] = T(sc * lp.dir[0]); v[1] = T(sc * lp.dir[1]); v[2] = T(sc * lp.dir[2]);
            zdir = 1.0;
        } else {
            zdir = -1.0;
        }
        zou_he_apply<Q, T>(p, z.kind, lp.face, v, T(lp.rho));
#pragma unroll
        for (int q = 0; q < Q; ++q) f[q] = unplain<S, Q>(p[q], q);
    }
    if constexpr (DRY) {
        double fp[Q];
#pragma unroll
        for (int q = 0; q < Q; ++q) fp[q] = (double)plain<S, Q>(f[q], q);
        double rho, ux, uy, uz;
        macro_ref<Q, double>(fp, rho, ux, uy, uz);
        const int64_t pos = (int64_t)a.out_pos[n];
        if (a.out_f) {
#pragma unroll
            for (int q = 0; q < Q; ++q) a.out_f[pos * Q + q] = fp[q];
        }
        if (a.out_rho) a.out_rho[pos] = rho;
        if (a.out_u) { a.out_u[3 * pos] = ux; a.out_u[3 * pos + 1] = uy; a.out_u[3 * pos + 2] = uz; }
        const double sp = sqrt(ux * ux + uy * uy + uz * uz);
        mon[0] = rho;
        mon[3] = sp;
        mon[4] = (isfinite(rho) && isfinite(sp)) ? 0.0 : 1.0;
        if (zl) {
            if (zdir > 0) mon[1] = rho * sp;
            else mon[2] = rho * sp;
        }
    } else {
        collide<Q, S>(f, a.insts[inst]);
    }
}

template <int Q, int S, int MODE, bool DRY, int RA>
__global__ void __launch_bounds__(256, 4) k_step(StepArgs a, Partials part) {
    using L = Lat<Q>;
    using X = Ax<Q, RA>;
    using T = typename Work<S>::T;
    const int lane = threadIdx.x & 31;
    const int64_t ci = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    double mon[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    if (ci < a.nchunks) {
        const Chunk* cp = a.chunks + ci;
        const int32_t n0 = __ldg(&cp->n0);
        const uint32_t li = __ldg(&cp->len_inst);
        const int len = (int)(li & 63u);
        if (lane < len) {
            const uint32_t wmask = __ldg(&cp->wmask), zmask = __ldg(&cp->zmask), bmask = __ldg(&cp->bmask);
            const int32_t n = n0 + lane;
            const uint32_t missing = lane_missing(a, cp, bmask, lane);
            int32_t K[8];
            if constexpr (MODE != MODE_AA_EVEN) {
#pragma unroll
                for (int c = 0; c < 8; ++c) K[c] = __ldg(&cp->K[c]);
            }
            const int64_t step = a.step + (a.step_base ? *a.step_base : 0);
            T f[Q];
            const void* A = a.src;
#pragma unroll
            for (int q = 0; q < Q; ++q) {
                const bool has = !((missing >> q) & 1u);
                if constexpr (MODE == MODE_PULL) {
                    const int32_t s = nb_id(K, n0, lane, -X::a(q), -X::b(q), -X::r(q));
                    f[q] = has ? ld<S, Q, true>(A, a.stride, q, s) : T(0);
                } else if constexpr (MODE == MODE_AA_EVEN) {
                    f[q] = ld<S, Q>(A, a.stride, q, n);
                } else {
                    const int32_t s = nb_id(K, n0, lane, -X::a(q), -X::b(q), -X::r(q));
                    f[q] = has ? ld<S, Q>(A, a.stride, L::opp(q), s) : T(0);
                }
            }
            node_update<Q, S, MODE, DRY>(a, zmask ? __ldg(&cp->zslot0) : 0, f, missing, wmask, zmask, lane, n,
                                         (int)(li >> 8), step, mon);
            if constexpr (!DRY) {
                void* D = a.dst;
#pragma unroll
                for (int q = 0; q < Q; ++q) {
                    if constexpr (MODE == MODE_PULL) {
                        st<S, Q>(D, a.stride, q, n, f[q]);
                    } else if constexpr (MODE == MODE_AA_EVEN) {
                        st<S, Q>(D, a.stride, L::opp(q), n, f[q]);
                    } else {
                        // branch-free: an absent destination receives the value (bounced
                        // or initial) in the node's own opposite slot
                        if (q == 0) {
#pragma unroll
                            for (int c = 0; c < 8; ++c) K[c] = ld_fresh(&cp->K[c]);
                        }
                        const bool back = (missing >> L::opp(q)) & 1u;
                        const bool keep = !back || bounce_back_pop<Q>(L::opp(q), (wmask >> lane) & 1u, a.corr);
                        st_sel<S, Q>(D, (uint32_t)a.stride, q, nb_id(K, n0, lane, X::a(q), X::b(q), X::r(q)), back, n,
                                     keep ? f[q] : init_work<S, Q>(q));
                    }
                }
            }
        }
    }
    if constexpr (DRY) {
        if (part.mass) {
            // deterministic block reduction: warp shuffles then thread 0
            __shared__ double sm[4][8];
            __shared__ int sb[8];
            double m_mass = mon[0], m_in = mon[1], m_out = mon[2], m_maxu = mon[3];
            int m_bad = mon[4] != 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                m_mass += __shfl_down_sync(0xffffffffu, m_mass, o);
                m_in += __shfl_down_sync(0xffffffffu, m_in, o);
                m_out += __shfl_down_sync(0xffffffffu, m_out, o);
                m_maxu = fmax(m_maxu, __shfl_down_sync(0xffffffffu, m_maxu, o));
                m_bad |= __shfl_down_sync(0xffffffffu, m_bad, o);
            }
            const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
            if (lane == 0) { sm[0][w] = m_mass; sm[1][w] = m_in; sm[2][w] = m_out; sm[3][w] = m_maxu; sb[w] = m_bad; }
            __syncthreads();
            if (threadIdx.x == 0) {
                double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
                int b = 0;
                for (int i = 0; i < nw; ++i) { s0 += sm[0][i]; s1 += sm[1][i]; s2 += sm[2][i]; s3 = fmax(s3, sm[3][i]); b |= sb[i]; }
                part.mass[blockIdx.x] = s0; part.inflow[blockIdx.x] = s1; part.outflow[blockIdx.x] = s2;
                part.maxu[blockIdx.x] = s3; part.bad[blockIdx.x] = b;
            }
        }
    }
}

}  // namespace lbm
