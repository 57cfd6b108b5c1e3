// Synthetic vessel geometries (host C++, OpenMP): a faceted cylinder and a
// marching-tetrahedra mesher for unions of capsules.  They produce the seeded
// inputs of the benchmark workloads (straight pipe, Y-bifurcation, tortuous
// vessels, binary vascular tree) as closed triangle surfaces whose inlet and
// outlet faces are axis-aligned planes, as the reference's Zou-He routines
// require (Boundary.cpp:129-148, Simulation.cpp:952-1348).
//
// Meshing: the signed distance of the union (min over capsules, each capsule
// optionally clipped by its own half-space) is sampled on a grid of pitch h;
// every grid cube is split into the six tetrahedra around its main diagonal
// (a triangulation that matches across cube faces) and each tetrahedron
// contributes 0, 1 or 2 triangles.  Edge crossing points are computed from
// the edge's end points in a fixed order, so neighbouring tetrahedra produce
// identical vertices and the surface is closed.  Output order is fixed by the
// grid walk, independent of the thread count.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "internal.h"

namespace lbm {
namespace {

struct Capsule {
    double a[3], b[3], r;
    int cut_axis;
    double cut_pos, cut_sign;
    double lo[3], hi[3];   // bounding box of the capsule
};

inline double capsule_sdf(const Capsule& c, const double p[3]) {
    double ab[3] = {c.b[0] - c.a[0], c.b[1] - c.a[1], c.b[2] - c.a[2]};
    double ap[3] = {p[0] - c.a[0], p[1] - c.a[1], p[2] - c.a[2]};
    double l2 = ab[0] * ab[0] + ab[1] * ab[1] + ab[2] * ab[2];
    double t = l2 > 0 ? (ap[0] * ab[0] + ap[1] * ab[1] + ap[2] * ab[2]) / l2 : 0.0;
    t = std::min(1.0, std::max(0.0, t));
    double d[3] = {ap[0] - t * ab[0], ap[1] - t * ab[1], ap[2] - t * ab[2]};
    double s = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) - c.r;
    if (c.cut_axis >= 0) s = std::max(s, c.cut_sign * (p[c.cut_axis] - c.cut_pos));
    return s;
}

// Kuhn triangulation: corner index = x + 2y + 4z; six tetrahedra sharing 0-7.
const int kTets[6][4] = {{0, 1, 3, 7}, {0, 1, 5, 7}, {0, 2, 3, 7}, {0, 2, 6, 7}, {0, 4, 5, 7}, {0, 4, 6, 7}};

}  // namespace

lbm_status mesh_capsules(const double* seg, size_t nseg, const double lo[3], const double hi[3], double h,
                         uint64_t seed, TriVec& out) {
    if (!(h > 0) || nseg == 0) return fail(LBM_ERR_ARG, "mesh_capsules: need h > 0 and at least one capsule");
    std::vector<Capsule> caps(nseg);
    for (size_t i = 0; i < nseg; ++i) {
        const double* s = seg + 10 * i;
        Capsule& c = caps[i];
        for (int a = 0; a < 3; ++a) { c.a[a] = s[a]; c.b[a] = s[3 + a]; }
        c.r = s[6];
        c.cut_axis = (int)s[7];
        c.cut_pos = s[8];
        c.cut_sign = s[9];
        if (c.cut_axis > 2) return fail(LBM_ERR_ARG, "mesh_capsules: cut axis %d", c.cut_axis);
        for (int a = 0; a < 3; ++a) {
            c.lo[a] = std::min(c.a[a], c.b[a]) - c.r - 2 * h;
            c.hi[a] = std::max(c.a[a], c.b[a]) + c.r + 2 * h;
        }
    }
    std::mt19937_64 rng(seed);
    std::uniform_real_distribution<double> u01(0.0, 1.0);
    double org[3];
    for (int a = 0; a < 3; ++a) org[a] = lo[a] + h * (0.1 + 0.3 * u01(rng));
    long n[3];
    for (int a = 0; a < 3; ++a) {
        n[a] = (long)std::ceil((hi[a] - org[a]) / h) + 1;   // vertices per axis
        if (n[a] < 2) return fail(LBM_ERR_ARG, "mesh_capsules: empty box");
    }
    const long nx = n[0], ny = n[1], nz = n[2];
    // brick culling: capsules overlapping each (x,y) brick column of B cells
    const long B = 8;
    const long bx = (nx + B - 1) / B, by = (ny + B - 1) / B;
    std::vector<std::vector<int>> brick(bx * by);
    for (size_t i = 0; i < nseg; ++i) {
        const Capsule& c = caps[i];
        long i0 = std::max(0L, (long)std::floor((c.lo[0] - org[0]) / h) / B);
        long i1 = std::min(bx - 1, (long)std::floor((c.hi[0] - org[0]) / h) / B);
        long j0 = std::max(0L, (long)std::floor((c.lo[1] - org[1]) / h) / B);
        long j1 = std::min(by - 1, (long)std::floor((c.hi[1] - org[1]) / h) / B);
        for (long p = i0; p <= i1; ++p)
            for (long q = j0; q <= j1; ++q) brick[p * by + q].push_back((int)i);
    }
    auto eval_plane = [&](long k, std::vector<double>& plane) {
        double z = org[2] + k * h;
#pragma omp parallel for schedule(dynamic, 4)
        for (long i = 0; i < nx; ++i) {
            double p[3] = {org[0] + i * h, 0.0, z};
            for (long j = 0; j < ny; ++j) {
                p[1] = org[1] + j * h;
                double v = 1e30;
                for (int ci : brick[(i / B) * by + (j / B)]) {
                    const Capsule& c = caps[ci];
                    if (p[0] < c.lo[0] || p[0] > c.hi[0] || p[1] < c.lo[1] || p[1] > c.hi[1] || z < c.lo[2] || z > c.hi[2])
                        continue;
                    v = std::min(v, capsule_sdf(c, p));
                }
                if (v == 0.0) v = 1e-9 * h;   // no vertex exactly on the surface
                plane[i * ny + j] = v;
            }
        }
    };
    std::vector<double> p0(nx * ny), p1(nx * ny);
    eval_plane(0, p0);
    std::vector<TriVec> rows(nx - 1);
    for (long k = 0; k + 1 < nz; ++k) {
        eval_plane(k + 1, p1);
#pragma omp parallel for schedule(dynamic, 4)
        for (long i = 0; i < nx - 1; ++i) {
            TriVec& tv = rows[i];
            tv.clear();
            for (long j = 0; j < ny - 1; ++j) {
                double v[8];
                long gid[8];
                double pos[8][3];
                bool anyin = false, anyout = false;
                for (int c = 0; c < 8; ++c) {
                    long di = c & 1, dj = (c >> 1) & 1, dk = (c >> 2) & 1;
                    const std::vector<double>& pl = dk ? p1 : p0;
                    v[c] = pl[(i + di) * ny + (j + dj)];
                    gid[c] = ((k + dk) * nx + (i + di)) * ny + (j + dj);
                    pos[c][0] = org[0] + (i + di) * h;
                    pos[c][1] = org[1] + (j + dj) * h;
                    pos[c][2] = org[2] + (k + dk) * h;
                    if (v[c] < 0) anyin = true; else anyout = true;
                }
                if (!anyin || !anyout) continue;
                for (const auto& T : kTets) {
                    int ins[4], outs[4], ni = 0, no = 0;
                    for (int m = 0; m < 4; ++m) (v[T[m]] < 0 ? ins[ni++] : outs[no++]) = T[m];
                    if (ni == 0 || no == 0) continue;
                    auto edge = [&](int A, int Bc, double* q) {
                        int P = gid[A] < gid[Bc] ? A : Bc, Qc = gid[A] < gid[Bc] ? Bc : A;
                        double t = v[P] / (v[P] - v[Qc]);
                        for (int a = 0; a < 3; ++a) q[a] = pos[P][a] + t * (pos[Qc][a] - pos[P][a]);
                    };
                    double dir[3] = {0, 0, 0};
                    for (int m = 0; m < no; ++m) for (int a = 0; a < 3; ++a) dir[a] += pos[outs[m]][a] / no;
                    for (int m = 0; m < ni; ++m) for (int a = 0; a < 3; ++a) dir[a] -= pos[ins[m]][a] / ni;
                    auto emit = [&](const double* A, const double* Bv, const double* C) {
                        double e1[3] = {Bv[0] - A[0], Bv[1] - A[1], Bv[2] - A[2]};
                        double e2[3] = {C[0] - A[0], C[1] - A[1], C[2] - A[2]};
                        double nrm[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                                         e1[0] * e2[1] - e1[1] * e2[0]};
                        double len = std::sqrt(nrm[0] * nrm[0] + nrm[1] * nrm[1] + nrm[2] * nrm[2]);
                        if (!(len > 1e-300)) return;
                        const double* Pb = Bv;
                        const double* Pc = C;
                        if (nrm[0] * dir[0] + nrm[1] * dir[1] + nrm[2] * dir[2] < 0) {
                            std::swap(Pb, Pc);
                            for (double& x : nrm) x = -x;
                        }
                        lbm_tri t = {A[0], A[1], A[2], Pb[0], Pb[1], Pb[2], Pc[0], Pc[1], Pc[2],
                                     nrm[0] / len, nrm[1] / len, nrm[2] / len};
                        tv.push_back(t);
                    };
                    if (ni == 1 || no == 1) {
                        int lone = ni == 1 ? ins[0] : outs[0];
                        const int* others = ni == 1 ? outs : ins;
                        double q[3][3];
                        for (int m = 0; m < 3; ++m) edge(lone, others[m], q[m]);
                        emit(q[0], q[1], q[2]);
                    } else {
                        double q00[3], q01[3], q10[3], q11[3];
                        edge(ins[0], outs[0], q00);
                        edge(ins[0], outs[1], q01);
                        edge(ins[1], outs[0], q10);
                        edge(ins[1], outs[1], q11);
                        // quad q00-q01-q11-q10
                        emit(q00, q01, q11);
                        emit(q00, q11, q10);
                    }
                }
            }
        }
        for (auto& r : rows) out.insert(out.end(), r.begin(), r.end());
        std::swap(p0, p1);
    }
    return LBM_OK;
}

}  // namespace lbm

using namespace lbm;

extern "C" {

lbm_status lbm_synth_cylinder(double r, double len, int32_t segments, int32_t axis, const double c[3],
                              lbm_tri** tris, size_t* n) {
    if (!tris || !n || !c || segments < 3 || axis < 0 || axis > 2 || !(r > 0) || !(len > 0))
        return fail(LBM_ERR_ARG, "lbm_synth_cylinder: bad argument");
    clear_error();
    const int ua = (axis + 1) % 3, va = (axis + 2) % 3;
    const double pi = 3.14159265358979323846;
    std::vector<std::array<double, 3>> bot(segments), top(segments);
    for (int k = 0; k < segments; ++k) {
        double th = 2.0 * pi * (k + 0.5) / segments;
        std::array<double, 3> p;
        p[axis] = c[axis] - 0.5 * len;
        p[ua] = c[ua] + r * std::cos(th);
        p[va] = c[va] + r * std::sin(th);
        bot[k] = p;
        p[axis] = c[axis] + 0.5 * len;
        top[k] = p;
    }
    std::array<double, 3> cb, ct;
    cb[axis] = c[axis] - 0.5 * len; cb[ua] = c[ua]; cb[va] = c[va];
    ct = cb; ct[axis] = c[axis] + 0.5 * len;
    TriVec out;
    auto emit = [&](const std::array<double, 3>& A, const std::array<double, 3>& B, const std::array<double, 3>& C) {
        double e1[3] = {B[0] - A[0], B[1] - A[1], B[2] - A[2]};
        double e2[3] = {C[0] - A[0], C[1] - A[1], C[2] - A[2]};
        double nr[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        double l = std::sqrt(nr[0] * nr[0] + nr[1] * nr[1] + nr[2] * nr[2]);
        lbm_tri t = {A[0], A[1], A[2], B[0], B[1], B[2], C[0], C[1], C[2], nr[0] / l, nr[1] / l, nr[2] / l};
        out.push_back(t);
    };
    // (u,v,axis) is right-handed, so counter-clockwise in (u,v) seen from +axis
    for (int k = 0; k < segments; ++k) {
        int k1 = (k + 1) % segments;
        emit(bot[k], bot[k1], top[k1]);   // outward side
        emit(bot[k], top[k1], top[k]);
        emit(ct, top[k], top[k1]);        // +axis cap
        emit(cb, bot[k1], bot[k]);        // -axis cap
    }
    return to_c_array(out, tris, n);
}

lbm_status lbm_synth_capsules(const double* seg, size_t nseg, const double lo[3], const double hi[3], double h,
                              uint64_t seed, lbm_tri** tris, size_t* n) {
    if (!seg || !lo || !hi || !tris || !n) return fail(LBM_ERR_ARG, "lbm_synth_capsules: null argument");
    clear_error();
    return guarded("lbm_synth_capsules", [&] {
        TriVec out;
        lbm_status st = mesh_capsules(seg, nseg, lo, hi, h, seed, out);
        if (st != LBM_OK) return st;
        return to_c_array(out, tris, n);
    });
}

}  // extern "C"
