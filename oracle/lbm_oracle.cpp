// CPU oracle for the GB300 lattice Boltzmann engine.  TEST INFRASTRUCTURE ONLY.
//
// This file restates, in plain C++ (FP64, OpenMP, structure-of-arrays), the
// algorithm of the PV2013 reference solver for the path the engine accelerates:
//   * ASCII STL reading            GeometryReader.cpp:33-117
//   * bounding box and grid dims   ComplexGeometry.cpp:40-73, :178-207
//   * +z ray-parity voxelization   ComplexGeometry.cpp:264-330, :334-357, :431-506
//   * boundary-point extraction    ComplexGeometry.cpp:509-556
//   * plane-predicate selection    ComplexGeometry.cpp:559-638
//   * node typing / links / init   Subdomain.cpp:375-505, :618-634, Node.cpp:30-37
//   * BGK collision (D3Q19/D3Q27)  Simulation.cpp:21-179
//   * push streaming               Simulation.cpp:184-198, Node.cpp:16-20
//   * Zou-He velocity inlet        Boundary.cpp:87-148
//   * halfway bounce-back          Simulation.cpp:1353-1370, Node.cpp:121-125
//   * Zou-He pressure outlets      Simulation.cpp:952-1348
//   * step order                   Simulation.cpp:903-932
//
// It is the checker the GPU engine is compared against; only the test suite,
// the smoke check and the CPU-baseline leg of the benchmark load it.  Nothing
// in the engine links or calls it.  Build with -ffp-contract=off so that no
// multiply-add is fused: the reference's FP64 results depend on it.
//
// Parity pins: the voxelizer/classifier output is checked against the eight
// boundary-point VTK files shipped with the reference (PV2013.stl, spacing
// 0.1); the LBM step is checked against the reference's own Simulation
// methods compiled from its sources (oracle/ref), on small lattices.

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>
#include <limits>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {

// ---------------------------------------------------------------------------
// STL reader: GeometryReader.cpp:33-117.  Same token grammar: a facet is only
// accepted when "facet normal", "outer loop", three "vertex" lines, "endloop"
// and "endfacet" parse in sequence; a failed vertex line leaves the remaining
// corners at their previous values (the reference breaks out of its loop).
// Numbers go through std::istream >> double, like the reference.
// Returns the number of triangles, or -1 when the file cannot be opened.
int64_t orc_read_stl_ascii(const char* path, double** tris_out) {
    std::ifstream file(path);
    *tris_out = nullptr;
    if (!file.is_open()) return -1;
    std::vector<double> out;
    std::string line, facet, normal, outer, loop, vertex, endloop, endfacet;
    std::stringstream ss;
    double t[12] = {0};
    while (std::getline(file, line)) {
        ss.clear(); ss.str(line);
        ss >> facet >> normal >> t[9] >> t[10] >> t[11];
        if (ss.fail() || facet != "facet" || normal != "normal") continue;
        std::getline(file, line);
        ss.clear(); ss.str(line);
        ss >> outer >> loop;
        if (ss.fail() || outer != "outer" || loop != "loop") continue;
        for (int i = 0; i < 3; ++i) {
            std::getline(file, line);
            ss.clear(); ss.str(line);
            double x, y, z;
            ss >> vertex >> x >> y >> z;
            if (ss.fail() || vertex != "vertex") break;
            t[3 * i + 0] = x; t[3 * i + 1] = y; t[3 * i + 2] = z;
        }
        std::getline(file, line);
        ss.clear(); ss.str(line);
        ss >> endloop;
        if (ss.fail() || endloop != "endloop") continue;
        std::getline(file, line);
        ss.clear(); ss.str(line);
        ss >> endfacet;
        if (ss.fail() || endfacet != "endfacet") continue;
        out.insert(out.end(), t, t + 12);
    }
    int64_t n = (int64_t)(out.size() / 12);
    *tris_out = (double*)std::malloc(sizeof(double) * (out.size() ? out.size() : 1));
    if (!out.empty()) std::memcpy(*tris_out, out.data(), sizeof(double) * out.size());
    return n;
}

void orc_free(void* p) { std::free(p); }

// GetBoundingbox: ComplexGeometry.cpp:45-72.  bbox = {min_x,max_x,min_y,max_y,min_z,max_z}
void orc_bbox(const double* tris, int64_t n, double bbox[6], int dims[3], double spacing) {
    double mn[3] = {std::numeric_limits<double>::infinity(), std::numeric_limits<double>::infinity(),
                    std::numeric_limits<double>::infinity()};
    double mx[3] = {-mn[0], -mn[1], -mn[2]};
    for (int64_t t = 0; t < n; ++t) {
        const double* T = tris + 12 * t;
        for (int a = 0; a < 3; ++a) {
            mn[a] = std::min(mn[a], std::min(T[a], std::min(T[3 + a], T[6 + a])));
            mx[a] = std::max(mx[a], std::max(T[a], std::max(T[3 + a], T[6 + a])));
        }
    }
    for (int a = 0; a < 3; ++a) { bbox[2 * a] = mn[a]; bbox[2 * a + 1] = mx[a]; }
    for (int a = 0; a < 3; ++a) dims[a] = (int)std::ceil((bbox[2 * a + 1] - bbox[2 * a]) / spacing) + 1;
}

// isPointInsideTriangle: ComplexGeometry.cpp:264-281 (inclusive xy test).
static inline bool inside2d(double x, double y, const double* T) {
    double x1 = T[0], y1 = T[1], x2 = T[3], y2 = T[4], x3 = T[6], y3 = T[7];
    double d1 = ((x - x2) * (y1 - y2) - (y - y2) * (x1 - x2));
    double d2 = ((x - x3) * (y2 - y3) - (y - y3) * (x2 - x3));
    double d3 = ((x - x1) * (y3 - y1) - (y - y1) * (x3 - x1));
    bool hasNeg = (d1 < 0) || (d2 < 0) || (d3 < 0);
    bool hasPos = (d1 > 0) || (d2 > 0) || (d3 > 0);
    return !(hasNeg && hasPos);
}

// Ray start after adjustLineCoordinates case 0 (ComplexGeometry.cpp:337-355).
static inline void nudge_xy(double& sx, double& sy, const double* bb) {
    const double off = 0.01;
    if (sx == bb[0]) sx += off;
    if (sx == bb[1]) sx -= off;
    if (sy == bb[2]) sy += off;
    if (sy == bb[3]) sy -= off;
}

// One crossing test of countIntersectinsTriangle (ComplexGeometry.cpp:303-325)
// for a ray starting at (sx, sy, pz) with end (sx, sy, (pz + L) + 0.1).
static inline bool crosses(double sx, double sy, double pz, double L, const double* T) {
    const double thr = 1e-7;
    double ez = pz + L + 0.1;
    double dx = sx - sx, dy = sy - sy, dz = ez - pz;
    double t = ((T[0] - sx) * T[9] + (T[1] - sy) * T[10] + (T[2] - pz) * T[11]) /
               (dx * T[9] + dy * T[10] + dz * T[11]);
    if (t >= -thr && t <= 1 + thr) {
        double ix = sx + t * dx;
        double iy = sy + t * dy;
        return inside2d(ix, iy, T);
    }
    return false;
}

// labelPoints: ComplexGeometry.cpp:431-506.  flags[i*Ny*Nz + j*Nz + k] = 1 for
// Fluid, 0 for NotFluid.  Per column the xy inside test does not depend on z
// (the ray is vertical), so triangles are first filtered with the exact xy
// test at the ray's (x, y), then the crossing test runs for every z.  The
// filter is brute force over all triangles unless `binned` is set, in which
// case a conservative column bin of the triangle's xy box is used.
int orc_voxelize_cols(const double* tris, int64_t n, const double bbox[6], double spacing, const int dims[3],
                      int binned, const int cols[4], uint8_t* flags);

int orc_voxelize(const double* tris, int64_t n, const double bbox[6], double spacing, const int dims[3],
                 int binned, uint8_t* flags) {
    const int cols[4] = {0, dims[0], 0, dims[1]};
    return orc_voxelize_cols(tris, n, bbox, spacing, dims, binned, cols, flags);
}

// Same, restricted to the grid columns i in [cols[0], cols[1]), j in
// [cols[2], cols[3]) (other columns are left untouched); rays, nudges and ray
// length are those of the full grid.
int orc_voxelize_cols(const double* tris, int64_t n, const double bbox[6], double spacing, const int dims[3],
                      int binned, const int cols[4], uint8_t* flags) {
    const int Nx = dims[0], Ny = dims[1], Nz = dims[2];
    const double L = bbox[5] - bbox[4];
    std::vector<std::vector<int64_t>> bins;
    std::vector<int64_t> global;
    if (binned) {
        bins.resize((size_t)Nx * Ny);
        double ext = (bbox[1] - bbox[0]) + (bbox[3] - bbox[2]) + 1.0;
        for (int64_t t = 0; t < n; ++t) {
            const double* T = tris + 12 * t;
            double area2 = (T[3] - T[0]) * (T[7] - T[1]) - (T[4] - T[1]) * (T[6] - T[0]);
            if (std::fabs(area2) <= 1e-9 * ext * ext) { global.push_back(t); continue; }
            double xmn = std::min(T[0], std::min(T[3], T[6])), xmx = std::max(T[0], std::max(T[3], T[6]));
            double ymn = std::min(T[1], std::min(T[4], T[7])), ymx = std::max(T[1], std::max(T[4], T[7]));
            int pad = 2 + (int)std::ceil(0.01 / spacing);
            long i0 = (long)std::floor((xmn - bbox[0]) / spacing) - pad, i1 = (long)std::ceil((xmx - bbox[0]) / spacing) + pad;
            long j0 = (long)std::floor((ymn - bbox[2]) / spacing) - pad, j1 = (long)std::ceil((ymx - bbox[2]) / spacing) + pad;
            i0 = std::max(i0, 0L); j0 = std::max(j0, 0L);
            i1 = std::min(i1, (long)Nx - 1); j1 = std::min(j1, (long)Ny - 1);
            for (long i = i0; i <= i1; ++i)
                for (long j = j0; j <= j1; ++j) bins[(size_t)i * Ny + j].push_back(t);
        }
    }
#pragma omp parallel for schedule(dynamic, 4)
    for (long col = 0; col < (long)Nx * Ny; ++col) {
        int i = (int)(col / Ny), j = (int)(col % Ny);
        if (i < cols[0] || i >= cols[1] || j < cols[2] || j >= cols[3]) continue;
        double sx = bbox[0] + i * spacing, sy = bbox[2] + j * spacing;
        nudge_xy(sx, sy, bbox);
        std::vector<int64_t> cand;
        if (binned) {
            for (int64_t t : bins[col]) if (inside2d(sx, sy, tris + 12 * t)) cand.push_back(t);
            for (int64_t t : global) if (inside2d(sx, sy, tris + 12 * t)) cand.push_back(t);
        } else {
            for (int64_t t = 0; t < n; ++t) if (inside2d(sx, sy, tris + 12 * t)) cand.push_back(t);
        }
        uint8_t* out = flags + (size_t)col * Nz;
        for (int k = 0; k < Nz; ++k) {
            double pz = bbox[4] + k * spacing;
            int cnt = 0;
            for (int64_t t : cand) cnt += crosses(sx, sy, pz, L, tris + 12 * t) ? 1 : 0;
            out[k] = (cnt % 2 == 1) ? 1 : 0;
        }
    }
    return 0;
}

// findBoundaryPoints: ComplexGeometry.cpp:509-556.  Writes x-major linear
// indices of boundary points; returns their count (or the count needed when
// cap is too small).
int64_t orc_boundary_points(const uint8_t* flags, const int dims[3], int64_t* out, int64_t cap) {
    const int Nx = dims[0], Ny = dims[1], Nz = dims[2];
    int64_t cnt = 0;
    for (int i = 0; i < Nx; ++i)
        for (int j = 0; j < Ny; ++j)
            for (int k = 0; k < Nz; ++k) {
                size_t id = ((size_t)i * Ny + j) * Nz + k;
                if (!flags[id]) continue;
                bool b = false;
                for (int dx = -1; dx <= 1 && !b; ++dx)
                    for (int dy = -1; dy <= 1 && !b; ++dy)
                        for (int dz = -1; dz <= 1 && !b; ++dz) {
                            int a = i + dx, c = j + dy, e = k + dz;
                            if (a >= 0 && a < Nx && c >= 0 && c < Ny && e >= 0 && e < Nz &&
                                !flags[((size_t)a * Ny + c) * Nz + e])
                                b = true;
                        }
                if (i == 0 || i == Nx - 1 || j == 0 || j == Ny - 1 || k == 0 || k == Nz - 1) b = true;
                if (b) { if (cnt < cap) out[cnt] = (int64_t)id; ++cnt; }
            }
    return cnt;
}

// Plane predicate of getInOutBP (ComplexGeometry.cpp:579-638): the point's
// coordinate on `axis` lies within `tol` of the plane (compared in long double
// like the reference), and the other coordinates lie strictly inside the open
// ranges lo/hi (NaN disables a bound).  The plane constant is passed as decimal
// text so it is rounded to long double exactly as the reference's literal.
typedef struct {
    int axis;
    char plane[40];
    double tol;
    double lo[3];
    double hi[3];
} orc_predicate;

// For each boundary point (x-major indices) writes a bitmask of the matching
// predicates (bit p for predicate p).  Coordinates are min + i*spacing
// (generatePointsInBoundingBox).
void orc_classify(const int64_t* bidx, int64_t nb, const int dims[3], const double bbox[6], double spacing,
                  const orc_predicate* preds, int np, uint32_t* mask) {
    const int Ny = dims[1], Nz = dims[2];
    std::vector<long double> planes(np);
    for (int p = 0; p < np; ++p) planes[p] = std::strtold(preds[p].plane, nullptr);
    for (int64_t b = 0; b < nb; ++b) {
        int64_t id = bidx[b];
        int i = (int)(id / ((int64_t)Ny * Nz)), j = (int)((id / Nz) % Ny), k = (int)(id % Nz);
        double c[3] = {bbox[0] + i * spacing, bbox[2] + j * spacing, bbox[4] + k * spacing};
        uint32_t m = 0;
        for (int p = 0; p < np; ++p) {
            const orc_predicate& P = preds[p];
            long double v = c[P.axis];
            long double tol = P.tol;
            bool ok = std::abs(v - planes[p]) <= tol;
            for (int a = 0; a < 3 && ok; ++a) {
                if (a == P.axis) continue;
                long double w = c[a];
                if (!std::isnan(P.lo[a]) && !(P.lo[a] < w)) ok = false;
                if (!std::isnan(P.hi[a]) && !(w < P.hi[a])) ok = false;
            }
            if (ok) m |= (1u << p);
        }
        mask[b] = m;
    }
}

// ---------------------------------------------------------------------------
// LBM restatement.

// D3Q19 tables: LatticeModel.cpp:51-151 (rest population is index 18).
static const int C19[19][3] = {{1, 0, 0},  {-1, 0, 0}, {0, 1, 0},  {0, -1, 0}, {0, 0, 1},   {0, 0, -1}, {1, 1, 0},
                               {1, -1, 0}, {1, 0, 1},  {1, 0, -1}, {-1, 1, 0}, {-1, -1, 0}, {-1, 0, 1}, {-1, 0, -1},
                               {0, 1, 1},  {0, 1, -1}, {0, -1, 1}, {0, -1, -1}, {0, 0, 0}};
static const int OPP19[19] = {1, 0, 3, 2, 5, 4, 11, 10, 13, 12, 7, 6, 9, 8, 17, 16, 15, 14, 18};
// D3Q27 tables: LatticeModel.cpp:208-334 (rest population is index 0).
static const int C27[27][3] = {{0, 0, 0},   {1, 0, 0},   {-1, 0, 0},  {0, 1, 0},   {0, -1, 0},  {0, 0, 1},
                               {0, 0, -1},  {1, 1, 0},   {1, -1, 0},  {-1, 1, 0},  {-1, -1, 0}, {1, 0, 1},
                               {-1, 0, 1},  {1, 0, -1},  {-1, 0, -1}, {0, 1, 1},   {0, 1, -1},  {0, -1, 1},
                               {0, -1, -1}, {1, 1, 1},   {-1, -1, -1}, {1, 1, -1}, {-1, -1, 1}, {1, -1, 1},
                               {-1, 1, -1}, {1, -1, -1}, {-1, 1, 1}};
static const int OPP27[27] = {0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15,
                              20, 19, 22, 21, 24, 23, 26, 25};

static double weight(int Q, int q) {
    if (Q == 19) return q < 6 ? 2.0 / 36.0 : (q < 18 ? 1.0 / 36.0 : 12.0 / 36.0);
    if (q == 0) return 8.0 / 27.0;
    if (q < 7) return 2.0 / 27.0;
    if (q < 19) return 1.0 / 54.0;
    return 1.0 / 216.0;
}

// Boundary-condition kinds, named after the reference routine they restate.
enum {
    ORC_BC_WALL = 0,            // ApplyWallBc, Simulation.cpp:1353-1370
    ORC_BC_VEL_NEGY = 1,        // Boundary::ApplyBc D3Q19, Boundary.cpp:129-148 (unknowns -y)
    ORC_BC_PRESS_NEGY = 2,      // outlet list 1, Simulation.cpp:966-1019 (unknowns -y)
    ORC_BC_PRESS_POSY = 3,      // outlet list 2, Simulation.cpp:1029-1083 (unknowns +y)
    ORC_BC_PRESS_POSX = 4,      // outlet lists 3-5, Simulation.cpp:1093-1279 (unknowns +x, f10 in Nxz)
    ORC_BC_PRESS_POSZ = 5,      // outlet list 6, Simulation.cpp:1290-1346 (unknowns +z)
    ORC_BC_VEL_POSX_Q27 = 6,    // Boundary::ApplyBc D3Q27, Boundary.cpp:87-123 (unknowns +x)
    ORC_BC_FACE_VEL = 7,        // any face: the velocity routines above with the axes relabelled
    ORC_BC_FACE_PRESS = 8,      // any face: the pressure routines above with the axes relabelled
};

struct OrcSim {
    int Q, Nx, Ny, Nz;
    int64_t N;
    double tau, omega;
    std::vector<int32_t> grid;        // node id or -1, x-major
    std::vector<int32_t> nbr;         // N*Q neighbour (x + c_q) node id or -1
    std::vector<double> f, fnew;      // N*Q, node-major (f[n*Q+q])
    std::vector<double> rho, u;       // collision macroscopic values (N, 3N)
    // boundary lists in x-major order; kind per list
    std::vector<std::vector<int32_t>> lists;
    std::vector<int> kinds;
    std::vector<double> list_rho;                 // outlet density per list
    std::vector<int> list_face;                   // face of ORC_BC_FACE_* lists (0..5 = +x,-x,+y,-y,+z,-z unknowns)
    int corr;                                     // corrections: 1 bounce back every direction, 2 list nodes too
    std::vector<std::vector<double>> list_vel;    // inlet velocity per node (3 per node)
    std::vector<int32_t> wall;                    // wall node ids
    int64_t zero_hits;                            // times the streaming "f != 0" test fired
    int64_t steps;
};

// Builds the node set from a dense role grid (x-major, one int8 per point):
// -1 no node (NotFluid), 0 interior fluid, 1 wall, 2+l member of list l.  This
// is CreateNodes (Subdomain.cpp:375-478) with the first-match typing resolved
// by the caller, Connectivity (:481-505) and Initialize (f = w, :618-634).
void* orc_sim_create(int Q, const int dims[3], const int8_t* role, int nlists, const int* kinds,
                     const double* list_rho, double tau) {
    OrcSim* s = new OrcSim();
    s->Q = Q; s->Nx = dims[0]; s->Ny = dims[1]; s->Nz = dims[2];
    s->tau = tau; s->omega = 1.0 / tau;
    s->zero_hits = 0; s->steps = 0;
    size_t P = (size_t)s->Nx * s->Ny * s->Nz;
    s->grid.assign(P, -1);
    int64_t n = 0;
    s->lists.resize(nlists);
    s->kinds.assign(kinds, kinds + nlists);
    s->list_rho.assign(list_rho, list_rho + nlists);
    s->list_face.assign(nlists, 0);
    s->corr = 0;
    for (size_t p = 0; p < P; ++p) {
        if (role[p] < 0) continue;
        s->grid[p] = (int32_t)n;
        if (role[p] == 1) s->wall.push_back((int32_t)n);
        else if (role[p] >= 2) s->lists[role[p] - 2].push_back((int32_t)n);
        ++n;
    }
    s->N = n;
    const int (*C)[3] = Q == 19 ? C19 : C27;
    s->nbr.assign((size_t)n * Q, -1);
    for (int i = 0; i < s->Nx; ++i)
        for (int j = 0; j < s->Ny; ++j)
            for (int k = 0; k < s->Nz; ++k) {
                int32_t id = s->grid[((size_t)i * s->Ny + j) * s->Nz + k];
                if (id < 0) continue;
                for (int q = 0; q < Q; ++q) {
                    int a = i + C[q][0], b = j + C[q][1], c = k + C[q][2];
                    if (a < 0 || b < 0 || c < 0 || a >= s->Nx || b >= s->Ny || c >= s->Nz) continue;
                    s->nbr[(size_t)id * Q + q] = s->grid[((size_t)a * s->Ny + b) * s->Nz + c];
                }
            }
    s->f.resize((size_t)n * Q);
    s->fnew.assign((size_t)n * Q, 0.0);
    for (int64_t m = 0; m < n; ++m)
        for (int q = 0; q < Q; ++q) s->f[(size_t)m * Q + q] = weight(Q, q);
    s->rho.assign(n, 0.0);
    s->u.assign((size_t)n * 3, 0.0);
    s->list_vel.resize(nlists);
    for (int l = 0; l < nlists; ++l) {
        s->list_vel[l].assign(s->lists[l].size() * 3, 0.0);
        // Boundary ctor default inlet velocity (0,-0.1,0): Boundary.cpp:9
        for (size_t m = 0; m < s->lists[l].size(); ++m) s->list_vel[l][3 * m + 1] = -0.1;
    }
    return s;
}

void orc_sim_destroy(void* h) { delete (OrcSim*)h; }
int64_t orc_sim_nodes(void* h) { return ((OrcSim*)h)->N; }
int64_t orc_sim_list_size(void* h, int l) { return (int64_t)((OrcSim*)h)->lists[l].size(); }
int64_t orc_sim_zero_hits(void* h) { return ((OrcSim*)h)->zero_hits; }
int64_t orc_sim_wall_count(void* h) { return (int64_t)((OrcSim*)h)->wall.size(); }

void orc_sim_set_face(void* h, int l, int face) { ((OrcSim*)h)->list_face[l] = face; }

// Corrections of the reference's boundary handling (off by default = parity):
// bit 0 bounces back every moving direction (the reference's ApplyWallBc
// starts at direction 1, Simulation.cpp:1361), bit 1 also bounces back the
// missing populations of inlet/outlet nodes, before their Zou-He routine.
void orc_sim_set_corrections(void* h, int corr) { ((OrcSim*)h)->corr = corr; }

// Sets the inlet velocity of every node of list l (3 doubles per node, list order).
void orc_sim_set_velocity(void* h, int l, const double* uvw) {
    OrcSim* s = (OrcSim*)h;
    std::memcpy(s->list_vel[l].data(), uvw, sizeof(double) * s->list_vel[l].size());
}

// Collision: Simulation.cpp:21-179.
static void collide(OrcSim* s) {
    const int Q = s->Q;
    const double om = s->omega;
    const int (*C)[3] = Q == 19 ? C19 : C27;
#pragma omp parallel for schedule(static)
    for (int64_t n = 0; n < s->N; ++n) {
        const double* f = &s->f[(size_t)n * Q];
        double rho = 0.0;
        for (int q = 0; q < Q; ++q) rho += f[q];
        double ux, uy, uz;
        if (Q == 19) {
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
        s->rho[n] = rho;
        s->u[3 * n] = ux; s->u[3 * n + 1] = uy; s->u[3 * n + 2] = uz;
        double* fn = &s->fnew[(size_t)n * Q];
        for (int q = 0; q < Q; ++q) {
            double du = ux * C[q][0] + uy * C[q][1] + uz * C[q][2];
            double usq = ux * ux + uy * uy + uz * uz;
            double feq = weight(Q, q) * rho * (1.0 + 3.0 * du + 9.0 / 2.0 * du * du - 3.0 / 2.0 * usq);
            fn[q] = om * feq + (1.0 - om) * f[q];
        }
    }
}

// Streaming: Simulation.cpp:184-198 pushes f*[q] to the neighbour x + c_q when
// it exists and the pushing node's own f[q] is not exactly 0.0.  With all
// populations nonzero (checked here, counted in zero_hits) the push order does
// not matter, so the restatement pulls in parallel.
static void stream(OrcSim* s) {
    const int Q = s->Q;
    const int64_t N = s->N;
    int64_t zh = 0;
#pragma omp parallel for reduction(+ : zh) schedule(static)
    for (int64_t i = 0; i < N * Q; ++i) zh += (s->f[i] == 0.0 || s->fnew[i] == 0.0) ? 1 : 0;
    s->zero_hits += zh;
    const int* opp = Q == 19 ? OPP19 : OPP27;
#pragma omp parallel for schedule(static)
    for (int64_t n = 0; n < N; ++n)
        for (int q = 0; q < Q; ++q) {
            int32_t src = s->nbr[(size_t)n * Q + opp[q]];   // x - c_q
            if (src >= 0) s->f[(size_t)n * Q + q] = s->fnew[(size_t)src * Q + q];
        }
}

static void bc_vel_negy(double* f, const double* v) {
    // Boundary::ApplyBc D3Q19 (Boundary.cpp:129-148), m_inletVel = v
    double rhoN = (f[0] + f[1] + f[4] + f[5] + f[8] + f[9] + f[12] + f[13] + f[18] +
                   2.0 * (f[2] + f[6] + f[10] + f[14] + f[15])) / (1 + v[1]);
    double Nx = 0.5 * (f[0] + f[8] + f[9] - (f[1] + f[12] + f[13])) - (1.0 / 3.0) * rhoN * v[0];
    double Nz = 0.5 * (f[4] + f[8] + f[12] - (f[5] + f[9] + f[13])) - (1.0 / 3.0) * rhoN * v[2];
    f[3] = f[2] - (1.0 / 3.0) * rhoN * v[1];
    f[11] = f[6] + (1.0 / 6.0) * rhoN * (-v[1] - v[0]) + Nx;
    f[7] = f[10] + (1.0 / 6.0) * rhoN * (-v[1] + v[0]) - Nx;
    f[17] = f[14] + (1.0 / 6.0) * rhoN * (-v[1] - v[2]) + Nz;
    f[16] = f[15] + (1.0 / 6.0) * rhoN * (-v[1] + v[2]) - Nz;
}

static void bc_vel_posx_q27(double* f, const double* v) {
    // Boundary::ApplyBc D3Q27 (Boundary.cpp:87-123)
    double rho = ((f[0] + f[3] + f[4] + f[5] + f[6] + f[15] + f[16] + f[17] + f[18]) +
                  2 * (f[2] + f[9] + f[10] + f[12] + f[14] + f[20] + f[22] + f[24] + f[26])) / (1 - v[0]);
    double Ny = (1.0 / 6) * (f[3] + f[15] + f[16] - f[4] - f[17] - f[18]) - (1.0 / 9) * (rho * v[1]);
    double Nz = (1.0 / 6) * (f[5] + f[15] + f[17] - f[6] - f[16] - f[18]) - (1.0 / 9) * (rho * v[2]);
    f[1] = f[2] + (4 / 9.0) * rho * v[0];
    f[7] = f[10] + (1 / 9.0) * rho * (v[0] + v[1]) - Ny;
    f[8] = f[9] + (1 / 9.0) * rho * (v[0] - v[1]) + Ny;
    f[11] = f[14] + (1 / 9.0) * rho * (v[0] + v[2]) - Nz;
    f[13] = f[12] + (1 / 9.0) * rho * (v[0] - v[2]) + Nz;
    f[19] = f[20] + (1 / 36.0) * rho * (v[0] + v[1] + v[2]) - Ny - Nz;
    f[21] = f[22] + (1 / 36.0) * rho * (v[0] + v[1] - v[2]) - Ny + Nz;
    f[23] = f[24] + (1 / 36.0) * rho * (v[0] - v[1] + v[2]) + Ny - Nz;
    f[25] = f[26] + (1 / 36.0) * rho * (v[0] - v[1] - v[2]) + Ny + Nz;
}

// ApplyOutletBc bodies (Simulation.cpp:952-1348); the transverse velocities
// are 0 in every loop of the reference.
static void bc_press(double* f, int kind, double rho) {
    const double vx = 0.0, vz = 0.0, vyz = 0.0;
    if (kind == ORC_BC_PRESS_NEGY) {
        double vy = -1 + (1.0 / rho) * (f[0] + f[1] + f[4] + f[5] + f[8] + f[9] + f[12] + f[13] + f[18] +
                                        2.0 * (f[2] + f[6] + f[10] + f[14] + f[15]));
        double Nyx = 0.5 * (f[0] + f[8] + f[9] - (f[1] + f[12] + f[13])) - (1.0 / 3.0) * rho * vx;
        double Nyz = 0.5 * (f[4] + f[8] + f[12] - (f[5] + f[9] + f[13])) - (1.0 / 3.0) * rho * vz;
        f[3] = f[2] - (1.0 / 3.0) * rho * vy;
        f[11] = f[6] + (1.0 / 6.0) * rho * (-vx - vy) + Nyx;
        f[7] = f[10] + (1.0 / 6.0) * rho * (vx - vy) - Nyx;
        f[17] = f[14] + (1.0 / 6.0) * rho * (-vy - vz) + Nyz;
        f[16] = f[15] + (1.0 / 6.0) * rho * (-vy + vz) - Nyz;
    } else if (kind == ORC_BC_PRESS_POSY) {
        double vy = 1 - (1.0 / rho) * (f[0] + f[1] + f[4] + f[5] + f[8] + f[9] + f[12] + f[13] + f[18] +
                                       2.0 * (f[3] + f[7] + f[11] + f[16] + f[17]));
        double Nyx = 0.5 * (f[0] + f[8] + f[9] - (f[1] + f[12] + f[13])) - (1.0 / 3.0) * rho * vx;
        double Nyz = 0.5 * (f[4] + f[8] + f[12] - (f[5] + f[9] + f[13])) - (1.0 / 3.0) * rho * vz;
        f[2] = f[3] + (1.0 / 3.0) * rho * vy;
        f[6] = f[11] + (1.0 / 6.0) * rho * (vx + vy) - Nyx;
        f[10] = f[7] + (1.0 / 6.0) * rho * (-vx + vy) + Nyx;
        f[14] = f[17] + (1.0 / 6.0) * rho * (vy + vz) - Nyz;
        f[15] = f[16] + (1.0 / 6.0) * rho * (vy - vz) + Nyz;
    } else if (kind == ORC_BC_PRESS_POSX) {
        const double vy = vyz;
        double vxx = 1 - (1.0 / rho) * (f[2] + f[3] + f[4] + f[5] + f[14] + f[15] + f[16] + f[17] + f[18] +
                                        2.0 * (f[1] + f[10] + f[11] + f[12] + f[13]));
        double Nxy = 0.5 * (f[2] + f[14] + f[15] - (f[3] + f[16] + f[17])) - (1.0 / 3.0) * rho * vy;
        double Nxz = 0.5 * (f[4] + f[10] + f[14] - (f[5] + f[15] + f[17])) - (1.0 / 3.0) * rho * vz;
        f[0] = f[1] + (1.0 / 3.0) * rho * vxx;
        f[7] = f[10] + (1.0 / 6.0) * rho * (vxx - vy) + Nxy;
        f[6] = f[11] + (1.0 / 6.0) * rho * (vxx + vy) - Nxy;
        f[8] = f[13] + (1.0 / 6.0) * rho * (vxx + vz) - Nxz;
        f[9] = f[12] + (1.0 / 6.0) * rho * (vxx - vz) + Nxz;
    } else if (kind == ORC_BC_PRESS_POSZ) {
        const double vy = vyz;
        double vzz = 1 - (1.0 / rho) * (f[0] + f[1] + f[2] + f[3] + f[6] + f[7] + f[10] + f[11] + f[18] +
                                        2.0 * (f[5] + f[9] + f[13] + f[15] + f[17]));
        double Nzx = 0.5 * (f[0] + f[6] + f[7] - (f[1] + f[10] + f[11])) - (1.0 / 3.0) * rho * vx;
        double Nzy = 0.5 * (f[2] + f[6] + f[10] - (f[3] + f[7] + f[11])) - (1.0 / 3.0) * rho * vy;
        f[4] = f[5] + (1.0 / 3.0) * rho * vzz;
        f[8] = f[13] + (1.0 / 6.0) * rho * (vzz + vx) - Nzx;
        f[12] = f[9] + (1.0 / 6.0) * rho * (vzz - vx) + Nzx;
        f[14] = f[17] + (1.0 / 6.0) * rho * (vzz + vy) - Nzy;
        f[16] = f[15] + (1.0 / 6.0) * rho * (vzz - vy) + Nzy;
    }
}

// Zou-He on an axis-aligned face of any orientation.  The reference writes
// one routine per orientation (D3Q19: unknowns -y velocity, Boundary.cpp:
// 129-148; -y/+y/+x/+z pressure, Simulation.cpp:952-1348; D3Q27: +x velocity,
// Boundary.cpp:87-123); all share one form, restated here over the lattice
// tables for unknowns sg along axis A (face = 2A + (sg < 0)):
//   S0 = sum of f over c_A = 0, Sk = sum of f over c_A = -sg
//   velocity: rho = (S0 + 2 Sk) / (1 - sg u_A)
//   pressure: u_A = sg (1 - (S0 + 2 Sk) / rho), transverse u = 0
//   N_T = a sum_{c_A = 0} c_T f - b rho u_T  (a, b = 1/2, 1/3 for D3Q19 and
//         1/6, 1/9 for D3Q27, the reference's coefficients)
//   unknown f_q (c_A(q) = sg) = f_opp(q) + 6 w_q rho (c_q . u) - sum_T c_T(q) N_T
// (the f10 term of outlets 3-5, Simulation.cpp:1124-1129, is the reference's
// own and stays with ORC_BC_PRESS_POSX).
static void bc_face(int Q, double* f, int face, bool vel, const double* v, double rho_in) {
    const int (*C)[3] = Q == 19 ? C19 : C27;
    const int* opp = Q == 19 ? OPP19 : OPP27;
    const int A = face >> 1, sg = (face & 1) ? -1 : 1;
    double S0 = 0.0, Sk = 0.0;
    for (int q = 0; q < Q; ++q) {
        if (C[q][A] == 0) S0 += f[q];
        else if (C[q][A] == -sg) Sk += f[q];
    }
    double u[3] = {0.0, 0.0, 0.0}, rho;
    if (vel) {
        u[0] = v[0]; u[1] = v[1]; u[2] = v[2];
        rho = (S0 + 2.0 * Sk) / (1.0 - sg * u[A]);
    } else {
        rho = rho_in;
        u[A] = sg * (1.0 - (S0 + 2.0 * Sk) / rho);
    }
    const double a = Q == 19 ? 0.5 : 1.0 / 6.0, b = Q == 19 ? 1.0 / 3.0 : 1.0 / 9.0;
    double N[3] = {0.0, 0.0, 0.0};
    for (int t = 0; t < 3; ++t) {
        if (t == A) continue;
        double m = 0.0;
        for (int q = 0; q < Q; ++q)
            if (C[q][A] == 0 && C[q][t] != 0) m += C[q][t] > 0 ? f[q] : -f[q];
        N[t] = a * m - b * rho * u[t];
    }
    for (int q = 0; q < Q; ++q) {
        if (C[q][A] != sg) continue;
        double cu = C[q][0] * u[0] + C[q][1] * u[1] + C[q][2] * u[2];
        double v2 = f[opp[q]] + 6.0 * weight(Q, q) * rho * cu;
        for (int t = 0; t < 3; ++t)
            if (t != A && C[q][t] != 0) v2 -= C[q][t] * N[t];
        f[q] = v2;
    }
}

// One node, any kind (tests): f (Q values) updated in place.
void orc_zou_he(int Q, int kind, int face, double* f, const double* v, double rho) {
    if (kind == ORC_BC_VEL_NEGY) bc_vel_negy(f, v);
    else if (kind == ORC_BC_VEL_POSX_Q27) bc_vel_posx_q27(f, v);
    else if (kind == ORC_BC_FACE_VEL) bc_face(Q, f, face, true, v, 0.0);
    else if (kind == ORC_BC_FACE_PRESS) bc_face(Q, f, face, false, nullptr, rho);
    else bc_press(f, kind, rho);
}

// One Iterate() body (Simulation.cpp:909-915): Collision, Streaming,
// ApplyZouHeBc (velocity lists), ApplyWallBc, ApplyOutletBc (pressure lists).
void orc_sim_step(void* h, int nsteps) {
    OrcSim* s = (OrcSim*)h;
    const int Q = s->Q;
    const int* opp = Q == 19 ? OPP19 : OPP27;
    const int d0 = (s->corr & 1) ? 0 : 1;
    auto bounce = [&](int32_t n) {
        for (int d = d0; d < Q; ++d)
            if (s->nbr[(size_t)n * Q + d] < 0) s->f[(size_t)n * Q + opp[d]] = s->fnew[(size_t)n * Q + d];
    };
    for (int it = 0; it < nsteps; ++it) {
        collide(s);
        stream(s);
        if (s->corr & 2)
            for (size_t l = 0; l < s->lists.size(); ++l)
                for (int32_t n : s->lists[l]) bounce(n);
        for (size_t l = 0; l < s->lists.size(); ++l) {
            int k = s->kinds[l];
            if (k != ORC_BC_VEL_NEGY && k != ORC_BC_VEL_POSX_Q27 && k != ORC_BC_FACE_VEL) continue;
            for (size_t m = 0; m < s->lists[l].size(); ++m) {
                double* f = &s->f[(size_t)s->lists[l][m] * Q];
                if (k == ORC_BC_VEL_NEGY) bc_vel_negy(f, &s->list_vel[l][3 * m]);
                else if (k == ORC_BC_VEL_POSX_Q27) bc_vel_posx_q27(f, &s->list_vel[l][3 * m]);
                else bc_face(Q, f, s->list_face[l], true, &s->list_vel[l][3 * m], 0.0);
            }
        }
#pragma omp parallel for schedule(static)
        for (size_t m = 0; m < s->wall.size(); ++m) bounce(s->wall[m]);
        for (size_t l = 0; l < s->lists.size(); ++l) {
            int k = s->kinds[l];
            if (k == ORC_BC_FACE_PRESS) {
                for (size_t m = 0; m < s->lists[l].size(); ++m)
                    bc_face(Q, &s->f[(size_t)s->lists[l][m] * Q], s->list_face[l], false, nullptr, s->list_rho[l]);
                continue;
            }
            if (k < ORC_BC_PRESS_NEGY || k > ORC_BC_PRESS_POSZ) continue;
            for (size_t m = 0; m < s->lists[l].size(); ++m)
                bc_press(&s->f[(size_t)s->lists[l][m] * Q], k, s->list_rho[l]);
        }
        s->steps++;
    }
}

// Wall shear stress of every wall node, wall-list order, from the velocities
// of the last collision (ComputeVelocityGradientAtWall and
// ComputeWallShearStress, Simulation.cpp:1374-1421).
void orc_sim_wss(void* h, double* out) {
    OrcSim* s = (OrcSim*)h;
    const int Q = s->Q;
    const double mu = 1.0 / 6.0 * (2.0 * s->tau - 1.0);
    for (size_t m = 0; m < s->wall.size(); ++m) {
        const int32_t n = s->wall[m];
        double g[3] = {0.0, 0.0, 0.0};
        int cnt = 0;
        for (int d = 0; d < Q; ++d) {
            const int32_t nb = s->nbr[(size_t)n * Q + d];
            if (nb < 0) continue;
            for (int k = 0; k < 3; ++k) g[k] += (s->u[3 * (size_t)nb + k] - s->u[3 * (size_t)n + k]);
            ++cnt;
        }
        if (cnt > 0)
            for (int k = 0; k < 3; ++k) g[k] /= cnt;
        const double s0 = mu * g[0], s1 = mu * g[1], s2 = mu * g[2];
        out[m] = std::sqrt(s0 * s0 + s1 * s1 + s2 * s2);
    }
}

// Copies populations (N*Q, node order), and optionally the macroscopic values
// of the last collision (rho N, u 3N).
void orc_sim_get(void* h, double* f, double* rho, double* u) {
    OrcSim* s = (OrcSim*)h;
    if (f) std::memcpy(f, s->f.data(), sizeof(double) * s->f.size());
    if (rho) std::memcpy(rho, s->rho.data(), sizeof(double) * s->rho.size());
    if (u) std::memcpy(u, s->u.data(), sizeof(double) * s->u.size());
}

void orc_sim_set_f(void* h, const double* f) {
    OrcSim* s = (OrcSim*)h;
    std::memcpy(s->f.data(), f, sizeof(double) * s->f.size());
}

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

}  // extern "C"
