// pv2013.hpp - header-only C++ facade over the C ABI (lbm_gb300.h) with the
// class names and constructor signatures of the PV2013 solver, so its driver
// (LBM.cpp:253-256)
//
//     auto velSet = std::make_shared<LatticeModel>();
//     Geometry Geometry("PV2013.stl", velSet, spacing, mdepth);
//     SubDomain SubDomain(Geometry);
//     Simulation(SubDomain, tau, pressure, dt);
//
// compiles unchanged against it (namespace pv2013) and runs on the GPU.
// Differences that a caller can see:
//   * Geometry's public lists hold the same points, in the same order, but are
//     filled on first access (they are copies of device data);
//   * Simulation's constructor runs the reference's 20000 iterations
//     (Simulation.cpp:908) only when `iterations` is left at its default;
//     Iterate(n) advances n more steps; Fields() returns rho, u, f;
//   * errors throw pv2013::Error carrying the lbm_status and message (the
//     reference printed and continued).
#pragma once
#include <cmath>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../lbm_gb300.h"

namespace pv2013 {

struct Error : std::runtime_error {
    lbm_status status;
    Error(lbm_status s, const std::string& what) : std::runtime_error(what), status(s) {}
};

inline void check(lbm_status s) {
    if (s != LBM_OK) throw Error(s, std::string(lbm_status_string(s)) + ": " + lbm_last_error());
}

// Point of the reference's Struct.h:41-64 (coordinates only).
struct Point {
    double x, y, z;
};

// Velocity sets of LatticeModel.cpp (D3Q19 :51-151, D3Q27 :208-334).
class LatticeModel {
public:
    explicit LatticeModel(int Q = 19) : Q_(Q) {
        if (Q != 19 && Q != 27) throw Error(LBM_ERR_ARG, "LatticeModel: Q must be 19 or 27");
    }
    int Get_nDirections() const { return Q_; }
    int Get_nDimensions() const { return 3; }
    double Get_c_square(int = 0) const { return 1.0 / 3.0; }
    double GetWeight(int d) const {
        if (Q_ == 19) return d < 6 ? 2.0 / 36.0 : (d < 18 ? 1.0 / 36.0 : 12.0 / 36.0);
        return d == 0 ? 8.0 / 27.0 : (d < 7 ? 2.0 / 27.0 : (d < 19 ? 1.0 / 54.0 : 1.0 / 216.0));
    }
    std::vector<int> GetDirection(int d) const {
        static const int c19[19][3] = {{1, 0, 0},  {-1, 0, 0}, {0, 1, 0},   {0, -1, 0},  {0, 0, 1},  {0, 0, -1}, {1, 1, 0},
                                       {1, -1, 0}, {1, 0, 1},  {1, 0, -1},  {-1, 1, 0},  {-1, -1, 0}, {-1, 0, 1}, {-1, 0, -1},
                                       {0, 1, 1},  {0, 1, -1}, {0, -1, 1},  {0, -1, -1}, {0, 0, 0}};
        static const int c27[27][3] = {{0, 0, 0},   {1, 0, 0},    {-1, 0, 0}, {0, 1, 0},   {0, -1, 0},  {0, 0, 1},
                                       {0, 0, -1},  {1, 1, 0},    {1, -1, 0}, {-1, 1, 0},  {-1, -1, 0}, {1, 0, 1},
                                       {-1, 0, 1},  {1, 0, -1},   {-1, 0, -1}, {0, 1, 1},  {0, 1, -1},  {0, -1, 1},
                                       {0, -1, -1}, {1, 1, 1},    {-1, -1, -1}, {1, 1, -1}, {-1, -1, 1}, {1, -1, 1},
                                       {-1, 1, -1}, {1, -1, -1},  {-1, 1, 1}};
        const int* v = Q_ == 19 ? c19[d] : c27[d];
        return {v[0], v[1], v[2]};
    }
    int OppositeDirection(int d) const {
        static const int o19[19] = {1, 0, 3, 2, 5, 4, 11, 10, 13, 12, 7, 6, 9, 8, 17, 16, 15, 14, 18};
        static const int o27[27] = {0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15,
                                    20, 19, 22, 21, 24, 23, 26, 25};
        return Q_ == 19 ? o19[d] : o27[d];
    }

private:
    int Q_;
};
using VelocitySet = LatticeModel;

struct BoundingBox {
    double min_x, max_x, min_y, max_y, min_z, max_z;
};

// Geometry(FileName, velSet, spacing, mdepth): ComplexGeometry.cpp:7-32.
// The predicates default to the reference's PV2013 preset (getInOutBP).
class Geometry {
public:
    Geometry(const std::string& FileName, std::shared_ptr<LatticeModel> velSet, double spacing, int mdepth = 1,
             std::vector<lbm_bc_predicate> preds = {}, const lbm_grid* grid = nullptr)
        : velSet_(std::move(velSet)), spacing(spacing), maxDepth(mdepth) {
        lbm_tri* tris = nullptr;
        size_t n = 0;
        // parsed on the GPU (the same triangles as the host reader, which takes
        // over for files outside the canonical facet layout)
        check(lbm_stl_read_ascii_device(FileName.c_str(), nullptr, &tris, &n, nullptr));
        std::unique_ptr<lbm_tri, void (*)(void*)> hold(tris, lbm_free);
        if (preds.empty()) {
            size_t np = 0;
            check(lbm_predicates_pv2013(nullptr, 0, &np));
            preds.resize(np);
            check(lbm_predicates_pv2013(preds.data(), np, &np));
        }
        lbm_geometry* g = nullptr;
        check(lbm_geometry_create(tris, n, spacing, grid, preds.data(), preds.size(), nullptr, &g));
        handle_.reset(g, lbm_geometry_destroy);
        check(lbm_geometry_info_get(g, &info_));
        GeomSize = {info_.dims[0], info_.dims[1], info_.dims[2]};
        boundingbox = {info_.bbox[0], info_.bbox[1], info_.bbox[2], info_.bbox[3], info_.bbox[4], info_.bbox[5]};
        globalNumtris = (int)n;
    }

    std::vector<int> GeomSize;
    BoundingBox boundingbox;
    int globalNumtris = 0;
    std::shared_ptr<LatticeModel> velSet_;
    double spacing;
    int maxDepth;

    // the reference's public point lists (ComplexGeometry.h:40-48)
    std::vector<Point> boundaryPoints() const { return points(LBM_LIST_BOUNDARY); }
    std::vector<Point> InletboundaryPoints() const { return points(0); }
    std::vector<Point> OutletboundaryPoints(int k) const { return points(k); }
    std::vector<Point> WallboundaryPoints() const { return points(LBM_LIST_WALL); }
    // Fluid/NotFluid field, x-major
    std::vector<uint8_t> flags() const {
        std::vector<uint8_t> f((size_t)info_.n_points);
        check(lbm_geometry_flags(handle_.get(), f.data(), f.size()));
        return f;
    }
    const lbm_geometry_info& info() const { return info_; }
    lbm_geometry* handle() const { return handle_.get(); }

private:
    std::vector<Point> points(int list) const {
        size_t n = 0;
        check(lbm_geometry_list(handle_.get(), list, nullptr, 0, &n));
        std::vector<int64_t> idx(n);
        if (n) check(lbm_geometry_list(handle_.get(), list, idx.data(), n, &n));
        std::vector<Point> out(n);
        const int64_t Ny = info_.dims[1], Nz = info_.dims[2];
        for (size_t m = 0; m < n; ++m) {
            const int64_t i = idx[m] / (Ny * Nz), j = (idx[m] / Nz) % Ny, k = idx[m] % Nz;
            out[m] = {info_.bbox[0] + i * spacing, info_.bbox[2] + j * spacing, info_.bbox[4] + k * spacing};
        }
        return out;
    }
    std::shared_ptr<lbm_geometry> handle_;
    lbm_geometry_info info_{};
};

// SubDomain(Geometry&): Subdomain.cpp:3-33.  Holds the lattice settings; the
// device lattice is built by Simulation.  The boundary routines default to the
// reference's: list 0 velocity inlet (0,-0.1,0) (Boundary.cpp:9, :129-148),
// lists 1-6 pressure outlets at rho 1.01 (Simulation.cpp:952-1348).
class SubDomain {
public:
    explicit SubDomain(Geometry& g) : Geometry_(&g) {
        params.Q = g.velSet_ ? g.velSet_->Get_nDirections() : 19;
        params.precision = LBM_F64;
        params.pattern = LBM_PULL;
        params.warps_per_block = 0;
        params.run_axis = 0;
        params.staging = 1;
        const int kinds[7] = {LBM_BC_VEL_NEGY,   LBM_BC_PRESS_NEGY, LBM_BC_PRESS_POSY, LBM_BC_PRESS_POSX,
                              LBM_BC_PRESS_POSX, LBM_BC_PRESS_POSX, LBM_BC_PRESS_POSZ};
        if (params.Q == 19) {
            for (int l = 0; l < 7; ++l) {
                lbm_list_bc b{};
                b.list_id = l;
                b.kind = kinds[l];
                b.rho = 1.01;
                b.dir[1] = -1.0;
                bcs.push_back(b);
            }
            inlet_speed = 0.1;
        }
    }
    Geometry* Geometry_;
    lbm_sim_params params{};
    std::vector<lbm_list_bc> bcs;
    double inlet_speed = 0.0;
};

// Simulation(SubDomain&, tau, pressure, dt): Simulation.cpp:3-13, 903-932.
class Simulation {
public:
    static constexpr long kReferenceIterations = 20000;

    Simulation(SubDomain& sd, double tau, double pressure, double dt, long iterations = kReferenceIterations)
        : m_relaxation(tau), pressure_(pressure), m_dt(dt), m_omega(1.0 / tau) {
        lbm_sim_params p = sd.params;
        p.tau = tau;
        std::vector<lbm_list_bc> bcs = sd.bcs;
        amp_ = {sd.inlet_speed};
        for (auto& b : bcs)
            if (b.kind == LBM_BC_VEL_NEGY || b.kind == LBM_BC_VEL_POSX) { b.amp = amp_.data(); b.amp_len = 1; }
        p.bcs = bcs.data();
        p.nbcs = bcs.size();
        lbm_sim* s = nullptr;
        check(lbm_sim_create(sd.Geometry_->handle(), &p, nullptr, &s));
        sim_.reset(s, lbm_sim_destroy);
        if (iterations > 0) Iterate(iterations);
    }

    // Advances n iterations (Collision .. ApplyOutletBc per step).
    void Iterate(long n) { check(lbm_sim_step(sim_.get(), n, LBM_STEP_GRAPH, nullptr)); }

    struct Fields {
        std::vector<double> rho, u, f;
    };
    Fields GetFields(bool with_f = false) {
        lbm_sim_info inf;
        check(lbm_sim_info_get(sim_.get(), &inf));
        Fields F;
        F.rho.resize(inf.n_nodes);
        F.u.resize(3 * inf.n_nodes);
        if (with_f) F.f.resize((size_t)inf.n_nodes * inf.Q);
        check(lbm_sim_fields(sim_.get(), F.rho.data(), F.u.data(), with_f ? F.f.data() : nullptr, inf.n_nodes, nullptr));
        return F;
    }
    lbm_monitors Monitors() {
        lbm_monitors m;
        check(lbm_sim_monitors(sim_.get(), &m, nullptr));
        return m;
    }
    lbm_sim* handle() const { return sim_.get(); }

    double m_relaxation, pressure_, m_dt, m_omega;

private:
    std::vector<double> amp_;
    std::shared_ptr<lbm_sim> sim_;
};

}  // namespace pv2013
