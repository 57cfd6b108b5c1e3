// Driver for the PV2013 reference compiled from its own sources (staged and
// patched by stage_ref.py).  TEST INFRASTRUCTURE ONLY: it produces the
// reference's outputs on small inputs so the CPU restatement
// (oracle/lbm_oracle.cpp) and the golden fixtures can be checked against them.
//
// It calls the reference's public members in the order of its constructors:
//   Geometry: GetBoundingbox, DistributeTriangles, generatePointsInBoundingBox,
//             labelPoints, findBoundaryPoints, getInOutBP (or harness
//             predicates), excludeInletOutlet    (ComplexGeometry.cpp:7-32)
//   SubDomain(Geometry&)                          (Subdomain.cpp:3-33)
//   Simulation(SubDomain&, tau, pressure, dt) with zero iterations, then per
//   step: Collision, Streaming, ApplyZouHeBc, ApplyWallBc, ApplyOutletBc
//                                                 (Simulation.cpp:909-915)
//
// Usage: pv2013_ref <run file>.  The run file is "key value..." lines:
//   stl <path>                 ASCII STL read by Reader::readSTLASCII
//   spacing <h>
//   box <minx> <miny> <minz> <Nx> <Ny> <Nz>   overrides the tight bounding box
//   preset pv2013              use the reference's own getInOutBP predicates
//   pred <list 0..6> <axis> <plane> <tol> <lox> <hix> <loy> <hiy> <loz> <hiz>
//                              plane predicate in getInOutBP form (nan = no bound);
//                              list 0 = inlet, 1..6 = outlet lists 1..6
//   vtk <dir>                  write the eight boundary-point VTK files there
//   tau <t>   outlet_rho <r>   steps <n>
//   warmup <n>                 untimed iterations before the <steps> timed ones
//                              (the outputs are the state after all of them)
//   inlet_dir <dx> <dy> <dz>   inlet_profile <file of doubles, one per inlet node>
//   amp_table <file of doubles> amplitude a(t) = table[t mod len]; the inlet
//                              velocity of node m at step t is (a*p_m)*dir
//   flags <file>               node-type field (uint8, x-major, 1 = Fluid) of the box
//                              grid, used instead of labelPoints (for timing the
//                              step loop on a sample of a large geometry)
//   wss 1                      after the steps, ComputeVelocityGradientAtWall and
//                              ComputeWallShearStress (Simulation.cpp:1374-1421):
//                              writes <prefix>.wss and <prefix>.wallnodes (grid
//                              indices), in WallBoundaryNode_ order
//   stl_binary <path>          only reads the binary STL with Reader::readSTLBinary
//                              (GeometryReader.cpp:119-176) and writes <prefix>.tris
//                              (12 doubles per triangle, Triangle's field order)
//   pulsatile <n>              only evaluates the reference's inlet waveform (the
//                              Pulsatile polynomials of pulsatile.h, selected as in
//                              Simulation::getInletVelocity, Simulation.cpp:875-900)
//                              at x = 0.9 s / n ... and writes <prefix>.pulsatile
//   out <prefix>               writes <prefix>.flags, .lists, .nodes, .f, .rho, .u
#include "ComplexGeometry.h"
#include "GeometryReader.h"
#include "LatticeModel.h"
#include "Simulation.h"
#include "Subdomain.h"
#include "pulsatile.h"

#include <chrono>
#include <cstdio>
#include <fstream>
#include <sstream>

int g_oracle_steps = 0;
double g_oracle_outlet_rho = 1.01;

namespace {

struct Pred {
    int list, axis;
    long double plane;
    long double tol;
    double lo[3], hi[3];
};

std::vector<double> read_doubles(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    std::vector<double> v;
    double d;
    while (f.read(reinterpret_cast<char*>(&d), sizeof d)) v.push_back(d);
    return v;
}

template <class T>
void write_vec(const std::string& path, const std::vector<T>& v) {
    std::ofstream f(path, std::ios::binary);
    f.write(reinterpret_cast<const char*>(v.data()), (std::streamsize)(v.size() * sizeof(T)));
}

bool pred_match(const Pred& p, const Point& pt) {
    long double c[3] = {pt.x, pt.y, pt.z};
    if (!(std::abs(c[p.axis] - p.plane) <= p.tol)) return false;
    for (int a = 0; a < 3; ++a) {
        if (a == p.axis) continue;
        if (!std::isnan(p.lo[a]) && !(p.lo[a] < c[a])) return false;
        if (!std::isnan(p.hi[a]) && !(c[a] < p.hi[a])) return false;
    }
    return true;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) { std::fprintf(stderr, "usage: %s <run file>\n", argv[0]); return 2; }
    MPI_Init(&argc, &argv);
    std::ifstream run(argv[1]);
    std::string line, stl, out = "ref", vtkdir, profile_path, amp_path, flags_path, stl_binary;
    bool want_wss = false;
    int pulsatile_n = 0;
    double spacing = 1.0, tau = 0.8, box[3] = {0, 0, 0};
    int dims[3] = {0, 0, 0}, steps = 0, warmup = 0;
    bool have_box = false, preset = false;
    double idir[3] = {0.0, -1.0, 0.0};
    std::vector<Pred> preds;
    while (std::getline(run, line)) {
        std::istringstream ss(line);
        std::string key;
        if (!(ss >> key) || key[0] == '#') continue;
        if (key == "stl") ss >> stl;
        else if (key == "spacing") ss >> spacing;
        else if (key == "box") { ss >> box[0] >> box[1] >> box[2] >> dims[0] >> dims[1] >> dims[2]; have_box = true; }
        else if (key == "preset") { std::string p; ss >> p; preset = (p == "pv2013"); }
        else if (key == "pred") {
            Pred p; std::string plane, tol, v[6];
            ss >> p.list >> p.axis >> plane >> tol >> v[0] >> v[1] >> v[2] >> v[3] >> v[4] >> v[5];
            p.plane = std::strtold(plane.c_str(), nullptr);
            p.tol = (long double)std::strtod(tol.c_str(), nullptr);
            for (int a = 0; a < 3; ++a) { p.lo[a] = std::strtod(v[2 * a].c_str(), nullptr); p.hi[a] = std::strtod(v[2 * a + 1].c_str(), nullptr); }
            preds.push_back(p);
        }
        else if (key == "vtk") ss >> vtkdir;
        else if (key == "tau") ss >> tau;
        else if (key == "outlet_rho") ss >> g_oracle_outlet_rho;
        else if (key == "steps") ss >> steps;
        else if (key == "warmup") ss >> warmup;
        else if (key == "inlet_dir") ss >> idir[0] >> idir[1] >> idir[2];
        else if (key == "inlet_profile") ss >> profile_path;
        else if (key == "amp_table") ss >> amp_path;
        else if (key == "out") ss >> out;
        else if (key == "flags") ss >> flags_path;
        else if (key == "wss") { int w = 0; ss >> w; want_wss = w != 0; }
        else if (key == "stl_binary") ss >> stl_binary;
        else if (key == "pulsatile") ss >> pulsatile_n;
    }
    if (pulsatile_n > 0) {
        Pulsatile P;
        std::vector<double> v;
        for (int s = 0; s < pulsatile_n; ++s) {
            const double x = P.period * s / pulsatile_n;
            const double nx = std::fmod(x, P.period);
            double vel = 0.0;
            if (nx >= 0 && nx < 0.1 * P.period) vel = P.InletVelequation1(nx);
            else if (nx >= 0.1 * P.period && nx < 0.3 * P.period) vel = P.InletVelequation2(nx);
            else if (nx >= 0.3 * P.period && nx < 0.9 * P.period) vel = P.InletVelequation3(nx);
            v.push_back(vel);
        }
        write_vec(out + ".pulsatile", v);
        MPI_Finalize();
        return 0;
    }
    if (!stl_binary.empty()) {
        Reader R;
        const std::vector<Triangle> tris = R.readSTLBinary(stl_binary);
        std::vector<double> v;
        for (const Triangle& t : tris)
            for (double x : {t.x1, t.y1, t.z1, t.x2, t.y2, t.z2, t.x3, t.y3, t.z3, t.nx, t.ny, t.nz}) v.push_back(x);
        write_vec(out + ".tris", v);
        MPI_Finalize();
        return 0;
    }

    auto t0 = std::chrono::steady_clock::now();
    std::shared_ptr<LatticeModel> velSet = std::make_shared<LatticeModel>();
    Geometry G;
    MPI_Comm_rank(MPI_COMM_WORLD, &G.myrank);
    MPI_Comm_size(MPI_COMM_WORLD, &G.num_procs);
    G.stlFileName = stl;
    G.velSet_ = velSet;
    G.spacing = spacing;
    G.maxDepth = 1;
    G.GetBoundingbox();
    if (have_box) {
        G.boundingbox = {box[0], box[0] + (dims[0] - 1) * spacing, box[1], box[1] + (dims[1] - 1) * spacing,
                         box[2], box[2] + (dims[2] - 1) * spacing};
    }
    G.DistributeTriangles();
    G.generatePointsInBoundingBox();
    if (have_box && (G.GeomSize[0] != dims[0] || G.GeomSize[1] != dims[1] || G.GeomSize[2] != dims[2])) {
        std::fprintf(stderr, "box override gives grid %d %d %d\n", G.GeomSize[0], G.GeomSize[1], G.GeomSize[2]);
        return 3;
    }
    if (flags_path.empty()) {
        G.labelPoints();
    } else {
        std::ifstream ff(flags_path, std::ios::binary);
        const int Nx = G.GeomSize[0], Ny = G.GeomSize[1], Nz = G.GeomSize[2];
        std::vector<uint8_t> fl((size_t)Nx * Ny * Nz);
        if (!ff.read(reinterpret_cast<char*>(fl.data()), (std::streamsize)fl.size())) {
            std::fprintf(stderr, "flags file %s is shorter than the grid\n", flags_path.c_str());
            return 5;
        }
        for (int i = 0; i < Nx; ++i)
            for (int j = 0; j < Ny; ++j)
                for (int k = 0; k < Nz; ++k)
                    G.pointsBox[i][j][k].Type =
                        fl[((size_t)i * Ny + j) * Nz + k] ? NodeType::Fluid : NodeType::NotFluid;
    }
    G.boundaryPoints = G.findBoundaryPoints();
    std::vector<Point>* lists[7] = {&G.InletboundaryPoints, &G.OutletboundaryPoints1, &G.OutletboundaryPoints2,
                                    &G.OutletboundaryPoints3, &G.OutletboundaryPoints4, &G.OutletboundaryPoints5,
                                    &G.OutletboundaryPoints6};
    if (preset) {
        G.getInOutBP();
    } else {
        for (const Point& p : G.boundaryPoints)
            for (const Pred& pr : preds)
                if (pred_match(pr, p)) lists[pr.list]->push_back(p);
    }
    G.WallboundaryPoints = G.excludeInletOutlet();
    auto t1 = std::chrono::steady_clock::now();
    std::fprintf(stderr, "geometry: %d x %d x %d grid, %zu triangles, %.2f s\n", G.GeomSize[0], G.GeomSize[1],
                 G.GeomSize[2], G.globalTriangles.size(), std::chrono::duration<double>(t1 - t0).count());

    if (!vtkdir.empty()) {
        const char* names[7] = {"InboundaryPointsFromGeometry.vtk", "OutboundaryPointsFromGeometry1.vtk",
                                "OutboundaryPointsFromGeometry2.vtk", "OutboundaryPointsFromGeometry3.vtk",
                                "OutboundaryPointsFromGeometry4.vtk", "OutboundaryPointsFromGeometry5.vtk",
                                "OutboundaryPointsFromGeometry6.vtk"};
        for (int l = 0; l < 7; ++l) G.Writer.writePointsToFile(*lists[l], vtkdir + "/" + names[l]);
        G.Writer.writePointsToFile(G.WallboundaryPoints, vtkdir + "/WallboundaryPointsFromGeometry.vtk");
    }

    // flags (x-major) and lists as x-major linear indices
    const int Nx = G.GeomSize[0], Ny = G.GeomSize[1], Nz = G.GeomSize[2];
    std::vector<uint8_t> flags((size_t)Nx * Ny * Nz);
    for (int i = 0; i < Nx; ++i)
        for (int j = 0; j < Ny; ++j)
            for (int k = 0; k < Nz; ++k)
                flags[((size_t)i * Ny + j) * Nz + k] = G.pointsBox[i][j][k].Type == NodeType::Fluid ? 1 : 0;
    write_vec(out + ".flags", flags);
    auto index_of = [&](const Point& p) -> int64_t {
        long i = std::lround((p.x - G.boundingbox.min_x) / spacing);
        long j = std::lround((p.y - G.boundingbox.min_y) / spacing);
        long k = std::lround((p.z - G.boundingbox.min_z) / spacing);
        return ((int64_t)i * Ny + j) * Nz + k;
    };
    std::vector<int64_t> lst;   // [n_boundary, n_l0..n_l6, n_wall, indices...]
    std::vector<const std::vector<Point>*> all = {&G.boundaryPoints};
    for (int l = 0; l < 7; ++l) all.push_back(lists[l]);
    all.push_back(&G.WallboundaryPoints);
    for (auto* v : all) lst.push_back((int64_t)v->size());
    for (auto* v : all) for (const Point& p : *v) lst.push_back(index_of(p));
    write_vec(out + ".lists", lst);
    {
        std::ofstream meta(out + ".meta");
        meta.precision(17);
        meta << Nx << " " << Ny << " " << Nz << "\n"
             << G.boundingbox.min_x << " " << G.boundingbox.max_x << " " << G.boundingbox.min_y << " "
             << G.boundingbox.max_y << " " << G.boundingbox.min_z << " " << G.boundingbox.max_z << "\n";
    }
    if (steps <= 0 && profile_path.empty()) { MPI_Finalize(); return 0; }

    SubDomain S(G);
    g_oracle_steps = 0;
    Simulation sim(S, tau, 1.0, 1.0);
    SubDomain& D = sim.SubDomain_;
    std::vector<double> profile = profile_path.empty() ? std::vector<double>() : read_doubles(profile_path);
    std::vector<double> amp = amp_path.empty() ? std::vector<double>{1.0} : read_doubles(amp_path);
    if (!profile.empty() && profile.size() != D.InletBoundaryNode_.size()) {
        std::fprintf(stderr, "inlet profile has %zu entries, inlet list %zu\n", profile.size(), D.InletBoundaryNode_.size());
        return 4;
    }
    auto iterate = [&](int it) {
        if (!profile.empty()) {
            double a = amp[(size_t)it % amp.size()];
            for (size_t m = 0; m < D.InletBoundaryNode_.size(); ++m) {
                double s = a * profile[m];
                std::dynamic_pointer_cast<Boundary>(D.InletBoundaryNode_[m])->SetInletVel(s * idir[0], s * idir[1], s * idir[2]);
            }
        }
        sim.Collision();
        sim.Streaming();
        sim.ApplyZouHeBc();
        sim.ApplyWallBc();
        sim.ApplyOutletBc();
    };
    for (int it = 0; it < warmup; ++it) iterate(it);
    auto t2 = std::chrono::steady_clock::now();
    for (int it = warmup; it < warmup + steps; ++it) iterate(it);
    auto t3 = std::chrono::steady_clock::now();
    double secs = std::chrono::duration<double>(t3 - t2).count();
    std::fprintf(stderr, "steps: %d over %zu nodes, %.3f s, %.4f MLUPS\n", steps, D.Involved_Lat_.size(), secs,
                 steps > 0 ? (double)steps * D.Involved_Lat_.size() / secs / 1e6 : 0.0);
    {
        std::ofstream t(out + ".time");
        t.precision(9);
        t << steps << " " << D.Involved_Lat_.size() << " " << secs << "\n";
    }
    std::vector<double> f, rho, u;
    std::vector<int64_t> nodes;
    for (auto& n : D.Involved_Lat_) {
        for (int q = 0; q < _nLatNodes; ++q) f.push_back(n->m_distributions[q]);
        rho.push_back(n->density);
        for (int a = 0; a < 3; ++a) u.push_back(n->velocity[a]);
        nodes.push_back(((int64_t)n->x_position * Ny + n->y_position) * Nz + n->z_position);
    }
    write_vec(out + ".f", f);
    write_vec(out + ".rho", rho);
    write_vec(out + ".u", u);
    write_vec(out + ".nodes", nodes);
    if (want_wss) {
        sim.ComputeVelocityGradientAtWall();
        sim.ComputeWallShearStress();
        std::vector<double> wss;
        std::vector<int64_t> wn;
        for (auto& n : D.WallBoundaryNode_) {
            wss.push_back(n->wall_shear_stress);
            wn.push_back(((int64_t)n->x_position * Ny + n->y_position) * Nz + n->z_position);
        }
        write_vec(out + ".wss", wss);
        write_vec(out + ".wallnodes", wn);
    }
    MPI_Finalize();
    return 0;
}
