// Drives the C++ facade the way the reference's main does (LBM.cpp:253-256):
// LatticeModel, Geometry(stl, velSet, spacing, mdepth), SubDomain(Geometry),
// Simulation(SubDomain, tau, pressure, dt, iterations).  Prints one line:
// "<fluid nodes> <wall points> <mass after the steps>" or "nodev".
#include <cstdio>
#include <cstdlib>

#include "pv2013/pv2013.hpp"

int main(int argc, char** argv) {
    using namespace pv2013;
    if (argc < 3) return 2;
    const long steps = std::atol(argv[2]);
    try {
        auto velSet = std::make_shared<LatticeModel>();
        Geometry geometry(argv[1], velSet, 0.1, 1);
        SubDomain subdomain(geometry);
        Simulation sim(subdomain, 0.66, 1.0, 1.0, steps);
        const auto F = sim.GetFields();
        double mass = 0.0;
        for (double r : F.rho) mass += r;
        std::printf("%lld %zu %.17g\n", (long long)geometry.info().n_fluid, geometry.WallboundaryPoints().size(), mass);
    } catch (const Error& e) {
        if (e.status == LBM_ERR_NODEV) {
            std::printf("nodev\n");
            return 0;
        }
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    return 0;
}
