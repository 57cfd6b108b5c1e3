// Prints the device lattice tables (Lat<19>, Lat<27> of device.cuh) from
// host code (test infrastructure, built with nvcc and run on the CPU by
// test_lattice_cpu.py; no kernel is launched).
#include <cstdio>

#include "device.cuh"

template <int Q>
static void dump() {
    using L = lbm::Lat<Q>;
    std::printf("Q %d %d %d\n", Q, L::REST, L::NO_BB_POP);
    for (int q = 0; q < Q; ++q) std::printf("%d %d %d %d %.17g\n", L::cx(q), L::cy(q), L::cz(q), L::opp(q), L::w(q));
}

int main() {
    dump<19>();
    dump<27>();
    return 0;
}
