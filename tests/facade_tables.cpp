// Prints the C++ facade's lattice tables (pv2013::LatticeModel), host only
// (test infrastructure for test_lattice_cpu.py).
#include <cstdio>

#include "pv2013/pv2013.hpp"

int main() {
    for (int Q : {19, 27}) {
        pv2013::LatticeModel L(Q);
        std::printf("Q %d\n", Q);
        for (int d = 0; d < Q; ++d) {
            const std::vector<int> c = L.GetDirection(d);
            std::printf("%d %d %d %d %.17g\n", c[0], c[1], c[2], L.OppositeDirection(d), L.GetWeight(d));
        }
    }
    return 0;
}
