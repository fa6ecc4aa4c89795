// Host-only parts of include/cosmos_gb300_compat.hpp (no device calls): the boundary-cell insertion of
// the Solvers classes, the spacetime's excision test and the status line.  Prints one line per check
// for tests/test_compat_host.py.
#include <cstdio>
#include <vector>

#include "cosmos_gb300_compat.hpp"

int main() {
    std::vector<EulerStateVector> row;
    for (int i = 0; i < 5; i++) row.push_back(EulerStateVector(i, 0.0, 0.0, 0.0, 1.0));
    for (int b = 1; b <= 2; b++) {
        std::vector<EulerStateVector> p = EulerSolvers::insertBoundaryCells(row, b);
        std::printf("1d%d", b);
        for (auto& s : p) std::printf(" %g", s.getDensity());
        std::printf("\n");
    }
    std::vector<std::vector<RelativisticEulerStateVector> > g(3, std::vector<RelativisticEulerStateVector>(4));
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 4; j++) g[i][j] = RelativisticEulerStateVector(10 * i + j, 0.0, 0.0, 0.0, 1.0);
    for (int b = 1; b <= 2; b++) {
        auto p = RelativisticEulerSolvers::insertBoundaryCells2D(g, b);
        std::printf("2d%d", b);
        for (auto& r : p)
            for (auto& s : r) std::printf(" %g", s.getDensity());
        std::printf("\n");
    }
    BlackHoleSpacetime bh(0.1, 0.99, 0.5, 0.5, 0.0);
    std::printf("excised %d %d %d\n", (int)bh.inExcisionRegion(0.5, 0.5, 0.0), (int)bh.inExcisionRegion(0.6, 0.5, 0.0),
                (int)bh.inExcisionRegion(0.61, 0.5, 0.0));
    EulerSolvers::outputStatus(3, 0.25, 0.001);
    return 0;
}
