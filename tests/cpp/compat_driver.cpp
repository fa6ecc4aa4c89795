// A reference-style driver (the shape of Tests/EulerTests.cpp:3-30 and friends) compiled against
// include/cosmos_gb300_compat.hpp instead of the reference's headers.  It runs a few scenarios and
// writes their final primitive grids as raw doubles to the directory given as argv[1], for
// tests/test_gpu_compat.py to compare with the oracle.
#include <cstdio>
#include <string>
#include <vector>

#include "cosmos_gb300_compat.hpp"

static void dump(const std::string& path, const std::vector<double>& v) {
    FILE* f = std::fopen(path.c_str(), "wb");
    std::fwrite(v.data(), sizeof(double), v.size(), f);
    std::fclose(f);
}
template <class S> static std::vector<double> flat1(std::vector<S> c) {
    std::vector<double> v;
    for (auto& s : c) {
        v.push_back(s.getDensity()); v.push_back(s.getXVelocity()); v.push_back(s.getYVelocity());
        v.push_back(s.getZVelocity()); v.push_back(s.getPressure());
    }
    return v;
}
template <class S> static std::vector<double> flat2(std::vector<std::vector<S> > g) {
    std::vector<double> v;
    for (auto& row : g) {
        std::vector<double> r = flat1(row);
        v.insert(v.end(), r.begin(), r.end());
    }
    return v;
}

int main(int argc, char** argv) {
    std::string dir = argc > 1 ? argv[1] : ".";
    // Sod shock tube, SLIC van Leer (the Toro test 1 setup with CFL 0.9)
    {
        int cellCount = 1000;
        double cellSpacing = 1.0 / cellCount;
        std::vector<EulerStateVector> initialCells(cellCount);
        EulerMaterialParameters materialParameters(1.4);
        for (int i = 0; i < cellCount; i++) {
            if (i <= (0.5 * cellCount)) initialCells[i] = EulerStateVector(1.0, 0.0, 0.0, 0.0, 1.0);
            else initialCells[i] = EulerStateVector(0.125, 0.0, 0.0, 0.0, 0.1);
        }
        dump(dir + "/sod.bin", flat1(EulerSecondOrderSolver::solve(initialCells, cellSpacing, 0.9, 0.25, 0.0, 1,
                                                                     materialParameters)));
    }
    // 2D cylindrical explosion (Tests/EulerTests.cpp:95-130 layout), FORCE, 40x40
    {
        int cellCount = 40;
        double cellSpacing = 1.0 / cellCount;
        std::vector<std::vector<EulerStateVector> > initialCells(cellCount, std::vector<EulerStateVector>(cellCount));
        EulerMaterialParameters materialParameters(1.4);
        for (int i = 0; i < cellCount; i++)
            for (int j = 0; j < cellCount; j++) {
                double r2 = ((i - (0.5 * cellCount)) * (i - (0.5 * cellCount))) + ((j - (0.5 * cellCount)) * (j - (0.5 * cellCount)));
                if (r2 <= (0.2 * cellCount) * (0.2 * cellCount)) initialCells[i][j] = EulerStateVector(1.0, 0.0, 0.0, 0.0, 1.0);
                else initialCells[i][j] = EulerStateVector(0.125, 0.0, 0.0, 0.0, 0.1);
            }
        dump(dir + "/cyl_force.bin", flat2(EulerFirstOrderSolver::solve2D(initialCells, cellSpacing, 0.9, 0.05,
                                                                           materialParameters)));
        EulerSecondOrderSolver::computeXSLICTimeStep2D(initialCells, cellSpacing, 0.001, 0.0, 2, materialParameters);
        dump(dir + "/cyl_xsweep.bin", flat2(initialCells));
    }
    // mildly relativistic shock tube (Tests/RelativisticEulerTests.cpp:3-30), 200 cells, t = 0.1
    {
        int cellCount = 200;
        double cellSpacing = 1.0 / cellCount;
        std::vector<RelativisticEulerStateVector> initialCells(cellCount);
        EulerMaterialParameters materialParameters(5.0 / 3.0);
        for (int i = 0; i < cellCount; i++) {
            if (i <= (0.5 * cellCount)) initialCells[i] = RelativisticEulerStateVector(10.0, 0.0, 0.0, 0.0, 13.3);
            else initialCells[i] = RelativisticEulerStateVector(1.0, 0.0, 0.0, 0.0, 1e-6);
        }
        dump(dir + "/sr_shock.bin", flat1(RelativisticEulerSecondOrderSolver::solve(initialCells, cellSpacing, 0.8, 0.1,
                                                                                      0.0, 1, materialParameters)));
    }
    // spherical accretion setup (Tests/BlackHoleEulerTests.cpp:3-30), 1D, 60 cells, a few steps
    {
        int cellCount = 60;
        double cellSpacing = 1.0 / cellCount;
        std::vector<BlackHoleEulerStateVector> initialCells(cellCount);
        EulerMaterialParameters materialParameters(5.0 / 3.0);
        BlackHoleSpacetime blackHole(0.05, 0.5, 0.0, 0.0);
        for (int i = 0; i < cellCount; i++) {
            if (i >= (0.1 * cellCount) && i <= (0.9 * cellCount)) initialCells[i] = BlackHoleEulerStateVector(10.0, 0.0, 0.0, 0.0, 0.1);
            else initialCells[i] = BlackHoleEulerStateVector(0.1, 0.0, 0.0, 0.0, 0.1);
        }
        dump(dir + "/bh_accretion.bin", flat1(BlackHoleEulerSecondOrderSolver::solve(
                                             initialCells, cellSpacing, 0.9, 0.02, 0.0, 1, 1, materialParameters, blackHole)));
    }
    // Level-1 AMR (AMR/EulerAMR.cpp:352-592): the cylindrical explosion on 20x20 coarse cells, SLIC
    {
        int cellCount = 20;
        double cellSpacing = 1.0 / cellCount;
        std::vector<std::vector<EulerStateVector> > initialCells(cellCount, std::vector<EulerStateVector>(cellCount));
        EulerMaterialParameters materialParameters(1.4);
        for (int i = 0; i < cellCount; i++)
            for (int j = 0; j < cellCount; j++) {
                double r2 = ((i - (0.5 * cellCount)) * (i - (0.5 * cellCount))) + ((j - (0.5 * cellCount)) * (j - (0.5 * cellCount)));
                if (r2 <= (0.2 * cellCount) * (0.2 * cellCount)) initialCells[i][j] = EulerStateVector(1.0, 0.0, 0.0, 0.0, 1.0);
                else initialCells[i][j] = EulerStateVector(0.125, 0.0, 0.0, 0.0, 0.1);
            }
        auto r = EulerAMR::solve2DLevel1AMR(initialCells, cellSpacing, 0.9, 0.05, 4.0, 2, materialParameters);
        dump(dir + "/amr_coarse.bin", flat2(std::get<0>(r)));
        dump(dir + "/amr_fine.bin", flat2(std::get<1>(r)));
        std::vector<double> flags;
        for (auto& row : std::get<2>(r)) for (bool b : row) flags.push_back(b ? 1.0 : 0.0);
        for (auto& row : std::get<3>(r)) for (bool b : row) flags.push_back(b ? 1.0 : 0.0);
        dump(dir + "/amr_flags.bin", flags);
    }
    // Level-2 AMR (AMR/RelativisticEulerAMR.cpp:604-929): the SR shock tube on 50 coarse cells, SLIC
    {
        int cellCount = 50;
        double cellSpacing = 1.0 / cellCount;
        std::vector<RelativisticEulerStateVector> initialCells(cellCount);
        EulerMaterialParameters materialParameters(5.0 / 3.0);
        for (int i = 0; i < cellCount; i++) {
            if (i <= (0.5 * cellCount)) initialCells[i] = RelativisticEulerStateVector(10.0, 0.0, 0.0, 0.0, 13.3);
            else initialCells[i] = RelativisticEulerStateVector(1.0, 0.0, 0.0, 0.0, 1e-6);
        }
        auto r = RelativisticEulerAMR::solveLevel2AMR(initialCells, cellSpacing, 0.8, 0.1, 20.0, 2, materialParameters);
        std::vector<double> all = flat1(std::get<0>(r)), m = flat1(std::get<1>(r)), f = flat1(std::get<2>(r));
        all.insert(all.end(), m.begin(), m.end());
        all.insert(all.end(), f.begin(), f.end());
        for (bool b : std::get<3>(r)) all.push_back(b ? 1.0 : 0.0);
        for (bool b : std::get<4>(r)) all.push_back(b ? 1.0 : 0.0);
        for (bool b : std::get<5>(r)) all.push_back(b ? 1.0 : 0.0);
        dump(dir + "/amr2_sr.bin", all);
    }
    std::printf("compat driver ok\n");
    return 0;
}
