// Test driver for include/cosmos_gb300_tests.hpp (the reference's scenario drivers and writers).
//
//   dat_tool write <kind> <system> <dims> <ny> <nx> <input.bin> <outdir>
//       calls the reference-named writer on the levels in input.bin (levels 0-2 as doubles, 5 per
//       cell, then the hole's 5 doubles, then the three flag sets as bytes); kind 0 plain
//       (outputSolution / outputSolution2D of the system), 1 Level-1 AMR, 2 Level-2 AMR
//   dat_tool problem <Class::method> <n> <out.bin>
//       writes the scenario's problem: ints system, dims, nx, ny; doubles dx, gamma, cfl, t_final[2],
//       t_amr, bh[5]; then the primitive cells
//   dat_tool run <Class::method> <n> <order> <subcycles> <tol> <level> <outdir>
//       runs the scenario on the GPU and writes its .dat files into outdir
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <map>
#include <string>
#include <vector>

#include "cosmos_gb300_tests.hpp"

using cosmos_tests::Problem;

namespace {

struct Entry {
    std::function<Problem(int)> build;
    std::function<void(int, int, int, double, int)> run;  // n, order, subcycles, tol, level
};

std::map<std::string, Entry> table() {
    std::map<std::string, Entry> t;
    using namespace cosmos_tests;
#define PLAIN(CLS, FN, BUILD) t[#CLS "::" #FN] = {BUILD, [](int n, int o, int, double, int) { CLS::FN(n, o); }};
#define GR(CLS, FN, BUILD) t[#CLS "::" #FN] = {BUILD, [](int n, int o, int s, double, int) { CLS::FN(n, o, s); }};
#define AMR(CLS, FN, BUILD) t[#CLS "::" #FN] = {BUILD, [](int n, int o, int, double tol, int l) { CLS::FN(n, o, tol, l); }};
    PLAIN(EulerTests, solveToroTest1, [](int n) { return toro_1d(n, 1); })
    PLAIN(EulerTests, solveToroTest2, [](int n) { return toro_1d(n, 2); })
    PLAIN(EulerTests, solveToroTest3, [](int n) { return toro_1d(n, 3); })
    PLAIN(EulerTests, solve2DToroTest1, [](int n) { return toro_2d(n, 1); })
    PLAIN(EulerTests, solve2DToroTest2, [](int n) { return toro_2d(n, 2); })
    PLAIN(EulerTests, solve2DToroTest3, [](int n) { return toro_2d(n, 3); })
    PLAIN(RelativisticEulerTests, solveMildlyRelativisticShock, [](int n) { return sr_1d(n, 1); })
    PLAIN(RelativisticEulerTests, solveStronglyRelativisticBlast, [](int n) { return sr_1d(n, 2); })
    PLAIN(RelativisticEulerTests, solvePerturbedDensityTest, [](int n) { return sr_1d(n, 3); })
    PLAIN(RelativisticEulerTests, solve2DMildlyRelativisticShock, [](int n) { return sr_2d(n, 1); })
    PLAIN(RelativisticEulerTests, solve2DStronglyRelativisticBlast, [](int n) { return sr_2d(n, 2); })
    PLAIN(RelativisticEulerTests, solve2DPerturbedDensityTest, [](int n) { return sr_2d(n, 3); })
    GR(BlackHoleEulerTests, solve1DSphericalAccretionTest, [](int n) { return bh_problem(1, n, 1); })
    GR(BlackHoleEulerTests, solve1DSpinningSphericalAccretionTest, [](int n) { return bh_problem(1, n, 2); })
    GR(BlackHoleEulerTests, solve2DSphericalAccretionTest, [](int n) { return bh_problem(2, n, 1); })
    GR(BlackHoleEulerTests, solve2DSpinningSphericalAccretionTest, [](int n) { return bh_problem(2, n, 2); })
    GR(BlackHoleEulerTests, solve2DSpheroidalAccretionTest, [](int n) { return bh_problem(2, n, 3); })
    GR(BlackHoleEulerTests, solve2DSpinningSpheroidalAccretionTest, [](int n) { return bh_problem(2, n, 4); })
    AMR(EulerAMRTests, solveToroTest1AMR, [](int n) { return toro_1d(n, 1); })
    AMR(EulerAMRTests, solve2DToroTest1AMR, [](int n) { return toro_2d(n, 1); })
    AMR(RelativisticEulerAMRTests, solveMildlyRelativisticShock, [](int n) { return sr_1d(n, 1); })
    AMR(RelativisticEulerAMRTests, solveStronglyRelativisticBlast, [](int n) { return sr_1d(n, 2); })
    AMR(RelativisticEulerAMRTests, solvePerturbedDensityTest, [](int n) { return sr_1d(n, 3); })
    AMR(RelativisticEulerAMRTests, solve2DMildlyRelativisticShock, [](int n) { return sr_2d(n, 1); })
    AMR(RelativisticEulerAMRTests, solve2DStronglyRelativisticBlast, [](int n) { return sr_2d(n, 2); })
    AMR(RelativisticEulerAMRTests, solve2DPerturbedDensityTest, [](int n) { return sr_2d(n, 3); })
#undef PLAIN
#undef GR
#undef AMR
    return t;
}

template <class S> std::vector<S> states(const double* p, size_t n) {
    std::vector<S> v(n);
    for (size_t i = 0; i < n; i++) v[i] = S(p[5 * i], p[5 * i + 1], p[5 * i + 2], p[5 * i + 3], p[5 * i + 4]);
    return v;
}
template <class S> std::vector<std::vector<S> > grid(const double* p, size_t ny, size_t nx) {
    std::vector<std::vector<S> > g(ny);
    for (size_t i = 0; i < ny; i++) g[i] = states<S>(p + 5 * i * nx, nx);
    return g;
}
std::vector<bool> bits(const unsigned char* f, size_t n) { return std::vector<bool>(f, f + n); }
std::vector<std::vector<bool> > bits2(const unsigned char* f, size_t ny, size_t nx) {
    std::vector<std::vector<bool> > g(ny);
    for (size_t i = 0; i < ny; i++) g[i] = bits(f + i * nx, nx);
    return g;
}

template <class S, class Tests, class AmrTests>
void write_kind(int kind, int dims, size_t ny, size_t nx, const double* const* lv, const unsigned char* const* fl,
                const BlackHoleSpacetime& bh, int system) {
    (void)bh;
    (void)system;
    if (kind == 0) {
        if (dims == 1) Tests::outputSolution(states<S>(lv[0], nx));
        else Tests::outputSolution2D(grid<S>(lv[0], ny, nx));
        return;
    }
    const size_t r = dims == 1 ? 1 : 2;
    if (kind == 1) {
        if (dims == 1) cosmos_tests::write_level1(states<S>(lv[0], nx), states<S>(lv[1], 2 * nx), bits(fl[0], nx), bits(fl[1], 2 * nx));
        else cosmos_tests::write_level1_2d(grid<S>(lv[0], ny, nx), grid<S>(lv[1], r * ny, 2 * nx), bits2(fl[0], ny, nx),
                                           bits2(fl[1], r * ny, 2 * nx), system == COSMOS_SR ? 1 : 5);
    } else if (dims == 1) {
        cosmos_tests::write_level2(states<S>(lv[0], nx), states<S>(lv[1], 2 * nx), states<S>(lv[2], 4 * nx), bits(fl[0], nx),
                                   bits(fl[1], 2 * nx), bits(fl[2], 4 * nx));
    } else {
        cosmos_tests::write_level2_2d(grid<S>(lv[0], ny, nx), grid<S>(lv[1], 2 * ny, 2 * nx), grid<S>(lv[2], 4 * ny, 4 * nx),
                                      bits2(fl[0], ny, nx), bits2(fl[1], 2 * ny, 2 * nx), bits2(fl[2], 4 * ny, 4 * nx));
    }
}

int do_write(char** a) {
    const int kind = atoi(a[0]), system = atoi(a[1]), dims = atoi(a[2]);
    const size_t ny = dims == 1 ? 1 : (size_t)atoi(a[3]), nx = (size_t)atoi(a[4]);
    FILE* in = fopen(a[5], "rb");
    if (!in) return 2;
    const size_t r = dims == 2 ? 4 : 2, n0 = ny * nx, sizes[3] = {n0, n0 * r, n0 * r * r};
    std::vector<double> lv[3];
    std::vector<unsigned char> fl[3];
    double bh[5];
    bool ok = true;
    for (int l = 0; l < 3; l++) {
        lv[l].resize(5 * sizes[l]);
        ok = ok && fread(lv[l].data(), sizeof(double), lv[l].size(), in) == lv[l].size();
    }
    ok = ok && fread(bh, sizeof(double), 5, in) == 5;
    for (int l = 0; l < 3; l++) {
        fl[l].resize(sizes[l]);
        ok = ok && fread(fl[l].data(), 1, sizes[l], in) == sizes[l];
    }
    fclose(in);
    if (!ok) return 2;
    cosmos_tests::set_output_directory(a[6]);
    const double* lp[3] = {lv[0].data(), lv[1].data(), lv[2].data()};
    const unsigned char* fp[3] = {fl[0].data(), fl[1].data(), fl[2].data()};
    const BlackHoleSpacetime hole(bh[0], bh[1], bh[2], bh[3], bh[4]);
    if (system == COSMOS_GR) {
        if (dims == 1) BlackHoleEulerTests::outputSolution(states<BlackHoleEulerStateVector>(lp[0], nx), hole);
        else BlackHoleEulerTests::outputSolution2D(grid<BlackHoleEulerStateVector>(lp[0], ny, nx), hole);
    } else if (system == COSMOS_SR) {
        write_kind<RelativisticEulerStateVector, RelativisticEulerTests, RelativisticEulerAMRTests>(kind, dims, ny, nx, lp,
                                                                                                    fp, hole, system);
    } else {
        write_kind<EulerStateVector, EulerTests, EulerAMRTests>(kind, dims, ny, nx, lp, fp, hole, system);
    }
    return 0;
}

int do_problem(char** a) {
    auto t = table();
    auto it = t.find(a[0]);
    if (it == t.end()) return 3;
    const Problem P = it->second.build(atoi(a[1]));
    FILE* out = fopen(a[2], "wb");
    if (!out) return 2;
    const int hdr[4] = {P.system, P.dims, P.nx, P.ny};
    const double par[11] = {P.dx, P.gamma, P.cfl, P.t_final[0], P.t_final[1], P.t_amr,
                            P.bh[0], P.bh[1], P.bh[2], P.bh[3], P.bh[4]};
    fwrite(hdr, sizeof(int), 4, out);
    fwrite(par, sizeof(double), 11, out);
    fwrite(P.prim.data(), sizeof(double), P.prim.size(), out);
    fclose(out);
    return 0;
}

int do_run(char** a) {
    auto t = table();
    auto it = t.find(a[0]);
    if (it == t.end()) return 3;
    cosmos_tests::set_output_directory(a[6]);
    it->second.run(atoi(a[1]), atoi(a[2]), atoi(a[3]), atof(a[4]), atoi(a[5]));
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) return 1;
    const std::string mode = argv[1];
    try {
        if (mode == "write" && argc == 9) return do_write(argv + 2);
        if (mode == "problem" && argc == 5) return do_problem(argv + 2);
        if (mode == "run" && argc == 9) return do_run(argv + 2);
    } catch (const std::exception& e) {
        fprintf(stderr, "%s\n", e.what());
        return 4;
    }
    return 1;
}
