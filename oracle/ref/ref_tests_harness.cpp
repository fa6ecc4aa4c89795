// Test infrastructure only: a C-ABI harness over the reference's scenario drivers and solution
// writers (Tests/*.cpp), compiled with oracle/ref/redirect_ofstream.hpp so that the files they write
// go to the directory set by ref_tests_set_dir.  Used to generate the golden .dat fixtures under
// tests/golden/ (tests/golden/make_dat_golden.py); nothing in the product links it.
#include "EulerTests.hpp"
#include "RelativisticEulerTests.hpp"
#include "BlackHoleEulerTests.hpp"
#include "EulerAMRTests.hpp"
#include "RelativisticEulerAMRTests.hpp"

namespace cosmos_ref_redirect {
static std::string g_dir = ".";
std::string map_path(const char* path) {
    std::string p(path);
    const size_t slash = p.find_last_of('/');
    return g_dir + "/" + (slash == std::string::npos ? p : p.substr(slash + 1));
}
}  // namespace cosmos_ref_redirect

namespace {
struct Quiet {  // the reference prints a status line per step
    std::streambuf* old;
    std::ostringstream sink;
    Quiet() { old = std::cout.rdbuf(sink.rdbuf()); }
    ~Quiet() { std::cout.rdbuf(old); }
};
template <class S> S st(const double* p) { return S(p[0], p[1], p[2], p[3], p[4]); }
template <class S> vector<S> v1(const double* p, int n) {
    vector<S> v(n);
    for (int i = 0; i < n; i++) v[i] = st<S>(p + 5 * i);
    return v;
}
template <class S> vector<vector<S> > v2(const double* p, int ny, int nx) {
    vector<vector<S> > g(ny, vector<S>(nx));
    for (int i = 0; i < ny; i++)
        for (int j = 0; j < nx; j++) g[i][j] = st<S>(p + 5 * ((size_t)i * nx + j));
    return g;
}
vector<bool> b1(const unsigned char* f, int n) { return vector<bool>(f, f + n); }
vector<vector<bool> > b2(const unsigned char* f, int ny, int nx) {
    vector<vector<bool> > g(ny, vector<bool>(nx));
    for (int i = 0; i < ny; i++)
        for (int j = 0; j < nx; j++) g[i][j] = f[(size_t)i * nx + j] != 0;
    return g;
}
}  // namespace

extern "C" {

void ref_tests_set_dir(const char* d) { cosmos_ref_redirect::g_dir = d; }

// Runs one of the reference's scenario drivers by name; returns 0, or -1 for an unknown name.
int ref_tests_run(const char* name, int n, int order, int sub, double tol, int level) {
    Quiet q;
    const std::string s(name);
#define RUN0(CLS, FN) if (s == #CLS "::" #FN) { CLS::FN(n, order); return 0; }
#define RUNB(CLS, FN) if (s == #CLS "::" #FN) { CLS::FN(n, order, sub); return 0; }
#define RUNA(CLS, FN) if (s == #CLS "::" #FN) { CLS::FN(n, order, tol, level); return 0; }
    RUN0(EulerTests, solveToroTest1) RUN0(EulerTests, solveToroTest2) RUN0(EulerTests, solveToroTest3)
    RUN0(EulerTests, solve2DToroTest1) RUN0(EulerTests, solve2DToroTest2) RUN0(EulerTests, solve2DToroTest3)
    RUN0(RelativisticEulerTests, solveMildlyRelativisticShock) RUN0(RelativisticEulerTests, solveStronglyRelativisticBlast)
    RUN0(RelativisticEulerTests, solvePerturbedDensityTest) RUN0(RelativisticEulerTests, solve2DMildlyRelativisticShock)
    RUN0(RelativisticEulerTests, solve2DStronglyRelativisticBlast) RUN0(RelativisticEulerTests, solve2DPerturbedDensityTest)
    RUNB(BlackHoleEulerTests, solve1DSphericalAccretionTest) RUNB(BlackHoleEulerTests, solve1DSpinningSphericalAccretionTest)
    RUNB(BlackHoleEulerTests, solve2DSphericalAccretionTest) RUNB(BlackHoleEulerTests, solve2DSpinningSphericalAccretionTest)
    RUNB(BlackHoleEulerTests, solve2DSpheroidalAccretionTest) RUNB(BlackHoleEulerTests, solve2DSpinningSpheroidalAccretionTest)
    RUNA(EulerAMRTests, solveToroTest1AMR) RUNA(EulerAMRTests, solve2DToroTest1AMR)
    RUNA(RelativisticEulerAMRTests, solveMildlyRelativisticShock) RUNA(RelativisticEulerAMRTests, solveStronglyRelativisticBlast)
    RUNA(RelativisticEulerAMRTests, solvePerturbedDensityTest) RUNA(RelativisticEulerAMRTests, solve2DMildlyRelativisticShock)
    RUNA(RelativisticEulerAMRTests, solve2DStronglyRelativisticBlast) RUNA(RelativisticEulerAMRTests, solve2DPerturbedDensityTest)
#undef RUN0
#undef RUNB
#undef RUNA
    return -1;
}

// Calls one of the reference's writers on caller data.  kind 0: outputSolution(2D) of the system
// (sys 2 with the hole bh = {M, a, x, y, z}); kind 1: the Level-1 AMR writer, kind 2: the Level-2
// writer (levels l0 coarse, l1, l2 with flags f0, f1, f2; Newtonian or SR class by sys).
int ref_tests_write(int kind, int sys, int dims, int ny, int nx, const double* l0, const double* l1, const double* l2,
                    const unsigned char* f0, const unsigned char* f1, const unsigned char* f2, const double* bh) {
    if (kind == 0) {
        if (sys == 0) {
            if (dims == 1) EulerTests::outputSolution(v1<EulerStateVector>(l0, nx));
            else EulerTests::outputSolution2D(v2<EulerStateVector>(l0, ny, nx));
        } else if (sys == 1) {
            if (dims == 1) RelativisticEulerTests::outputSolution(v1<RelativisticEulerStateVector>(l0, nx));
            else RelativisticEulerTests::outputSolution2D(v2<RelativisticEulerStateVector>(l0, ny, nx));
        } else {
            BlackHoleSpacetime h(bh[0], bh[1], bh[2], bh[3], bh[4]);
            if (dims == 1) BlackHoleEulerTests::outputSolution(v1<BlackHoleEulerStateVector>(l0, nx), h);
            else BlackHoleEulerTests::outputSolution2D(v2<BlackHoleEulerStateVector>(l0, ny, nx), h);
        }
        return 0;
    }
#define AMR_WRITERS(CLS, S)                                                                                       \
    if (kind == 1 && dims == 1)                                                                                   \
        CLS::outputSolutionLevel1AMR(make_tuple(v1<S>(l0, nx), v1<S>(l1, 2 * nx), b1(f0, nx), b1(f1, 2 * nx)));   \
    else if (kind == 1)                                                                                           \
        CLS::outputSolution2DLevel1AMR(make_tuple(v2<S>(l0, ny, nx), v2<S>(l1, 2 * ny, 2 * nx), b2(f0, ny, nx),    \
                                                  b2(f1, 2 * ny, 2 * nx)));                                       \
    else if (dims == 1)                                                                                           \
        CLS::outputSolutionLevel2AMR(make_tuple(v1<S>(l0, nx), v1<S>(l1, 2 * nx), v1<S>(l2, 4 * nx), b1(f0, nx),  \
                                                b1(f1, 2 * nx), b1(f2, 4 * nx)));                                 \
    else                                                                                                          \
        CLS::outputSolution2DLevel2AMR(make_tuple(v2<S>(l0, ny, nx), v2<S>(l1, 2 * ny, 2 * nx),                    \
                                                  v2<S>(l2, 4 * ny, 4 * nx), b2(f0, ny, nx), b2(f1, 2 * ny, 2 * nx), \
                                                  b2(f2, 4 * ny, 4 * nx)));
    if (sys == 0) { AMR_WRITERS(EulerAMRTests, EulerStateVector) }
    else { AMR_WRITERS(RelativisticEulerAMRTests, RelativisticEulerStateVector) }
#undef AMR_WRITERS
    return 0;
}

}  // extern "C"
