// Test infrastructure only: a C-ABI harness over the reference's own public static API.
//
// This file is compiled together with the reference's sources (read in place from the
// reference tree by oracle/ref/Makefile) into oracle/_ref/libcosmos_ref.so.  It converts
// flat arrays of primitive states (rho, vx, vy, vz, p; row-major [ny][nx]) into the
// reference's vector<StateVector> grids, calls the reference's solver functions unchanged,
// and converts back.  It is used only to pin the C++ restatement in oracle/ and to
// generate the golden fixtures under tests/golden/; nothing in the product links it.
//
// Periodic boundaries are not part of the reference (Solvers/EulerSolvers.cpp:3-85 only
// fills transmissive ghosts).  For them the harness fills periodic ghost cells itself and
// calls the reference's public per-interface functions (computeXSLICFlux,
// computeFORCEUpdate, ...) exactly as the reference's own sweep loops do
// (Solvers/EulerSecondOrderSolver.cpp:48-100).

#include <iostream>
#include <sstream>
#include <streambuf>
#include <tuple>
#include <vector>

#include "EulerSecondOrderSolver.hpp"
#include "RelativisticEulerSecondOrderSolver.hpp"
#include "BlackHoleEulerSecondOrderSolver.hpp"
#include "BlackHoleEulerForcingSolver.hpp"
#include "EulerAMR.hpp"
#include "RelativisticEulerAMR.hpp"

using namespace std;

namespace {

// The reference prints a status line per step (Solvers/EulerSolvers.cpp:225-228);
// silence std::cout for the duration of a call.
struct Quiet {
    std::streambuf* old;
    std::ostringstream sink;
    Quiet() { old = std::cout.rdbuf(sink.rdbuf()); }
    ~Quiet() { std::cout.rdbuf(old); }
};

template <class S> S make_state(const double* p) { return S(p[0], p[1], p[2], p[3], p[4]); }
template <class S> void put_state(S s, double* p) {
    p[0] = s.getDensity(); p[1] = s.getXVelocity(); p[2] = s.getYVelocity();
    p[3] = s.getZVelocity(); p[4] = s.getPressure();
}
template <class S> vector<S> to1d(const double* prim, int n) {
    vector<S> v(n);
    for (int i = 0; i < n; i++) v[i] = make_state<S>(prim + 5 * i);
    return v;
}
template <class S> void from1d(const vector<S>& v, double* prim) {
    for (size_t i = 0; i < v.size(); i++) put_state(v[i], prim + 5 * i);
}
template <class S> vector<vector<S> > to2d(const double* prim, int ny, int nx) {
    vector<vector<S> > g(ny, vector<S>(nx));
    for (int i = 0; i < ny; i++)
        for (int j = 0; j < nx; j++) g[i][j] = make_state<S>(prim + 5 * ((size_t)i * nx + j));
    return g;
}
template <class S> void from2d(const vector<vector<S> >& g, double* prim) {
    int ny = (int)g.size(), nx = (int)g[0].size();
    for (int i = 0; i < ny; i++)
        for (int j = 0; j < nx; j++) put_state(g[i][j], prim + 5 * ((size_t)i * nx + j));
}
inline int wrap(int i, int n) { return ((i % n) + n) % n; }
void vec5(const vector<double>& v, double* out) { for (int k = 0; k < 5; k++) out[k] = v[k]; }
void vec3(const vector<double>& v, double* out) { for (int k = 0; k < 3; k++) out[k] = v[k]; }
vector<double> mk5(const double* p) { return vector<double>(p, p + 5); }

}  // namespace

extern "C" {

// ---------------------------------------------------------------- Newtonian + SR sweeps
// sys: 0 = Newtonian (Euler*), 1 = special relativistic (RelativisticEuler*)
// dims 1: prim is [nx]; dims 2: prim is [ny][nx]; axis 0 = x (columns), 1 = y (rows).
// order 1 = FORCE sweep, 2 = SLIC sweep.  bc 0 = transmissive (reference), 1 = periodic.

static void euler_sweep(double* prim, int ny, int nx, int dims, int axis, int order, double dx,
                        double dt, double bias, int lim, double gamma, int bc) {
    EulerMaterialParameters mp(gamma);
    if (bc == 0) {
        if (dims == 1) {
            vector<EulerStateVector> c = to1d<EulerStateVector>(prim, nx);
            if (order == 2) EulerSecondOrderSolver::computeSLICTimeStep(c, dx, dt, bias, lim, mp);
            else EulerFirstOrderSolver::computeFORCETimeStep(c, dx, dt, mp);
            from1d(c, prim);
        } else {
            vector<vector<EulerStateVector> > g = to2d<EulerStateVector>(prim, ny, nx);
            if (order == 2) {
                if (axis == 0) EulerSecondOrderSolver::computeXSLICTimeStep2D(g, dx, dt, bias, lim, mp);
                else EulerSecondOrderSolver::computeYSLICTimeStep2D(g, dx, dt, bias, lim, mp);
            } else {
                if (axis == 0) EulerFirstOrderSolver::computeXFORCETimeStep2D(g, dx, dt, mp);
                else EulerFirstOrderSolver::computeYFORCETimeStep2D(g, dx, dt, mp);
            }
            from2d(g, prim);
        }
        return;
    }
    // periodic: same loop structure as the reference's sweeps, periodic ghosts
    if (dims == 1) { ny = 1; axis = 0; }
    vector<vector<EulerStateVector> > g = to2d<EulerStateVector>(prim, ny, nx);
    vector<vector<EulerStateVector> > out = g;
    for (int i = 0; i < ny; i++) {
        for (int j = 0; j < nx; j++) {
            auto at = [&](int d) -> EulerStateVector {
                return axis == 0 ? g[i][wrap(j + d, nx)] : g[wrap(i + d, ny)][j];
            };
            vector<double> u = g[i][j].computeConservedVariableVector(mp);
            vector<double> fl, fr;
            if (order == 2) {
                if (axis == 0) {
                    fl = EulerSecondOrderSolver::computeXSLICFlux(at(-2), at(-1), at(0), at(1), dx, dt, bias, lim, mp);
                    fr = EulerSecondOrderSolver::computeXSLICFlux(at(-1), at(0), at(1), at(2), dx, dt, bias, lim, mp);
                } else {
                    fl = EulerSecondOrderSolver::computeYSLICFlux(at(-2), at(-1), at(0), at(1), dx, dt, bias, lim, mp);
                    fr = EulerSecondOrderSolver::computeYSLICFlux(at(-1), at(0), at(1), at(2), dx, dt, bias, lim, mp);
                }
            } else {
                if (axis == 0) {
                    fl = EulerFirstOrderSolver::computeXFORCEFlux(at(-1), at(0), dx, dt, mp);
                    fr = EulerFirstOrderSolver::computeXFORCEFlux(at(0), at(1), dx, dt, mp);
                } else {
                    fl = EulerFirstOrderSolver::computeYFORCEFlux(at(-1), at(0), dx, dt, mp);
                    fr = EulerFirstOrderSolver::computeYFORCEFlux(at(0), at(1), dx, dt, mp);
                }
            }
            out[i][j].setConservedVariableVector(EulerFirstOrderSolver::computeFORCEUpdate(u, fl, fr, dx, dt), mp);
        }
    }
    from2d(out, prim);
}

static void sr_sweep(double* prim, int ny, int nx, int dims, int axis, int order, double dx,
                     double dt, double bias, int lim, double gamma, int bc) {
    typedef RelativisticEulerStateVector S;
    EulerMaterialParameters mp(gamma);
    if (bc == 0) {
        if (dims == 1) {
            vector<S> c = to1d<S>(prim, nx);
            if (order == 2) RelativisticEulerSecondOrderSolver::computeSLICTimeStep(c, dx, dt, bias, lim, mp);
            else RelativisticEulerFirstOrderSolver::computeFORCETimeStep(c, dx, dt, mp);
            from1d(c, prim);
        } else {
            vector<vector<S> > g = to2d<S>(prim, ny, nx);
            if (order == 2) {
                if (axis == 0) RelativisticEulerSecondOrderSolver::computeXSLICTimeStep2D(g, dx, dt, bias, lim, mp);
                else RelativisticEulerSecondOrderSolver::computeYSLICTimeStep2D(g, dx, dt, bias, lim, mp);
            } else {
                if (axis == 0) RelativisticEulerFirstOrderSolver::computeXFORCETimeStep2D(g, dx, dt, mp);
                else RelativisticEulerFirstOrderSolver::computeYFORCETimeStep2D(g, dx, dt, mp);
            }
            from2d(g, prim);
        }
        return;
    }
    if (dims == 1) { ny = 1; axis = 0; }
    vector<vector<S> > g = to2d<S>(prim, ny, nx);
    vector<vector<S> > out = g;
    for (int i = 0; i < ny; i++) {
        for (int j = 0; j < nx; j++) {
            auto at = [&](int d) -> S { return axis == 0 ? g[i][wrap(j + d, nx)] : g[wrap(i + d, ny)][j]; };
            vector<double> u = g[i][j].computeConservedVariableVector(mp);
            vector<double> fl, fr;
            if (order == 2) {
                if (axis == 0) {
                    fl = RelativisticEulerSecondOrderSolver::computeXSLICFlux(at(-2), at(-1), at(0), at(1), dx, dt, bias, lim, mp);
                    fr = RelativisticEulerSecondOrderSolver::computeXSLICFlux(at(-1), at(0), at(1), at(2), dx, dt, bias, lim, mp);
                } else {
                    fl = RelativisticEulerSecondOrderSolver::computeYSLICFlux(at(-2), at(-1), at(0), at(1), dx, dt, bias, lim, mp);
                    fr = RelativisticEulerSecondOrderSolver::computeYSLICFlux(at(-1), at(0), at(1), at(2), dx, dt, bias, lim, mp);
                }
            } else {
                if (axis == 0) {
                    fl = RelativisticEulerFirstOrderSolver::computeXFORCEFlux(at(-1), at(0), dx, dt, mp);
                    fr = RelativisticEulerFirstOrderSolver::computeXFORCEFlux(at(0), at(1), dx, dt, mp);
                } else {
                    fl = RelativisticEulerFirstOrderSolver::computeYFORCEFlux(at(-1), at(0), dx, dt, mp);
                    fr = RelativisticEulerFirstOrderSolver::computeYFORCEFlux(at(0), at(1), dx, dt, mp);
                }
            }
            out[i][j].setConservedVariableVector(EulerFirstOrderSolver::computeFORCEUpdate(u, fl, fr, dx, dt), mp);
        }
    }
    from2d(out, prim);
}

void ref_sweep(int sys, double* prim, int ny, int nx, int dims, int axis, int order, double dx, double dt,
               double bias, int lim, double gamma, int bc) {
    if (sys == 0) euler_sweep(prim, ny, nx, dims, axis, order, dx, dt, bias, lim, gamma, bc);
    else sr_sweep(prim, ny, nx, dims, axis, order, dx, dt, bias, lim, gamma, bc);
}

double ref_stable_dt(int sys, const double* prim, int ny, int nx, int dims, double dx, double cfl,
                     double t, double tfinal, int it, double gamma) {
    EulerMaterialParameters mp(gamma);
    if (sys == 0) {
        if (dims == 1) return EulerSolvers::computeStableTimeStep(to1d<EulerStateVector>(prim, nx), dx, cfl, t, tfinal, it, mp);
        return EulerSolvers::computeStableTimeStep2D(to2d<EulerStateVector>(prim, ny, nx), dx, cfl, t, tfinal, it, mp);
    }
    typedef RelativisticEulerStateVector S;
    if (dims == 1) return RelativisticEulerSolvers::computeStableTimeStep(to1d<S>(prim, nx), dx, cfl, t, tfinal, it, mp);
    return RelativisticEulerSolvers::computeStableTimeStep2D(to2d<S>(prim, ny, nx), dx, cfl, t, tfinal, it, mp);
}

double ref_max_wavespeed(int sys, const double* prim, int ny, int nx, int dims, double gamma) {
    EulerMaterialParameters mp(gamma);
    if (sys == 0) {
        if (dims == 1) { auto c = to1d<EulerStateVector>(prim, nx); return EulerSolvers::computeMaximumWaveSpeed(c, mp); }
        auto g = to2d<EulerStateVector>(prim, ny, nx); return EulerSolvers::computeMaximumWaveSpeed2D(g, mp);
    }
    typedef RelativisticEulerStateVector S;
    if (dims == 1) { auto c = to1d<S>(prim, nx); return RelativisticEulerSolvers::computeMaximumWaveSpeed(c, mp); }
    auto g = to2d<S>(prim, ny, nx); return RelativisticEulerSolvers::computeMaximumWaveSpeed2D(g, mp);
}

// Full solve through the reference's solve / solve2D (transmissive only).  Returns the step
// count (counted from the reference's own status lines).
int ref_solve(int sys, double* prim, int ny, int nx, int dims, int order, double dx, double cfl,
              double tfinal, double bias, int lim, double gamma) {
    EulerMaterialParameters mp(gamma);
    Quiet q;
    if (sys == 0) {
        if (dims == 1) {
            auto c = to1d<EulerStateVector>(prim, nx);
            c = order == 2 ? EulerSecondOrderSolver::solve(c, dx, cfl, tfinal, bias, lim, mp)
                           : EulerFirstOrderSolver::solve(c, dx, cfl, tfinal, mp);
            from1d(c, prim);
        } else {
            auto g = to2d<EulerStateVector>(prim, ny, nx);
            g = order == 2 ? EulerSecondOrderSolver::solve2D(g, dx, cfl, tfinal, bias, lim, mp)
                           : EulerFirstOrderSolver::solve2D(g, dx, cfl, tfinal, mp);
            from2d(g, prim);
        }
    } else {
        typedef RelativisticEulerStateVector S;
        if (dims == 1) {
            auto c = to1d<S>(prim, nx);
            c = order == 2 ? RelativisticEulerSecondOrderSolver::solve(c, dx, cfl, tfinal, bias, lim, mp)
                           : RelativisticEulerFirstOrderSolver::solve(c, dx, cfl, tfinal, mp);
            from1d(c, prim);
        } else {
            auto g = to2d<S>(prim, ny, nx);
            g = order == 2 ? RelativisticEulerSecondOrderSolver::solve2D(g, dx, cfl, tfinal, bias, lim, mp)
                           : RelativisticEulerFirstOrderSolver::solve2D(g, dx, cfl, tfinal, mp);
            from2d(g, prim);
        }
    }
    std::string s = q.sink.str();
    int steps = 0;
    for (size_t pos = 0; (pos = s.find("Iteration = ", pos)) != std::string::npos; pos += 12) steps++;
    return steps;
}

// ---------------------------------------------------------------- state-level functions
void ref_euler_cons(const double* prim, double gamma, double* out) {
    EulerMaterialParameters mp(gamma);
    vec5(make_state<EulerStateVector>(prim).computeConservedVariableVector(mp), out);
}
void ref_euler_prim(const double* cons, double gamma, double* out) {
    EulerMaterialParameters mp(gamma);
    EulerStateVector s; s.setConservedVariableVector(mk5(cons), mp); put_state(s, out);
}
void ref_euler_flux(const double* cons, int axis, double gamma, double* out) {
    EulerMaterialParameters mp(gamma);
    vec5(axis == 0 ? EulerStateVector::computeXFluxVector(mk5(cons), mp) : EulerStateVector::computeYFluxVector(mk5(cons), mp), out);
}
void ref_sr_cons(const double* prim, double gamma, double* out) {
    EulerMaterialParameters mp(gamma);
    vec5(make_state<RelativisticEulerStateVector>(prim).computeConservedVariableVector(mp), out);
}
void ref_sr_prim(const double* cons, double gamma, double* out) {
    EulerMaterialParameters mp(gamma);
    RelativisticEulerStateVector s; s.setConservedVariableVector(mk5(cons), mp); put_state(s, out);
}
void ref_sr_flux(const double* cons, int axis, double gamma, double* out) {
    EulerMaterialParameters mp(gamma);
    vec5(axis == 0 ? RelativisticEulerStateVector::computeXFluxVector(mk5(cons), mp)
                   : RelativisticEulerStateVector::computeYFluxVector(mk5(cons), mp), out);
}
double ref_limiter(double r, double bias, int lim) { return SlopeLimiters::computeSlopeLimiter(r, bias, lim); }
void ref_slope(const double* ul, const double* uc, const double* ur, double bias, int lim, double* out) {
    vec5(SlopeLimiters::computeSlopeVector(mk5(ul), mk5(uc), mk5(ur), bias, lim), out);
}

// ---------------------------------------------------------------- black-hole (GR) system
static BlackHoleSpacetime mkbh(const double* bh) { return BlackHoleSpacetime(bh[0], bh[1], bh[2], bh[3], bh[4]); }

// bh = {mass, spin, x, y, z}.  out receives: [0] det gamma_ij, [1] lapse, [2..4] shift,
// [5..13] gamma_ij, [14..29] inverse spacetime metric, [30..38] K_ij (FD spacing h),
// [39..41] d lapse, [42] excised flag, [43] Kerr-Schild scalar, [44..47] spacetime vector,
// [48..56] inverse spatial metric
void ref_gr_metric(double x, double y, double z, double h, const double* bh, double* out) {
    BlackHoleSpacetime b = mkbh(bh);
    out[0] = b.computeSpatialMetricDeterminant(x, y, z);
    out[1] = b.computeLapseFunction(x, y, z);
    vector<double> s = b.computeShiftVector(x, y, z);
    for (int i = 0; i < 3; i++) out[2 + i] = s[i];
    vector<vector<double> > g = b.computeSpatialMetricTensor(x, y, z);
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) out[5 + 3 * i + j] = g[i][j];
    vector<vector<double> > gi = b.computeInverseSpacetimeMetricTensor(x, y, z);
    for (int i = 0; i < 4; i++) for (int j = 0; j < 4; j++) out[14 + 4 * i + j] = gi[i][j];
    vector<vector<double> > K = b.computeExtrinsicCurvatureTensor(x, y, z, h);
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) out[30 + 3 * i + j] = K[i][j];
    vector<double> da = b.computeLapseFunctionDerivative(x, y, z, h);
    for (int i = 0; i < 3; i++) out[39 + i] = da[i];
    out[42] = b.inExcisionRegion(x, y, z) ? 1.0 : 0.0;
    out[43] = b.computeKerrSchildScalar(x, y, z);
    vector<double> l = b.computeKerrSchildSpacetimeVector(x, y, z);
    for (int i = 0; i < 4; i++) out[44 + i] = l[i];
    vector<vector<double> > gs = b.computeInverseSpatialMetricTensor(x, y, z);
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) out[48 + 3 * i + j] = gs[i][j];
}
// every public quantity of the reference's BlackHoleSpacetime at (x, y, z), in the layout of
// orc_spacetime_record (oracle/cosmos_oracle.cpp)
void ref_spacetime_record(double x, double y, double z, double h, const double* bhp, double* o) {
    BlackHoleSpacetime b = mkbh(bhp);
    auto put = [&](int at, const vector<double>& v) { for (size_t i = 0; i < v.size(); i++) o[at + i] = v[i]; };
    auto put2 = [&](int at, const vector<vector<double> >& m) {
        int k = at;
        for (auto& r : m) for (double v : r) o[k++] = v;
    };
    o[0] = b.computeKerrSchildScalar(x, y, z);
    put(1, b.computeKerrSchildVector(x, y, z));
    put(4, b.computeKerrSchildSpacetimeVector(x, y, z));
    put(8, b.computeKerrSchildScalarDerivative(x, y, z, h));
    put2(11, b.computeKerrSchildVectorDerivative(x, y, z, h));
    put2(20, b.computeSpatialMetricTensor(x, y, z));
    put2(29, b.computeSpacetimeMetricTensor(x, y, z));
    put2(45, b.computeInverseSpatialMetricTensor(x, y, z));
    put2(54, b.computeInverseSpacetimeMetricTensor(x, y, z));
    o[70] = b.computeSpatialMetricDeterminant(x, y, z);
    o[71] = b.computeSpacetimeMetricDeterminant(x, y, z);
    vector<vector<vector<double> > > d = b.computeSpatialMetricTensorDerivative(x, y, z, h);
    int k = 72;
    for (auto& m : d) for (auto& r : m) for (double v : r) o[k++] = v;
    o[99] = b.computeLapseFunction(x, y, z);
    put(100, b.computeShiftVector(x, y, z));
    put(103, b.computeLapseFunctionDerivative(x, y, z, h));
    put2(106, b.computeShiftVectorDerivative(x, y, z, h));
    put2(115, b.computeExtrinsicCurvatureTensor(x, y, z, h));
    o[124] = b.inExcisionRegion(x, y, z) ? 1.0 : 0.0;
}
// BlackHoleEulerEigenvalues (material, fast acoustic, slow acoustic; 3 each) of primitives p
void ref_gr_eigenvalues(const double* p, double x, double y, double z, double gamma, const double* bhp, double* o) {
    EulerMaterialParameters mp(gamma);
    BlackHoleSpacetime b = mkbh(bhp);
    vec3(BlackHoleEulerEigenvalues::computeMaterialWaveEigenvalues(x, y, z, p[1], p[2], p[3], mp, b), o);
    vec3(BlackHoleEulerEigenvalues::computeFastAcousticWaveEigenvalues(x, y, z, p[0], p[4], p[1], p[2], p[3], mp, b), o + 3);
    vec3(BlackHoleEulerEigenvalues::computeSlowAcousticWaveEigenvalues(x, y, z, p[0], p[4], p[1], p[2], p[3], mp, b), o + 6);
}
void ref_gr_cons(const double* prim, double x, double y, double z, double gamma, const double* bh, double* out) {
    EulerMaterialParameters mp(gamma);
    vec5(make_state<BlackHoleEulerStateVector>(prim).computeConservedVariableVector(x, y, z, mp, mkbh(bh)), out);
}
void ref_gr_prim(const double* cons, double x, double y, double z, double gamma, const double* bh, double* out) {
    EulerMaterialParameters mp(gamma);
    BlackHoleEulerStateVector s; s.setConservedVariableVector(mk5(cons), x, y, z, mp, mkbh(bh)); put_state(s, out);
}
void ref_gr_flux(const double* cons, int axis, double x, double y, double z, double gamma, const double* bh, double* out) {
    EulerMaterialParameters mp(gamma);
    vec5(axis == 0 ? BlackHoleEulerStateVector::computeXFluxVector(mk5(cons), x, y, z, mp, mkbh(bh))
                   : BlackHoleEulerStateVector::computeYFluxVector(mk5(cons), x, y, z, mp, mkbh(bh)), out);
}
void ref_gr_source(const double* cons, double x, double y, double z, double h, double gamma, const double* bh, double* out) {
    EulerMaterialParameters mp(gamma);
    vec5(BlackHoleEulerStateVector::computeSourceTermVector(mk5(cons), x, y, z, h, mp, mkbh(bh)), out);
}
double ref_gr_sound_speed(const double* prim, double x, double y, double z, double gamma, const double* bh) {
    EulerMaterialParameters mp(gamma);
    return make_state<BlackHoleEulerStateVector>(prim).computeSoundSpeed(x, y, z, mp, mkbh(bh));
}

// ---------------------------------------------------------------- per-interface solver functions
// The reference's static building blocks applied to n items: in holds the op's inputs per item
// (vectors of 5 doubles: conserved vectors, flux vectors or primitive states, see
// orc_interface_eval in oracle/cosmos_oracle.cpp for the op list), xyz the coordinate arguments
// (black hole only), out 5 doubles per item (a vector, or the primitives of the returned state).
}  // extern "C"

namespace {
const int kIfaceWidth[23] = {20, 20, 10, 15, 10, 10, 10, 10, 10, 10, 10, 10, 20, 20, 15, 15, 15, 15, 15, 15, 10, 15, 25};

// ops 0..5: system-independent vector forms
bool vector_op(int op, const double* a, double dx, double dt, double frac, double* o) {
    auto v = [&](int k) { return mk5(a + 5 * k); };
    switch (op) {
        case 0: vec5(EulerFirstOrderSolver::computeLaxFriedrichsFlux(v(0), v(1), v(2), v(3), dx, dt), o); return true;
        case 1: vec5(EulerFirstOrderSolver::computeRichtmyerFlux(v(0), v(1), v(2), v(3), dx, dt), o); return true;
        case 2: vec5(EulerFirstOrderSolver::computeFORCEFlux(v(0), v(1)), o); return true;
        case 3: vec5(EulerFirstOrderSolver::computeFORCEUpdate(v(0), v(1), v(2), dx, dt), o); return true;
        case 4: vec5(EulerSolvers::computeFractionalEvolutionVector(frac, v(0), v(1), dx, dt), o); return true;
        case 5: vec5(EulerSolvers::computeEvolutionVector(v(0), v(1), dx, dt), o); return true;
        default: return false;
    }
}

// Newtonian and special-relativistic state forms (the same signatures in both families)
template <class S, class First, class Second, class Solvers>
int flat_op(int op, const double* a, double dx, double dt, double bias, int lim, int side, double gamma, double* o) {
    EulerMaterialParameters mp(gamma);
    auto st = [&](int k) { return make_state<S>(a + 5 * k); };
    auto v = [&](int k) { return mk5(a + 5 * k); };
    switch (op) {
        case 6: vec5(First::computeXLaxFriedrichsFlux(st(0), st(1), dx, dt, mp), o); return 0;
        case 7: vec5(First::computeYLaxFriedrichsFlux(st(0), st(1), dx, dt, mp), o); return 0;
        case 8: vec5(First::computeXRichtmyerFlux(st(0), st(1), dx, dt, mp), o); return 0;
        case 9: vec5(First::computeYRichtmyerFlux(st(0), st(1), dx, dt, mp), o); return 0;
        case 10: vec5(First::computeXFORCEFlux(st(0), st(1), dx, dt, mp), o); return 0;
        case 11: vec5(First::computeYFORCEFlux(st(0), st(1), dx, dt, mp), o); return 0;
        case 12: vec5(Second::computeXSLICFlux(st(0), st(1), st(2), st(3), dx, dt, bias, lim, mp), o); return 0;
        case 13: vec5(Second::computeYSLICFlux(st(0), st(1), st(2), st(3), dx, dt, bias, lim, mp), o); return 0;
        case 14: put_state(Solvers::evolveStateByHalfXTimeStep(st(0), st(1), st(2), dx, dt, bias, lim, side, mp), o); return 0;
        case 15: put_state(Solvers::evolveStateByHalfYTimeStep(st(0), st(1), st(2), dx, dt, bias, lim, side, mp), o); return 0;
        case 16: case 17: put_state(Solvers::evolveStateByHalfTimeStep(v(0), v(1), v(2), side, mp), o); return 0;
        default: return -1;
    }
}

int gr_op(int op, const double* a, const double* q, double dx, double dt, double bias, int lim, double frac, int side,
          double gamma, const double* bhp, double* o) {
    typedef BlackHoleEulerStateVector S;
    EulerMaterialParameters mp(gamma);
    BlackHoleSpacetime bh = mkbh(bhp);
    const double x = q[0], y = q[1], z = q[2];
    auto st = [&](int k) { return make_state<S>(a + 5 * k); };
    auto v = [&](int k) { return mk5(a + 5 * k); };
    typedef BlackHoleEulerFirstOrderSolver F;
    typedef BlackHoleEulerSolvers V;
    switch (op) {
        case 6: vec5(F::computeXLaxFriedrichsFlux(st(0), st(1), x, y, z, dx, dt, mp, bh), o); return 0;
        case 7: vec5(F::computeYLaxFriedrichsFlux(st(0), st(1), x, y, z, dx, dt, mp, bh), o); return 0;
        case 8: vec5(F::computeXRichtmyerFlux(st(0), st(1), x, y, z, dx, dt, mp, bh), o); return 0;
        case 9: vec5(F::computeYRichtmyerFlux(st(0), st(1), x, y, z, dx, dt, mp, bh), o); return 0;
        case 10: vec5(F::computeXFORCEFlux(st(0), st(1), x, y, z, dx, dt, mp, bh), o); return 0;
        case 11: vec5(F::computeYFORCEFlux(st(0), st(1), x, y, z, dx, dt, mp, bh), o); return 0;
        case 12: vec5(BlackHoleEulerSecondOrderSolver::computeXSLICFlux(st(0), st(1), st(2), st(3), dx, dt, bias, lim, x, y, z, mp, bh), o); return 0;
        case 13: vec5(BlackHoleEulerSecondOrderSolver::computeYSLICFlux(st(0), st(1), st(2), st(3), dx, dt, bias, lim, x, y, z, mp, bh), o); return 0;
        case 14: put_state(V::evolveStateByHalfXTimeStep(st(0), st(1), st(2), dx, dt, bias, lim, side, x, y, z, mp, bh), o); return 0;
        case 15: put_state(V::evolveStateByHalfYTimeStep(st(0), st(1), st(2), dx, dt, bias, lim, side, x, y, z, mp, bh), o); return 0;
        case 16: put_state(V::evolveStateByHalfXTimeStep(v(0), v(1), v(2), side, dx, x, y, z, mp, bh), o); return 0;
        case 17: put_state(V::evolveStateByHalfYTimeStep(v(0), v(1), v(2), side, dx, x, y, z, mp, bh), o); return 0;
        case 18: put_state(V::evolveStateByFractionalXTimeStep(frac, st(0), st(1), st(2), dx, dt, bias, lim, x, y, z, mp, bh), o); return 0;
        case 19: put_state(V::evolveStateByFractionalYTimeStep(frac, st(0), st(1), st(2), dx, dt, bias, lim, x, y, z, mp, bh), o); return 0;
        case 20: put_state(V::evolveStateByFractionalTimeStep(v(0), v(1), x, y, z, mp, bh), o); return 0;
        case 21: vec5(BlackHoleEulerForcingSolver::evolveConservedVariableVector(v(0), v(1), v(2), x, y, z, dx, dt, bias, lim, mp, bh), o); return 0;
        case 22: vec5(BlackHoleEulerForcingSolver::evolveConservedVariableVector2D(v(0), v(1), v(2), v(3), v(4), x, y, z, dx, dt, bias, lim, mp, bh), o); return 0;
        default: return -1;
    }
}
}  // namespace

extern "C" {

int ref_interface_eval(int op, int sys, size_t n, const double* in, const double* xyz, double gamma, const double* bh,
                       double dx, double dt, double bias, int lim, double frac, int side, double* out) {
    if (op < 0 || op > 22) return -1;
    const int iw = kIfaceWidth[op];
    for (size_t i = 0; i < n; i++) {
        const double* a = in + (size_t)iw * i;
        double* o = out + 5 * i;
        if (vector_op(op, a, dx, dt, frac, o)) continue;
        int rc;
        if (sys == 0)
            rc = flat_op<EulerStateVector, EulerFirstOrderSolver, EulerSecondOrderSolver, EulerSolvers>(op, a, dx, dt, bias, lim, side, gamma, o);
        else if (sys == 1)
            rc = flat_op<RelativisticEulerStateVector, RelativisticEulerFirstOrderSolver, RelativisticEulerSecondOrderSolver,
                         RelativisticEulerSolvers>(op, a, dx, dt, bias, lim, side, gamma, o);
        else
            rc = gr_op(op, a, xyz + 3 * i, dx, dt, bias, lim, frac, side, gamma, bh, o);
        if (rc) return rc;
    }
    return 0;
}

void ref_gr_sweep(double* prim, int ny, int nx, int dims, int axis, int order, double dx, double dt,
                  double bias, int lim, double gamma, const double* bh) {
    typedef BlackHoleEulerStateVector S;
    EulerMaterialParameters mp(gamma);
    BlackHoleSpacetime b = mkbh(bh);
    if (dims == 1) {
        vector<S> c = to1d<S>(prim, nx);
        if (order == 2) BlackHoleEulerSecondOrderSolver::computeSLICTimeStep(c, dx, dt, bias, lim, mp, b);
        else BlackHoleEulerFirstOrderSolver::computeFORCETimeStep(c, dx, dt, mp, b);
        from1d(c, prim);
    } else {
        vector<vector<S> > g = to2d<S>(prim, ny, nx);
        if (order == 2) {
            if (axis == 0) BlackHoleEulerSecondOrderSolver::computeXSLICTimeStep2D(g, dx, dt, bias, lim, mp, b);
            else BlackHoleEulerSecondOrderSolver::computeYSLICTimeStep2D(g, dx, dt, bias, lim, mp, b);
        } else {
            if (axis == 0) BlackHoleEulerFirstOrderSolver::computeXFORCETimeStep2D(g, dx, dt, mp, b);
            else BlackHoleEulerFirstOrderSolver::computeYFORCETimeStep2D(g, dx, dt, mp, b);
        }
        from2d(g, prim);
    }
}

void ref_gr_rk_source(double* prim, int ny, int nx, int dims, double dx, double dt, double bias, int lim,
                      double gamma, const double* bh) {
    typedef BlackHoleEulerStateVector S;
    EulerMaterialParameters mp(gamma);
    BlackHoleSpacetime b = mkbh(bh);
    if (dims == 1) {
        vector<S> c = to1d<S>(prim, nx);
        BlackHoleEulerForcingSolver::computeRungeKuttaTimeStep(c, dx, dt, bias, lim, mp, b);
        from1d(c, prim);
    } else {
        vector<vector<S> > g = to2d<S>(prim, ny, nx);
        BlackHoleEulerForcingSolver::computeRungeKuttaTimeStep2D(g, dx, dt, bias, lim, mp, b);
        from2d(g, prim);
    }
}

double ref_gr_stable_dt(const double* prim, int ny, int nx, int dims, double dx, double cfl, double t,
                        double tfinal, int it, double gamma, const double* bh) {
    typedef BlackHoleEulerStateVector S;
    EulerMaterialParameters mp(gamma);
    if (dims == 1) return BlackHoleEulerSolvers::computeStableTimeStep(to1d<S>(prim, nx), dx, cfl, t, tfinal, it, mp, mkbh(bh));
    return BlackHoleEulerSolvers::computeStableTimeStep2D(to2d<S>(prim, ny, nx), dx, cfl, t, tfinal, it, mp, mkbh(bh));
}

int ref_gr_solve(double* prim, int ny, int nx, int dims, int order, double dx, double cfl, double tfinal,
                 double bias, int lim, int subcycles, double gamma, const double* bh) {
    typedef BlackHoleEulerStateVector S;
    EulerMaterialParameters mp(gamma);
    BlackHoleSpacetime b = mkbh(bh);
    Quiet q;
    if (dims == 1) {
        auto c = to1d<S>(prim, nx);
        c = order == 2 ? BlackHoleEulerSecondOrderSolver::solve(c, dx, cfl, tfinal, bias, lim, subcycles, mp, b)
                       : BlackHoleEulerFirstOrderSolver::solve(c, dx, cfl, tfinal, subcycles, mp, b);
        from1d(c, prim);
    } else {
        auto g = to2d<S>(prim, ny, nx);
        g = order == 2 ? BlackHoleEulerSecondOrderSolver::solve2D(g, dx, cfl, tfinal, bias, lim, subcycles, mp, b)
                       : BlackHoleEulerFirstOrderSolver::solve2D(g, dx, cfl, tfinal, subcycles, mp, b);
        from2d(g, prim);
    }
    std::string s = q.sink.str();
    int steps = 0;
    for (size_t pos = 0; (pos = s.find("Iteration = ", pos)) != std::string::npos; pos += 12) steps++;
    return steps;
}

// ---------------------------------------------------------------- AMR (level 1)
// Runs the reference's Level-1 AMR driver and returns its final coarse/fine grids and flags.
// sys: 0 Newtonian, 1 SR (the GR driver's file does not compile).  flags as 0/1 bytes.
int ref_amr_level1(int sys, const double* prim, int ny, int nx, int dims, double dx, double cfl, double tfinal,
                   double tol, int order, double gamma, const double* bh, double* coarse_out, double* fine_out,
                   unsigned char* coarse_flags, unsigned char* fine_flags) {
    EulerMaterialParameters mp(gamma);
    Quiet q;
    auto put_flags1 = [](const vector<bool>& f, unsigned char* o) { for (size_t i = 0; i < f.size(); i++) o[i] = f[i] ? 1 : 0; };
    auto put_flags2 = [](const vector<vector<bool> >& f, unsigned char* o) {
        size_t k = 0;
        for (size_t i = 0; i < f.size(); i++) for (size_t j = 0; j < f[i].size(); j++) o[k++] = f[i][j] ? 1 : 0;
    };
#define AMR_CASE(S, CALL1, CALL2)                                                          \
    if (dims == 1) {                                                                       \
        auto r = CALL1;                                                                    \
        from1d(get<0>(r), coarse_out); from1d(get<1>(r), fine_out);                        \
        put_flags1(get<2>(r), coarse_flags); put_flags1(get<3>(r), fine_flags);            \
    } else {                                                                               \
        auto r = CALL2;                                                                    \
        from2d(get<0>(r), coarse_out); from2d(get<1>(r), fine_out);                        \
        put_flags2(get<2>(r), coarse_flags); put_flags2(get<3>(r), fine_flags);            \
    }
    if (sys == 0) {
        typedef EulerStateVector S;
        AMR_CASE(S, EulerAMR::solveLevel1AMR(to1d<S>(prim, nx), dx, cfl, tfinal, tol, order, mp),
                 EulerAMR::solve2DLevel1AMR(to2d<S>(prim, ny, nx), dx, cfl, tfinal, tol, order, mp))
    } else if (sys == 1) {
        typedef RelativisticEulerStateVector S;
        AMR_CASE(S, RelativisticEulerAMR::solveLevel1AMR(to1d<S>(prim, nx), dx, cfl, tfinal, tol, order, mp),
                 RelativisticEulerAMR::solve2DLevel1AMR(to2d<S>(prim, ny, nx), dx, cfl, tfinal, tol, order, mp))
    } else {
        // AMR/BlackHoleEulerAMR.cpp does not compile (see oracle/ref/Makefile); no GR driver.
        (void)bh;
        return -1;
    }
#undef AMR_CASE
    std::string s = q.sink.str();
    int steps = 0;
    for (size_t pos = 0; (pos = s.find("Coarse Grid Iteration", pos)) != std::string::npos; pos += 10) steps++;
    return steps;
}

// ---------------------------------------------------------------- AMR (level 2)
// Runs the reference's Level-2 AMR driver (three levels) and returns its final coarse,
// intermediate and fine grids and flags.  sys: 0 Newtonian, 1 SR.  Returns the number of coarse
// steps (status lines counted), -1 for other systems.
int ref_amr_level2(int sys, const double* prim, int ny, int nx, int dims, double dx, double cfl, double tfinal,
                   double tol, int order, double gamma, double* coarse_out, double* mid_out, double* fine_out,
                   unsigned char* coarse_flags, unsigned char* mid_flags, unsigned char* fine_flags) {
    EulerMaterialParameters mp(gamma);
    Quiet q;
    auto put_flags1 = [](const vector<bool>& f, unsigned char* o) { for (size_t i = 0; i < f.size(); i++) o[i] = f[i] ? 1 : 0; };
    auto put_flags2 = [](const vector<vector<bool> >& f, unsigned char* o) {
        size_t k = 0;
        for (size_t i = 0; i < f.size(); i++) for (size_t j = 0; j < f[i].size(); j++) o[k++] = f[i][j] ? 1 : 0;
    };
#define AMR2_CASE(S, CALL1, CALL2)                                                                   \
    if (dims == 1) {                                                                                 \
        auto r = CALL1;                                                                              \
        from1d(get<0>(r), coarse_out); from1d(get<1>(r), mid_out); from1d(get<2>(r), fine_out);      \
        put_flags1(get<3>(r), coarse_flags); put_flags1(get<4>(r), mid_flags);                       \
        put_flags1(get<5>(r), fine_flags);                                                           \
    } else {                                                                                         \
        auto r = CALL2;                                                                              \
        from2d(get<0>(r), coarse_out); from2d(get<1>(r), mid_out); from2d(get<2>(r), fine_out);      \
        put_flags2(get<3>(r), coarse_flags); put_flags2(get<4>(r), mid_flags);                       \
        put_flags2(get<5>(r), fine_flags);                                                           \
    }
    if (sys == 0) {
        typedef EulerStateVector S;
        AMR2_CASE(S, EulerAMR::solveLevel2AMR(to1d<S>(prim, nx), dx, cfl, tfinal, tol, order, mp),
                  EulerAMR::solve2DLevel2AMR(to2d<S>(prim, ny, nx), dx, cfl, tfinal, tol, order, mp))
    } else if (sys == 1) {
        typedef RelativisticEulerStateVector S;
        AMR2_CASE(S, RelativisticEulerAMR::solveLevel2AMR(to1d<S>(prim, nx), dx, cfl, tfinal, tol, order, mp),
                  RelativisticEulerAMR::solve2DLevel2AMR(to2d<S>(prim, ny, nx), dx, cfl, tfinal, tol, order, mp))
    } else {
        return -1;
    }
#undef AMR2_CASE
    std::string s = q.sink.str();
    int steps = 0;
    for (size_t pos = 0; (pos = s.find("Coarse Grid Iteration", pos)) != std::string::npos; pos += 10) steps++;
    return steps;
}

}  // extern "C"
