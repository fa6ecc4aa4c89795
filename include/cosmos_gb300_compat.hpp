// C++ drop-in shim: the reference's class and method names over the cosmos_gb300 C ABI.
//
// Code written against the reference (JonathanGorard/Cosmos) -- e.g. its Tests/*.cpp drivers --
// compiles against this header instead of the reference's Euler/, RelativisticEuler/,
// BlackHoleEuler/ and Solvers/ headers.  Grid-level methods (solve, solve2D, the per-sweep
// compute*TimeStep*, computeMaximumWaveSpeed*, computeStableTimeStep*, the forcing step) run on
// the GPU through the C ABI with the reference's arguments; the state classes keep the
// reference's primitive storage (density, x/y/z velocity, pressure) and accessors.
//
// Differences a caller can see: every grid call returns the same values as the reference (FP64
// path, bit-identical); failures throw std::runtime_error with cosmos_last_error()'s text (the
// reference has no error reporting); no per-step status line is printed.
#pragma once

#include <cmath>
#include <iostream>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "cosmos_gb300.h"

namespace cosmos_compat_detail {

inline void check(int rc) {
    if (rc != COSMOS_OK) throw std::runtime_error(std::string("cosmos_gb300: ") + cosmos_last_error());
}

struct Ctx {
    cosmos_ctx* c = nullptr;
    Ctx() { check(cosmos_ctx_create(0, &c)); }
    ~Ctx() { cosmos_ctx_destroy(c); }
};
inline cosmos_ctx* ctx() {
    static thread_local Ctx c;
    return c.c;
}

// A device grid for the duration of one call.
struct Grid {
    cosmos_grid* g = nullptr;
    Grid(int system, int dims, int nx, int ny, double dx, double gamma, const double* bh) {
        cosmos_params p;
        cosmos_params_default(&p);
        p.system = system;
        p.dims = dims;
        p.nx = nx;
        p.ny = dims == 1 ? 1 : ny;
        p.dx = dx;
        p.gamma = gamma;
        if (bh) { p.bh_mass = bh[0]; p.bh_spin = bh[1]; p.bh_x = bh[2]; p.bh_y = bh[3]; p.bh_z = bh[4]; }
        check(cosmos_grid_create(ctx(), &p, &g));
    }
    ~Grid() { cosmos_grid_destroy(g); }
};

template <class S> std::vector<double> pack1(const std::vector<S>& c) {
    std::vector<double> a(c.size() * 5);
    for (size_t i = 0; i < c.size(); i++) {
        S s = c[i];
        a[5 * i] = s.getDensity(); a[5 * i + 1] = s.getXVelocity(); a[5 * i + 2] = s.getYVelocity();
        a[5 * i + 3] = s.getZVelocity(); a[5 * i + 4] = s.getPressure();
    }
    return a;
}
template <class S> void unpack1(const std::vector<double>& a, std::vector<S>& c) {
    for (size_t i = 0; i < c.size(); i++) c[i] = S(a[5 * i], a[5 * i + 1], a[5 * i + 2], a[5 * i + 3], a[5 * i + 4]);
}
template <class S> std::vector<double> pack2(const std::vector<std::vector<S> >& g) {
    std::vector<double> a;
    a.reserve(g.size() * g[0].size() * 5);
    for (const auto& row : g) {
        std::vector<double> r = pack1(row);
        a.insert(a.end(), r.begin(), r.end());
    }
    return a;
}
template <class S> void unpack2(const std::vector<double>& a, std::vector<std::vector<S> >& g) {
    size_t k = 0;
    for (auto& row : g)
        for (auto& s : row) { s = S(a[k], a[k + 1], a[k + 2], a[k + 3], a[k + 4]); k += 5; }
}

}  // namespace cosmos_compat_detail

// ----------------------------------------------------------------------------- material, spacetime
class EulerMaterialParameters {  // Euler/EulerMaterialParameters.hpp
public:
    EulerMaterialParameters() : adiabaticIndex(1.0) {}
    EulerMaterialParameters(double g) : adiabaticIndex(g) {}
    void setAdiabaticIndex(double g) { adiabaticIndex = g; }
    double getAdiabaticIndex() { return adiabaticIndex; }
private:
    double adiabaticIndex;
};

class BlackHoleSpacetime {  // BlackHoleEuler/BlackHoleSpacetime.hpp (parameters; the metric lives on the GPU)
public:
    BlackHoleSpacetime() : m(1.0), a(0.0), x(0.5), y(0.5), z(0.0) {}
    BlackHoleSpacetime(double M) : m(M), a(0.0), x(0.5), y(0.5), z(0.0) {}
    BlackHoleSpacetime(double M, double X, double Y, double Z) : m(M), a(0.0), x(X), y(Y), z(Z) {}
    BlackHoleSpacetime(double M, double A) : m(M), a(A), x(0.5), y(0.5), z(0.0) {}
    BlackHoleSpacetime(double M, double A, double X, double Y, double Z) : m(M), a(A), x(X), y(Y), z(Z) {}
    void setBlackHoleMass(double v) { m = v; }
    void setBlackHoleSpin(double v) { a = v; }
    void setBlackHoleXPosition(double v) { x = v; }
    void setBlackHoleYPosition(double v) { y = v; }
    void setBlackHoleZPosition(double v) { z = v; }
    double getBlackHoleMass() { return m; }
    double getBlackHoleSpin() { return a; }
    double getBlackHoleXPosition() { return x; }
    double getBlackHoleYPosition() { return y; }
    double getBlackHoleZPosition() { return z; }
    // BlackHoleEuler/BlackHoleSpacetime.cpp:372-386: Euclidean distance within M (1 + sqrt(1 - a^2))
    bool inExcisionRegion(double X, double Y, double Z) const {
        const double r = std::sqrt((((X - x) * (X - x)) + ((Y - y) * (Y - y))) + ((Z - z) * (Z - z)));
        return r <= (m * (1.0 + std::sqrt(1.0 - (a * a))));
    }
    void pack(double* o) const { o[0] = m; o[1] = a; o[2] = x; o[3] = y; o[4] = z; }

    // The metric methods (BlackHoleEuler/BlackHoleSpacetime.hpp:16-40), evaluated on the device
    // (cosmos_spacetime_eval), bit for bit with the reference.
    double computeKerrSchildScalar(double X, double Y, double Z) { return rec(X, Y, Z)[COSMOS_ST_KS_SCALAR]; }
    std::vector<double> computeKerrSchildVector(double X, double Y, double Z) { return vec(rec(X, Y, Z), COSMOS_ST_KS_VECTOR, 3); }
    std::vector<double> computeKerrSchildSpacetimeVector(double X, double Y, double Z) {
        return vec(rec(X, Y, Z), COSMOS_ST_KS_SPACETIME_VECTOR, 4);
    }
    std::vector<double> computeKerrSchildScalarDerivative(double X, double Y, double Z, double h) {
        return vec(rec(X, Y, Z, h), COSMOS_ST_KS_SCALAR_DERIVATIVE, 3);
    }
    std::vector<std::vector<double> > computeKerrSchildVectorDerivative(double X, double Y, double Z, double h) {
        return mat(rec(X, Y, Z, h), COSMOS_ST_KS_VECTOR_DERIVATIVE, 3);
    }
    std::vector<std::vector<double> > computeSpatialMetricTensor(double X, double Y, double Z) {
        return mat(rec(X, Y, Z), COSMOS_ST_SPATIAL_METRIC, 3);
    }
    std::vector<std::vector<double> > computeSpacetimeMetricTensor(double X, double Y, double Z) {
        return mat(rec(X, Y, Z), COSMOS_ST_SPACETIME_METRIC, 4);
    }
    std::vector<std::vector<double> > computeInverseSpatialMetricTensor(double X, double Y, double Z) {
        return mat(rec(X, Y, Z), COSMOS_ST_INVERSE_SPATIAL_METRIC, 3);
    }
    std::vector<std::vector<double> > computeInverseSpacetimeMetricTensor(double X, double Y, double Z) {
        return mat(rec(X, Y, Z), COSMOS_ST_INVERSE_SPACETIME_METRIC, 4);
    }
    double computeSpatialMetricDeterminant(double X, double Y, double Z) { return rec(X, Y, Z)[COSMOS_ST_SPATIAL_DETERMINANT]; }
    double computeSpacetimeMetricDeterminant(double X, double Y, double Z) {
        return rec(X, Y, Z)[COSMOS_ST_SPACETIME_DETERMINANT];
    }
    std::vector<std::vector<std::vector<double> > > computeSpatialMetricTensorDerivative(double X, double Y, double Z, double h) {
        const std::vector<double> r = rec(X, Y, Z, h);
        std::vector<std::vector<std::vector<double> > > d(3);
        for (int k = 0; k < 3; k++) d[k] = mat(r, COSMOS_ST_SPATIAL_METRIC_DERIVATIVE + 9 * k, 3);
        return d;
    }
    double computeLapseFunction(double X, double Y, double Z) { return rec(X, Y, Z)[COSMOS_ST_LAPSE]; }
    std::vector<double> computeShiftVector(double X, double Y, double Z) { return vec(rec(X, Y, Z), COSMOS_ST_SHIFT, 3); }
    std::vector<double> computeLapseFunctionDerivative(double X, double Y, double Z, double h) {
        return vec(rec(X, Y, Z, h), COSMOS_ST_LAPSE_DERIVATIVE, 3);
    }
    std::vector<std::vector<double> > computeShiftVectorDerivative(double X, double Y, double Z, double h) {
        return mat(rec(X, Y, Z, h), COSMOS_ST_SHIFT_DERIVATIVE, 3);
    }
    std::vector<std::vector<double> > computeExtrinsicCurvatureTensor(double X, double Y, double Z, double h) {
        return mat(rec(X, Y, Z, h), COSMOS_ST_EXTRINSIC_CURVATURE, 3);
    }

private:
    std::vector<double> rec(double X, double Y, double Z, double h = 1.0) const {
        cosmos_params p;
        cosmos_params_default(&p);
        p.system = COSMOS_GR;
        p.dx = h;
        p.bh_mass = m; p.bh_spin = a; p.bh_x = x; p.bh_y = y; p.bh_z = z;
        std::vector<double> o(COSMOS_SPACETIME_WIDTH);
        const double q[3] = {X, Y, Z};
        cosmos_compat_detail::check(cosmos_spacetime_eval(cosmos_compat_detail::ctx(), &p, 1, q, o.data()));
        return o;
    }
    static std::vector<double> vec(const std::vector<double>& r, int at, int n) {
        return std::vector<double>(r.begin() + at, r.begin() + at + n);
    }
    static std::vector<std::vector<double> > mat(const std::vector<double>& r, int at, int n) {
        std::vector<std::vector<double> > o(n, std::vector<double>(n));
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++) o[i][j] = r[at + n * i + j];
        return o;
    }
    double m, a, x, y, z;
};

// ----------------------------------------------------------------------------- state-level functions
// One state (or three, for slopes) through cosmos_state_eval: the device's reference-exact kernels.
namespace cosmos_compat_detail {
inline std::vector<double> state_op(int sys, int op, const std::vector<double>& in, double gamma,
                                    const double* xyz = nullptr, const BlackHoleSpacetime* bh = nullptr,
                                    double dx = 0.0, double bias = 0.0, int lim = 1) {
    cosmos_params p;
    cosmos_params_default(&p);
    p.system = sys;
    p.gamma = gamma;
    p.dx = dx;
    if (bh) {
        double b[5];
        bh->pack(b);
        p.bh_mass = b[0]; p.bh_spin = b[1]; p.bh_x = b[2]; p.bh_y = b[3]; p.bh_z = b[4];
    }
    size_t wi = 0, wo = 0;
    check(cosmos_state_width(op, &wi, &wo));
    std::vector<double> out(wo);
    check(cosmos_state_eval(ctx(), &p, op, 1, in.data(), xyz, bias, lim, out.data()));
    return out;
}

// One item of a per-interface solver function (cosmos_interface_eval): `in` holds the function's
// vector and state arguments back to back (states as primitive vectors).
inline std::vector<double> iface_op(int sys, int op, const std::vector<double>& in, double gamma, double dx, double dt,
                                    double bias = 0.0, int lim = 1, double frac = 0.5, int side = 0,
                                    const double* xyz = nullptr, const BlackHoleSpacetime* bh = nullptr) {
    cosmos_params p;
    cosmos_params_default(&p);
    p.system = sys;
    p.gamma = gamma;
    p.dx = dx;
    if (bh) {
        double b[5];
        bh->pack(b);
        p.bh_mass = b[0]; p.bh_spin = b[1]; p.bh_x = b[2]; p.bh_y = b[3]; p.bh_z = b[4];
    }
    std::vector<double> out(5);
    check(cosmos_interface_eval(ctx(), &p, op, 1, in.data(), xyz, dt, bias, lim, frac, side, out.data()));
    return out;
}
inline void cat_into(std::vector<double>&) {}
template <class... R>
inline void cat_into(std::vector<double>& o, const std::vector<double>& v, const R&... rest) {
    o.insert(o.end(), v.begin(), v.end());
    cat_into(o, rest...);
}
template <class... V> inline std::vector<double> cat(const V&... v) {
    std::vector<double> o;
    cat_into(o, v...);
    return o;
}
template <class S> inline std::vector<double> pv(S s) { return s.computePrimitiveVariableVector(); }
template <class S> inline S from_prim(const std::vector<double>& p) { return S(p[0], p[1], p[2], p[3], p[4]); }
}  // namespace cosmos_compat_detail

// ----------------------------------------------------------------------------- state vectors
// Primitive storage and accessors as in Euler/EulerStateVector.hpp:8-48 (and the SR/GR twins); the
// physics methods (conserved variables, fluxes, sound speed, ...) evaluate on the GPU.
#define COSMOS_COMPAT_STATE(NAME, METHODS)                                                                 \
    class NAME {                                                                                           \
    public:                                                                                                \
        NAME() : density(1.0), xVelocity(0.0), yVelocity(0.0), zVelocity(0.0), pressure(1.0) {}          \
        NAME(double r, double vx, double vy, double vz, double p)                                          \
            : density(r), xVelocity(vx), yVelocity(vy), zVelocity(vz), pressure(p) {}                      \
        void setPrimitiveVariableVector(std::vector<double> v) {                                           \
            density = v[0]; xVelocity = v[1]; yVelocity = v[2]; zVelocity = v[3]; pressure = v[4];         \
        }                                                                                                  \
        std::vector<double> computePrimitiveVariableVector() {                                             \
            return std::vector<double>{density, xVelocity, yVelocity, zVelocity, pressure};                \
        }                                                                                                  \
        void setDensity(double v) { density = v; }                                                         \
        void setXVelocity(double v) { xVelocity = v; }                                                     \
        void setYVelocity(double v) { yVelocity = v; }                                                     \
        void setZVelocity(double v) { zVelocity = v; }                                                     \
        void setPressure(double v) { pressure = v; }                                                       \
        double getDensity() { return density; }                                                            \
        double getXVelocity() { return xVelocity; }                                                        \
        double getYVelocity() { return yVelocity; }                                                        \
        double getZVelocity() { return zVelocity; }                                                        \
        double getPressure() { return pressure; }                                                          \
        METHODS                                                                                            \
    private:                                                                                               \
        double density, xVelocity, yVelocity, zVelocity, pressure;                                         \
    };

// Newtonian and SR: Euler/EulerStateVector.hpp:14-28, RelativisticEuler/RelativisticEulerStateVector.hpp:14-26
// (the member flux methods take the flux of the state's own conserved vector, as the reference's do).
#define COSMOS_COMPAT_FLAT_METHODS(SYS)                                                                    \
    std::vector<double> computeConservedVariableVector(EulerMaterialParameters mp) {                       \
        return cosmos_compat_detail::state_op(SYS, COSMOS_STATE_CONS, computePrimitiveVariableVector(),    \
                                              mp.getAdiabaticIndex());                                     \
    }                                                                                                      \
    void setConservedVariableVector(std::vector<double> u, EulerMaterialParameters mp) {                   \
        setPrimitiveVariableVector(cosmos_compat_detail::state_op(SYS, COSMOS_STATE_PRIM, u, mp.getAdiabaticIndex())); \
    }                                                                                                      \
    static std::vector<double> computeXFluxVector(std::vector<double> u, EulerMaterialParameters mp) {     \
        return cosmos_compat_detail::state_op(SYS, COSMOS_STATE_FLUX_X, u, mp.getAdiabaticIndex());        \
    }                                                                                                      \
    std::vector<double> computeXFluxVector(EulerMaterialParameters mp) {                                   \
        return computeXFluxVector(computeConservedVariableVector(mp), mp);                                 \
    }                                                                                                      \
    static std::vector<double> computeYFluxVector(std::vector<double> u, EulerMaterialParameters mp) {     \
        return cosmos_compat_detail::state_op(SYS, COSMOS_STATE_FLUX_Y, u, mp.getAdiabaticIndex());        \
    }                                                                                                      \
    std::vector<double> computeYFluxVector(EulerMaterialParameters mp) {                                   \
        return computeYFluxVector(computeConservedVariableVector(mp), mp);                                 \
    }                                                                                                      \
    double computeSoundSpeed(EulerMaterialParameters mp) {                                                 \
        return cosmos_compat_detail::state_op(SYS, COSMOS_STATE_SOUND, computePrimitiveVariableVector(),   \
                                              mp.getAdiabaticIndex())[0];                                  \
    }
#define COSMOS_COMPAT_EULER_METHODS                                                                        \
    COSMOS_COMPAT_FLAT_METHODS(COSMOS_NEWTONIAN)                                                           \
    double computeSpecificInternalEnergy(EulerMaterialParameters mp) {                                     \
        return cosmos_compat_detail::state_op(COSMOS_NEWTONIAN, COSMOS_STATE_INTERNAL_ENERGY,              \
                                              computePrimitiveVariableVector(), mp.getAdiabaticIndex())[0]; \
    }                                                                                                      \
    double computeTotalEnergy(EulerMaterialParameters mp) {                                                \
        return cosmos_compat_detail::state_op(COSMOS_NEWTONIAN, COSMOS_STATE_TOTAL_ENERGY,                 \
                                              computePrimitiveVariableVector(), mp.getAdiabaticIndex())[0]; \
    }
// Black hole: BlackHoleEuler/BlackHoleEulerStateVector.hpp:14-37, functions of the coordinates.
#define COSMOS_COMPAT_BH_METHODS                                                                           \
    std::vector<double> computeConservedVariableVector(double x, double y, double z, EulerMaterialParameters mp, \
                                                       BlackHoleSpacetime bh) {                            \
        const double q[3] = {x, y, z};                                                                     \
        return cosmos_compat_detail::state_op(COSMOS_GR, COSMOS_STATE_CONS, computePrimitiveVariableVector(), \
                                              mp.getAdiabaticIndex(), q, &bh);                             \
    }                                                                                                      \
    void setConservedVariableVector(std::vector<double> u, double x, double y, double z, EulerMaterialParameters mp, \
                                    BlackHoleSpacetime bh) {                                               \
        const double q[3] = {x, y, z};                                                                     \
        setPrimitiveVariableVector(cosmos_compat_detail::state_op(COSMOS_GR, COSMOS_STATE_PRIM, u,         \
                                                                  mp.getAdiabaticIndex(), q, &bh));        \
    }                                                                                                      \
    static std::vector<double> computeXFluxVector(std::vector<double> u, double x, double y, double z,     \
                                                  EulerMaterialParameters mp, BlackHoleSpacetime bh) {     \
        const double q[3] = {x, y, z};                                                                     \
        return cosmos_compat_detail::state_op(COSMOS_GR, COSMOS_STATE_FLUX_X, u, mp.getAdiabaticIndex(), q, &bh); \
    }                                                                                                      \
    std::vector<double> computeXFluxVector(double x, double y, double z, EulerMaterialParameters mp,       \
                                           BlackHoleSpacetime bh) {                                        \
        return computeXFluxVector(computeConservedVariableVector(x, y, z, mp, bh), x, y, z, mp, bh);       \
    }                                                                                                      \
    static std::vector<double> computeYFluxVector(std::vector<double> u, double x, double y, double z,     \
                                                  EulerMaterialParameters mp, BlackHoleSpacetime bh) {     \
        const double q[3] = {x, y, z};                                                                     \
        return cosmos_compat_detail::state_op(COSMOS_GR, COSMOS_STATE_FLUX_Y, u, mp.getAdiabaticIndex(), q, &bh); \
    }                                                                                                      \
    std::vector<double> computeYFluxVector(double x, double y, double z, EulerMaterialParameters mp,       \
                                           BlackHoleSpacetime bh) {                                        \
        return computeYFluxVector(computeConservedVariableVector(x, y, z, mp, bh), x, y, z, mp, bh);       \
    }                                                                                                      \
    static std::vector<double> computeSourceTermVector(std::vector<double> u, double x, double y, double z, \
                                                       double h, EulerMaterialParameters mp, BlackHoleSpacetime bh) { \
        const double q[3] = {x, y, z};                                                                     \
        return cosmos_compat_detail::state_op(COSMOS_GR, COSMOS_STATE_SOURCE, u, mp.getAdiabaticIndex(), q, &bh, h); \
    }                                                                                                      \
    std::vector<double> computeSourceTermVector(double x, double y, double z, double h, EulerMaterialParameters mp, \
                                                BlackHoleSpacetime bh) {                                   \
        return computeSourceTermVector(computeConservedVariableVector(x, y, z, mp, bh), x, y, z, h, mp, bh); \
    }                                                                                                      \
    double computeSoundSpeed(double x, double y, double z, EulerMaterialParameters mp, BlackHoleSpacetime bh) { \
        const double q[3] = {x, y, z};                                                                     \
        return cosmos_compat_detail::state_op(COSMOS_GR, COSMOS_STATE_SOUND, computePrimitiveVariableVector(), \
                                              mp.getAdiabaticIndex(), q, &bh)[0];                          \
    }

COSMOS_COMPAT_STATE(EulerStateVector, COSMOS_COMPAT_EULER_METHODS)
COSMOS_COMPAT_STATE(RelativisticEulerStateVector, COSMOS_COMPAT_FLAT_METHODS(COSMOS_SR))
COSMOS_COMPAT_STATE(BlackHoleEulerStateVector, COSMOS_COMPAT_BH_METHODS)
#undef COSMOS_COMPAT_STATE
#undef COSMOS_COMPAT_FLAT_METHODS
#undef COSMOS_COMPAT_EULER_METHODS
#undef COSMOS_COMPAT_BH_METHODS

// ----------------------------------------------------------------------------- equations of state
class EulerEquationOfState {  // Euler/EulerEquationOfState.hpp
public:
    static double computeSpecificInternalEnergy(double rho, double p, EulerMaterialParameters mp) {
        return cosmos_compat_detail::state_op(COSMOS_NEWTONIAN, COSMOS_STATE_INTERNAL_ENERGY, {rho, 0.0, 0.0, 0.0, p},
                                              mp.getAdiabaticIndex())[0];
    }
    static double computePressure(double rho, double e, EulerMaterialParameters mp) {
        return cosmos_compat_detail::state_op(COSMOS_NEWTONIAN, COSMOS_STATE_PRESSURE, {rho, 0.0, 0.0, 0.0, e},
                                              mp.getAdiabaticIndex())[0];
    }
    static double computeSoundSpeed(double rho, double p, EulerMaterialParameters mp) {
        return cosmos_compat_detail::state_op(COSMOS_NEWTONIAN, COSMOS_STATE_SOUND, {rho, 0.0, 0.0, 0.0, p},
                                              mp.getAdiabaticIndex())[0];
    }
};

class RelativisticEulerEquationOfState {  // RelativisticEuler/RelativisticEulerEquationOfState.hpp
public:
    static double computeSpecificEnthalpy(double rho, double p, EulerMaterialParameters mp) {
        return cosmos_compat_detail::state_op(COSMOS_SR, COSMOS_STATE_ENTHALPY, {rho, 0.0, 0.0, 0.0, p},
                                              mp.getAdiabaticIndex())[0];
    }
    static double computeSoundSpeed(double rho, double p, EulerMaterialParameters mp) {
        return cosmos_compat_detail::state_op(COSMOS_SR, COSMOS_STATE_SOUND, {rho, 0.0, 0.0, 0.0, p},
                                              mp.getAdiabaticIndex())[0];
    }
};

// ----------------------------------------------------------------------------- slope limiters
class SlopeLimiters {  // Solvers/SlopeLimiters.hpp (0 SuperBee, 1 van Leer, anything else MinBee)
public:
    static double computeGradientRatio(double r, double bias) {
        return cosmos_compat_detail::state_op(COSMOS_NEWTONIAN, COSMOS_STATE_GRADIENT_RATIO, {r}, 1.4, nullptr, nullptr,
                                              0.0, bias)[0];
    }
    static double computeSlopeLimiter(double r, double bias, int limiter) {
        return cosmos_compat_detail::state_op(COSMOS_NEWTONIAN, COSMOS_STATE_LIMITER, {r}, 1.4, nullptr, nullptr, 0.0,
                                              bias, limiter)[0];
    }
    static double computeSuperBeeSlopeLimiter(double r, double bias) { return computeSlopeLimiter(r, bias, 0); }
    static double computeVanLeerSlopeLimiter(double r, double bias) { return computeSlopeLimiter(r, bias, 1); }
    static double computeMinBeeSlopeLimiter(double r, double bias) { return computeSlopeLimiter(r, bias, 2); }
    static std::vector<double> computeSlopeVector(std::vector<double> l, std::vector<double> m, std::vector<double> r,
                                                  double bias, int limiter) {
        std::vector<double> in(l);
        in.insert(in.end(), m.begin(), m.end());
        in.insert(in.end(), r.begin(), r.end());
        return cosmos_compat_detail::state_op(COSMOS_NEWTONIAN, COSMOS_STATE_SLOPE, in, 1.4, nullptr, nullptr, 0.0, bias,
                                              limiter);
    }
    static std::vector<double> computeSlopeVector(EulerStateVector l, EulerStateVector m, EulerStateVector r, double bias,
                                                  int limiter, EulerMaterialParameters mp) {
        return computeSlopeVector(l.computeConservedVariableVector(mp), m.computeConservedVariableVector(mp),
                                  r.computeConservedVariableVector(mp), bias, limiter);
    }
    static std::vector<double> computeSlopeVector(RelativisticEulerStateVector l, RelativisticEulerStateVector m,
                                                  RelativisticEulerStateVector r, double bias, int limiter,
                                                  EulerMaterialParameters mp) {
        return computeSlopeVector(l.computeConservedVariableVector(mp), m.computeConservedVariableVector(mp),
                                  r.computeConservedVariableVector(mp), bias, limiter);
    }
    // Solvers/SlopeLimiters.cpp:103-147: neighbours evaluated one spacing away along the axis
    static std::vector<double> computeSlopeVectorX(BlackHoleEulerStateVector l, BlackHoleEulerStateVector m,
                                                   BlackHoleEulerStateVector r, double dx, double bias, int limiter,
                                                   double x, double y, double z, EulerMaterialParameters mp,
                                                   BlackHoleSpacetime bh) {
        return computeSlopeVector(l.computeConservedVariableVector(x - dx, y, z, mp, bh),
                                  m.computeConservedVariableVector(x, y, z, mp, bh),
                                  r.computeConservedVariableVector(x + dx, y, z, mp, bh), bias, limiter);
    }
    static std::vector<double> computeSlopeVectorY(BlackHoleEulerStateVector t, BlackHoleEulerStateVector m,
                                                   BlackHoleEulerStateVector b, double dx, double bias, int limiter,
                                                   double x, double y, double z, EulerMaterialParameters mp,
                                                   BlackHoleSpacetime bh) {
        return computeSlopeVector(t.computeConservedVariableVector(x, y - dx, z, mp, bh),
                                  m.computeConservedVariableVector(x, y, z, mp, bh),
                                  b.computeConservedVariableVector(x, y + dx, z, mp, bh), bias, limiter);
    }
};

// ----------------------------------------------------------------------------- black-hole eigenvalues
class BlackHoleEulerEigenvalues {  // BlackHoleEuler/BlackHoleEulerEigenvalues.hpp
public:
    static std::vector<double> computeMaterialWaveEigenvalues(double x, double y, double z, double vx, double vy, double vz,
                                                              EulerMaterialParameters mp, BlackHoleSpacetime bh) {
        return part(x, y, z, 1.0, 1.0, vx, vy, vz, mp, bh, 0);
    }
    static std::vector<double> computeFastAcousticWaveEigenvalues(double x, double y, double z, double rho, double p,
                                                                  double vx, double vy, double vz,
                                                                  EulerMaterialParameters mp, BlackHoleSpacetime bh) {
        return part(x, y, z, rho, p, vx, vy, vz, mp, bh, 1);
    }
    static std::vector<double> computeSlowAcousticWaveEigenvalues(double x, double y, double z, double rho, double p,
                                                                  double vx, double vy, double vz,
                                                                  EulerMaterialParameters mp, BlackHoleSpacetime bh) {
        return part(x, y, z, rho, p, vx, vy, vz, mp, bh, 2);
    }
private:
    static std::vector<double> part(double x, double y, double z, double rho, double p, double vx, double vy, double vz,
                                    EulerMaterialParameters mp, BlackHoleSpacetime bh, int which) {
        const double q[3] = {x, y, z};
        std::vector<double> all = cosmos_compat_detail::state_op(COSMOS_GR, COSMOS_STATE_EIGENVALUES, {rho, vx, vy, vz, p},
                                                                 mp.getAdiabaticIndex(), q, &bh);
        return std::vector<double>(all.begin() + 3 * which, all.begin() + 3 * which + 3);
    }
};

// ----------------------------------------------------------------------------- solvers
namespace cosmos_compat_detail {

template <class S>
std::vector<S> solve1(int sys, std::vector<S> cells, double dx, double cfl, double T, int order, double bias, int lim,
                      EulerMaterialParameters mp, int sub = 1, const BlackHoleSpacetime* bh = nullptr) {
    double b[5];
    if (bh) bh->pack(b);
    Grid g(sys, 1, (int)cells.size(), 1, dx, mp.getAdiabaticIndex(), bh ? b : nullptr);
    std::vector<double> a = pack1(cells);
    check(cosmos_grid_set_prim(g.g, a.data(), a.size()));
    cosmos_solve_opts o;
    cosmos_solve_opts_default(&o);
    o.order = order; o.cfl = cfl; o.t_final = T; o.bias = bias; o.limiter = lim; o.subcycles = sub;
    cosmos_solve_result r;
    check(cosmos_grid_solve(g.g, &o, &r));
    check(cosmos_grid_get_prim(g.g, a.data(), a.size()));
    unpack1(a, cells);
    return cells;
}
template <class S>
std::vector<std::vector<S> > solve2(int sys, std::vector<std::vector<S> > cells, double dx, double cfl, double T,
                                    int order, double bias, int lim, EulerMaterialParameters mp, int sub = 1,
                                    const BlackHoleSpacetime* bh = nullptr) {
    double b[5];
    if (bh) bh->pack(b);
    Grid g(sys, 2, (int)cells[0].size(), (int)cells.size(), dx, mp.getAdiabaticIndex(), bh ? b : nullptr);
    std::vector<double> a = pack2(cells);
    check(cosmos_grid_set_prim(g.g, a.data(), a.size()));
    cosmos_solve_opts o;
    cosmos_solve_opts_default(&o);
    o.order = order; o.cfl = cfl; o.t_final = T; o.bias = bias; o.limiter = lim; o.subcycles = sub;
    cosmos_solve_result r;
    check(cosmos_grid_solve(g.g, &o, &r));
    check(cosmos_grid_get_prim(g.g, a.data(), a.size()));
    unpack2(a, cells);
    return cells;
}
template <class S>
void sweep1(int sys, std::vector<S>& cells, double dx, double dt, int order, double bias, int lim,
            EulerMaterialParameters mp, const BlackHoleSpacetime* bh = nullptr) {
    double b[5];
    if (bh) bh->pack(b);
    Grid g(sys, 1, (int)cells.size(), 1, dx, mp.getAdiabaticIndex(), bh ? b : nullptr);
    std::vector<double> a = pack1(cells);
    check(cosmos_grid_set_prim(g.g, a.data(), a.size()));
    check(cosmos_grid_sweep(g.g, 0, order, dt, bias, lim));
    check(cosmos_grid_get_prim(g.g, a.data(), a.size()));
    unpack1(a, cells);
}
template <class S>
void sweep2(int sys, std::vector<std::vector<S> >& cells, double dx, double dt, int axis, int order, double bias,
            int lim, EulerMaterialParameters mp, const BlackHoleSpacetime* bh = nullptr) {
    double b[5];
    if (bh) bh->pack(b);
    Grid g(sys, 2, (int)cells[0].size(), (int)cells.size(), dx, mp.getAdiabaticIndex(), bh ? b : nullptr);
    std::vector<double> a = pack2(cells);
    check(cosmos_grid_set_prim(g.g, a.data(), a.size()));
    check(cosmos_grid_sweep(g.g, axis, order, dt, bias, lim));
    check(cosmos_grid_get_prim(g.g, a.data(), a.size()));
    unpack2(a, cells);
}
template <class S, class Cells>
double max_speed(int sys, Cells& cells, int dims, EulerMaterialParameters mp, const BlackHoleSpacetime* bh = nullptr);
template <class S>
double max_speed1(int sys, std::vector<S>& c, EulerMaterialParameters mp, const BlackHoleSpacetime* bh = nullptr) {
    double b[5];
    if (bh) bh->pack(b);
    Grid g(sys, 1, (int)c.size(), 1, 1.0, mp.getAdiabaticIndex(), bh ? b : nullptr);
    std::vector<double> a = pack1(c);
    check(cosmos_grid_set_prim(g.g, a.data(), a.size()));
    double s;
    check(cosmos_grid_max_wavespeed(g.g, &s));
    return s;
}
template <class S>
double max_speed2(int sys, std::vector<std::vector<S> >& c, EulerMaterialParameters mp,
                  const BlackHoleSpacetime* bh = nullptr) {
    double b[5];
    if (bh) bh->pack(b);
    Grid g(sys, 2, (int)c[0].size(), (int)c.size(), 1.0, mp.getAdiabaticIndex(), bh ? b : nullptr);
    std::vector<double> a = pack2(c);
    check(cosmos_grid_set_prim(g.g, a.data(), a.size()));
    double s;
    check(cosmos_grid_max_wavespeed(g.g, &s));
    return s;
}

// EulerSolvers::insertBoundaryCells(2D) (Solvers/EulerSolvers.cpp:3-85; the SR and black-hole
// twins are the same): a copy with 1 or 2 transmissive ghost cells per side (mirrored order for 2);
// the 2D corners keep default-constructed states, as in the reference.
template <class S> std::vector<S> insert_boundary(const std::vector<S>& c, int b) {
    const long n = (long)c.size();
    std::vector<S> o(n + 2 * b);
    if (b == 1) {
        o[0] = c[0];
        o[n + 1] = c[n - 1];
    } else if (b == 2) {
        o[0] = c[1]; o[1] = c[0];
        o[n + 2] = c[n - 1]; o[n + 3] = c[n - 2];
    }
    for (long i = 0; i < n; i++) o[i + b] = c[i];
    return o;
}
template <class S> std::vector<std::vector<S> > insert_boundary_2d(const std::vector<std::vector<S> >& c, int b) {
    const long rows = (long)c.size(), cols = (long)c[0].size();
    std::vector<std::vector<S> > o(rows + 2 * b, std::vector<S>(cols + 2 * b));
    if (b == 1) {
        for (long i = 0; i < rows; i++) { o[i + 1][0] = c[i][0]; o[i + 1][cols + 1] = c[i][cols - 1]; }
        for (long j = 0; j < cols; j++) { o[0][j + 1] = c[0][j]; o[rows + 1][j + 1] = c[rows - 1][j]; }
    } else if (b == 2) {
        for (long i = 0; i < rows; i++) {
            o[i + 2][0] = c[i][1]; o[i + 2][1] = c[i][0];
            o[i + 2][cols + 2] = c[i][cols - 1]; o[i + 2][cols + 3] = c[i][cols - 2];
        }
        for (long j = 0; j < cols; j++) {
            o[0][j + 2] = c[1][j]; o[1][j + 2] = c[0][j];
            o[rows + 2][j + 2] = c[rows - 1][j]; o[rows + 3][j + 2] = c[rows - 2][j];
        }
    }
    for (long i = 0; i < rows; i++)
        for (long j = 0; j < cols; j++) o[i + b][j + b] = c[i][j];
    return o;
}

}  // namespace cosmos_compat_detail

// Per-interface building blocks (evolveStateByHalf*, compute*Flux): one item each through
// cosmos_interface_eval, bit for bit with the reference.  VEC_SOLVERS / VEC_FIRST add the vector
// forms the Newtonian classes declare (Solvers/EulerSolvers.hpp:25-27, EulerFirstOrderSolver.hpp:11-15, :31).
#define COSMOS_COMPAT_EULER_VEC_SOLVERS                                                                        \
    static std::vector<double> computeFractionalEvolutionVector(double f, std::vector<double> FL, std::vector<double> FR, \
                                                                double dx, double dt) {                        \
        using namespace cosmos_compat_detail;                                                                  \
        return iface_op(COSMOS_NEWTONIAN, COSMOS_IF_FRACTIONAL_EVOLUTION, cat(FL, FR), 1.4, dx, dt, 0.0, 1, f); \
    }                                                                                                          \
    static std::vector<double> computeEvolutionVector(std::vector<double> FL, std::vector<double> FR, double dx,  \
                                                      double dt) {                                             \
        using namespace cosmos_compat_detail;                                                                  \
        return iface_op(COSMOS_NEWTONIAN, COSMOS_IF_EVOLUTION, cat(FL, FR), 1.4, dx, dt);                      \
    }
#define COSMOS_COMPAT_EULER_VEC_FIRST                                                                          \
    static std::vector<double> computeLaxFriedrichsFlux(std::vector<double> UL, std::vector<double> UR,        \
                                                        std::vector<double> FL, std::vector<double> FR, double dx, \
                                                        double dt) {                                           \
        using namespace cosmos_compat_detail;                                                                  \
        return iface_op(COSMOS_NEWTONIAN, COSMOS_IF_LAX_FRIEDRICHS, cat(UL, UR, FL, FR), 1.4, dx, dt);         \
    }                                                                                                          \
    static std::vector<double> computeRichtmyerFlux(std::vector<double> UL, std::vector<double> UR,            \
                                                    std::vector<double> FL, std::vector<double> FR, double dx, double dt) { \
        using namespace cosmos_compat_detail;                                                                  \
        return iface_op(COSMOS_NEWTONIAN, COSMOS_IF_RICHTMYER, cat(UL, UR, FL, FR), 1.4, dx, dt);              \
    }                                                                                                          \
    static std::vector<double> computeFORCEFlux(std::vector<double> LF, std::vector<double> RI) {              \
        using namespace cosmos_compat_detail;                                                                  \
        return iface_op(COSMOS_NEWTONIAN, COSMOS_IF_FORCE, cat(LF, RI), 1.4, 1.0, 1.0);                        \
    }                                                                                                          \
    static std::vector<double> computeFORCEUpdate(std::vector<double> U, std::vector<double> FL,               \
                                                  std::vector<double> FR, double dx, double dt) {              \
        using namespace cosmos_compat_detail;                                                                  \
        return iface_op(COSMOS_NEWTONIAN, COSMOS_IF_FORCE_UPDATE, cat(U, FL, FR), 1.4, dx, dt);                \
    }
#define COSMOS_COMPAT_SOLVERS(PREFIX, STATE, SYS, VEC_SOLVERS, VEC_FIRST)                                      \
    class PREFIX##Solvers {                                                                                    \
    public:                                                                                                    \
        VEC_SOLVERS                                                                                            \
        static STATE evolveStateByHalfTimeStep(std::vector<double> UL, std::vector<double> UR, std::vector<double> ev, \
                                               int side, EulerMaterialParameters mp) {                         \
            using namespace cosmos_compat_detail;                                                              \
            return from_prim<STATE>(iface_op(SYS, COSMOS_IF_EVOLVE_HALF_VECTOR_X, cat(UL, UR, ev),             \
                                             mp.getAdiabaticIndex(), 1.0, 1.0, 0.0, 1, 0.5, side));            \
        }                                                                                                      \
        static STATE evolveStateByHalfXTimeStep(STATE l, STATE m, STATE r, double dx, double dt, double bias,   \
                                                int lim, int side, EulerMaterialParameters mp) {               \
            using namespace cosmos_compat_detail;                                                              \
            return from_prim<STATE>(iface_op(SYS, COSMOS_IF_EVOLVE_HALF_X, cat(pv(l), pv(m), pv(r)),           \
                                             mp.getAdiabaticIndex(), dx, dt, bias, lim, 0.5, side));           \
        }                                                                                                      \
        static STATE evolveStateByHalfYTimeStep(STATE t, STATE m, STATE b, double dx, double dt, double bias,   \
                                                int lim, int side, EulerMaterialParameters mp) {               \
            using namespace cosmos_compat_detail;                                                              \
            return from_prim<STATE>(iface_op(SYS, COSMOS_IF_EVOLVE_HALF_Y, cat(pv(t), pv(m), pv(b)),           \
                                             mp.getAdiabaticIndex(), dx, dt, bias, lim, 0.5, side));           \
        }                                                                                                      \
        static std::vector<STATE> insertBoundaryCells(std::vector<STATE>& c, int b) {                          \
            return cosmos_compat_detail::insert_boundary(c, b);                                                \
        }                                                                                                      \
        static std::vector<std::vector<STATE> > insertBoundaryCells2D(std::vector<std::vector<STATE> >& c, int b) { \
            return cosmos_compat_detail::insert_boundary_2d(c, b);                                             \
        }                                                                                                      \
        /* Solvers/EulerSolvers.cpp:225-228 */                                                                 \
        static void outputStatus(int it, double t, double dt) {                                                \
            std::cout << "Iteration = " << it << "; Time = " << t << "; Timestep = " << dt << std::endl;       \
        }                                                                                                      \
        static double computeMaximumWaveSpeed(std::vector<STATE>& c, EulerMaterialParameters mp) {             \
            return cosmos_compat_detail::max_speed1(SYS, c, mp);                                               \
        }                                                                                                      \
        static double computeMaximumWaveSpeed2D(std::vector<std::vector<STATE> >& c, EulerMaterialParameters mp) { \
            return cosmos_compat_detail::max_speed2(SYS, c, mp);                                               \
        }                                                                                                      \
        static double computeStableTimeStep(double dt, double t, double T, int it) {                          \
            return cosmos_stable_dt_rule(dt, t, T, it);                                                        \
        }                                                                                                      \
        static double computeStableTimeStep(std::vector<STATE> c, double dx, double cfl, double t, double T,   \
                                            int it, EulerMaterialParameters mp) {                              \
            return cosmos_stable_dt_rule(cfl * (dx / computeMaximumWaveSpeed(c, mp)), t, T, it);              \
        }                                                                                                      \
        static double computeStableTimeStep2D(std::vector<std::vector<STATE> > c, double dx, double cfl,       \
                                              double t, double T, int it, EulerMaterialParameters mp) {        \
            return cosmos_stable_dt_rule(cfl * (dx / computeMaximumWaveSpeed2D(c, mp)), t, T, it);            \
        }                                                                                                      \
    };                                                                                                         \
    class PREFIX##FirstOrderSolver {                                                                           \
    public:                                                                                                    \
        VEC_FIRST                                                                                              \
        static std::vector<double> computeXLaxFriedrichsFlux(STATE L, STATE R, double dx, double dt,           \
                                                             EulerMaterialParameters mp) {                     \
            using namespace cosmos_compat_detail;                                                              \
            return iface_op(SYS, COSMOS_IF_X_LAX_FRIEDRICHS_FLUX, cat(pv(L), pv(R)), mp.getAdiabaticIndex(), dx, dt); \
        }                                                                                                      \
        static std::vector<double> computeYLaxFriedrichsFlux(STATE T, STATE B, double dx, double dt,           \
                                                             EulerMaterialParameters mp) {                     \
            using namespace cosmos_compat_detail;                                                              \
            return iface_op(SYS, COSMOS_IF_Y_LAX_FRIEDRICHS_FLUX, cat(pv(T), pv(B)), mp.getAdiabaticIndex(), dx, dt); \
        }                                                                                                      \
        static std::vector<double> computeXRichtmyerFlux(STATE L, STATE R, double dx, double dt,               \
                                                         EulerMaterialParameters mp) {                         \
            using namespace cosmos_compat_detail;                                                              \
            return iface_op(SYS, COSMOS_IF_X_RICHTMYER_FLUX, cat(pv(L), pv(R)), mp.getAdiabaticIndex(), dx, dt); \
        }                                                                                                      \
        static std::vector<double> computeYRichtmyerFlux(STATE T, STATE B, double dx, double dt,               \
                                                         EulerMaterialParameters mp) {                         \
            using namespace cosmos_compat_detail;                                                              \
            return iface_op(SYS, COSMOS_IF_Y_RICHTMYER_FLUX, cat(pv(T), pv(B)), mp.getAdiabaticIndex(), dx, dt); \
        }                                                                                                      \
        static std::vector<double> computeXFORCEFlux(STATE L, STATE R, double dx, double dt,                   \
                                                     EulerMaterialParameters mp) {                             \
            using namespace cosmos_compat_detail;                                                              \
            return iface_op(SYS, COSMOS_IF_X_FORCE_FLUX, cat(pv(L), pv(R)), mp.getAdiabaticIndex(), dx, dt);   \
        }                                                                                                      \
        static std::vector<double> computeYFORCEFlux(STATE T, STATE B, double dx, double dt,                   \
                                                     EulerMaterialParameters mp) {                             \
            using namespace cosmos_compat_detail;                                                              \
            return iface_op(SYS, COSMOS_IF_Y_FORCE_FLUX, cat(pv(T), pv(B)), mp.getAdiabaticIndex(), dx, dt);   \
        }                                                                                                      \
        static void computeFORCETimeStep(std::vector<STATE>& c, double dx, double dt, EulerMaterialParameters mp) { \
            cosmos_compat_detail::sweep1(SYS, c, dx, dt, 1, 0.0, 1, mp);                                       \
        }                                                                                                      \
        static void computeXFORCETimeStep2D(std::vector<std::vector<STATE> >& c, double dx, double dt,          \
                                            EulerMaterialParameters mp) {                                      \
            cosmos_compat_detail::sweep2(SYS, c, dx, dt, 0, 1, 0.0, 1, mp);                                    \
        }                                                                                                      \
        static void computeYFORCETimeStep2D(std::vector<std::vector<STATE> >& c, double dx, double dt,          \
                                            EulerMaterialParameters mp) {                                      \
            cosmos_compat_detail::sweep2(SYS, c, dx, dt, 1, 1, 0.0, 1, mp);                                    \
        }                                                                                                      \
        static std::vector<STATE> solve(std::vector<STATE> c, double dx, double cfl, double T,                  \
                                        EulerMaterialParameters mp) {                                          \
            return cosmos_compat_detail::solve1(SYS, c, dx, cfl, T, 1, 0.0, 1, mp);                            \
        }                                                                                                      \
        static std::vector<std::vector<STATE> > solve2D(std::vector<std::vector<STATE> > c, double dx,           \
                                                        double cfl, double T, EulerMaterialParameters mp) {    \
            return cosmos_compat_detail::solve2(SYS, c, dx, cfl, T, 1, 0.0, 1, mp);                            \
        }                                                                                                      \
    };                                                                                                         \
    class PREFIX##SecondOrderSolver {                                                                          \
    public:                                                                                                    \
        static std::vector<double> computeXSLICFlux(STATE ll, STATE l, STATE r, STATE rr, double dx, double dt, \
                                                    double bias, int lim, EulerMaterialParameters mp) {        \
            using namespace cosmos_compat_detail;                                                              \
            return iface_op(SYS, COSMOS_IF_X_SLIC_FLUX, cat(pv(ll), pv(l), pv(r), pv(rr)), mp.getAdiabaticIndex(), \
                            dx, dt, bias, lim);                                                                \
        }                                                                                                      \
        static std::vector<double> computeYSLICFlux(STATE tt, STATE t, STATE b, STATE bb, double dx, double dt, \
                                                    double bias, int lim, EulerMaterialParameters mp) {        \
            using namespace cosmos_compat_detail;                                                              \
            return iface_op(SYS, COSMOS_IF_Y_SLIC_FLUX, cat(pv(tt), pv(t), pv(b), pv(bb)), mp.getAdiabaticIndex(), \
                            dx, dt, bias, lim);                                                                \
        }                                                                                                      \
        static void computeSLICTimeStep(std::vector<STATE>& c, double dx, double dt, double bias, int lim,      \
                                        EulerMaterialParameters mp) {                                          \
            cosmos_compat_detail::sweep1(SYS, c, dx, dt, 2, bias, lim, mp);                                    \
        }                                                                                                      \
        static void computeXSLICTimeStep2D(std::vector<std::vector<STATE> >& c, double dx, double dt, double bias, \
                                           int lim, EulerMaterialParameters mp) {                              \
            cosmos_compat_detail::sweep2(SYS, c, dx, dt, 0, 2, bias, lim, mp);                                 \
        }                                                                                                      \
        static void computeYSLICTimeStep2D(std::vector<std::vector<STATE> >& c, double dx, double dt, double bias, \
                                           int lim, EulerMaterialParameters mp) {                              \
            cosmos_compat_detail::sweep2(SYS, c, dx, dt, 1, 2, bias, lim, mp);                                 \
        }                                                                                                      \
        static std::vector<STATE> solve(std::vector<STATE> c, double dx, double cfl, double T, double bias,    \
                                        int lim, EulerMaterialParameters mp) {                                 \
            return cosmos_compat_detail::solve1(SYS, c, dx, cfl, T, 2, bias, lim, mp);                         \
        }                                                                                                      \
        static std::vector<std::vector<STATE> > solve2D(std::vector<std::vector<STATE> > c, double dx,           \
                                                        double cfl, double T, double bias, int lim,            \
                                                        EulerMaterialParameters mp) {                          \
            return cosmos_compat_detail::solve2(SYS, c, dx, cfl, T, 2, bias, lim, mp);                         \
        }                                                                                                      \
    };
COSMOS_COMPAT_SOLVERS(Euler, EulerStateVector, COSMOS_NEWTONIAN, COSMOS_COMPAT_EULER_VEC_SOLVERS,
                      COSMOS_COMPAT_EULER_VEC_FIRST)
COSMOS_COMPAT_SOLVERS(RelativisticEuler, RelativisticEulerStateVector, COSMOS_SR, , )
#undef COSMOS_COMPAT_SOLVERS
#undef COSMOS_COMPAT_EULER_VEC_SOLVERS
#undef COSMOS_COMPAT_EULER_VEC_FIRST

// GR solvers take (..., subcyclingIterations, EulerMaterialParameters, BlackHoleSpacetime)
// (Solvers/BlackHoleEulerSecondOrderSolver.hpp:10-32, Solvers/BlackHoleEulerForcingSolver.hpp:19-22).
namespace cosmos_compat_detail {
typedef BlackHoleEulerStateVector BHS;
inline std::vector<double> bh_op(int op, const std::vector<double>& in, double x, double y, double z, double dx,
                                 double dt, EulerMaterialParameters mp, const BlackHoleSpacetime& bh, double bias = 0.0,
                                 int lim = 1, double frac = 0.5, int side = 0) {
    const double q[3] = {x, y, z};
    return iface_op(COSMOS_GR, op, in, mp.getAdiabaticIndex(), dx, dt, bias, lim, frac, side, q, &bh);
}
}  // namespace cosmos_compat_detail

class BlackHoleEulerSolvers {
public:
    // Solvers/BlackHoleEulerSolvers.hpp:22-49: evolutions at (x, y, z), one item through cosmos_interface_eval
    static BlackHoleEulerStateVector evolveStateByFractionalTimeStep(std::vector<double> U, std::vector<double> ev, double x,
                                                                     double y, double z, EulerMaterialParameters mp,
                                                                     BlackHoleSpacetime bh) {
        using namespace cosmos_compat_detail;
        return from_prim<BHS>(bh_op(COSMOS_IF_EVOLVE_FRACTION_VECTOR, cat(U, ev), x, y, z, 1.0, 1.0, mp, bh));
    }
    static BlackHoleEulerStateVector evolveStateByFractionalXTimeStep(double f, BlackHoleEulerStateVector l,
                                                                      BlackHoleEulerStateVector m, BlackHoleEulerStateVector r,
                                                                      double dx, double dt, double bias, int lim, double x,
                                                                      double y, double z, EulerMaterialParameters mp,
                                                                      BlackHoleSpacetime bh) {
        using namespace cosmos_compat_detail;
        return from_prim<BHS>(bh_op(COSMOS_IF_EVOLVE_FRACTION_X, cat(pv(l), pv(m), pv(r)), x, y, z, dx, dt, mp, bh, bias, lim, f));
    }
    static BlackHoleEulerStateVector evolveStateByFractionalYTimeStep(double f, BlackHoleEulerStateVector t,
                                                                      BlackHoleEulerStateVector m, BlackHoleEulerStateVector b,
                                                                      double dx, double dt, double bias, int lim, double x,
                                                                      double y, double z, EulerMaterialParameters mp,
                                                                      BlackHoleSpacetime bh) {
        using namespace cosmos_compat_detail;
        return from_prim<BHS>(bh_op(COSMOS_IF_EVOLVE_FRACTION_Y, cat(pv(t), pv(m), pv(b)), x, y, z, dx, dt, mp, bh, bias, lim, f));
    }
    static BlackHoleEulerStateVector evolveStateByHalfXTimeStep(std::vector<double> UL, std::vector<double> UR,
                                                                std::vector<double> ev, int side, double dx, double x,
                                                                double y, double z, EulerMaterialParameters mp,
                                                                BlackHoleSpacetime bh) {
        using namespace cosmos_compat_detail;
        return from_prim<BHS>(bh_op(COSMOS_IF_EVOLVE_HALF_VECTOR_X, cat(UL, UR, ev), x, y, z, dx, 1.0, mp, bh, 0.0, 1, 0.5, side));
    }
    static BlackHoleEulerStateVector evolveStateByHalfXTimeStep(BlackHoleEulerStateVector l, BlackHoleEulerStateVector m,
                                                                BlackHoleEulerStateVector r, double dx, double dt, double bias,
                                                                int lim, int side, double x, double y, double z,
                                                                EulerMaterialParameters mp, BlackHoleSpacetime bh) {
        using namespace cosmos_compat_detail;
        return from_prim<BHS>(bh_op(COSMOS_IF_EVOLVE_HALF_X, cat(pv(l), pv(m), pv(r)), x, y, z, dx, dt, mp, bh, bias, lim, 0.5, side));
    }
    static BlackHoleEulerStateVector evolveStateByHalfYTimeStep(std::vector<double> UT, std::vector<double> UB,
                                                                std::vector<double> ev, int side, double dx, double x,
                                                                double y, double z, EulerMaterialParameters mp,
                                                                BlackHoleSpacetime bh) {
        using namespace cosmos_compat_detail;
        return from_prim<BHS>(bh_op(COSMOS_IF_EVOLVE_HALF_VECTOR_Y, cat(UT, UB, ev), x, y, z, dx, 1.0, mp, bh, 0.0, 1, 0.5, side));
    }
    static BlackHoleEulerStateVector evolveStateByHalfYTimeStep(BlackHoleEulerStateVector t, BlackHoleEulerStateVector m,
                                                                BlackHoleEulerStateVector b, double dx, double dt, double bias,
                                                                int lim, int side, double x, double y, double z,
                                                                EulerMaterialParameters mp, BlackHoleSpacetime bh) {
        using namespace cosmos_compat_detail;
        return from_prim<BHS>(bh_op(COSMOS_IF_EVOLVE_HALF_Y, cat(pv(t), pv(m), pv(b)), x, y, z, dx, dt, mp, bh, bias, lim, 0.5, side));
    }
    static std::vector<BlackHoleEulerStateVector> insertBoundaryCells(std::vector<BlackHoleEulerStateVector>& c, int b) {
        return cosmos_compat_detail::insert_boundary(c, b);
    }
    static std::vector<std::vector<BlackHoleEulerStateVector> > insertBoundaryCells2D(
        std::vector<std::vector<BlackHoleEulerStateVector> >& c, int b) {
        return cosmos_compat_detail::insert_boundary_2d(c, b);
    }
    static double computeMaximumWaveSpeed(std::vector<BlackHoleEulerStateVector>& c, EulerMaterialParameters mp,
                                          BlackHoleSpacetime bh) {
        return cosmos_compat_detail::max_speed1(COSMOS_GR, c, mp, &bh);
    }
    static double computeMaximumWaveSpeed2D(std::vector<std::vector<BlackHoleEulerStateVector> >& c,
                                            EulerMaterialParameters mp, BlackHoleSpacetime bh) {
        return cosmos_compat_detail::max_speed2(COSMOS_GR, c, mp, &bh);
    }
    static double computeStableTimeStep(std::vector<BlackHoleEulerStateVector> c, double dx, double cfl, double t,
                                        double T, int it, EulerMaterialParameters mp, BlackHoleSpacetime bh) {
        return cosmos_stable_dt_rule(cfl * (dx / cosmos_compat_detail::max_speed1(COSMOS_GR, c, mp, &bh)), t, T, it);
    }
    static double computeStableTimeStep2D(std::vector<std::vector<BlackHoleEulerStateVector> > c, double dx,
                                          double cfl, double t, double T, int it, EulerMaterialParameters mp,
                                          BlackHoleSpacetime bh) {
        return cosmos_stable_dt_rule(cfl * (dx / cosmos_compat_detail::max_speed2(COSMOS_GR, c, mp, &bh)), t, T, it);
    }
};
#define COSMOS_COMPAT_BH_FLUX(NAME, OP)                                                                         \
    static std::vector<double> NAME(BlackHoleEulerStateVector a, BlackHoleEulerStateVector b, double x, double y, \
                                    double z, double dx, double dt, EulerMaterialParameters mp, BlackHoleSpacetime bh) { \
        using namespace cosmos_compat_detail;                                                                  \
        return bh_op(OP, cat(pv(a), pv(b)), x, y, z, dx, dt, mp, bh);                                          \
    }
class BlackHoleEulerFirstOrderSolver {
public:
    // Solvers/BlackHoleEulerFirstOrderSolver.hpp:11-28: fluxes at the interface point (x, y, z)
    COSMOS_COMPAT_BH_FLUX(computeXLaxFriedrichsFlux, COSMOS_IF_X_LAX_FRIEDRICHS_FLUX)
    COSMOS_COMPAT_BH_FLUX(computeYLaxFriedrichsFlux, COSMOS_IF_Y_LAX_FRIEDRICHS_FLUX)
    COSMOS_COMPAT_BH_FLUX(computeXRichtmyerFlux, COSMOS_IF_X_RICHTMYER_FLUX)
    COSMOS_COMPAT_BH_FLUX(computeYRichtmyerFlux, COSMOS_IF_Y_RICHTMYER_FLUX)
    COSMOS_COMPAT_BH_FLUX(computeXFORCEFlux, COSMOS_IF_X_FORCE_FLUX)
    COSMOS_COMPAT_BH_FLUX(computeYFORCEFlux, COSMOS_IF_Y_FORCE_FLUX)
    static void computeFORCETimeStep(std::vector<BlackHoleEulerStateVector>& c, double dx, double dt,
                                     EulerMaterialParameters mp, BlackHoleSpacetime bh) {
        cosmos_compat_detail::sweep1(COSMOS_GR, c, dx, dt, 1, 0.0, 1, mp, &bh);
    }
    static void computeXFORCETimeStep2D(std::vector<std::vector<BlackHoleEulerStateVector> >& c, double dx, double dt,
                                        EulerMaterialParameters mp, BlackHoleSpacetime bh) {
        cosmos_compat_detail::sweep2(COSMOS_GR, c, dx, dt, 0, 1, 0.0, 1, mp, &bh);
    }
    static void computeYFORCETimeStep2D(std::vector<std::vector<BlackHoleEulerStateVector> >& c, double dx, double dt,
                                        EulerMaterialParameters mp, BlackHoleSpacetime bh) {
        cosmos_compat_detail::sweep2(COSMOS_GR, c, dx, dt, 1, 1, 0.0, 1, mp, &bh);
    }
    static std::vector<BlackHoleEulerStateVector> solve(std::vector<BlackHoleEulerStateVector> c, double dx, double cfl,
                                                        double T, int sub, EulerMaterialParameters mp,
                                                        BlackHoleSpacetime bh) {
        return cosmos_compat_detail::solve1(COSMOS_GR, c, dx, cfl, T, 1, 0.0, 1, mp, sub, &bh);
    }
    static std::vector<std::vector<BlackHoleEulerStateVector> > solve2D(
        std::vector<std::vector<BlackHoleEulerStateVector> > c, double dx, double cfl, double T, int sub,
        EulerMaterialParameters mp, BlackHoleSpacetime bh) {
        return cosmos_compat_detail::solve2(COSMOS_GR, c, dx, cfl, T, 1, 0.0, 1, mp, sub, &bh);
    }
};
#undef COSMOS_COMPAT_BH_FLUX
class BlackHoleEulerSecondOrderSolver {
public:
    // Solvers/BlackHoleEulerSecondOrderSolver.hpp:9-16
    static std::vector<double> computeXSLICFlux(BlackHoleEulerStateVector ll, BlackHoleEulerStateVector l,
                                                BlackHoleEulerStateVector r, BlackHoleEulerStateVector rr, double dx, double dt,
                                                double bias, int lim, double x, double y, double z, EulerMaterialParameters mp,
                                                BlackHoleSpacetime bh) {
        using namespace cosmos_compat_detail;
        return bh_op(COSMOS_IF_X_SLIC_FLUX, cat(pv(ll), pv(l), pv(r), pv(rr)), x, y, z, dx, dt, mp, bh, bias, lim);
    }
    static std::vector<double> computeYSLICFlux(BlackHoleEulerStateVector tt, BlackHoleEulerStateVector t,
                                                BlackHoleEulerStateVector b, BlackHoleEulerStateVector bb, double dx, double dt,
                                                double bias, int lim, double x, double y, double z, EulerMaterialParameters mp,
                                                BlackHoleSpacetime bh) {
        using namespace cosmos_compat_detail;
        return bh_op(COSMOS_IF_Y_SLIC_FLUX, cat(pv(tt), pv(t), pv(b), pv(bb)), x, y, z, dx, dt, mp, bh, bias, lim);
    }
    static void computeSLICTimeStep(std::vector<BlackHoleEulerStateVector>& c, double dx, double dt, double bias,
                                    int lim, EulerMaterialParameters mp, BlackHoleSpacetime bh) {
        cosmos_compat_detail::sweep1(COSMOS_GR, c, dx, dt, 2, bias, lim, mp, &bh);
    }
    static void computeXSLICTimeStep2D(std::vector<std::vector<BlackHoleEulerStateVector> >& c, double dx, double dt,
                                       double bias, int lim, EulerMaterialParameters mp, BlackHoleSpacetime bh) {
        cosmos_compat_detail::sweep2(COSMOS_GR, c, dx, dt, 0, 2, bias, lim, mp, &bh);
    }
    static void computeYSLICTimeStep2D(std::vector<std::vector<BlackHoleEulerStateVector> >& c, double dx, double dt,
                                       double bias, int lim, EulerMaterialParameters mp, BlackHoleSpacetime bh) {
        cosmos_compat_detail::sweep2(COSMOS_GR, c, dx, dt, 1, 2, bias, lim, mp, &bh);
    }
    static std::vector<BlackHoleEulerStateVector> solve(std::vector<BlackHoleEulerStateVector> c, double dx, double cfl,
                                                        double T, double bias, int lim, int sub,
                                                        EulerMaterialParameters mp, BlackHoleSpacetime bh) {
        return cosmos_compat_detail::solve1(COSMOS_GR, c, dx, cfl, T, 2, bias, lim, mp, sub, &bh);
    }
    static std::vector<std::vector<BlackHoleEulerStateVector> > solve2D(
        std::vector<std::vector<BlackHoleEulerStateVector> > c, double dx, double cfl, double T, double bias, int lim,
        int sub, EulerMaterialParameters mp, BlackHoleSpacetime bh) {
        return cosmos_compat_detail::solve2(COSMOS_GR, c, dx, cfl, T, 2, bias, lim, mp, sub, &bh);
    }
};
class BlackHoleEulerForcingSolver {
public:
    // Solvers/BlackHoleEulerForcingSolver.hpp:9-17: one cell's RK4 source update (conserved vectors)
    static std::vector<double> evolveConservedVariableVector(std::vector<double> l, std::vector<double> m,
                                                             std::vector<double> r, double x, double y, double z, double dx,
                                                             double dt, double bias, int lim, EulerMaterialParameters mp,
                                                             BlackHoleSpacetime bh) {
        using namespace cosmos_compat_detail;
        return bh_op(COSMOS_IF_RK_CELL_1D, cat(l, m, r), x, y, z, dx, dt, mp, bh, bias, lim);
    }
    static std::vector<double> evolveConservedVariableVector2D(std::vector<double> l, std::vector<double> m,
                                                               std::vector<double> r, std::vector<double> t,
                                                               std::vector<double> b, double x, double y, double z,
                                                               double dx, double dt, double bias, int lim,
                                                               EulerMaterialParameters mp, BlackHoleSpacetime bh) {
        using namespace cosmos_compat_detail;
        return bh_op(COSMOS_IF_RK_CELL_2D, cat(l, m, r, t, b), x, y, z, dx, dt, mp, bh, bias, lim);
    }
    static void computeRungeKuttaTimeStep(std::vector<BlackHoleEulerStateVector>& c, double dx, double dt, double bias,
                                          int lim, EulerMaterialParameters mp, BlackHoleSpacetime bh) {
        double b[5];
        bh.pack(b);
        cosmos_compat_detail::Grid g(COSMOS_GR, 1, (int)c.size(), 1, dx, mp.getAdiabaticIndex(), b);
        std::vector<double> a = cosmos_compat_detail::pack1(c);
        cosmos_compat_detail::check(cosmos_grid_set_prim(g.g, a.data(), a.size()));
        cosmos_compat_detail::check(cosmos_grid_rk_source(g.g, dt, bias, lim));
        cosmos_compat_detail::check(cosmos_grid_get_prim(g.g, a.data(), a.size()));
        cosmos_compat_detail::unpack1(a, c);
    }
    static void computeRungeKuttaTimeStep2D(std::vector<std::vector<BlackHoleEulerStateVector> >& c, double dx,
                                            double dt, double bias, int lim, EulerMaterialParameters mp,
                                            BlackHoleSpacetime bh) {
        double b[5];
        bh.pack(b);
        cosmos_compat_detail::Grid g(COSMOS_GR, 2, (int)c[0].size(), (int)c.size(), dx, mp.getAdiabaticIndex(), b);
        std::vector<double> a = cosmos_compat_detail::pack2(c);
        cosmos_compat_detail::check(cosmos_grid_set_prim(g.g, a.data(), a.size()));
        cosmos_compat_detail::check(cosmos_grid_rk_source(g.g, dt, bias, lim));
        cosmos_compat_detail::check(cosmos_grid_get_prim(g.g, a.data(), a.size()));
        cosmos_compat_detail::unpack2(a, c);
    }
};

// ----------------------------------------------------------------------------- AMR drivers
// AMR/EulerAMR.hpp and AMR/RelativisticEulerAMR.hpp: solveLevel1AMR / solve2DLevel1AMR return
// (coarse cells, fine cells, coarse flags, fine flags); solveLevel2AMR / solve2DLevel2AMR return
// (coarse, intermediate, fine cells, and the three flag sets).
namespace cosmos_compat_detail {

struct Amr {
    cosmos_amr* a = nullptr;
    Amr(int system, int dims, int nx, int ny, double dx, double gamma, int levels = 1) {
        cosmos_params p;
        cosmos_params_default(&p);
        p.system = system;
        p.dims = dims;
        p.nx = nx;
        p.ny = dims == 1 ? 1 : ny;
        p.dx = dx;
        p.gamma = gamma;
        check(levels == 1 ? cosmos_amr_create(ctx(), &p, &a) : cosmos_amr_create_level2(ctx(), &p, &a));
    }
    ~Amr() { cosmos_amr_destroy(a); }
    // runs the driver and fills the host copies of both levels and their flags
    void run(const std::vector<double>& prim, double cfl, double T, double tol, int order, std::vector<double>& c,
             std::vector<double>& f, std::vector<unsigned char>& cf, std::vector<unsigned char>& ff) {
        check(cosmos_amr_set_prim(a, prim.data(), prim.size()));
        cosmos_amr_result r;
        check(cosmos_amr_solve(a, cfl, T, tol, order, &r));
        check(cosmos_amr_get(a, c.data(), f.data(), cf.data(), ff.data()));
    }
};

template <class S>
std::tuple<std::vector<S>, std::vector<S>, std::vector<bool>, std::vector<bool> >
amr1(int sys, std::vector<S> cells, double dx, double cfl, double T, double tol, int order,
     EulerMaterialParameters mp) {
    const size_t n = cells.size();
    Amr d(sys, 1, (int)n, 1, dx, mp.getAdiabaticIndex());
    std::vector<double> c(5 * n), f(10 * n);
    std::vector<unsigned char> cf(n), ff(2 * n);
    d.run(pack1(cells), cfl, T, tol, order, c, f, cf, ff);
    std::vector<S> coarse(n), fine(2 * n);
    unpack1(c, coarse);
    unpack1(f, fine);
    return std::make_tuple(coarse, fine, std::vector<bool>(cf.begin(), cf.end()), std::vector<bool>(ff.begin(), ff.end()));
}

template <class S>
std::tuple<std::vector<std::vector<S> >, std::vector<std::vector<S> >, std::vector<std::vector<bool> >,
           std::vector<std::vector<bool> > >
amr2(int sys, std::vector<std::vector<S> > cells, double dx, double cfl, double T, double tol, int order,
     EulerMaterialParameters mp) {
    const size_t ny = cells.size(), nx = cells[0].size();
    Amr d(sys, 2, (int)nx, (int)ny, dx, mp.getAdiabaticIndex());
    std::vector<double> c(5 * nx * ny), f(20 * nx * ny);
    std::vector<unsigned char> cf(nx * ny), ff(4 * nx * ny);
    d.run(pack2(cells), cfl, T, tol, order, c, f, cf, ff);
    std::vector<std::vector<S> > coarse(ny, std::vector<S>(nx)), fine(2 * ny, std::vector<S>(2 * nx));
    unpack2(c, coarse);
    unpack2(f, fine);
    std::vector<std::vector<bool> > cb(ny, std::vector<bool>(nx)), fb(2 * ny, std::vector<bool>(2 * nx));
    for (size_t i = 0; i < ny; i++)
        for (size_t j = 0; j < nx; j++) cb[i][j] = cf[i * nx + j] != 0;
    for (size_t i = 0; i < 2 * ny; i++)
        for (size_t j = 0; j < 2 * nx; j++) fb[i][j] = ff[i * 2 * nx + j] != 0;
    return std::make_tuple(coarse, fine, cb, fb);
}

// Level-2 run: level l of the three, as primitives and flags.
struct Amr2Out {
    std::vector<double> c[3];
    std::vector<unsigned char> f[3];
};
inline Amr2Out amr2_run(int sys, int dims, int nx, int ny, const std::vector<double>& prim, double dx, double cfl,
                        double T, double tol, int order, double gamma) {
    Amr d(sys, dims, nx, ny, dx, gamma, 2);
    check(cosmos_amr_set_prim(d.a, prim.data(), prim.size()));
    cosmos_amr_result r;
    check(cosmos_amr_solve(d.a, cfl, T, tol, order, &r));
    Amr2Out o;
    const size_t n = (size_t)nx * (dims == 2 ? ny : 1);
    for (int l = 0; l < 3; l++) {
        const size_t m = n << (dims == 2 ? 2 * l : l);
        o.c[l].resize(5 * m);
        o.f[l].resize(m);
        check(cosmos_amr_get_level(d.a, l, o.c[l].data(), o.f[l].data()));
    }
    return o;
}

template <class S>
std::tuple<std::vector<S>, std::vector<S>, std::vector<S>, std::vector<bool>, std::vector<bool>, std::vector<bool> >
amr1_level2(int sys, std::vector<S> cells, double dx, double cfl, double T, double tol, int order,
            EulerMaterialParameters mp) {
    const size_t n = cells.size();
    Amr2Out o = amr2_run(sys, 1, (int)n, 1, pack1(cells), dx, cfl, T, tol, order, mp.getAdiabaticIndex());
    std::vector<S> lv[3] = {std::vector<S>(n), std::vector<S>(2 * n), std::vector<S>(4 * n)};
    for (int l = 0; l < 3; l++) unpack1(o.c[l], lv[l]);
    auto b = [](const std::vector<unsigned char>& f) { return std::vector<bool>(f.begin(), f.end()); };
    return std::make_tuple(lv[0], lv[1], lv[2], b(o.f[0]), b(o.f[1]), b(o.f[2]));
}

template <class S>
std::tuple<std::vector<std::vector<S> >, std::vector<std::vector<S> >, std::vector<std::vector<S> >,
           std::vector<std::vector<bool> >, std::vector<std::vector<bool> >, std::vector<std::vector<bool> > >
amr2_level2(int sys, std::vector<std::vector<S> > cells, double dx, double cfl, double T, double tol, int order,
            EulerMaterialParameters mp) {
    const size_t ny = cells.size(), nx = cells[0].size();
    Amr2Out o = amr2_run(sys, 2, (int)nx, (int)ny, pack2(cells), dx, cfl, T, tol, order, mp.getAdiabaticIndex());
    std::vector<std::vector<S> > lv[3];
    std::vector<std::vector<bool> > fb[3];
    for (int l = 0; l < 3; l++) {
        const size_t r = ny << l, c = nx << l;
        lv[l].assign(r, std::vector<S>(c));
        unpack2(o.c[l], lv[l]);
        fb[l].assign(r, std::vector<bool>(c));
        for (size_t i = 0; i < r; i++)
            for (size_t j = 0; j < c; j++) fb[l][i][j] = o.f[l][i * c + j] != 0;
    }
    return std::make_tuple(lv[0], lv[1], lv[2], fb[0], fb[1], fb[2]);
}

}  // namespace cosmos_compat_detail

#define COSMOS_COMPAT_AMR(PREFIX, STATE, SYS)                                                                   \
    class PREFIX##AMR {                                                                                        \
    public:                                                                                                    \
        static std::tuple<std::vector<STATE>, std::vector<STATE>, std::vector<bool>, std::vector<bool> >       \
        solveLevel1AMR(std::vector<STATE> c, double dx, double cfl, double T, double tol, int order,          \
                       EulerMaterialParameters mp) {                                                           \
            return cosmos_compat_detail::amr1(SYS, c, dx, cfl, T, tol, order, mp);                             \
        }                                                                                                      \
        static std::tuple<std::vector<std::vector<STATE> >, std::vector<std::vector<STATE> >,                  \
                          std::vector<std::vector<bool> >, std::vector<std::vector<bool> > >                   \
        solve2DLevel1AMR(std::vector<std::vector<STATE> > c, double dx, double cfl, double T, double tol,      \
                         int order, EulerMaterialParameters mp) {                                              \
            return cosmos_compat_detail::amr2(SYS, c, dx, cfl, T, tol, order, mp);                             \
        }                                                                                                      \
        static std::tuple<std::vector<STATE>, std::vector<STATE>, std::vector<STATE>, std::vector<bool>,       \
                          std::vector<bool>, std::vector<bool> >                                               \
        solveLevel2AMR(std::vector<STATE> c, double dx, double cfl, double T, double tol, int order,          \
                       EulerMaterialParameters mp) {                                                           \
            return cosmos_compat_detail::amr1_level2(SYS, c, dx, cfl, T, tol, order, mp);                      \
        }                                                                                                      \
        static std::tuple<std::vector<std::vector<STATE> >, std::vector<std::vector<STATE> >,                  \
                          std::vector<std::vector<STATE> >, std::vector<std::vector<bool> >,                   \
                          std::vector<std::vector<bool> >, std::vector<std::vector<bool> > >                   \
        solve2DLevel2AMR(std::vector<std::vector<STATE> > c, double dx, double cfl, double T, double tol,      \
                         int order, EulerMaterialParameters mp) {                                              \
            return cosmos_compat_detail::amr2_level2(SYS, c, dx, cfl, T, tol, order, mp);                      \
        }                                                                                                      \
    };
COSMOS_COMPAT_AMR(Euler, EulerStateVector, COSMOS_NEWTONIAN)
COSMOS_COMPAT_AMR(RelativisticEuler, RelativisticEulerStateVector, COSMOS_SR)
#undef COSMOS_COMPAT_AMR
