// TEST INFRASTRUCTURE ONLY -- the CPU oracle.  Only tests/, __graft_entry__.smoke() and
// bench.py's CPU-baseline leg may load or run anything under oracle/.  The product library
// never links, calls or falls back to it.
//
// A scalar FP64 restatement of the reference's finite-volume SLIC/FORCE path
// (JonathanGorard/Cosmos), in the reference's own operation order so that it reproduces the
// reference bit for bit when built with -ffp-contract=off.  It is pinned against the
// reference itself (oracle/ref/ builds the reference from its sources into oracle/_ref/) and
// against the golden fixtures in tests/golden/ generated from that build.
//
// Every function cites the reference file:line it restates.  Grids are flat arrays of
// primitive states (rho, vx, vy, vz, p), row-major [ny][nx], as in the reference's
// vector<vector<StateVector>> indexed [row i = y][column j = x].
#pragma once
#include <cmath>
#include <cstddef>

namespace orc {

// ----------------------------------------------------------------- a differentiable scalar
// Forward-mode dual number used for the tangent-linear reference gradient of the Newtonian
// SLIC step (the adjoint's CPU check).  Comparisons act on the value part; every branch of the
// reference (limiter regions, clamps) is therefore taken exactly as in the FP64 forward run.
struct Dual {
    double v, d;
    Dual() : v(0), d(0) {}
    Dual(double a) : v(a), d(0) {}
    Dual(double a, double b) : v(a), d(b) {}
};
inline Dual operator+(Dual a, Dual b) { return Dual(a.v + b.v, a.d + b.d); }
inline Dual operator-(Dual a, Dual b) { return Dual(a.v - b.v, a.d - b.d); }
inline Dual operator-(Dual a) { return Dual(-a.v, -a.d); }
inline Dual operator*(Dual a, Dual b) { return Dual(a.v * b.v, a.d * b.v + a.v * b.d); }
inline Dual operator/(Dual a, Dual b) { double q = a.v / b.v; return Dual(q, (a.d - q * b.d) / b.v); }
inline bool operator<(Dual a, Dual b) { return a.v < b.v; }
inline bool operator>(Dual a, Dual b) { return a.v > b.v; }
inline bool operator<=(Dual a, Dual b) { return a.v <= b.v; }
inline bool operator>=(Dual a, Dual b) { return a.v >= b.v; }
inline Dual sqrt(Dual a) { double s = std::sqrt(a.v); return Dual(s, a.d / (2.0 * s)); }
inline Dual fabs(Dual a) { return a.v < 0 ? -a : a; }
inline double val(Dual a) { return a.v; }
inline double val(double a) { return a; }
// A root xv of f(x; c) with its tangent by the implicit-function theorem: given f evaluated at
// x = xv held fixed (its tangent is the coefficients' part) and f'(xv), dx = -df / f'(xv).
inline double ift_root(double xv, double, double) { return xv; }
inline Dual ift_root(double xv, Dual f_at_xv, double fp) { return Dual(xv, -f_at_xv.d / fp); }

// std::min / std::max semantics (the reference uses them with doubles).
template <class T> inline T mn(T a, T b) { return (b < a) ? b : a; }
template <class T> inline T mx(T a, T b) { return (a < b) ? b : a; }

}  // namespace orc
