// TEST INFRASTRUCTURE ONLY -- the CPU oracle (see cosmos_oracle.hpp).  Only tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline leg may load this library.
//
// Restates the reference's SLIC/FORCE path in FP64 with the reference's operation order.
// Every expression below is written with explicit parentheses matching C++'s left-to-right
// evaluation of the reference's source line it cites; build with -ffp-contract=off.
//
// Restructuring relative to the reference (results are bit-identical, only work is saved):
//  * Each interface flux is computed once and shared by its two cells.  The reference
//    computes it twice with identical arguments (Solvers/EulerSecondOrderSolver.cpp:60-65 and
//    the neighbouring cell's call), so the values are the same doubles.
//  * For the coordinate-free systems (Newtonian, SR) a cell's half-step evolution is computed
//    once and gives both its left- and right-face states; the reference recomputes the same
//    slope for each side (Solvers/EulerSolvers.cpp:208-223).  The GR system evaluates the two
//    sides at two separately rounded coordinates, so it keeps one evolution per side.
#include "cosmos_oracle.hpp"

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

namespace orc {

struct Pt { double x, y, z; };

static inline Pt shift(Pt p, int axis, double d) {
    if (axis == 0) p.x = p.x + d; else p.y = p.y + d;
    return p;
}

// ========================================================================= slope limiters
// Solvers/SlopeLimiters.cpp:3-6
template <class T> static T gradient_ratio(T r, double w) { return T(2.0) / (T(1.0 - w) + (T(1.0 + w) * r)); }

// Solvers/SlopeLimiters.cpp:8-69 (0 = SuperBee, 1 = van Leer, else MinBee)
template <class T> static T limiter(T r, double w, int lim) {
    if (lim == 0) {
        if (r < T(0.0)) return T(0.0);
        else if (r >= T(0.0) && r < T(0.5)) return T(2.0) * r;
        else if (r >= T(0.5) && r < T(1.0)) return T(1.0);
        return mn(mn(r, gradient_ratio(r, w)), T(2.0));
    } else if (lim == 1) {
        if (r < T(0.0)) return T(0.0);
        return mn((T(2.0) * r) / (T(1.0) + r), gradient_ratio(r, w));
    }
    if (r < T(0.0)) return T(0.0);
    else if (r >= T(0.0) && r < T(1.0)) return r;
    return mn(T(1.0), gradient_ratio(r, w));
}

// Solvers/SlopeLimiters.cpp:71-101.  pow(10.0, -5.0) == 1e-5 exactly.
template <class T> static void slope_vector(const T* ul, const T* uc, const T* ur, double w, int lim, T* s) {
    T dl[5], dr[5];
    for (int k = 0; k < 5; k++) { dl[k] = uc[k] - ul[k]; dr[k] = ur[k] - uc[k]; }
    const T a = T(0.5 * (1.0 + w)), b = T(0.5 * (1.0 - w));
    for (int k = 0; k < 5; k++) s[k] = (a * dl[k]) + (b * dr[k]);
    for (int k = 0; k < 5; k++) {
        T num = dl[k], den = dr[k];
        if (fabs(num) < T(1e-5)) num = T(1e-5);
        if (fabs(den) < T(1e-5)) den = T(1e-5);
        T r = num / den;
        s[k] = s[k] * limiter(r, w, lim);
    }
}

// ========================================================================= Newtonian Euler
template <class T> struct Newton {
    double g;
    static constexpr bool coords = false;
    // Euler/EulerStateVector.cpp:55-66 with computeTotalEnergy :129-134 and
    // Euler/EulerEquationOfState.cpp:3-8
    void cons(const T* p, Pt, T* u) const {
        T rho = p[0], vx = p[1], vy = p[2], vz = p[3], pr = p[4];
        u[0] = rho; u[1] = rho * vx; u[2] = rho * vy; u[3] = rho * vz;
        T v2 = ((vx * vx) + (vy * vy)) + (vz * vz);
        T e = pr / (T(g - 1.0) * rho);
        u[4] = rho * ((T(0.5) * v2) + e);
    }
    // Euler/EulerStateVector.cpp:30-40, computePressure Euler/EulerEquationOfState.cpp:10-15
    void prim(const T* u, Pt, T* p) const {
        T rho = u[0];
        T vx = u[1] / rho, vy = u[2] / rho, vz = u[3] / rho;
        T v2 = ((vx * vx) + (vy * vy)) + (vz * vz);
        T e = (u[4] / rho) - (T(0.5) * v2);
        p[0] = rho; p[1] = vx; p[2] = vy; p[3] = vz; p[4] = (e * T(g - 1.0)) * rho;
    }
    // Euler/EulerStateVector.cpp:68-89 (x) and :96-117 (y)
    void flux(const T* u, int axis, Pt, T* f) const {
        T rho = u[0];
        T vx = u[1] / rho, vy = u[2] / rho, vz = u[3] / rho;
        T v2 = ((vx * vx) + (vy * vy)) + (vz * vz);
        T et = u[4] / rho;
        T e = et - (T(0.5) * v2);
        T pr = (e * T(g - 1.0)) * rho;
        if (axis == 0) {
            f[0] = rho * vx; f[1] = (rho * (vx * vx)) + pr; f[2] = rho * (vx * vy); f[3] = rho * (vx * vz);
            f[4] = (rho * (vx * et)) + (vx * pr);
        } else {
            f[0] = rho * vy; f[1] = rho * (vy * vx); f[2] = (rho * (vy * vy)) + pr; f[3] = rho * (vy * vz);
            f[4] = (rho * (vy * et)) + (vy * pr);
        }
    }
    // Euler/EulerEquationOfState.cpp:17-22
    double sound(const double* p) const { return std::sqrt((g * p[4]) / p[0]); }
    // Solvers/EulerSolvers.cpp:87-104 (1D) and :106-128 (2D: max(|vx|, |vy| + c) as written)
    double wavespeed(const double* p, int dims, Pt) const {
        double c = std::fabs(sound(p));
        if (dims == 1) return std::fabs(p[1]) + c;
        return mx(std::fabs(p[1]), std::fabs(p[2]) + c);
    }
};

// ========================================================================= SR Euler
// Conserved -> primitive Newton solve shared by RelativisticEulerStateVector.cpp:30-101
// (setConservedVariableVector), :138-220 / :227-309 (fluxes) and the densitised GR versions
// BlackHoleEulerStateVector.cpp:30-103, :159-350, :359-430.  tol is 1e-8 everywhere except the
// GR x-flux (BlackHoleEulerStateVector.cpp:205, 1e-10).  Results: rho, v, p, W, h.
// Templated on the scalar: double for the restatement, Dual for the tangent-linear model (whose
// comparisons act on values, so every branch is the FP64 run's; the root's derivative is the
// implicit-function theorem's at the final iterate; the floors have derivative 0).
template <class T> struct C2PT { T rho, vx, vy, vz, p, W, h; };
template <class T>
static C2PT<T> con2prim_t(T D, T Sx, T Sy, T Sz, T tau, double g, double tol) {
    using std::sqrt;
    using std::fabs;
    T q = ((tau + D) * (tau + D)) - (((Sx * Sx) + (Sy * Sy)) + (Sz * Sz));
    T dc = D / sqrt(q);
    T ec = (D + tau) / sqrt(q);
    if (q < T(1e-8)) {
        dc = D / T(std::sqrt(1e-8));
        ec = (D + tau) / T(std::sqrt(1e-8));
    }
    const T constant = T(-1.0 / (g * g));
    T linear = (T(-2.0) * dc) * T((g - 1.0) / (g * g));
    T quadratic = (((T((g - 2.0) / g) * ((ec * ec) - T(1.0))) + T(1.0)) -
                   (((dc * dc) * T((g - 1.0) / g)) * T((g - 1.0) / g)));
    T quartic = (ec * ec) - T(1.0);
    T eta = (T(2.0) * dc) * T((g - 1.0) / g);
    // Newton on the values (the reference's iteration); for the tangent-linear model the root's
    // tangent comes from the implicit-function theorem at the final iterate (ift_root).
    const double qv = val(quartic), ev = val(eta), dv = val(quadratic), lv = val(linear), cv = val(constant);
    double xv = 1.0;
    int it = 0;
    while (it < 1000) {
        double f = ((((qv * ((xv * xv) * xv)) * (xv - ev)) + (dv * (xv * xv))) + (lv * xv)) + cv;
        double fp = ((lv + ((2.0 * dv) * xv)) + ((4.0 * qv) * ((xv * xv) * xv))) - (((3.0 * ev) * qv) * (xv * xv));
        double nx = xv - (f / fp);
        if (std::fabs(xv - nx) < tol) it = 1000;
        else { it += 1; xv = nx; }
    }
    const double fpv = ((lv + ((2.0 * dv) * xv)) + ((4.0 * qv) * ((xv * xv) * xv))) - (((3.0 * ev) * qv) * (xv * xv));
    const T X = T(xv);
    const T fx = ((((quartic * ((X * X) * X)) * (X - eta)) + (quadratic * (X * X))) + (linear * X)) + constant;
    T x = ift_root(xv, fx, fpv);
    C2PT<T> r;
    r.W = ((T(0.5) * ec) * x) *
          (T(1.0) + sqrt(T(1.0) + ((T(4.0) * T((g - 1.0) / g)) * ((T(1.0) - (dc * x)) / ((ec * ec) * (x * x))))));
    r.h = T(1.0) / (dc * x);
    r.rho = D / r.W;
    T rhw = (r.rho * r.h) * (r.W * r.W);
    r.vx = Sx / rhw; r.vy = Sy / rhw; r.vz = Sz / rhw;
    r.p = (rhw - D) - tau;
    if (r.rho < T(1e-8)) r.rho = T(1e-8);
    if (r.p < T(1e-8)) r.p = T(1e-8);
    return r;
}
typedef C2PT<double> C2P;
static C2P con2prim(double D, double Sx, double Sy, double Sz, double tau, double g, double tol) {
    return con2prim_t<double>(D, Sx, Sy, Sz, tau, g, tol);
}

// RelativisticEuler/RelativisticEulerEquationOfState.cpp:3-8
static inline double sr_enthalpy(double rho, double p, double g) { return 1.0 + ((p / rho) * (g / (g - 1.0))); }
// RelativisticEuler/RelativisticEulerEquationOfState.cpp:10-18
static inline double sr_sound(double rho, double p, double g) {
    double num = (g * p) / rho;
    double den = 1.0 + ((p / rho) * (g / (g - 1.0)));
    return std::sqrt(num / den);
}

template <class T> struct SRT {
    double g;
    static constexpr bool coords = false;
    // RelativisticEuler/RelativisticEulerStateVector.cpp:116-136
    void cons(const T* p, Pt, T* u) const {
        using std::sqrt;
        T rho = p[0], vx = p[1], vy = p[2], vz = p[3], pr = p[4];
        T v2 = ((vx * vx) + (vy * vy)) + (vz * vz);
        T W = T(1.0) / sqrt(T(1.0) - v2);
        if (v2 > T(1.0 - 1e-8)) W = T(1.0 / std::sqrt(1.0 - 1e-8));
        T h = T(1.0) + ((pr / rho) * T(g / (g - 1.0)));  // sr_enthalpy
        T rhw = (rho * h) * (W * W);
        u[0] = rho * W; u[1] = rhw * vx; u[2] = rhw * vy; u[3] = rhw * vz;
        u[4] = (rhw - pr) - (rho * W);
    }
    // RelativisticEuler/RelativisticEulerStateVector.cpp:30-101
    void prim(const T* u, Pt, T* p) const {
        C2PT<T> c = con2prim_t<T>(u[0], u[1], u[2], u[3], u[4], g, 1e-8);
        p[0] = c.rho; p[1] = c.vx; p[2] = c.vy; p[3] = c.vz; p[4] = c.p;
    }
    // RelativisticEuler/RelativisticEulerStateVector.cpp:138-220 (x), :227-309 (y)
    void flux(const T* u, int axis, Pt, T* f) const {
        C2PT<T> c = con2prim_t<T>(u[0], u[1], u[2], u[3], u[4], g, 1e-8);
        T rhw = (c.rho * c.h) * (c.W * c.W);
        T vn = axis == 0 ? c.vx : c.vy;
        f[0] = (c.rho * c.W) * vn;
        if (axis == 0) {
            f[1] = (rhw * (c.vx * c.vx)) + c.p; f[2] = rhw * (c.vy * c.vx); f[3] = rhw * (c.vz * c.vx);
        } else {
            f[1] = rhw * (c.vx * c.vy); f[2] = (rhw * (c.vy * c.vy)) + c.p; f[3] = rhw * (c.vz * c.vy);
        }
        f[4] = (((rhw - c.p) - (c.rho * c.W)) * vn) + (c.p * vn);
    }
    double sound(const double* p) const { return sr_sound(p[0], p[4], g); }
    // Solvers/RelativisticEulerSolvers.cpp:87-104 (1D) and :106-128 (2D: max(|vx|,|vy|) + c)
    double wavespeed(const double* p, int dims, Pt) const {
        double c = std::fabs(sound(p));
        if (dims == 1) return std::fabs(p[1]) + c;
        return mx(std::fabs(p[1]), std::fabs(p[2])) + c;
    }
};
typedef SRT<double> SR;

// ========================================================================= Kerr-Schild spacetime
struct BH {
    double M, a, bx, by, bz;

    // BlackHoleSpacetime.cpp:54-68 (the Kerr radius as written at :59-63)
    double radius(double dx, double dy, double dz) const {
        double n2 = ((dx * dx) + (dy * dy)) + (dz * dz);
        double ma2 = (M * M) * (a * a);
        return std::sqrt(0.5 * ((n2 - ma2) + std::sqrt(((n2 - ma2) * (n2 - ma2)) + (4.0 * (ma2 * (dz * dz))))));
    }
    double H(double x, double y, double z) const {
        double dx = x - bx, dy = y - by, dz = z - bz;
        double r = radius(dx, dy, dz);
        double ma2 = (M * M) * (a * a);
        return -(M * ((r * r) * r)) / ((((r * r) * r) * r) + (ma2 * (dz * dz)));
    }
    // BlackHoleSpacetime.cpp:70-90
    void l(double x, double y, double z, double* o) const {
        double dx = x - bx, dy = y - by, dz = z - bz;
        double r = radius(dx, dy, dz);
        double ma2 = (M * M) * (a * a);
        o[0] = -((r * dx) + ((a * M) * dy)) / ((r * r) + ma2);
        o[1] = -((r * dy) - ((a * M) * dx)) / ((r * r) + ma2);
        o[2] = -dz / r;
    }
    // BlackHoleSpacetime.cpp:92-113, including the "r + (y - y_BH)" of :108 as written
    void L4(double x, double y, double z, double* o) const {
        double dx = x - bx, dy = y - by, dz = z - bz;
        double r = radius(dx, dy, dz);
        double ma2 = (M * M) * (a * a);
        o[0] = -1.0;
        o[1] = -((r * dx) + ((a * M) * dy)) / ((r * r) + ma2);
        o[2] = -((r + dy) - ((a * M) * dx)) / ((r * r) + ma2);
        o[3] = -dz / r;
    }
    // BlackHoleSpacetime.cpp:153-186
    void gamma(double x, double y, double z, double* m) const {
        double h = H(x, y, z), v[3];
        l(x, y, z, v);
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) m[3 * i + j] = (i == j ? 1.0 : 0.0) - (((2.0 * h) * v[i]) * v[j]);
    }
    // BlackHoleSpacetime.cpp:188-228
    void g4(double x, double y, double z, double* m) const {
        double h = H(x, y, z), v[4];
        L4(x, y, z, v);
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++) {
                double eta = (i == j) ? ((i == 0) ? -1.0 : 1.0) : 0.0;
                m[4 * i + j] = eta - (((2.0 * h) * v[i]) * v[j]);
            }
    }
    double lapse(double x, double y, double z) const { return 1.0 / std::sqrt(1.0 - (2.0 * H(x, y, z))); }  // :278-281
    void shiftv(double x, double y, double z, double* b) const {  // :283-296
        double h = H(x, y, z), v[3];
        l(x, y, z, v);
        for (int i = 0; i < 3; i++) b[i] = ((2.0 * h) / (1.0 - (2.0 * h))) * v[i];
    }
    bool excised(double x, double y, double z) const {  // :372-386
        double r = std::sqrt((((x - bx) * (x - bx)) + ((y - by) * (y - by))) + ((z - bz) * (z - bz)));
        return r <= (M * (1.0 + std::sqrt(1.0 - (a * a))));
    }
};

// Mathematics/MatrixAlgebra.cpp:106-149 (cofactor expansion along row 0; 2x2 base case)
static double det2(const double* m) { return (m[0] * m[3]) - (m[2] * m[1]); }
static double det_n(const double* m, int n) {
    if (n == 2) return det2(m);
    double d = 0.0;
    double c[9];
    for (int i = 0; i < n; i++) {
        for (int j = 0; j < n - 1; j++)
            for (int k = 0; k < n - 1; k++) c[(n - 1) * j + k] = (k < i) ? m[n * (j + 1) + k] : m[n * (j + 1) + k + 1];
        if (i % 2 == 0) d = d + (m[i] * det_n(c, n - 1));
        else d = d - (m[i] * det_n(c, n - 1));
    }
    return d;
}
// Mathematics/MatrixAlgebra.cpp:63-93 (products accumulate from 0.0 in k order)
static void matmul(const double* a, const double* b, double* c, int n) {
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
            double s = 0.0;
            for (int k = 0; k < n; k++) s = s + (a[n * i + k] * b[n * k + j]);
            c[n * i + j] = s;
        }
}
static double trace(const double* m, int n) { double t = 0.0; for (int i = 0; i < n; i++) t = t + m[n * i + i]; return t; }
// Mathematics/MatrixAlgebra.cpp:151-194 (Cayley-Hamilton inverses for n = 3, 4)
static void inverse_n(const double* m, int n, double* o) {
    double d = det_n(m, n), tr = trace(m, n);
    double m2[16];
    matmul(m, m, m2, n);
    double tr2 = trace(m2, n);
    if (n == 3) {
        double s = 0.5 * ((tr * tr) - tr2);
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                double e = ((s * (i == j ? 1.0 : 0.0)) - (tr * m[3 * i + j])) + m2[3 * i + j];
                o[3 * i + j] = (1.0 / d) * e;
            }
    } else {
        double m3[16];
        matmul(m2, m, m3, 4);
        double tr3 = trace(m3, 4);
        double c0 = (1.0 / 6.0) * ((((tr * tr) * tr) - ((3.0 * tr) * tr2)) + (2.0 * tr3));
        double c1 = 0.5 * ((tr * tr) - tr2);
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++) {
                double e = (((c0 * (i == j ? 1.0 : 0.0)) - (c1 * m[4 * i + j])) + (tr * m2[4 * i + j])) - m3[4 * i + j];
                o[4 * i + j] = (1.0 / d) * e;
            }
    }
}

template <class Num> struct GRT {
    double g;
    BH bh;
    double h;  // finite-difference spacing for metric derivatives (the grid's cell spacing)
    static constexpr bool coords = true;

    double detg(Pt p) const { double m[9]; bh.gamma(p.x, p.y, p.z, m); return det_n(m, 3); }  // :240-243

    // BlackHoleEuler/BlackHoleEulerStateVector.cpp:118-157 (energy uses W, not W^2, at :154).  The
    // metric is FP64 data; the state may be a dual number (tangent-linear model).
    void cons(const Num* p, Pt q, Num* u) const {
        using std::sqrt;
        double m[9];
        bh.gamma(q.x, q.y, q.z, m);
        double dg = detg(q);
        Num v[3] = {p[1], p[2], p[3]};
        Num v2 = Num(0.0);
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) v2 = v2 + ((Num(m[3 * i + j]) * v[i]) * v[j]);
        Num W = Num(1.0) / sqrt(Num(1.0) - v2);
        if (v2 > Num(1.0 - 1e-8)) W = Num(1.0 / std::sqrt(1.0 - 1e-8));
        Num hh = Num(1.0) + ((p[4] / p[0]) * Num(g / (g - 1.0)));  // sr_enthalpy
        Num sg = Num(std::sqrt(dg));
        u[0] = (sg * p[0]) * W;
        for (int k = 0; k < 3; k++) u[1 + k] = (((sg * p[0]) * hh) * (W * W)) * v[k];
        u[4] = sg * ((((p[0] * hh) * W) - p[4]) - (p[0] * W));
    }
    C2PT<Num> c2p(const Num* u, Pt q, double tol) const {
        Num sg = Num(std::sqrt(detg(q)));
        return con2prim_t<Num>(u[0] / sg, u[1] / sg, u[2] / sg, u[3] / sg, u[4] / sg, g, tol);
    }
    // BlackHoleEuler/BlackHoleEulerStateVector.cpp:30-103
    void prim(const Num* u, Pt q, Num* p) const {
        C2PT<Num> c = c2p(u, q, 1e-8);
        p[0] = c.rho; p[1] = c.vx; p[2] = c.vy; p[3] = c.vz; p[4] = c.p;
    }
    // BlackHoleEuler/BlackHoleEulerStateVector.cpp:159-250 (x, Newton tol 1e-10) and :259-350 (y)
    void flux(const Num* u, int axis, Pt q, Num* f) const {
        double dg = detg(q);
        double al = bh.lapse(q.x, q.y, q.z);
        double be[3];
        bh.shiftv(q.x, q.y, q.z, be);
        C2PT<Num> c = c2p(u, q, axis == 0 ? 1e-10 : 1e-8);
        Num as = Num(al * std::sqrt(dg));
        Num rhw = (c.rho * c.h) * (c.W * c.W);
        Num vn = axis == 0 ? c.vx : c.vy;
        Num w = vn - Num(be[axis] / al);
        f[0] = as * ((c.rho * c.W) * w);
        if (axis == 0) {
            f[1] = as * ((rhw * (c.vx * w)) + c.p);
            f[2] = as * (rhw * (c.vy * w));
        } else {
            f[1] = as * (rhw * (c.vx * w));
            f[2] = as * ((rhw * (c.vy * w)) + c.p);
        }
        f[3] = as * (rhw * (c.vz * w));
        f[4] = as * ((((rhw - c.p) - (c.rho * c.W)) * w) + (c.p * vn));
    }

    // ---- metric derivatives, BlackHoleSpacetime.cpp:115-151, :250-370
    void dH(Pt q, double* o) const {
        double hs = 0.5 * h;
        o[0] = (bh.H(q.x + hs, q.y, q.z) - bh.H(q.x - hs, q.y, q.z)) / h;
        o[1] = (bh.H(q.x, q.y + hs, q.z) - bh.H(q.x, q.y - hs, q.z)) / h;
        o[2] = (bh.H(q.x, q.y, q.z + hs) - bh.H(q.x, q.y, q.z - hs)) / h;
    }
    void dl(Pt q, double* o) const {  // o[3*dir + comp]
        double hs = 0.5 * h, a[3], b[3];
        for (int d = 0; d < 3; d++) {
            Pt p1 = q, p0 = q;
            if (d == 0) { p1.x = q.x + hs; p0.x = q.x - hs; }
            if (d == 1) { p1.y = q.y + hs; p0.y = q.y - hs; }
            if (d == 2) { p1.z = q.z + hs; p0.z = q.z - hs; }
            bh.l(p1.x, p1.y, p1.z, a); bh.l(p0.x, p0.y, p0.z, b);
            for (int c = 0; c < 3; c++) o[3 * d + c] = (1.0 / h) * (a[c] - b[c]);
        }
    }
    void dgamma(Pt q, double* o) const {  // o[9*dir + 3*i + j]
        double hs = 0.5 * h, a[9], b[9];
        for (int d = 0; d < 3; d++) {
            Pt p1 = q, p0 = q;
            if (d == 0) { p1.x = q.x + hs; p0.x = q.x - hs; }
            if (d == 1) { p1.y = q.y + hs; p0.y = q.y - hs; }
            if (d == 2) { p1.z = q.z + hs; p0.z = q.z - hs; }
            bh.gamma(p1.x, p1.y, p1.z, a); bh.gamma(p0.x, p0.y, p0.z, b);
            for (int c = 0; c < 9; c++) o[9 * d + c] = (1.0 / h) * (a[c] - b[c]);
        }
    }
    void dalpha(Pt q, double* o) const {
        double hs = 0.5 * h;
        o[0] = (bh.lapse(q.x + hs, q.y, q.z) - bh.lapse(q.x - hs, q.y, q.z)) / h;
        o[1] = (bh.lapse(q.x, q.y + hs, q.z) - bh.lapse(q.x, q.y - hs, q.z)) / h;
        o[2] = (bh.lapse(q.x, q.y, q.z + hs) - bh.lapse(q.x, q.y, q.z - hs)) / h;
    }
    void dbeta(Pt q, double* o) const {  // o[3*dir + comp]
        double hs = 0.5 * h, a[3], b[3];
        for (int d = 0; d < 3; d++) {
            Pt p1 = q, p0 = q;
            if (d == 0) { p1.x = q.x + hs; p0.x = q.x - hs; }
            if (d == 1) { p1.y = q.y + hs; p0.y = q.y - hs; }
            if (d == 2) { p1.z = q.z + hs; p0.z = q.z - hs; }
            bh.shiftv(p1.x, p1.y, p1.z, a); bh.shiftv(p0.x, p0.y, p0.z, b);
            for (int c = 0; c < 3; c++) o[3 * d + c] = (1.0 / h) * (a[c] - b[c]);
        }
    }
    void Kij(Pt q, double* K) const {  // BlackHoleSpacetime.cpp:336-370
        double al = bh.lapse(q.x, q.y, q.z), Hs = bh.H(q.x, q.y, q.z), v[3], dh[3], dv[9];
        bh.l(q.x, q.y, q.z, v);
        dH(q, dh);
        dl(q, dv);
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                double k = al * ((((-(v[i] * dh[j])) - (v[j] * dh[i])) - (Hs * dv[3 * j + i])) - (Hs * dv[3 * i + j]));
                for (int c = 0; c < 3; c++) {
                    k = k + (((al * 2.0) * (Hs * Hs)) * (((v[i] * v[c]) * dv[3 * c + j]) + ((v[j] * v[c]) * dv[3 * c + i])));
                    k = k + ((((((al * 2.0) * Hs) * v[i]) * v[j]) * v[c]) * dh[c]);
                }
                K[3 * i + j] = k;
            }
    }
    // BlackHoleEuler/BlackHoleEulerStateVector.cpp:359-510
    // State-dependent parts in Num (the tangent-linear model's dual numbers), the metric in FP64.
    void source(const Num* u, Pt q, Num* s) const {
        double dg = detg(q);
        double al = bh.lapse(q.x, q.y, q.z), be[3];
        bh.shiftv(q.x, q.y, q.z, be);
        C2PT<Num> c = c2p(u, q, 1e-8);
        double g4m[16], gi[16];
        bh.g4(q.x, q.y, q.z, g4m);
        inverse_n(g4m, 4, gi);
        Num uu[4];
        uu[0] = c.W / Num(al);
        uu[1] = ((Num(al) * uu[0]) * c.vx) - (Num(be[0]) * uu[0]);
        uu[2] = ((Num(al) * uu[0]) * c.vy) - (Num(be[1]) * uu[0]);
        uu[3] = ((Num(al) * uu[0]) * c.vz) - (Num(be[2]) * uu[0]);
        Num T[16];
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++) T[4 * i + j] = (((c.rho * c.h) * uu[i]) * uu[j]) + (c.p * Num(gi[4 * i + j]));
        double da[3], db[9], gm[9], dgm[27], K[9];
        dalpha(q, da);
        dbeta(q, db);
        bh.gamma(q.x, q.y, q.z, gm);
        dgamma(q, dgm);
        Kij(q, K);
        Num S[5] = {Num(0.0), Num(0.0), Num(0.0), Num(0.0), Num(0.0)};
        Num vc[3];
        for (int i = 0; i < 3; i++) vc[i] = ((Num(gm[3 * i + 0]) * c.vx) + (Num(gm[3 * i + 1]) * c.vy)) + (Num(gm[3 * i + 2]) * c.vz);
        Num rhw = (c.rho * c.h) * (c.W * c.W);
        for (int i = 0; i < 3; i++) {
            for (int j = 0; j < 3; j++) {
                for (int k = 0; k < 3; k++) {
                    double dgijk = dgm[9 * i + 3 * j + k];
                    S[i + 1] = S[i + 1] + (T[0] * Num(((0.5 * be[j]) * be[k]) * dgijk));
                    S[i + 1] = S[i + 1] + ((T[j + 1] * Num(be[k])) * Num(dgijk));
                    S[i + 1] = S[i + 1] + (Num(0.5) * (T[4 * (j + 1) + (k + 1)] * Num(dgijk)));
                }
                S[i + 1] = S[i + 1] + (((rhw * vc[j]) / Num(al)) * Num(db[3 * i + j]));
            }
            S[i + 1] = S[i + 1] - ((T[0] * Num(al)) * Num(da[i]));
        }
        for (int i = 0; i < 3; i++) {
            for (int j = 0; j < 3; j++) {
                S[4] = S[4] + (T[0] * Num((be[i] * be[j]) * K[3 * i + j]));
                S[4] = S[4] + (T[i + 1] * Num((2.0 * be[j]) * K[3 * i + j]));
                S[4] = S[4] + (T[4 * (i + 1) + (j + 1)] * Num(K[3 * i + j]));
            }
            S[4] = S[4] - (T[0] * Num(be[i] * da[i]));
            S[4] = S[4] - (T[i + 1] * Num(da[i]));
        }
        Num f = Num(al * std::sqrt(dg));
        for (int k = 0; k < 5; k++) s[k] = f * S[k];
    }
    // BlackHoleEuler/BlackHoleEulerStateVector.cpp:519-549 with
    // BlackHoleEuler/BlackHoleEulerEigenvalues.cpp:3-96 (maximum signed eigenvalue)
    double sound_speed(const double* p, Pt q) const {
        double al = bh.lapse(q.x, q.y, q.z), be[3];
        bh.shiftv(q.x, q.y, q.z, be);
        double gm[9], gs[9];
        bh.gamma(q.x, q.y, q.z, gm);
        inverse_n(gm, 3, gs);
        double cs = sr_sound(p[0], p[4], g);
        double v[3] = {p[1], p[2], p[3]};
        double v2 = 0.0;
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) v2 = v2 + ((gm[3 * i + j] * v[i]) * v[j]);
        double s = 0.0;
        for (int i = 0; i < 3; i++) {
            double mat = (al * v[i]) - be[i];
            double rt = std::sqrt((1.0 - v2) * ((gs[3 * i + i] * (1.0 - (v2 * (cs * cs)))) - ((v[i] * v[i]) * (1.0 - (cs * cs)))));
            double pre = al / (1.0 - (v2 * (cs * cs)));
            double fast = (pre * ((v[i] * (1.0 - (cs * cs))) + (cs * rt))) - be[i];
            double slow = (pre * ((v[i] * (1.0 - (cs * cs))) - (cs * rt))) - be[i];
            if (mat > s) s = mat;
            if (fast > s) s = fast;
            if (slow > s) s = slow;
        }
        return s;
    }
};
typedef GRT<double> GR;

// ========================================================================= generic sweep
// Half-step evolution of the middle state, Solvers/EulerSolvers.cpp:174-223 (Newtonian),
// Solvers/RelativisticEulerSolvers.cpp:148-199 (SR), Solvers/BlackHoleEulerSolvers.cpp:234-307
// (GR: slopes from conserved states at xc -/+ dx, face fluxes at xc -/+ dx/2, and the evolved
// state converted at its face).  side 0 = left face, 1 = right face; both produced here.
template <class Sys, class T>
static void evolve_half(const Sys& S, const T* l, const T* m, const T* r, Pt xc, int axis, double dx, double dt,
                        double w, int lim, T* left_face, T* right_face) {
    T ul[5], um[5], ur[5], sl[5];
    S.cons(l, shift(xc, axis, -dx), ul);
    S.cons(m, xc, um);
    S.cons(r, shift(xc, axis, dx), ur);
    slope_vector(ul, um, ur, w, lim, sl);
    T UL[5], UR[5], FL[5], FR[5], ev[5];
    for (int k = 0; k < 5; k++) { UL[k] = um[k] - (T(0.5) * sl[k]); UR[k] = um[k] + (T(0.5) * sl[k]); }
    S.flux(UL, axis, shift(xc, axis, -(dx * 0.5)), FL);
    S.flux(UR, axis, shift(xc, axis, dx * 0.5), FR);
    const T s = T(0.5 * (dt / dx));  // computeEvolutionVector, Solvers/EulerSolvers.cpp:163-172
    for (int k = 0; k < 5; k++) ev[k] = s * (FL[k] - FR[k]);
    T a[5], b[5];
    for (int k = 0; k < 5; k++) { a[k] = UL[k] + ev[k]; b[k] = UR[k] + ev[k]; }
    if (left_face) S.prim(a, shift(xc, axis, -(dx * 0.5)), left_face);
    if (right_face) S.prim(b, shift(xc, axis, dx * 0.5), right_face);
}

// FORCE flux of two primitive states at interface xf: Solvers/EulerFirstOrderSolver.cpp:3-59
// (Lax-Friedrichs :3-11, Richtmyer :13-19, FORCE :21-24); GR twin
// Solvers/BlackHoleEulerFirstOrderSolver.cpp:3-47 (states at xf -/+ dx/2, Richtmyer flux at xf).
template <class Sys, class T>
static void force_flux(const Sys& S, const T* L, const T* R, Pt xf, int axis, double dx, double dt, T* F) {
    T uL[5], uR[5], fL[5], fR[5], us[5], fs[5];
    Pt pl = shift(xf, axis, -(dx * 0.5)), pr = shift(xf, axis, dx * 0.5);
    S.cons(L, pl, uL);
    S.cons(R, pr, uR);
    S.flux(uL, axis, pl, fL);
    S.flux(uR, axis, pr, fR);
    const T c = T(dx / dt), d = T(dt / dx);
    T lf[5];
    for (int k = 0; k < 5; k++) lf[k] = T(0.5) * ((fL[k] + fR[k]) + (c * (uL[k] - uR[k])));
    for (int k = 0; k < 5; k++) us[k] = T(0.5) * ((uL[k] + uR[k]) + (d * (fL[k] - fR[k])));
    S.flux(us, axis, xf, fs);
    for (int k = 0; k < 5; k++) F[k] = T(0.5) * (lf[k] + fs[k]);
}

// Cell coordinates: x = j*dx, y = i*dx (Solvers/BlackHoleEulerSecondOrderSolver.cpp:88-100).
static inline Pt cell_pt(int i, int j, double dx) { return Pt{j * dx, i * dx, 0.0}; }

// Ghost-cell index for a line of n cells: transmissive mirrors (Solvers/EulerSolvers.cpp:13-19:
// g[-1]=c[0], g[-2]=c[1], g[n]=c[n-1], g[n+1]=c[n-2]) or periodic wrap (the build's extension).
static inline int ghost(int k, int n, int bc) {
    if (bc == 1) return ((k % n) + n) % n;
    if (k < 0) return -1 - k;
    if (k >= n) return 2 * n - 1 - k;
    return k;
}

// Thread count for the line-parallel sweeps (1 by default; set by orc_set_threads).
static int g_threads = 1;

template <class F>
static void parallel_lines(int nlines, F&& body) {
    int nt = g_threads < 1 ? 1 : g_threads;
    if (nt > nlines) nt = nlines;
    if (nt <= 1) { body(0, nlines); return; }
    std::vector<std::thread> pool;
    for (int t = 0; t < nt; t++) {
        int a = (int)((long long)nlines * t / nt), b = (int)((long long)nlines * (t + 1) / nt);
        pool.emplace_back([&body, a, b]() { body(a, b); });
    }
    for (auto& th : pool) th.join();
}

// One dimensional sweep over the whole grid.  Solvers/EulerSecondOrderSolver.cpp:27-100 (SLIC),
// Solvers/EulerFirstOrderSolver.cpp:103-155 (FORCE), GR twins with excision masks
// Solvers/BlackHoleEulerSecondOrderSolver.cpp:39-179, Solvers/BlackHoleEulerFirstOrderSolver.cpp:89-165.
// mask (optional, one byte per cell): only cells with mask != 0 are updated (the AMR drivers'
// masked steps, AMR/EulerAMR.cpp:83-167).
template <class Sys, class T>
static void sweep(const Sys& S, T* prim, int ny, int nx, int dims, int axis, int order, double dx, double dt,
                  double w, int lim, int bc, const unsigned char* mask, const BH* exc) {
    if (dims == 1) { ny = 1; axis = 0; }
    const int nlines = axis == 0 ? ny : nx, n = axis == 0 ? nx : ny;
    // Lines are independent (each stencil stays inside its line), so they are split across
    // threads; the result does not depend on the thread count.
    parallel_lines(nlines, [&](int L0, int L1) {
    std::vector<T> line((size_t)(n + 4) * 5), out((size_t)n * 5);
    std::vector<T> flux((size_t)(n + 1) * 5), faceL((size_t)(n + 2) * 5), faceR((size_t)(n + 2) * 5);
    std::vector<char> needf(n + 1), active(n);
    for (int L = L0; L < L1; L++) {
        auto idx = [&](int k) -> size_t { return axis == 0 ? ((size_t)L * nx + k) : ((size_t)k * nx + L); };
        auto cpt = [&](int k) -> Pt { return axis == 0 ? cell_pt(L, k, dx) : cell_pt(k, L, dx); };
        for (int k = -2; k < n + 2; k++) {
            const T* src = prim + 5 * idx(ghost(k, n, bc));
            std::memcpy(&line[5 * (k + 2)], src, 5 * sizeof(T));
        }
        auto cell = [&](int k) -> const T* { return &line[5 * (k + 2)]; };
        // which cells update (mask, GR excision of the stencil)
        for (int k = 0; k < n; k++) {
            bool on = mask ? mask[idx(k)] != 0 : true;
            if (on && exc) {
                int reach = order == 2 ? 2 : 1;
                Pt c = cpt(k);
                if (dims == 1) {
                    for (int d = -reach; d <= reach && on; d++) on = !exc->excised((k + d) * dx, 0.0, 0.0);
                } else {
                    int i = axis == 0 ? L : k, j = axis == 0 ? k : L;
                    (void)c;
                    on = !exc->excised(j * dx, i * dx, 0.0);
                    for (int d = 1; d <= reach && on; d++)
                        on = !exc->excised((j - d) * dx, i * dx, 0.0) && !exc->excised((j + d) * dx, i * dx, 0.0) &&
                             !exc->excised(j * dx, (i - d) * dx, 0.0) && !exc->excised(j * dx, (i + d) * dx, 0.0);
                }
            }
            active[k] = on;
        }
        for (int f = 0; f <= n; f++) needf[f] = (f > 0 && active[f - 1]) || (f < n && active[f]);
        // interface f sits between cells f-1 and f, at coordinate (k - 0.5)*dx for k = f
        auto fpt = [&](int f) -> Pt {
            if (dims == 1) return Pt{(f - 0.5) * dx, 0.0, 0.0};
            return axis == 0 ? Pt{(f - 0.5) * dx, L * dx, 0.0} : Pt{L * dx, (f - 0.5) * dx, 0.0};
        };
        if (order == 2 && !Sys::coords) {
            for (int k = -1; k <= n; k++) {
                bool want = (k >= 0 && k <= n && needf[k]) || (k + 1 <= n && needf[k + 1]);
                if (!want) continue;
                evolve_half(S, cell(k - 1), cell(k), cell(k + 1), Pt{0, 0, 0}, axis, dx, dt, w, lim,
                            &faceL[5 * (k + 1)], &faceR[5 * (k + 1)]);
            }
        }
        for (int f = 0; f <= n; f++) {
            if (!needf[f]) continue;
            Pt xf = fpt(f);
            if (order == 1) {
                force_flux(S, cell(f - 1), cell(f), xf, axis, dx, dt, &flux[5 * f]);
            } else if (!Sys::coords) {
                force_flux(S, &faceR[5 * f], &faceL[5 * (f + 1)], xf, axis, dx, dt, &flux[5 * f]);
            } else {
                // Solvers/BlackHoleEulerSecondOrderSolver.cpp:3-37: left cell evolved at
                // xf - dx/2 (its right face), right cell at xf + dx/2 (its left face)
                T er[5], el[5];
                evolve_half(S, cell(f - 2), cell(f - 1), cell(f), shift(xf, axis, -(dx * 0.5)), axis, dx, dt, w, lim,
                            (T*)nullptr, er);
                evolve_half(S, cell(f - 1), cell(f), cell(f + 1), shift(xf, axis, dx * 0.5), axis, dx, dt, w, lim, el,
                            (T*)nullptr);
                force_flux(S, er, el, xf, axis, dx, dt, &flux[5 * f]);
            }
        }
        const T d = T(dt / dx);
        for (int k = 0; k < n; k++) {
            T* o = &out[5 * k];
            if (!active[k]) { std::memcpy(o, cell(k), 5 * sizeof(T)); continue; }
            Pt c = dims == 1 ? Pt{k * dx, 0.0, 0.0} : cpt(k);
            T u[5], nu[5];
            S.cons(cell(k), c, u);
            // computeFORCEUpdate, Solvers/EulerFirstOrderSolver.cpp:96-101
            for (int q = 0; q < 5; q++) nu[q] = u[q] + (d * (flux[5 * k + q] - flux[5 * (k + 1) + q]));
            S.prim(nu, c, o);
        }
        for (int k = 0; k < n; k++) std::memcpy(prim + 5 * idx(k), &out[5 * k], 5 * sizeof(T));
    }
    });
}

// Solvers/EulerSolvers.cpp:130-145
static double stable_dt_rule(double dt, double t, double tf, int it) {
    double n = dt;
    if (it <= 5) n = n * 0.2;
    if ((t + n) > tf) n = tf - t;
    return n;
}

template <class Sys>
static double max_wavespeed(const Sys& S, const double* prim, int ny, int nx, int dims) {
    double m = 0.0;
    size_t N = (size_t)(dims == 1 ? 1 : ny) * nx;
    for (size_t c = 0; c < N; c++) {
        double w = S.wavespeed(prim + 5 * c, dims, Pt{0, 0, 0});
        if (w > m) m = w;
    }
    return m;
}

// Solvers/BlackHoleEulerSolvers.cpp:87-131: coordinates i/N (1D) and, in 2D, excision tested at
// (j/ncol, i/nrow) while the speed is evaluated at (i/nrow, j/ncol) -- both as written.
static double gr_max_wavespeed(const GR& S, const double* prim, int ny, int nx, int dims) {
    double m = 0.0;
    if (dims == 1) {
        double cs = 1.0 / nx;
        for (int i = 0; i < nx; i++) {
            if (!S.bh.excised(i * cs, 0.0, 0.0)) {
                double w = std::fabs(S.sound_speed(prim + 5 * i, Pt{i * cs, 0.0, 0.0}));
                if (w > m) m = w;
            }
        }
        return m;
    }
    double rs = 1.0 / ny, cs = 1.0 / nx;
    for (int i = 0; i < ny; i++)
        for (int j = 0; j < nx; j++)
            if (!S.bh.excised(j * cs, i * rs, 0.0)) {
                double w = std::fabs(S.sound_speed(prim + 5 * ((size_t)i * nx + j), Pt{i * rs, j * cs, 0.0}));
                if (w > m) m = w;
            }
    return m;
}

// ---------------------------------------------------------------- GR source RK step
// Solvers/BlackHoleEulerSolvers.cpp:159-232: fractional evolution with face fluxes at xc -/+ dx
template <class Sys, class T, class P>
static void evolve_fraction(const Sys& S, double frac, const T* l, const T* m, const T* r, P xc, int axis, double dx,
                            double dt, double w, int lim, T* out) {
    T ul[5], um[5], ur[5], sl[5];
    S.cons(l, shift(xc, axis, -dx), ul);
    S.cons(m, xc, um);
    S.cons(r, shift(xc, axis, dx), ur);
    slope_vector(ul, um, ur, w, lim, sl);
    T UL[5], UR[5], FL[5], FR[5];
    for (int k = 0; k < 5; k++) { UL[k] = um[k] - (T(0.5) * sl[k]); UR[k] = um[k] + (T(0.5) * sl[k]); }
    S.flux(UL, axis, shift(xc, axis, -dx), FL);
    S.flux(UR, axis, shift(xc, axis, dx), FR);
    const T s = T(frac * (dt / dx));
    T nu[5];
    for (int k = 0; k < 5; k++) nu[k] = um[k] + (s * (FL[k] - FR[k]));
    S.prim(nu, xc, out);
}

// Solvers/BlackHoleEulerForcingSolver.cpp:3-70 (1D) and :72-185 (2D): classical RK4 on the
// source with interleaved fractional flux sweeps on frozen neighbours.
template <class Sys, class T>
static void rk_cell(const Sys& S, int dims, const T* cl, const T* cm, const T* cr, const T* ct, const T* cb, Pt q,
                    double dx, double dt, double w, int lim, T* out_cons) {
    T L[5], R[5], Tp[5], B[5], Mp[5], E1[5], E2[5], E[5];
    S.prim(cl, shift(q, 0, -dx), L);
    S.prim(cr, shift(q, 0, dx), R);
    if (dims == 2) {
        S.prim(ct, shift(q, 1, -dx), Tp);
        S.prim(cb, shift(q, 1, dx), B);
    }
    T k[4][5], st[5], c[5];
    auto src = [&](const T* u, T* o) {
        T s[5];
        S.source(u, q, s);
        for (int i = 0; i < 5; i++) o[i] = T(dt) * s[i];
    };
    src(cm, k[0]);
    const double fx1[3] = {0.5, 0.5, 1.0};                                     // 1D fractions
    const double fx2[3] = {0.25, 0.25, 0.5}, fy2[3] = {0.5, 0.5, 1.0};        // 2D fractions
    for (int stage = 0; stage < 3; stage++) {
        for (int i = 0; i < 5; i++) st[i] = stage < 2 ? (cm[i] + (T(0.5) * k[stage][i])) : (cm[i] + k[stage][i]);
        S.prim(st, q, Mp);
        if (dims == 1) {
            evolve_fraction(S, fx1[stage], L, Mp, R, q, 0, dx, dt, w, lim, E);
        } else {
            evolve_fraction(S, fx2[stage], L, Mp, R, q, 0, dx, dt, w, lim, E1);
            evolve_fraction(S, fy2[stage], Tp, E1, B, q, 1, dx, dt, w, lim, E2);
            evolve_fraction(S, fx2[stage], L, E2, R, q, 0, dx, dt, w, lim, E);
        }
        S.cons(E, q, c);
        src(c, k[stage + 1]);
    }
    for (int i = 0; i < 5; i++)
        out_cons[i] = cm[i] + (T(1.0 / 6.0) * (k[0][i] + ((T(2.0) * k[1][i]) + ((T(2.0) * k[2][i]) + k[3][i]))));
}

// Solvers/BlackHoleEulerForcingSolver.cpp:187-250 (transmissive 1-ghost neighbours)
template <class Sys, class T>
static void rk_source(const Sys& S, T* prim, int ny, int nx, int dims, double dx, double dt, double w, int lim) {
    if (dims == 1) ny = 1;
    std::vector<T> out((size_t)ny * nx * 5);
    std::memcpy(out.data(), prim, out.size() * sizeof(T));
    for (int i = 0; i < ny; i++)
        for (int j = 0; j < nx; j++) {
            bool on;
            if (dims == 1)
                on = !S.bh.excised(j * dx, 0.0, 0.0) && !S.bh.excised((j - 1) * dx, 0.0, 0.0) &&
                     !S.bh.excised((j + 1) * dx, 0.0, 0.0);
            else
                on = !S.bh.excised(j * dx, i * dx, 0.0) && !S.bh.excised((j - 1) * dx, i * dx, 0.0) &&
                     !S.bh.excised((j + 1) * dx, i * dx, 0.0) && !S.bh.excised(j * dx, (i - 1) * dx, 0.0) &&
                     !S.bh.excised(j * dx, (i + 1) * dx, 0.0);
            if (!on) continue;
            auto P = [&](int ii, int jj) -> const T* {
                return prim + 5 * ((size_t)ghost(ii, ny, 0) * nx + ghost(jj, nx, 0));
            };
            Pt q = dims == 1 ? Pt{j * dx, 0.0, 0.0} : Pt{j * dx, i * dx, 0.0};
            T cl[5], cm[5], cr[5], ct[5], cb[5], nc[5];
            S.cons(P(i, j - 1), dims == 1 ? Pt{(j - 1) * dx, 0.0, 0.0} : Pt{(j - 1) * dx, i * dx, 0.0}, cl);
            S.cons(P(i, j), q, cm);
            S.cons(P(i, j + 1), dims == 1 ? Pt{(j + 1) * dx, 0.0, 0.0} : Pt{(j + 1) * dx, i * dx, 0.0}, cr);
            if (dims == 2) {
                S.cons(P(i - 1, j), Pt{j * dx, (i - 1) * dx, 0.0}, ct);
                S.cons(P(i + 1, j), Pt{j * dx, (i + 1) * dx, 0.0}, cb);
            }
            rk_cell(S, dims, cl, cm, cr, ct, cb, q, dx, dt, w, lim, nc);
            S.prim(nc, q, &out[5 * ((size_t)i * nx + j)]);
        }
    std::memcpy(prim, out.data(), out.size() * sizeof(T));
}

}  // namespace orc

using namespace orc;

// ========================================================================= C ABI
extern "C" {

void orc_set_threads(int n) { g_threads = n < 1 ? 1 : n; }

// sys: 0 Newtonian, 1 SR, 2 GR.  bh = {M, a, x, y, z} (GR only).
void orc_sweep(int sys, double* prim, int ny, int nx, int dims, int axis, int order, double dx, double dt,
               double bias, int lim, double gamma, int bc, const unsigned char* mask, const double* bh) {
    if (sys == 0) sweep(Newton<double>{gamma}, prim, ny, nx, dims, axis, order, dx, dt, bias, lim, bc, mask, nullptr);
    else if (sys == 1) sweep(SR{gamma}, prim, ny, nx, dims, axis, order, dx, dt, bias, lim, bc, mask, nullptr);
    else {
        GR S{gamma, BH{bh[0], bh[1], bh[2], bh[3], bh[4]}, dx};
        sweep(S, prim, ny, nx, dims, axis, order, dx, dt, bias, lim, 0, mask, &S.bh);
    }
}

double orc_max_wavespeed(int sys, const double* prim, int ny, int nx, int dims, double gamma, const double* bh) {
    if (sys == 0) return max_wavespeed(Newton<double>{gamma}, prim, ny, nx, dims);
    if (sys == 1) return max_wavespeed(SR{gamma}, prim, ny, nx, dims);
    GR S{gamma, BH{bh[0], bh[1], bh[2], bh[3], bh[4]}, 0.0};
    return gr_max_wavespeed(S, prim, ny, nx, dims);
}

double orc_stable_dt_rule(double dt, double t, double tf, int it) { return stable_dt_rule(dt, t, tf, it); }

// Solvers/EulerSolvers.cpp:147-161
double orc_stable_dt(int sys, const double* prim, int ny, int nx, int dims, double dx, double cfl, double t,
                     double tf, int it, double gamma, const double* bh) {
    double dt = cfl * (dx / orc_max_wavespeed(sys, prim, ny, nx, dims, gamma, bh));
    return stable_dt_rule(dt, t, tf, it);
}

void orc_rk_source(double* prim, int ny, int nx, int dims, double dx, double dt, double bias, int lim, double gamma,
                   const double* bh) {
    GR S{gamma, BH{bh[0], bh[1], bh[2], bh[3], bh[4]}, dx};
    rk_source(S, prim, ny, nx, dims, dx, dt, bias, lim);
}

// Full solver loop: Solvers/EulerSecondOrderSolver.cpp:102-147 (and the first-order, SR and GR
// twins).  2D uses Strang splitting X(dt/2) Y(dt) X(dt/2); GR wraps it in `subcycles` RK source
// half-steps before and after (Solvers/BlackHoleEulerSecondOrderSolver.cpp:181-218).
// max_steps < 0 runs to t_final; otherwise stops after max_steps.  dts (optional) receives
// each step's dt.  Returns the number of steps; *t_out the final time.
int orc_solve(int sys, double* prim, int ny, int nx, int dims, int order, double dx, double cfl, double tf,
              double bias, int lim, double gamma, int bc, int subcycles, const double* bh, int max_steps,
              double* dts, double* t_out) {
    double t = 0.0;
    int it = 0;
    while (t < tf && (max_steps < 0 || it < max_steps)) {
        double dt = orc_stable_dt(sys, prim, ny, nx, dims, dx, cfl, t, tf, it, gamma, bh);
        if (sys == 2)
            for (int s = 0; s < subcycles; s++) orc_rk_source(prim, ny, nx, dims, dx, 0.5 * (dt / subcycles), 0.0, 1, gamma, bh);
        if (dims == 1) {
            orc_sweep(sys, prim, ny, nx, 1, 0, order, dx, dt, bias, lim, gamma, bc, nullptr, bh);
        } else {
            orc_sweep(sys, prim, ny, nx, 2, 0, order, dx, 0.5 * dt, bias, lim, gamma, bc, nullptr, bh);
            orc_sweep(sys, prim, ny, nx, 2, 1, order, dx, dt, bias, lim, gamma, bc, nullptr, bh);
            orc_sweep(sys, prim, ny, nx, 2, 0, order, dx, 0.5 * dt, bias, lim, gamma, bc, nullptr, bh);
        }
        if (sys == 2)
            for (int s = 0; s < subcycles; s++) orc_rk_source(prim, ny, nx, dims, dx, 0.5 * (dt / subcycles), 0.0, 1, gamma, bh);
        if (dts) dts[it] = dt;
        t = t + dt;
        it += 1;
    }
    if (t_out) *t_out = t;
    return it;
}

// ---------------------------------------------------------------- state-level functions
void orc_cons(int sys, const double* p, double x, double y, double gamma, const double* bh, double h, double* u) {
    if (sys == 0) Newton<double>{gamma}.cons(p, Pt{x, y, 0}, u);
    else if (sys == 1) SR{gamma}.cons(p, Pt{x, y, 0}, u);
    else GR{gamma, BH{bh[0], bh[1], bh[2], bh[3], bh[4]}, h}.cons(p, Pt{x, y, 0}, u);
}
void orc_prim(int sys, const double* u, double x, double y, double gamma, const double* bh, double h, double* p) {
    if (sys == 0) Newton<double>{gamma}.prim(u, Pt{x, y, 0}, p);
    else if (sys == 1) SR{gamma}.prim(u, Pt{x, y, 0}, p);
    else GR{gamma, BH{bh[0], bh[1], bh[2], bh[3], bh[4]}, h}.prim(u, Pt{x, y, 0}, p);
}
void orc_flux(int sys, const double* u, int axis, double x, double y, double gamma, const double* bh, double h, double* f) {
    if (sys == 0) Newton<double>{gamma}.flux(u, axis, Pt{x, y, 0}, f);
    else if (sys == 1) SR{gamma}.flux(u, axis, Pt{x, y, 0}, f);
    else GR{gamma, BH{bh[0], bh[1], bh[2], bh[3], bh[4]}, h}.flux(u, axis, Pt{x, y, 0}, f);
}
void orc_gr_source(const double* u, double x, double y, double h, double gamma, const double* bh, double* s) {
    GR{gamma, BH{bh[0], bh[1], bh[2], bh[3], bh[4]}, h}.source(u, Pt{x, y, 0}, s);
}
double orc_gr_sound_speed(const double* p, double x, double y, double gamma, const double* bh) {
    return GR{gamma, BH{bh[0], bh[1], bh[2], bh[3], bh[4]}, 0.0}.sound_speed(p, Pt{x, y, 0});
}
double orc_limiter(double r, double bias, int lim) { return limiter(r, bias, lim); }
void orc_slope(const double* ul, const double* uc, const double* ur, double bias, int lim, double* s) {
    slope_vector(ul, uc, ur, bias, lim, s);
}
// ---------------------------------------------------------------- per-interface solver functions
// One reference building block per op, applied to n items (in: in_width doubles per item, out: 5
// per item; xyz: the reference's coordinate arguments per item, black-hole system only).  The op
// numbers are the public COSMOS_IF_* values.  Vector forms restate the reference's VectorAlgebra
// compositions in its operation order:
//   0 computeLaxFriedrichsFlux  Solvers/EulerFirstOrderSolver.cpp:3-11   (UL, UR, FL, FR)
//   1 computeRichtmyerFlux      :13-19 (the intermediate state)          (UL, UR, FL, FR)
//   2 computeFORCEFlux          :21-24                                   (LF, RI)
//   3 computeFORCEUpdate        :96-101                                  (U, FL, FR)
//   4 computeFractionalEvolutionVector  Solvers/EulerSolvers.cpp:163-167 (FL, FR; frac)
//   5 computeEvolutionVector    Solvers/EulerSolvers.cpp:169-172         (FL, FR)
// State forms (primitive states in, flux or primitive state out):
//   6/7 computeX/YLaxFriedrichsFlux, 8/9 computeX/YRichtmyerFlux, 10/11 computeX/YFORCEFlux
//       Solvers/EulerFirstOrderSolver.cpp:26-94; SR Solvers/RelativisticEulerFirstOrderSolver.cpp;
//       black hole Solvers/BlackHoleEulerFirstOrderSolver.cpp:3-94 (states at x -/+ dx/2, the
//       Richtmyer state's flux at x)                                   (L, R)
//   12/13 computeX/YSLICFlux  Solvers/EulerSecondOrderSolver.cpp:3-25, SR twin, black hole
//       Solvers/BlackHoleEulerSecondOrderSolver.cpp:3-39                 (LL, L, R, RR)
//   14/15 evolveStateByHalfX/YTimeStep (states; side)  Solvers/EulerSolvers.cpp:190-223, SR
//       Solvers/RelativisticEulerSolvers.cpp:166-199, black hole Solvers/BlackHoleEulerSolvers.cpp:250-307
//                                                                      (l, m, r)
//   16/17 evolveStateByHalfTimeStep (vector form; side)  Solvers/EulerSolvers.cpp:174-188, SR :148-164;
//       black hole evolveStateByHalfX/YTimeStep vector forms Solvers/BlackHoleEulerSolvers.cpp:234-248,
//       :281-295 (the evolved state converted at x -/+ dx/2)           (UL, UR, evolution)
// Black hole only:
//   18/19 evolveStateByFractionalX/YTimeStep  Solvers/BlackHoleEulerSolvers.cpp:171-232 (l, m, r; frac)
//   20 evolveStateByFractionalTimeStep  Solvers/BlackHoleEulerSolvers.cpp:159-169       (U, evolution)
//   21 BlackHoleEulerForcingSolver::evolveConservedVariableVector    :3-70  (conserved l, m, r)
//   22 BlackHoleEulerForcingSolver::evolveConservedVariableVector2D  :72-185 (conserved l, m, r, t, b)
// Returns 0, or -1 for an op this system does not have.
int orc_interface_width(int op, int* in_w) {
    static const int w[23] = {20, 20, 10, 15, 10, 10, 10, 10, 10, 10, 10, 10, 20, 20, 15, 15, 15, 15, 15, 15, 10, 15, 25};
    if (op < 0 || op > 22) return -1;
    *in_w = w[op];
    return 0;
}

}  // extern "C"

template <class Sys>
static int interface_item(const Sys& S, bool gr, int op, const double* a, Pt q, double dx, double dt, double w, int lim,
                          double frac, int side, double* o) {
    const double* b = a + 5;
    const double* c = a + 10;
    const double* d = a + 15;
    const int axis = (op & 1) ? 1 : 0;  // ops 6..19 alternate X (even) and Y (odd)
    switch (op) {
        case 0: { const double r = dx / dt; for (int k = 0; k < 5; k++) o[k] = 0.5 * ((c[k] + d[k]) + (r * (a[k] - b[k]))); return 0; }
        case 1: { const double r = dt / dx; for (int k = 0; k < 5; k++) o[k] = 0.5 * ((a[k] + b[k]) + (r * (c[k] - d[k]))); return 0; }
        case 2: for (int k = 0; k < 5; k++) o[k] = 0.5 * (a[k] + b[k]); return 0;
        case 3: { const double r = dt / dx; for (int k = 0; k < 5; k++) o[k] = a[k] + (r * (b[k] - c[k])); return 0; }
        case 4: case 5: {
            const double r = (op == 4 ? frac : 0.5) * (dt / dx);
            for (int k = 0; k < 5; k++) o[k] = r * (a[k] - b[k]);
            return 0;
        }
        case 6: case 7: case 8: case 9: {
            double uL[5], uR[5], fL[5], fR[5], us[5];
            const Pt pl = shift(q, axis, -(dx * 0.5)), pr = shift(q, axis, dx * 0.5);
            S.cons(a, pl, uL);
            S.cons(b, pr, uR);
            S.flux(uL, axis, pl, fL);
            S.flux(uR, axis, pr, fR);
            if (op <= 7) {
                const double r = dx / dt;
                for (int k = 0; k < 5; k++) o[k] = 0.5 * ((fL[k] + fR[k]) + (r * (uL[k] - uR[k])));
                return 0;
            }
            const double r = dt / dx;
            for (int k = 0; k < 5; k++) us[k] = 0.5 * ((uL[k] + uR[k]) + (r * (fL[k] - fR[k])));
            S.flux(us, axis, q, o);
            return 0;
        }
        case 10: case 11: force_flux(S, a, b, q, axis, dx, dt, o); return 0;
        case 12: case 13: {
            double eR[5], eL[5];
            evolve_half(S, a, b, c, shift(q, axis, -(dx * 0.5)), axis, dx, dt, w, lim, (double*)nullptr, eR);
            evolve_half(S, b, c, d, shift(q, axis, dx * 0.5), axis, dx, dt, w, lim, eL, (double*)nullptr);
            force_flux(S, eR, eL, q, axis, dx, dt, o);
            return 0;
        }
        case 14: case 15:
            evolve_half(S, a, b, c, q, axis, dx, dt, w, lim, side == 0 ? o : nullptr, side == 0 ? nullptr : o);
            return 0;
        case 16: case 17: {
            double u[5];
            const double* x = side == 0 ? a : b;
            for (int k = 0; k < 5; k++) u[k] = x[k] + c[k];
            S.prim(u, gr ? shift(q, axis, side == 0 ? -(dx * 0.5) : dx * 0.5) : q, o);
            return 0;
        }
        default: return -1;
    }
}

extern "C" {

int orc_interface_eval(int op, int sys, size_t n, const double* in, const double* xyz, double gamma, const double* bh,
                       double dx, double dt, double bias, int lim, double frac, int side, double* out) {
    int iw = 0;
    if (orc_interface_width(op, &iw)) return -1;
    for (size_t i = 0; i < n; i++) {
        const double* a = in + iw * i;
        double* o = out + 5 * i;
        Pt q = xyz ? Pt{xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]} : Pt{0.0, 0.0, 0.0};
        int rc;
        if (sys == 0) rc = op > 17 ? -1 : interface_item(Newton<double>{gamma}, false, op, a, q, dx, dt, bias, lim, frac, side, o);
        else if (sys == 1) rc = op > 17 ? -1 : interface_item(SR{gamma}, false, op, a, q, dx, dt, bias, lim, frac, side, o);
        else {
            GR S{gamma, BH{bh[0], bh[1], bh[2], bh[3], bh[4]}, dx};
            if (op <= 17) rc = interface_item(S, true, op, a, q, dx, dt, bias, lim, frac, side, o);
            else if (op <= 19) { evolve_fraction(S, frac, a, a + 5, a + 10, q, op - 18, dx, dt, bias, lim, o); rc = 0; }
            else if (op == 20) {
                double u[5];
                for (int k = 0; k < 5; k++) u[k] = a[k] + a[5 + k];
                S.prim(u, q, o);
                rc = 0;
            } else if (op == 21) { rk_cell(S, 1, a, a + 5, a + 10, a, a, q, dx, dt, bias, lim, o); rc = 0; }
            else { rk_cell(S, 2, a, a + 5, a + 10, a + 15, a + 20, q, dx, dt, bias, lim, o); rc = 0; }
        }
        if (rc) return rc;
    }
    return 0;
}

// metric probe with the same layout as the reference harness's ref_gr_metric
void orc_gr_metric(double x, double y, double z, double h, const double* bhp, double* out) {
    BH b{bhp[0], bhp[1], bhp[2], bhp[3], bhp[4]};
    GR S{5.0 / 3.0, b, h};
    double m[9], g4m[16], gi[16], K[9], da[3], gs[9], L[4];
    b.gamma(x, y, z, m);
    out[0] = det_n(m, 3);
    out[1] = b.lapse(x, y, z);
    b.shiftv(x, y, z, out + 2);
    for (int i = 0; i < 9; i++) out[5 + i] = m[i];
    b.g4(x, y, z, g4m);
    inverse_n(g4m, 4, gi);
    for (int i = 0; i < 16; i++) out[14 + i] = gi[i];
    S.Kij(Pt{x, y, z}, K);
    for (int i = 0; i < 9; i++) out[30 + i] = K[i];
    S.dalpha(Pt{x, y, z}, da);
    for (int i = 0; i < 3; i++) out[39 + i] = da[i];
    out[42] = b.excised(x, y, z) ? 1.0 : 0.0;
    out[43] = b.H(x, y, z);
    b.L4(x, y, z, L);
    for (int i = 0; i < 4; i++) out[44 + i] = L[i];
    inverse_n(m, 3, gs);
    for (int i = 0; i < 9; i++) out[48 + i] = gs[i];
}

// Every public quantity of BlackHoleSpacetime (BlackHoleEuler/BlackHoleSpacetime.hpp:16-42) at one
// point, derivatives with spacing h, in the layout of the public COSMOS_ST_* offsets:
//   0 computeKerrSchildScalar, 1 computeKerrSchildVector (3), 4 computeKerrSchildSpacetimeVector (4),
//   8 computeKerrSchildScalarDerivative (3), 11 computeKerrSchildVectorDerivative ([dir][comp], 9),
//   20 computeSpatialMetricTensor (9), 29 computeSpacetimeMetricTensor (16),
//   45 computeInverseSpatialMetricTensor (9), 54 computeInverseSpacetimeMetricTensor (16),
//   70 computeSpatialMetricDeterminant, 71 computeSpacetimeMetricDeterminant,
//   72 computeSpatialMetricTensorDerivative ([dir][i][j], 27), 99 computeLapseFunction,
//   100 computeShiftVector (3), 103 computeLapseFunctionDerivative (3),
//   106 computeShiftVectorDerivative ([dir][comp], 9), 115 computeExtrinsicCurvatureTensor (9),
//   124 inExcisionRegion (1 or 0).
void orc_spacetime_record(double x, double y, double z, double h, const double* bhp, double* o) {
    BH b{bhp[0], bhp[1], bhp[2], bhp[3], bhp[4]};
    GR S{5.0 / 3.0, b, h};
    const Pt q{x, y, z};
    double m[9], g4m[16];
    o[0] = b.H(x, y, z);
    b.l(x, y, z, o + 1);
    b.L4(x, y, z, o + 4);
    S.dH(q, o + 8);
    S.dl(q, o + 11);
    b.gamma(x, y, z, m);
    for (int i = 0; i < 9; i++) o[20 + i] = m[i];
    b.g4(x, y, z, g4m);
    for (int i = 0; i < 16; i++) o[29 + i] = g4m[i];
    inverse_n(m, 3, o + 45);
    inverse_n(g4m, 4, o + 54);
    o[70] = det_n(m, 3);
    o[71] = det_n(g4m, 4);
    S.dgamma(q, o + 72);
    o[99] = b.lapse(x, y, z);
    b.shiftv(x, y, z, o + 100);
    S.dalpha(q, o + 103);
    S.dbeta(q, o + 106);
    S.Kij(q, o + 115);
    o[124] = b.excised(x, y, z) ? 1.0 : 0.0;
}

// BlackHoleEuler/BlackHoleEulerEigenvalues.cpp:3-96: material (3), fast acoustic (3) and slow
// acoustic (3) eigenvalues of primitives p at (x, y, z)
void orc_gr_eigenvalues(const double* p, double x, double y, double z, double gamma, const double* bhp, double* o) {
    BH b{bhp[0], bhp[1], bhp[2], bhp[3], bhp[4]};
    double al = b.lapse(x, y, z), be[3], gm[9], gs[9];
    b.shiftv(x, y, z, be);
    b.gamma(x, y, z, gm);
    inverse_n(gm, 3, gs);
    const double cs = sr_sound(p[0], p[4], gamma);
    const double v[3] = {p[1], p[2], p[3]};
    double v2 = 0.0;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) v2 = v2 + ((gm[3 * i + j] * v[i]) * v[j]);
    for (int i = 0; i < 3; i++) {
        const double rt = std::sqrt((1.0 - v2) * ((gs[3 * i + i] * (1.0 - (v2 * (cs * cs)))) - ((v[i] * v[i]) * (1.0 - (cs * cs)))));
        const double pre = al / (1.0 - (v2 * (cs * cs)));
        o[i] = (al * v[i]) - be[i];
        o[3 + i] = (pre * ((v[i] * (1.0 - (cs * cs))) + (cs * rt))) - be[i];
        o[6 + i] = (pre * ((v[i] * (1.0 - (cs * cs))) - (cs * rt))) - be[i];
    }
}

// ---------------------------------------------------------------- AMR flagging
// Refinement pass of the Level-1 drivers: AMR/EulerAMR.cpp:207-229 (1D), :394-431 (2D);
// SR twins AMR/RelativisticEulerAMR.cpp (2D bottom neighbour read at [i+2][j+2], :422);
// GR AMR/BlackHoleEulerAMR.cpp:276-300 (1D) and :484-515 (2D, same [i+2][j+2] and its
// coordinates ((j+1)dx, (i+1)dx)).  Transmissive 1-ghost neighbours.  A cell whose
// one-sided conserved gradient |dU/dx| reaches tol in any component gets coarse=0 and its
// 2 (1D) or 4 (2D) fine children fine=1; other flags are left as they are.
void orc_amr_flags(int sys, const double* prim, int ny, int nx, int dims, double dx, double tol, double gamma,
                   const double* bh, unsigned char* coarse, unsigned char* fine) {
    if (dims == 1) ny = 1;
    GR G{gamma, bh ? BH{bh[0], bh[1], bh[2], bh[3], bh[4]} : BH{1, 0, 0, 0, 0}, dx};
    auto cons = [&](int i, int j, Pt q, double* u) {
        const double* p = prim + 5 * ((size_t)ghost(i, ny, 0) * nx + ghost(j, nx, 0));
        if (sys == 0) Newton<double>{gamma}.cons(p, q, u);
        else if (sys == 1) SR{gamma}.cons(p, q, u);
        else G.cons(p, q, u);
    };
    for (int i = 0; i < ny; i++)
        for (int j = 0; j < nx; j++) {
            double c[5], l[5], r[5], t[5], b[5];
            bool hit = false;
            if (dims == 1) {
                cons(0, j - 1, Pt{(j - 1) * dx, 0.0, 0.0}, l);
                cons(0, j, Pt{j * dx, 0.0, 0.0}, c);
                cons(0, j + 1, Pt{(j + 1) * dx, 0.0, 0.0}, r);
                for (int k = 0; k < 5; k++)
                    if (std::fabs((c[k] - l[k]) / dx) >= tol || std::fabs((r[k] - c[k]) / dx) >= tol) hit = true;
            } else {
                cons(i - 1, j, Pt{j * dx, (i - 1) * dx, 0.0}, t);
                cons(i, j - 1, Pt{(j - 1) * dx, i * dx, 0.0}, l);
                cons(i, j, Pt{j * dx, i * dx, 0.0}, c);
                cons(i, j + 1, Pt{(j + 1) * dx, i * dx, 0.0}, r);
                if (sys == 0) cons(i + 1, j, Pt{j * dx, (i + 1) * dx, 0.0}, b);
                else if (i == ny - 1 && j == nx - 1) {
                    // the diagonal read lands on the bottom-right corner ghost, which
                    // insertBoundaryCells2D never fills (Solvers/EulerSolvers.cpp:30-85): it keeps
                    // the default-constructed state (1, 0, 0, 0, 1)
                    // (RelativisticEuler/RelativisticEulerStateVector.cpp:3-10)
                    const double dflt[5] = {1.0, 0.0, 0.0, 0.0, 1.0};
                    Pt q{(j + 1) * dx, (i + 1) * dx, 0.0};
                    if (sys == 1) SR{gamma}.cons(dflt, q, b); else G.cons(dflt, q, b);
                } else cons(i + 1, j + 1, Pt{(j + 1) * dx, (i + 1) * dx, 0.0}, b);
                for (int k = 0; k < 5; k++)
                    if (std::fabs((c[k] - t[k]) / dx) >= tol || std::fabs((b[k] - c[k]) / dx) >= tol ||
                        std::fabs((c[k] - l[k]) / dx) >= tol || std::fabs((r[k] - c[k]) / dx) >= tol)
                        hit = true;
            }
            if (!hit) continue;
            if (dims == 1) {
                coarse[j] = 0;
                fine[2 * j] = 1; fine[2 * j + 1] = 1;
            } else {
                coarse[(size_t)i * nx + j] = 0;
                size_t fw = 2 * (size_t)nx;
                fine[(2 * i) * fw + 2 * j] = 1; fine[(2 * i) * fw + 2 * j + 1] = 1;
                fine[(2 * i + 1) * fw + 2 * j] = 1; fine[(2 * i + 1) * fw + 2 * j + 1] = 1;
            }
        }
}

// Derefinement pass: AMR/EulerAMR.cpp:310-345 (1D) and :538-586 (2D).  Tests the fine grid
// (1-ghost transmissive) with the coarse dx at tol/2; where no component reaches it and the
// first fine child is flagged, the children are unflagged, the coarse cell flagged and the
// coarse state restricted from the children's conserved average.  The Newtonian neighbour
// pattern is used for every system (the SR/GR 2D derefinement passes read the same cells).
void orc_amr_derefine(int sys, double* coarse_prim, const double* fine_prim, int ny, int nx, int dims, double dx,
                      double tol, double gamma, const double* bh, unsigned char* coarse, unsigned char* fine) {
    if (dims == 1) ny = 1;
    const int fny = dims == 1 ? 1 : 2 * ny, fnx = 2 * nx;
    GR G{gamma, bh ? BH{bh[0], bh[1], bh[2], bh[3], bh[4]} : BH{1, 0, 0, 0, 0}, dx};
    auto consf = [&](int i, int j, Pt q, double* u) {
        const double* p = fine_prim + 5 * ((size_t)ghost(i, fny, 0) * fnx + ghost(j, fnx, 0));
        if (sys == 0) Newton<double>{gamma}.cons(p, q, u);
        else if (sys == 1) SR{gamma}.cons(p, q, u);
        else G.cons(p, q, u);
    };
    auto prim_of = [&](const double* u, Pt q, double* p) {
        if (sys == 0) Newton<double>{gamma}.prim(u, q, p);
        else if (sys == 1) SR{gamma}.prim(u, q, p);
        else G.prim(u, q, p);
    };
    const double half = tol * 0.5;
    for (int i = 0; i < ny; i++)
        for (int j = 0; j < nx; j++) {
            bool marked = false;
            double c[5], l[5], r[5], t[5], b[5];
            if (dims == 1) {
                // GR, AMR/BlackHoleEulerAMR.cpp:388-393: fine cells 2j, 2j+1, 2j+2 evaluated at
                // fine coordinates (2j-1), 2j, (2j+1) times dx/2 (shifted by one, as written)
                double fdx = dx * 0.5;
                consf(0, 2 * j, Pt{((j * 2) - 1) * fdx, 0.0, 0.0}, l);
                consf(0, 2 * j + 1, Pt{(j * 2) * fdx, 0.0, 0.0}, c);
                consf(0, 2 * j + 2, Pt{((j * 2) + 1) * fdx, 0.0, 0.0}, r);
                for (int k = 0; k < 5; k++)
                    if (std::fabs((c[k] - l[k]) / dx) >= half || std::fabs((r[k] - c[k]) / dx) >= half) marked = true;
                if (!marked && fine[2 * j]) {
                    fine[2 * j] = 0; fine[2 * j + 1] = 0; coarse[j] = 1;
                    double a[5], bb[5], avg[5];
                    consf(0, 2 * j, Pt{(2 * j) * fdx, 0.0, 0.0}, a);
                    consf(0, 2 * j + 1, Pt{(2 * j + 1) * fdx, 0.0, 0.0}, bb);
                    for (int k = 0; k < 5; k++) avg[k] = 0.5 * (a[k] + bb[k]);
                    prim_of(avg, Pt{j * dx, 0.0, 0.0}, coarse_prim + 5 * j);
                }
            } else {
                double fdx = dx * 0.5;
                consf(2 * i, 2 * j + 1, Pt{(2 * j + 1) * fdx, (2 * i) * fdx, 0.0}, t);
                consf(2 * i + 1, 2 * j, Pt{(2 * j) * fdx, (2 * i + 1) * fdx, 0.0}, l);
                consf(2 * i + 1, 2 * j + 1, Pt{(2 * j + 1) * fdx, (2 * i + 1) * fdx, 0.0}, c);
                consf(2 * i + 1, 2 * j + 2, Pt{(2 * j + 2) * fdx, (2 * i + 1) * fdx, 0.0}, r);
                consf(2 * i + 2, 2 * j + 1, Pt{(2 * j + 1) * fdx, (2 * i + 2) * fdx, 0.0}, b);
                for (int k = 0; k < 5; k++)
                    if (std::fabs((c[k] - t[k]) / dx) >= half || std::fabs((b[k] - c[k]) / dx) >= half ||
                        std::fabs((c[k] - l[k]) / dx) >= half || std::fabs((r[k] - c[k]) / dx) >= half)
                        marked = true;
                size_t fw = (size_t)fnx;
                if (!marked && fine[(2 * i) * fw + 2 * j]) {
                    fine[(2 * i) * fw + 2 * j] = 0; fine[(2 * i) * fw + 2 * j + 1] = 0;
                    fine[(2 * i + 1) * fw + 2 * j] = 0; fine[(2 * i + 1) * fw + 2 * j + 1] = 0;
                    coarse[(size_t)i * nx + j] = 1;
                    double a[5], bb[5], cc[5], dd[5], avg[5];
                    consf(2 * i, 2 * j, Pt{(2 * j) * fdx, (2 * i) * fdx, 0.0}, a);
                    consf(2 * i, 2 * j + 1, Pt{(2 * j + 1) * fdx, (2 * i) * fdx, 0.0}, bb);
                    consf(2 * i + 1, 2 * j, Pt{(2 * j) * fdx, (2 * i + 1) * fdx, 0.0}, cc);
                    consf(2 * i + 1, 2 * j + 1, Pt{(2 * j + 1) * fdx, (2 * i + 1) * fdx, 0.0}, dd);
                    for (int k = 0; k < 5; k++) avg[k] = 0.25 * (((a[k] + bb[k]) + cc[k]) + dd[k]);
                    prim_of(avg, Pt{j * dx, i * dx, 0.0}, coarse_prim + 5 * ((size_t)i * nx + j));
                }
            }
        }
}

// ---------------------------------------------------------------- AMR Level-1 driver
// EulerAMR::solveLevel1AMR (AMR/EulerAMR.cpp:169-350) and solve2DLevel1AMR (:352-592); the SR
// drivers (AMR/RelativisticEulerAMR.cpp) are the same loop with the SR state (their only other
// difference, the 2D flag pass's bottom neighbour, is inside orc_amr_flags).  Per coarse step:
// dt from the coarse grid with the TOTAL fine iteration count (:197-198); flag pass (:200-229);
// masked coarse step with bias 0 and limiter 1 (:231-239); while any fine flag is set, fine steps
// of dx/2 until the fine time passes (t + dt) - 1e-4, each dt from the whole fine grid (:253-277);
// otherwise the fine count still advances (:279-282); restriction of flagged-off coarse cells and
// injection into unflagged fine cells (:287-307); derefinement (:309-345).  coarse/fine receive
// the final primitive grids, cflags/fflags the final flags; *fine_steps the fine step count (the
// reference's fineTotalIteration), *fine_run the fine steps actually taken (optional).  Returns
// the number of coarse steps.
int orc_amr_level1(int sys, const double* prim, int ny, int nx, int dims, double dx, double cfl, double tf,
                   double tol, int order, double gamma, double* coarse, double* fine, unsigned char* cflags,
                   unsigned char* fflags, int* fine_steps, int* fine_run) {
    if (dims == 1) ny = 1;
    const int fny = dims == 1 ? 1 : 2 * ny, fnx = 2 * nx;
    const size_t nc = (size_t)ny * nx;
    auto kids = [&](int i, int j, size_t* k) -> int {
        if (dims == 1) { k[0] = 2 * (size_t)j; k[1] = 2 * (size_t)j + 1; return 2; }
        const size_t fw = (size_t)fnx;
        k[0] = (2 * (size_t)i) * fw + 2 * j; k[1] = k[0] + 1;
        k[2] = (2 * (size_t)i + 1) * fw + 2 * j; k[3] = k[2] + 1;
        return 4;
    };
    auto cons_of = [&](const double* p, double* u) {
        if (sys == 0) Newton<double>{gamma}.cons(p, Pt{0, 0, 0}, u); else SR{gamma}.cons(p, Pt{0, 0, 0}, u);
    };
    auto prim_of = [&](const double* u, double* p) {
        if (sys == 0) Newton<double>{gamma}.prim(u, Pt{0, 0, 0}, p); else SR{gamma}.prim(u, Pt{0, 0, 0}, p);
    };
    std::memcpy(coarse, prim, nc * 5 * sizeof(double));
    for (int i = 0; i < ny; i++)
        for (int j = 0; j < nx; j++) {
            size_t k[4];
            const int nk = kids(i, j, k);
            cflags[(size_t)i * nx + j] = 1;
            for (int q = 0; q < nk; q++) {
                fflags[k[q]] = 0;
                std::memcpy(fine + 5 * k[q], coarse + 5 * ((size_t)i * nx + j), 5 * sizeof(double));
            }
        }
    auto step = [&](double* p, int gy, int gx, double h, double dt, const unsigned char* m) {
        if (dims == 1) {
            orc_sweep(sys, p, 1, gx, 1, 0, order, h, dt, 0.0, 1, gamma, 0, m, nullptr);
        } else {
            orc_sweep(sys, p, gy, gx, 2, 0, order, h, dt * 0.5, 0.0, 1, gamma, 0, m, nullptr);
            orc_sweep(sys, p, gy, gx, 2, 1, order, h, dt, 0.0, 1, gamma, 0, m, nullptr);
            orc_sweep(sys, p, gy, gx, 2, 0, order, h, dt * 0.5, 0.0, 1, gamma, 0, m, nullptr);
        }
    };
    double t = 0.0;
    int it = 0, fit = 0, run = 0;
    while (t < tf) {
        const double dt = orc_stable_dt(sys, coarse, ny, nx, dims, dx, cfl, t, tf, fit, gamma, nullptr);
        orc_amr_flags(sys, coarse, ny, nx, dims, dx, tol, gamma, nullptr, cflags, fflags);
        step(coarse, ny, nx, dx, dt, cflags);
        bool refined = false;
        for (size_t q = 0; q < (size_t)fny * fnx; q++) refined = refined || fflags[q];
        if (refined) {
            double ft = t;
            while (ft < (t + dt - 1e-4)) {
                const double fdt = orc_stable_dt(sys, fine, fny, fnx, dims, dx * 0.5, cfl, ft, t + dt, fit, gamma, nullptr);
                step(fine, fny, fnx, dx * 0.5, fdt, fflags);
                ft += fdt;
                fit += 1;
                run += 1;
            }
        } else {
            fit += 1;
        }
        t += dt;
        it += 1;
        for (int i = 0; i < ny; i++)
            for (int j = 0; j < nx; j++) {
                size_t k[4];
                const int nk = kids(i, j, k);
                double* cp = coarse + 5 * ((size_t)i * nx + j);
                if (!cflags[(size_t)i * nx + j]) {
                    double u[4][5], avg[5];
                    for (int q = 0; q < nk; q++) cons_of(fine + 5 * k[q], u[q]);
                    for (int f = 0; f < 5; f++)
                        avg[f] = nk == 2 ? 0.5 * (u[0][f] + u[1][f]) : 0.25 * (((u[0][f] + u[1][f]) + u[2][f]) + u[3][f]);
                    prim_of(avg, cp);
                }
                for (int q = 0; q < nk; q++)
                    if (!fflags[k[q]]) std::memcpy(fine + 5 * k[q], cp, 5 * sizeof(double));
            }
        orc_amr_derefine(sys, coarse, fine, ny, nx, dims, dx, tol, gamma, nullptr, cflags, fflags);
    }
    if (fine_steps) *fine_steps = fit;
    if (fine_run) *fine_run = run;
    return it;
}

// ---------------------------------------------------------------- AMR Level-2 driver
// Pieces of the Level-2 drivers (Newtonian and SR), on primitive grids of gny x gnx cells (1D: gny = 1).
namespace amr2 {

struct Sys2 {
    int sys;
    double gamma;
    void cons(const double* p, double* u) const {
        if (sys == 0) Newton<double>{gamma}.cons(p, Pt{0, 0, 0}, u); else SR{gamma}.cons(p, Pt{0, 0, 0}, u);
    }
    void prim(const double* u, double* p) const {
        if (sys == 0) Newton<double>{gamma}.prim(u, Pt{0, 0, 0}, p); else SR{gamma}.prim(u, Pt{0, 0, 0}, p);
    }
};

// The drivers' gradient test of cell (ci, cj) against its 1-ghost transmissive neighbours:
// |dU/dx| >= thr for any component on any side (top, bottom, left, right; 1D left, right).
static bool hit(const Sys2& S, const double* g, int gny, int gnx, int dims, int ci, int cj, double dx, double thr) {
    auto at = [&](int i, int j, double* u) { S.cons(g + 5 * ((size_t)ghost(i, gny, 0) * gnx + ghost(j, gnx, 0)), u); };
    double c[5], l[5], r[5], t[5], b[5];
    at(ci, cj, c);
    at(ci, cj - 1, l);
    at(ci, cj + 1, r);
    if (dims == 2) { at(ci - 1, cj, t); at(ci + 1, cj, b); }
    for (int k = 0; k < 5; k++) {
        if (std::fabs((c[k] - l[k]) / dx) >= thr || std::fabs((r[k] - c[k]) / dx) >= thr) return true;
        if (dims == 2 && (std::fabs((c[k] - t[k]) / dx) >= thr || std::fabs((b[k] - c[k]) / dx) >= thr)) return true;
    }
    return false;
}

// Children of parent cell (i, j) on a grid of child width cnx: 2 in 1D, 4 in 2D (tl, tr, bl, br).
static int kids(int dims, int i, int j, int cnx, size_t* k) {
    if (dims == 1) { k[0] = 2 * (size_t)j; k[1] = k[0] + 1; return 2; }
    k[0] = (2 * (size_t)i) * cnx + 2 * j; k[1] = k[0] + 1;
    k[2] = (2 * (size_t)i + 1) * cnx + 2 * j; k[3] = k[2] + 1;
    return 4;
}

static void restrict_into(const Sys2& S, const double* child, const size_t* k, int nk, double* parent) {
    double u[4][5], avg[5];
    for (int q = 0; q < nk; q++) S.cons(child + 5 * k[q], u[q]);
    for (int f = 0; f < 5; f++)
        avg[f] = nk == 2 ? 0.5 * (u[0][f] + u[1][f]) : 0.25 * (((u[0][f] + u[1][f]) + u[2][f]) + u[3][f]);
    S.prim(avg, parent);
}

// Refinement flags: a parent cell that passes the gradient test (and, with need_on, is itself on)
// is switched off and its children on.
static void flag(const Sys2& S, const double* g, int gny, int gnx, int dims, double dx, double thr, bool need_on,
                 unsigned char* pf, unsigned char* cf) {
    for (int i = 0; i < gny; i++)
        for (int j = 0; j < gnx; j++) {
            unsigned char& on = pf[(size_t)i * gnx + j];
            if (need_on && !on) continue;
            if (!hit(S, g, gny, gnx, dims, i, j, dx, thr)) continue;
            on = 0;
            size_t k[4];
            const int nk = kids(dims, i, j, 2 * gnx, k);
            for (int q = 0; q < nk; q++) cf[k[q]] = 1;
        }
}

// Level exchange: restriction into an off parent (strict: only when every child is on), then
// injection into each off child (strict: only when the parent is on).
static void exchange(const Sys2& S, double* parent, double* child, int gny, int gnx, int dims, const unsigned char* pf,
                     const unsigned char* cf, bool strict) {
    for (int i = 0; i < gny; i++)
        for (int j = 0; j < gnx; j++) {
            size_t k[4];
            const int nk = kids(dims, i, j, 2 * gnx, k);
            const size_t pc = (size_t)i * gnx + j;
            bool all = true;
            for (int q = 0; q < nk; q++) all = all && cf[k[q]];
            if (!pf[pc] && (!strict || all)) restrict_into(S, child, k, nk, parent + 5 * pc);
            for (int q = 0; q < nk; q++)
                if (!cf[k[q]] && (!strict || pf[pc])) std::memcpy(child + 5 * k[q], parent + 5 * pc, 5 * sizeof(double));
        }
}

// Derefinement: the child-grid gradient test at cell (2i+1, 2j+1) (1D 2j+1) with divisor dx and
// threshold thr; where nothing is marked and the children are on (strict: all of them; else the
// first), the children go off, the parent on, and the parent is restricted from its children.
static void derefine(const Sys2& S, double* parent, const double* child, int gny, int gnx, int dims, double dx,
                     double thr, bool strict, unsigned char* pf, unsigned char* cf) {
    const int cny = dims == 1 ? 1 : 2 * gny, cnx = 2 * gnx;
    for (int i = 0; i < gny; i++)
        for (int j = 0; j < gnx; j++) {
            const bool marked = hit(S, child, cny, cnx, dims, dims == 1 ? 0 : 2 * i + 1, 2 * j + 1, dx, thr);
            size_t k[4];
            const int nk = kids(dims, i, j, cnx, k);
            bool on = cf[k[0]] != 0;
            if (strict)
                for (int q = 1; q < nk; q++) on = on && cf[k[q]];
            if (marked || !on) continue;
            for (int q = 0; q < nk; q++) cf[k[q]] = 0;
            pf[(size_t)i * gnx + j] = 1;
            restrict_into(S, child, k, nk, parent + 5 * ((size_t)i * gnx + j));
        }
}

}  // namespace amr2

// EulerAMR::solveLevel2AMR (AMR/EulerAMR.cpp:593-917) and solve2DLevel2AMR (:918-1379); the SR
// drivers (AMR/RelativisticEulerAMR.cpp:604-1392) are the same code with the SR state, including the
// coarse flag pass's bottom neighbour [i+2][j+1] (:1008; the Level-1 SR driver reads [i+2][j+2]).
// Three levels (coarse; intermediate at dx/2; fine at dx/4), each with flags.  Per coarse step: dt
// (total fine count), coarse flags (tol), masked coarse step; while the intermediate level has a
// flag on: intermediate dt, intermediate flags (tol * 2 * order with the coarse dx, only on cells
// that are on), masked intermediate step, fine sub-steps while a fine flag is on (the total fine
// count advances per fine step, or once when none runs), then once more per intermediate step;
// strict exchange and derefinement (tol, coarse dx) between intermediate and fine; after the coarse
// step: exchange and derefinement (tol * 0.5 / order) between coarse and intermediate.
// counts (optional): [0] total fine count, [1] intermediate steps taken, [2] fine steps taken.
int orc_amr_level2(int sys, const double* prim, int ny, int nx, int dims, double dx, double cfl, double tf,
                   double tol, int order, double gamma, double* coarse, double* mid, double* fine, unsigned char* cflags,
                   unsigned char* mflags, unsigned char* fflags, int* counts) {
    if (dims == 1) ny = 1;
    const amr2::Sys2 S{sys, gamma};
    const int mny = dims == 1 ? 1 : 2 * ny, mnx = 2 * nx, fny = dims == 1 ? 1 : 4 * ny, fnx = 4 * nx;
    const size_t nc = (size_t)ny * nx, nm = (size_t)mny * mnx, nf = (size_t)fny * fnx;
    std::memcpy(coarse, prim, nc * 5 * sizeof(double));
    std::memset(cflags, 1, nc);
    std::memset(mflags, 0, nm);
    std::memset(fflags, 0, nf);
    for (int i = 0; i < mny; i++)
        for (int j = 0; j < mnx; j++)
            std::memcpy(mid + 5 * ((size_t)i * mnx + j), coarse + 5 * ((size_t)(i / 2) * nx + j / 2), 5 * sizeof(double));
    for (int i = 0; i < fny; i++)
        for (int j = 0; j < fnx; j++)
            std::memcpy(fine + 5 * ((size_t)i * fnx + j), coarse + 5 * ((size_t)(i / 4) * nx + j / 4), 5 * sizeof(double));
    auto step = [&](double* p, int gy, int gx, double h, double dt, const unsigned char* m) {
        if (dims == 1) {
            orc_sweep(sys, p, 1, gx, 1, 0, order, h, dt, 0.0, 1, gamma, 0, m, nullptr);
        } else {
            orc_sweep(sys, p, gy, gx, 2, 0, order, h, dt * 0.5, 0.0, 1, gamma, 0, m, nullptr);
            orc_sweep(sys, p, gy, gx, 2, 1, order, h, dt, 0.0, 1, gamma, 0, m, nullptr);
            orc_sweep(sys, p, gy, gx, 2, 0, order, h, dt * 0.5, 0.0, 1, gamma, 0, m, nullptr);
        }
    };
    auto any = [](const unsigned char* f, size_t n) {
        for (size_t q = 0; q < n; q++)
            if (f[q]) return true;
        return false;
    };
    double t = 0.0;
    int it = 0, fit = 0, mrun = 0, frun = 0;
    while (t < tf) {
        const double dt = orc_stable_dt(sys, coarse, ny, nx, dims, dx, cfl, t, tf, fit, gamma, nullptr);
        amr2::flag(S, coarse, ny, nx, dims, dx, tol, false, cflags, mflags);
        step(coarse, ny, nx, dx, dt, cflags);
        if (any(mflags, nm)) {
            double mt = t;
            while (mt < (t + dt - 1e-4)) {
                const double mdt = orc_stable_dt(sys, mid, mny, mnx, dims, dx * 0.5, cfl, mt, t + dt, fit, gamma, nullptr);
                amr2::flag(S, mid, mny, mnx, dims, dx, tol * 2.0 * order, true, mflags, fflags);
                step(mid, mny, mnx, dx * 0.5, mdt, mflags);
                if (any(fflags, nf)) {
                    double ft = mt;
                    while (ft < (mt + mdt - 1e-4)) {
                        const double fdt = orc_stable_dt(sys, fine, fny, fnx, dims, dx * 0.25, cfl, ft, mt + mdt, fit, gamma,
                                                         nullptr);
                        step(fine, fny, fnx, dx * 0.25, fdt, fflags);
                        ft += fdt;
                        fit += 1;
                        frun += 1;
                    }
                } else {
                    fit += 1;
                }
                mt += mdt;
                fit += 1;
                mrun += 1;
                amr2::exchange(S, mid, fine, mny, mnx, dims, mflags, fflags, true);
                amr2::derefine(S, mid, fine, mny, mnx, dims, dx, tol, true, mflags, fflags);
            }
        } else {
            fit += 1;
        }
        t += dt;
        it += 1;
        amr2::exchange(S, coarse, mid, ny, nx, dims, cflags, mflags, false);
        amr2::derefine(S, coarse, mid, ny, nx, dims, dx, tol * 0.5 * (1.0 / order), true, cflags, mflags);
    }
    if (counts) { counts[0] = fit; counts[1] = mrun; counts[2] = frun; }
    return it;
}

// ---------------------------------------------------------------- tangent-linear (Newtonian)
// Directional derivative of the SLIC loss L = 1/2 sum_cells (rho_T - rho_target)^2 after
// `nsteps` steps with the step sizes dts[] held fixed (the adjoint's convention), along the
// initial-state direction dprim (primitive variables).  Runs the FP64 forward in dual numbers.
// Strang splitting for 2D.  Returns L; *dL receives the directional derivative.
}  // extern "C"
template <class Sys>
static double tlm_run(const Sys& S, const double* prim0, const double* dprim, const double* target, int ny, int nx,
                      int dims, double dx, const double* dts, int nsteps, double bias, int lim, int bc, double* dL,
                      const BH* exc = nullptr, int subcycles = 0) {
    size_t N = (size_t)(dims == 1 ? 1 : ny) * nx;
    std::vector<Dual> p(5 * N);
    for (size_t i = 0; i < 5 * N; i++) p[i] = Dual(prim0[i], dprim ? dprim[i] : 0.0);
    for (int s = 0; s < nsteps; s++) {
        double dt = dts[s];
        // black hole: `subcycles` RK source half-steps (bias 0, limiter 1) around the flux step
        auto source_steps = [&]() {
            if constexpr (Sys::coords)
                for (int c = 0; c < subcycles; c++) rk_source(S, p.data(), ny, nx, dims, dx, 0.5 * (dt / subcycles), 0.0, 1);
        };
        source_steps();
        if (dims == 1) sweep(S, p.data(), ny, nx, 1, 0, 2, dx, dt, bias, lim, bc, nullptr, exc);
        else {
            sweep(S, p.data(), ny, nx, 2, 0, 2, dx, 0.5 * dt, bias, lim, bc, nullptr, exc);
            sweep(S, p.data(), ny, nx, 2, 1, 2, dx, dt, bias, lim, bc, nullptr, exc);
            sweep(S, p.data(), ny, nx, 2, 0, 2, dx, 0.5 * dt, bias, lim, bc, nullptr, exc);
        }
        source_steps();
    }
    Dual L(0.0);
    for (size_t c = 0; c < N; c++) {
        Dual e = p[5 * c] - Dual(target[c]);
        L = L + (Dual(0.5) * (e * e));
    }
    if (dL) *dL = L.d;
    return L.v;
}
extern "C" {

double orc_tlm_newton(const double* prim0, const double* dprim, const double* target, int ny, int nx, int dims,
                      double dx, const double* dts, int nsteps, double bias, int lim, double gamma, int bc,
                      double* dL) {
    return tlm_run(Newton<Dual>{gamma}, prim0, dprim, target, ny, nx, dims, dx, dts, nsteps, bias, lim, bc, dL);
}

// The same for the special-relativistic system (RelativisticEulerSecondOrderSolver's step,
// Solvers/RelativisticEulerSecondOrderSolver.cpp:102-156): every primitive recovery runs its
// Newton iteration on dual numbers, whose derivative part converges with the iterates to the
// implicit-function derivative of the recovered primitives.
double orc_tlm_sr(const double* prim0, const double* dprim, const double* target, int ny, int nx, int dims, double dx,
                  const double* dts, int nsteps, double bias, int lim, double gamma, int bc, double* dL) {
    return tlm_run(SRT<Dual>{gamma}, prim0, dprim, target, ny, nx, dims, dx, dts, nsteps, bias, lim, bc, dL);
}

// The same for the black-hole step (BlackHoleEulerSecondOrderSolver's step,
// Solvers/BlackHoleEulerSecondOrderSolver.cpp:181-218): `subcycles` RK source half-steps
// (Solvers/BlackHoleEulerForcingSolver.cpp:3-250, the source term of
// BlackHoleEulerStateVector.cpp:359-510 in dual numbers) before and after the flux step; 0 gives
// the flux step alone.  The metric and its derivatives enter as FP64 data, cells whose stencil
// touches the excision region keep their state (derivative carried through unchanged),
// transmissive boundaries.  bh = {M, a, x, y, z}.
double orc_tlm_gr(const double* prim0, const double* dprim, const double* target, int ny, int nx, int dims, double dx,
                  const double* dts, int nsteps, double bias, int lim, double gamma, const double* bh, int subcycles,
                  double* dL) {
    GRT<Dual> S{gamma, BH{bh[0], bh[1], bh[2], bh[3], bh[4]}, dx};
    return tlm_run(S, prim0, dprim, target, ny, nx, dims, dx, dts, nsteps, bias, lim, 0, dL, &S.bh, subcycles);
}

}  // extern "C"
