// Adjoint (vector-Jacobian product) of one relativistic SLIC sweep, FP64, gather form: the
// special-relativistic sweep and the black-hole flux sweep (excision); and of one black-hole RK
// source step (rk_cell_adjoint, at the end).
//
// Forward map of a sweep along a line of n cells (primitive states P, dt and dx fixed):
//   SR  (Solvers/RelativisticEulerSecondOrderSolver.cpp:3-100, the half-step evolution of
//        Solvers/RelativisticEulerSolvers.cpp:148-199): A_k, B_k = the left- and right-face
//        primitives of cell k's half-step evolution from P_{k-1..k+1};  F_f = FORCE(B_{f-1}, A_f)
//   GR  (Solvers/BlackHoleEulerSecondOrderSolver.cpp:3-179, Solvers/BlackHoleEulerSolvers.cpp:234-307):
//        face f at x_f = (f - 1/2) dx gets F_f = FORCE(B, A) with B the right face of the evolution
//        of P_{f-2..f} centred at x_f - dx/2 and A the left face of that of P_{f-1..f+1} centred at
//        x_f + dx/2, every state converted with the Kerr-Schild metric at its own point
//   P'_k = prim(cons(P_k) + (dt/dx) (F_k - F_{k+1})), or P'_k = P_k for a black-hole cell whose
//   stencil touches the excision region;
// with the FORCE flux of Solvers/EulerFirstOrderSolver.cpp:3-59 (BlackHoleEulerFirstOrderSolver.cpp:3-47),
// the state functions of RelativisticEulerStateVector.cpp and BlackHoleEulerStateVector.cpp, and
// the slope limiters of Solvers/SlopeLimiters.cpp:3-101.  So P'_k depends on P_{k-2} .. P_{k+2},
// where positions outside the line read the interior cell they copy (transmissive mirror or
// periodic wrap).  Given the adjoint Pbar' of the output, the adjoint of input cell j is
//   Pbar_j = sum over the outputs k whose five-cell window holds j of (dP'_k / dP_j)^T Pbar'_k.
// One thread owns one input cell: it evaluates the window of each such k in dual numbers whose
// five tangent lanes are seeded on cell j's primitives, so the derivative is that of the arithmetic
// the forward runs -- every primitive recovery's Newton iteration, the limiter branch taken, the
// 1e-5 clamp and the floors (derivative 0) -- and no two threads write the same cell.
//
// Host and device code: the same cell function runs in the kernel and in host builds.
#pragma once
#include <cmath>
#include <cstddef>

#ifdef __CUDACC__
#define RADJ_HD __host__ __device__ inline
#else
#define RADJ_HD inline
#endif

namespace cg {
namespace radj {

// ---- dual numbers: value and five tangent lanes; comparisons act on values
struct D5 {
    double v, d[5];
    RADJ_HD D5() : v(0.0), d{0.0, 0.0, 0.0, 0.0, 0.0} {}
    RADJ_HD D5(double x) : v(x), d{0.0, 0.0, 0.0, 0.0, 0.0} {}
};
RADJ_HD D5 operator+(const D5& a, const D5& b) {
    D5 r(a.v + b.v);
    for (int i = 0; i < 5; i++) r.d[i] = a.d[i] + b.d[i];
    return r;
}
RADJ_HD D5 operator-(const D5& a, const D5& b) {
    D5 r(a.v - b.v);
    for (int i = 0; i < 5; i++) r.d[i] = a.d[i] - b.d[i];
    return r;
}
RADJ_HD D5 operator-(const D5& a) {
    D5 r(-a.v);
    for (int i = 0; i < 5; i++) r.d[i] = -a.d[i];
    return r;
}
RADJ_HD D5 operator*(const D5& a, const D5& b) {
    D5 r(a.v * b.v);
    for (int i = 0; i < 5; i++) r.d[i] = (a.d[i] * b.v) + (a.v * b.d[i]);
    return r;
}
// The value part of a quotient is the IEEE quotient (the forward's arithmetic); the tangents take
// one reciprocal instead of five divisions (an FP64 division is a long instruction sequence).
RADJ_HD D5 operator/(const D5& a, const D5& b) {
    D5 r(a.v / b.v);
    const double ib = 1.0 / b.v;
    for (int i = 0; i < 5; i++) r.d[i] = (a.d[i] - (r.v * b.d[i])) * ib;
    return r;
}
RADJ_HD D5 sqrt(const D5& a) {
    D5 r(::sqrt(a.v));
    const double ih = 1.0 / (2.0 * r.v);
    for (int i = 0; i < 5; i++) r.d[i] = a.d[i] * ih;
    return r;
}
// A constant operand (no tangents): the product and sum of the dual forms without the zero lanes.
RADJ_HD D5 operator*(double a, const D5& b) {
    D5 r(a * b.v);
    for (int i = 0; i < 5; i++) r.d[i] = a * b.d[i];
    return r;
}
RADJ_HD D5 operator*(const D5& a, double b) {
    D5 r(a.v * b);
    for (int i = 0; i < 5; i++) r.d[i] = a.d[i] * b;
    return r;
}
RADJ_HD D5 operator+(double a, const D5& b) {
    D5 r(a + b.v);
    for (int i = 0; i < 5; i++) r.d[i] = b.d[i];
    return r;
}
RADJ_HD D5 operator+(const D5& a, double b) {
    D5 r(a.v + b);
    for (int i = 0; i < 5; i++) r.d[i] = a.d[i];
    return r;
}
RADJ_HD D5 operator-(const D5& a, double b) {
    D5 r(a.v - b);
    for (int i = 0; i < 5; i++) r.d[i] = a.d[i];
    return r;
}
RADJ_HD D5 operator-(double a, const D5& b) {
    D5 r(a - b.v);
    for (int i = 0; i < 5; i++) r.d[i] = -b.d[i];
    return r;
}
RADJ_HD D5 operator/(double a, const D5& b) {
    D5 r(a / b.v);
    const double ib = 1.0 / b.v;
    for (int i = 0; i < 5; i++) r.d[i] = -(r.v * b.d[i]) * ib;
    return r;
}
RADJ_HD D5 operator/(const D5& a, double b) {
    D5 r(a.v / b);
    const double ib = 1.0 / b;
    for (int i = 0; i < 5; i++) r.d[i] = a.d[i] * ib;
    return r;
}
RADJ_HD D5 fabs(const D5& a) { return a.v < 0.0 ? -a : a; }
RADJ_HD bool operator<(const D5& a, const D5& b) { return a.v < b.v; }
RADJ_HD bool operator>(const D5& a, const D5& b) { return a.v > b.v; }

RADJ_HD D5 mn(const D5& a, const D5& b) { return (b < a) ? b : a; }

// ---- slope limiters, Solvers/SlopeLimiters.cpp:3-101 (0 = SuperBee, 1 = van Leer, else MinBee)
RADJ_HD D5 gradient_ratio(const D5& r, double w) { return 2.0 / ((1.0 - w) + ((1.0 + w) * r)); }
RADJ_HD D5 limiter(const D5& r, double w, int lim) {
    if (r < D5(0.0)) return D5(0.0);
    if (lim == 0) {
        if (r < D5(0.5)) return 2.0 * r;
        if (r < D5(1.0)) return D5(1.0);
        return mn(mn(r, gradient_ratio(r, w)), D5(2.0));
    }
    if (lim == 1) return mn((2.0 * r) / (1.0 + r), gradient_ratio(r, w));
    if (r < D5(1.0)) return r;
    return mn(D5(1.0), gradient_ratio(r, w));
}
RADJ_HD void slope_vector(const D5* ul, const D5* uc, const D5* ur, double w, int lim, D5* s) {
    const double a = 0.5 * (1.0 + w), b = 0.5 * (1.0 - w);
    for (int k = 0; k < 5; k++) {
        const D5 dl = uc[k] - ul[k], dr = ur[k] - uc[k];
        s[k] = (a * dl) + (b * dr);
        D5 num = dl, den = dr;
        if (fabs(num) < D5(1e-5)) num = D5(1e-5);
        if (fabs(den) < D5(1e-5)) den = D5(1e-5);
        s[k] = s[k] * limiter(num / den, w, lim);
    }
}

// ---- primitive recovery, RelativisticEulerStateVector.cpp:30-101 (BlackHoleEulerStateVector.cpp
// divides the densitised state by sqrt(det gamma) first): the quartic in x = 1 / (h W) by Newton
// from x = 1, stopping when a step moves x by less than tol; floors at 1e-8 (derivative 0).
struct Prim { D5 rho, vx, vy, vz, p, W, h; };
RADJ_HD Prim con2prim(const D5* u, double g, double tol) {
    const D5 D = u[0], Sx = u[1], Sy = u[2], Sz = u[3], tau = u[4];
    const D5 q = ((tau + D) * (tau + D)) - (((Sx * Sx) + (Sy * Sy)) + (Sz * Sz));
    D5 dc, ec;
    if (q < D5(1e-8)) {
        dc = D / ::sqrt(1e-8);
        ec = (D + tau) / ::sqrt(1e-8);
    } else {
        dc = D / sqrt(q);
        ec = (D + tau) / sqrt(q);
    }
    const double gm = (g - 1.0) / g;
    const D5 cst = D5(-1.0 / (g * g));
    const D5 lin = (-2.0 * dc) * ((g - 1.0) / (g * g));
    const D5 quad = ((((g - 2.0) / g) * ((ec * ec) - 1.0)) + 1.0) - (((dc * dc) * gm) * gm);
    const D5 quart = (ec * ec) - 1.0;
    const D5 eta = (2.0 * dc) * gm;
    // The Newton iterations run on the values, the forward's arithmetic operation for operation;
    // the root's tangents come from the implicit-function theorem at the final iterate xv:
    // f(x; c) = 0 gives dx = -(the tangent of f with x held at xv) / f'(xv), the quartic's
    // coefficients c carrying the tangents.
    const double qv = quart.v, ev = eta.v, dv = quad.v, lv = lin.v, cv = cst.v;
    double xv = 1.0;
    for (int it = 0; it < 1000; it++) {
        const double f = ((((qv * ((xv * xv) * xv)) * (xv - ev)) + (dv * (xv * xv))) + (lv * xv)) + cv;
        const double fp = ((lv + ((2.0 * dv) * xv)) + ((4.0 * qv) * ((xv * xv) * xv))) - (((3.0 * ev) * qv) * (xv * xv));
        const double nx = xv - (f / fp);
        if (::fabs(xv - nx) < tol) break;
        xv = nx;
    }
    const double fpv = ((lv + ((2.0 * dv) * xv)) + ((4.0 * qv) * ((xv * xv) * xv))) - (((3.0 * ev) * qv) * (xv * xv));
    const D5 X(xv);
    const D5 fx = ((((quart * ((X * X) * X)) * (X - eta)) + (quad * (X * X))) + (lin * X)) + cst;
    D5 x(xv);
    const double ifp = 1.0 / fpv;
    for (int i = 0; i < 5; i++) x.d[i] = -fx.d[i] * ifp;
    Prim r;
    r.W = ((0.5 * ec) * x) * (1.0 + sqrt(1.0 + ((4.0 * gm) * ((1.0 - (dc * x)) / ((ec * ec) * (x * x))))));
    r.h = 1.0 / (dc * x);
    r.rho = D / r.W;
    const D5 rhw = (r.rho * r.h) * (r.W * r.W);
    r.vx = Sx / rhw;
    r.vy = Sy / rhw;
    r.vz = Sz / rhw;
    r.p = (rhw - D) - tau;
    if (r.rho < D5(1e-8)) r.rho = D5(1e-8);
    if (r.p < D5(1e-8)) r.p = D5(1e-8);
    return r;
}
// RelativisticEulerEquationOfState.cpp:3-8
RADJ_HD D5 enthalpy(const D5& rho, const D5& p, double g) { return 1.0 + ((p / rho) * (g / (g - 1.0))); }

struct Pt { double x, y, z; };
RADJ_HD Pt shift(Pt p, int axis, double d) {
    if (axis == 0) p.x = p.x + d;
    else p.y = p.y + d;
    return p;
}

// ---- special-relativistic state, RelativisticEulerStateVector.cpp:116-309
struct SRSys {
    double g;
    static constexpr bool coords = false;
    RADJ_HD void cons(const D5* p, Pt, D5* u) const {
        const D5 v2 = ((p[1] * p[1]) + (p[2] * p[2])) + (p[3] * p[3]);
        D5 W = D5(1.0 / ::sqrt(1.0 - 1e-8));
        if (!(v2 > D5(1.0 - 1e-8))) W = 1.0 / sqrt(1.0 - v2);
        const D5 rhw = (p[0] * enthalpy(p[0], p[4], g)) * (W * W);
        u[0] = p[0] * W;
        u[1] = rhw * p[1];
        u[2] = rhw * p[2];
        u[3] = rhw * p[3];
        u[4] = (rhw - p[4]) - (p[0] * W);
    }
    RADJ_HD void prim(const D5* u, Pt, D5* p) const {
        const Prim c = con2prim(u, g, 1e-8);
        p[0] = c.rho; p[1] = c.vx; p[2] = c.vy; p[3] = c.vz; p[4] = c.p;
    }
    RADJ_HD void flux(const D5* u, int axis, Pt, D5* f) const {
        const Prim c = con2prim(u, g, 1e-8);
        const D5 rhw = (c.rho * c.h) * (c.W * c.W);
        const D5 vn = axis == 0 ? c.vx : c.vy;
        f[0] = (c.rho * c.W) * vn;
        f[1] = (rhw * (c.vx * vn)) + (axis == 0 ? c.p : D5(0.0));
        f[2] = (rhw * (c.vy * vn)) + (axis == 1 ? c.p : D5(0.0));
        f[3] = rhw * (c.vz * vn);
        f[4] = (((rhw - c.p) - (c.rho * c.W)) * vn) + (c.p * vn);
    }
    RADJ_HD bool active(int, int, int, int, double) const { return true; }
};

// ---- Kerr-Schild spacetime (BlackHoleSpacetime.cpp:54-186, :372-386), the arithmetic of the
// sweeps' FP64 metric: mass M, spin a, position (bx, by, bz).
struct KerrSchild {
    double M, a, bx, by, bz;
    RADJ_HD void Hl(double x, double y, double z, double& h, double* l) const {
        const double dx = x - bx, dy = y - by, dz = z - bz;
        const double n2 = ((dx * dx) + (dy * dy)) + (dz * dz);
        const double ma2 = (M * M) * (a * a);
        const double r = ::sqrt(0.5 * ((n2 - ma2) + ::sqrt(((n2 - ma2) * (n2 - ma2)) + (4.0 * (ma2 * (dz * dz))))));
        h = -(M * ((r * r) * r)) / ((((r * r) * r) * r) + (ma2 * (dz * dz)));
        l[0] = -((r * dx) + ((a * M) * dy)) / ((r * r) + ma2);
        l[1] = -((r * dy) - ((a * M) * dx)) / ((r * r) + ma2);
        l[2] = -dz / r;
    }
    RADJ_HD void gamma(Pt q, double* m) const {
        double h, l[3];
        Hl(q.x, q.y, q.z, h, l);
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) m[3 * i + j] = (i == j ? 1.0 : 0.0) - (((2.0 * h) * l[i]) * l[j]);
    }
    RADJ_HD void lapse_shift(Pt q, double& al, double* b) const {
        double h, l[3];
        Hl(q.x, q.y, q.z, h, l);
        al = 1.0 / ::sqrt(1.0 - (2.0 * h));
        for (int i = 0; i < 3; i++) b[i] = ((2.0 * h) / (1.0 - (2.0 * h))) * l[i];
    }
    // Mathematics/MatrixAlgebra.cpp:106-149, cofactor expansion along row 0
    RADJ_HD static double det3(const double* m) {
        double d = 0.0;
        d = d + (m[0] * ((m[4] * m[8]) - (m[7] * m[5])));
        d = d - (m[1] * ((m[3] * m[8]) - (m[6] * m[5])));
        d = d + (m[2] * ((m[3] * m[7]) - (m[6] * m[4])));
        return d;
    }
    RADJ_HD double sqrt_det(Pt q) const {
        double m[9];
        gamma(q, m);
        return ::sqrt(det3(m));
    }
    RADJ_HD bool excised(double x, double y, double z) const {
        const double r = ::sqrt((((x - bx) * (x - bx)) + ((y - by) * (y - by))) + ((z - bz) * (z - bz)));
        return r <= (M * (1.0 + ::sqrt(1.0 - (a * a))));
    }
    // BlackHoleSpacetime.cpp:92-113 with "r + (y - y_BH)" of :108 as written, and :188-228
    RADJ_HD void g4(Pt q, double* m) const {
        const double dx = q.x - bx, dy = q.y - by, dz = q.z - bz;
        const double n2 = ((dx * dx) + (dy * dy)) + (dz * dz);
        const double ma2 = (M * M) * (a * a);
        const double r = ::sqrt(0.5 * ((n2 - ma2) + ::sqrt(((n2 - ma2) * (n2 - ma2)) + (4.0 * (ma2 * (dz * dz))))));
        const double h = -(M * ((r * r) * r)) / ((((r * r) * r) * r) + (ma2 * (dz * dz)));
        const double l[4] = {-1.0, -((r * dx) + ((a * M) * dy)) / ((r * r) + ma2),
                             -((r + dy) - ((a * M) * dx)) / ((r * r) + ma2), -dz / r};
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++) {
                const double eta = (i == j) ? ((i == 0) ? -1.0 : 1.0) : 0.0;
                m[4 * i + j] = eta - (((2.0 * h) * l[i]) * l[j]);
            }
    }
    // Mathematics/MatrixAlgebra.cpp:106-194: cofactor determinant, Cayley-Hamilton inverse
    RADJ_HD static double det4(const double* m) {
        double d = 0.0;
        for (int i = 0; i < 4; i++) {
            double c[9];
            for (int j = 0; j < 3; j++)
                for (int k = 0; k < 3; k++) c[3 * j + k] = (k < i) ? m[4 * (j + 1) + k] : m[4 * (j + 1) + k + 1];
            if (i % 2 == 0) d = d + (m[i] * det3(c));
            else d = d - (m[i] * det3(c));
        }
        return d;
    }
    RADJ_HD static void inverse4(const double* m, double* o) {
        double m2[16], m3[16];
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++) {
                double s = 0.0;
                for (int k = 0; k < 4; k++) s = s + (m[4 * i + k] * m[4 * k + j]);
                m2[4 * i + j] = s;
            }
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++) {
                double s = 0.0;
                for (int k = 0; k < 4; k++) s = s + (m2[4 * i + k] * m[4 * k + j]);
                m3[4 * i + j] = s;
            }
        double tr = 0.0, tr2 = 0.0, tr3 = 0.0;
        for (int i = 0; i < 4; i++) tr = tr + m[5 * i];
        for (int i = 0; i < 4; i++) tr2 = tr2 + m2[5 * i];
        for (int i = 0; i < 4; i++) tr3 = tr3 + m3[5 * i];
        const double c0 = (1.0 / 6.0) * ((((tr * tr) * tr) - ((3.0 * tr) * tr2)) + (2.0 * tr3));
        const double c1 = 0.5 * ((tr * tr) - tr2);
        const double inv = 1.0 / det4(m);
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++)
                o[4 * i + j] = inv * ((((c0 * (i == j ? 1.0 : 0.0)) - (c1 * m[4 * i + j])) + (tr * m2[4 * i + j])) - m3[4 * i + j]);
    }
};

// ---- black-hole state, BlackHoleEulerStateVector.cpp:30-350 (energy with W, not W^2, at :154;
// x-flux Newton tolerance 1e-10 at :205)
struct GRSys {
    double g;
    KerrSchild bh;
    int dims;
    double h;  // spacing of the metric's centred derivatives (the cell spacing)
    static constexpr bool coords = true;
    RADJ_HD void cons(const D5* p, Pt q, D5* u) const {
        double m[9];
        bh.gamma(q, m);
        const double sg = ::sqrt(KerrSchild::det3(m));
        D5 v2 = D5(0.0);
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) v2 = v2 + ((m[3 * i + j] * p[1 + i]) * p[1 + j]);
        D5 W = D5(1.0 / ::sqrt(1.0 - 1e-8));
        if (!(v2 > D5(1.0 - 1e-8))) W = 1.0 / sqrt(1.0 - v2);
        const D5 hh = enthalpy(p[0], p[4], g);
        const D5 sr = sg * p[0];
        u[0] = sr * W;
        for (int k = 0; k < 3; k++) u[1 + k] = ((sr * hh) * (W * W)) * p[1 + k];
        u[4] = sg * ((((p[0] * hh) * W) - p[4]) - (p[0] * W));
    }
    RADJ_HD Prim c2p(const D5* u, Pt q, double tol) const {
        const double sg = bh.sqrt_det(q);
        const D5 us[5] = {u[0] / sg, u[1] / sg, u[2] / sg, u[3] / sg, u[4] / sg};
        return con2prim(us, g, tol);
    }
    RADJ_HD void prim(const D5* u, Pt q, D5* p) const {
        const Prim c = c2p(u, q, 1e-8);
        p[0] = c.rho; p[1] = c.vx; p[2] = c.vy; p[3] = c.vz; p[4] = c.p;
    }
    RADJ_HD void flux(const D5* u, int axis, Pt q, D5* f) const {
        const double sg = bh.sqrt_det(q);
        double al, be[3];
        bh.lapse_shift(q, al, be);
        const Prim c = c2p(u, q, axis == 0 ? 1e-10 : 1e-8);
        const double as = al * sg;
        const D5 rhw = (c.rho * c.h) * (c.W * c.W);
        const D5 vn = axis == 0 ? c.vx : c.vy;
        const D5 w = vn - (be[axis] / al);
        f[0] = as * ((c.rho * c.W) * w);
        f[1] = as * ((rhw * (c.vx * w)) + (axis == 0 ? c.p : D5(0.0)));
        f[2] = as * ((rhw * (c.vy * w)) + (axis == 1 ? c.p : D5(0.0)));
        f[3] = as * (rhw * (c.vz * w));
        f[4] = as * ((((rhw - c.p) - (c.rho * c.W)) * w) + (c.p * vn));
    }
    // ---- the source term, BlackHoleEuler/BlackHoleEulerStateVector.cpp:359-510, with the metric's
    // centred derivatives (spacing h) and extrinsic curvature, BlackHoleSpacetime.cpp:115-151, :230-370
    RADJ_HD static Pt off(Pt q, int d, double s) {
        if (d == 0) q.x = q.x + s;
        else if (d == 1) q.y = q.y + s;
        else q.z = q.z + s;
        return q;
    }
    RADJ_HD void Kij(Pt q, double al, double* K) const {
        double Hs, v[3], dh[3], dv[9];
        bh.Hl(q.x, q.y, q.z, Hs, v);
        const double hs = 0.5 * h;
        for (int d = 0; d < 3; d++) {
            const Pt p1 = off(q, d, hs), p0 = off(q, d, -hs);
            double h1, h0, a1[3], a0[3];
            bh.Hl(p1.x, p1.y, p1.z, h1, a1);
            bh.Hl(p0.x, p0.y, p0.z, h0, a0);
            dh[d] = (h1 - h0) / h;
            for (int c = 0; c < 3; c++) dv[3 * d + c] = (1.0 / h) * (a1[c] - a0[c]);
        }
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
    RADJ_HD void source(const D5* u, Pt q, D5* s) const {
        double gm[9];
        bh.gamma(q, gm);
        const double dg = KerrSchild::det3(gm);
        double al, be[3];
        bh.lapse_shift(q, al, be);
        const double sg = ::sqrt(dg);
        const D5 us[5] = {u[0] / sg, u[1] / sg, u[2] / sg, u[3] / sg, u[4] / sg};
        const Prim c = con2prim(us, g, 1e-8);
        double g4m[16], gi[16], da[3], db[9], dgm[27], K[9];
        bh.g4(q, g4m);
        KerrSchild::inverse4(g4m, gi);
        const double hs = 0.5 * h;
        for (int d = 0; d < 3; d++) {
            const Pt p1 = off(q, d, hs), p0 = off(q, d, -hs);
            double a1, a0, b1[3], b0[3], g1[9], g0[9];
            bh.lapse_shift(p1, a1, b1);
            bh.lapse_shift(p0, a0, b0);
            bh.gamma(p1, g1);
            bh.gamma(p0, g0);
            da[d] = (a1 - a0) / h;
            for (int k = 0; k < 3; k++) db[3 * d + k] = (1.0 / h) * (b1[k] - b0[k]);
            for (int k = 0; k < 9; k++) dgm[9 * d + k] = (1.0 / h) * (g1[k] - g0[k]);
        }
        Kij(q, al, K);
        D5 uu[4];
        uu[0] = c.W / al;
        uu[1] = ((al * uu[0]) * c.vx) - (be[0] * uu[0]);
        uu[2] = ((al * uu[0]) * c.vy) - (be[1] * uu[0]);
        uu[3] = ((al * uu[0]) * c.vz) - (be[2] * uu[0]);
        D5 T[16];
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++) T[4 * i + j] = (((c.rho * c.h) * uu[i]) * uu[j]) + (c.p * gi[4 * i + j]);
        D5 S[5];
        D5 vc[3];
        for (int i = 0; i < 3; i++)
            vc[i] = ((gm[3 * i + 0] * c.vx) + (gm[3 * i + 1] * c.vy)) + (gm[3 * i + 2] * c.vz);
        const D5 rhw = (c.rho * c.h) * (c.W * c.W);
        for (int i = 0; i < 3; i++) {
            for (int j = 0; j < 3; j++) {
                for (int k = 0; k < 3; k++) {
                    const double dgijk = dgm[9 * i + 3 * j + k];
                    S[i + 1] = S[i + 1] + (T[0] * (((0.5 * be[j]) * be[k]) * dgijk));
                    S[i + 1] = S[i + 1] + ((T[j + 1] * be[k]) * dgijk);
                    S[i + 1] = S[i + 1] + (0.5 * (T[4 * (j + 1) + (k + 1)] * dgijk));
                }
                S[i + 1] = S[i + 1] + (((rhw * vc[j]) / al) * db[3 * i + j]);
            }
            S[i + 1] = S[i + 1] - ((T[0] * al) * da[i]);
        }
        for (int i = 0; i < 3; i++) {
            for (int j = 0; j < 3; j++) {
                S[4] = S[4] + (T[0] * ((be[i] * be[j]) * K[3 * i + j]));
                S[4] = S[4] + (T[i + 1] * ((2.0 * be[j]) * K[3 * i + j]));
                S[4] = S[4] + (T[4 * (i + 1) + (j + 1)] * K[3 * i + j]);
            }
            S[4] = S[4] - (T[0] * (be[i] * da[i]));
            S[4] = S[4] - (T[i + 1] * da[i]);
        }
        const double f = al * ::sqrt(dg);
        for (int k = 0; k < 5; k++) s[k] = f * S[k];
    }
    // Cell k of line L is updated unless a cell of its stencil (two cells out along the line in
    // 1D; the cell and two cells out along both axes in 2D, Solvers/BlackHoleEulerSecondOrderSolver.cpp:39-100)
    // lies in the excision region, tested at the unmirrored positions x = j dx, y = i dx.
    RADJ_HD bool active(int axis, int L, int k, int, double dx) const {
        if (dims == 1) {
            for (int d = -2; d <= 2; d++)
                if (bh.excised((k + d) * dx, 0.0, 0.0)) return false;
            return true;
        }
        const int i = axis == 0 ? L : k, j = axis == 0 ? k : L;
        if (bh.excised(j * dx, i * dx, 0.0)) return false;
        for (int d = 1; d <= 2; d++)
            if (bh.excised((j - d) * dx, i * dx, 0.0) || bh.excised((j + d) * dx, i * dx, 0.0) ||
                bh.excised(j * dx, (i - d) * dx, 0.0) || bh.excised(j * dx, (i + d) * dx, 0.0))
                return false;
        return true;
    }
};

struct Step {
    double dx, dt, w;
    int lim, axis;
};

// Half-step evolution of the middle state centred at xc to its two face primitives (either may be
// null); the faces sit at xc -/+ dx/2.
template <class Sys>
RADJ_HD void evolve(const Sys& S, const Step& s, const D5* l, const D5* m, const D5* r, Pt xc, D5* left, D5* right) {
    D5 ul[5], um[5], ur[5], sl[5];
    S.cons(l, shift(xc, s.axis, -s.dx), ul);
    S.cons(m, xc, um);
    S.cons(r, shift(xc, s.axis, s.dx), ur);
    slope_vector(ul, um, ur, s.w, s.lim, sl);
    D5 UL[5], UR[5], FL[5], FR[5];
    for (int k = 0; k < 5; k++) {
        UL[k] = um[k] - (0.5 * sl[k]);
        UR[k] = um[k] + (0.5 * sl[k]);
    }
    const Pt pl = shift(xc, s.axis, -(s.dx * 0.5)), pr = shift(xc, s.axis, s.dx * 0.5);
    S.flux(UL, s.axis, pl, FL);
    S.flux(UR, s.axis, pr, FR);
    const double hs = 0.5 * (s.dt / s.dx);
    D5 a[5], b[5];
    for (int k = 0; k < 5; k++) {
        const D5 ev = hs * (FL[k] - FR[k]);
        a[k] = UL[k] + ev;
        b[k] = UR[k] + ev;
    }
    if (left) S.prim(a, pl, left);
    if (right) S.prim(b, pr, right);
}

// FORCE flux at face point xf between face primitives L (at xf - dx/2) and R (at xf + dx/2): the
// mean of the Lax-Friedrichs flux and the flux of the Richtmyer state (at xf).
template <class Sys> RADJ_HD void force(const Sys& S, const Step& s, const D5* L, const D5* R, Pt xf, D5* F) {
    D5 uL[5], uR[5], fL[5], fR[5], us[5], fs[5];
    const Pt pl = shift(xf, s.axis, -(s.dx * 0.5)), pr = shift(xf, s.axis, s.dx * 0.5);
    S.cons(L, pl, uL);
    S.cons(R, pr, uR);
    S.flux(uL, s.axis, pl, fL);
    S.flux(uR, s.axis, pr, fR);
    const double c = s.dx / s.dt, d = s.dt / s.dx;
    for (int k = 0; k < 5; k++) us[k] = 0.5 * ((uL[k] + uR[k]) + (d * (fL[k] - fR[k])));
    S.flux(us, s.axis, xf, fs);
    for (int k = 0; k < 5; k++) F[k] = 0.5 * ((0.5 * ((fL[k] + fR[k]) + (c * (uL[k] - uR[k])))) + fs[k]);
}

// Position k of a line of n cells that a stencil position reads: transmissive mirror
// (g[-1] = c[0], g[-2] = c[1], g[n] = c[n-1], g[n+1] = c[n-2]) or periodic wrap.  n >= 2.
RADJ_HD int ghost(int k, int n, bool periodic) {
    if (periodic) return ((k % n) + n) % n;
    if (k < 0) return -1 - k;
    if (k >= n) return 2 * n - 1 - k;
    return k;
}

// One sweep's adjoint over a grid in structure-of-arrays storage: field f of cell (i, j) at
// f * fstride + i * pitch + j, for the state (the sweep's input primitives), the output adjoint
// and the input adjoint alike.  system 1 = SR, 2 = black hole (bh = M, a, x, y, z).
struct Params {
    int system, dims, nx, ny, pitch, periodic;
    size_t fstride;
    double gamma, bh[5];
    Step s;
    const double* state;
    const double* pbar_out;
    double* pbar_in;
};

// The input adjoint of cell c = i * nx + j.  The output windows of one input cell overlap, and every
// half-step evolution and face flux in them carries the same seeds whichever window uses it, so
// each is evaluated once: the states at line positions [kmin - 2, kmax + 2] for the outputs
// kmin..kmax, the evolutions and fluxes of the faces that an updated output reads.
template <class Sys> RADJ_HD void cell_adjoint_sys(const Sys& S, const Params& P, size_t c) {
    const int i = (int)(c / (size_t)P.nx), j = (int)(c % (size_t)P.nx);
    const int axis = P.s.axis;
    const bool per = P.periodic != 0;
    const int n = axis == 0 ? P.nx : P.ny;
    const int me = axis == 0 ? j : i, line = axis == 0 ? i : j;
    const double dx = P.s.dx;
    // storage offset of line cell k: base + k * step
    const size_t base = axis == 0 ? (size_t)i * P.pitch : (size_t)j;
    const size_t step = axis == 0 ? 1 : (size_t)P.pitch;
    // outputs: line positions me - 2 .. me + 2 inside the line (periodic: each distinct cell once)
    int kpos[5], nk = 0;
    bool act[5];
    for (int t = -2; t <= 2; t++) {
        const int k = me + t;
        if (!per && (k < 0 || k >= n)) continue;
        bool dup = false;
        for (int q = 0; q < nk; q++) dup = dup || ghost(kpos[q], n, per) == ghost(k, n, per);
        if (dup) continue;
        act[nk] = S.active(axis, line, ghost(k, n, per), n, dx);
        kpos[nk++] = k;
    }
    const int kmin = kpos[0], kmax = kpos[nk - 1];
    const int lo = kmin - 2;  // states at positions lo .. kmax + 2 (at most 9)
    D5 W[9][5];
    for (int p = lo; p <= kmax + 2; p++) {
        const int src = ghost(p, n, per);
        const size_t off = base + (size_t)src * step;
        for (int f = 0; f < 5; f++) W[p - lo][f] = D5(P.state[f * P.fstride + off]);
        if (src == me)
            for (int f = 0; f < 5; f++) W[p - lo][f].d[f] = 1.0;
    }
    auto at = [&](int p) -> const D5* { return W[p - lo]; };
    // faces kmin .. kmax + 1 (face f between positions f - 1 and f); a face is needed when an
    // updated output reads it
    bool need[6] = {false, false, false, false, false, false};
    for (int q = 0; q < nk; q++)
        if (act[q]) {
            need[kpos[q] - kmin] = true;
            need[kpos[q] + 1 - kmin] = true;
        }
    auto face_pt = [&](int f) -> Pt {
        return axis == 0 ? Pt{(f - 0.5) * dx, line * dx, 0.0} : Pt{line * dx, (f - 0.5) * dx, 0.0};
    };
    auto cell_pt = [&](int k) -> Pt { return axis == 0 ? Pt{k * dx, line * dx, 0.0} : Pt{line * dx, k * dx, 0.0}; };
    D5 F[6][5];
    if (Sys::coords) {  // each face evolves its two cells at its own points
        for (int f = kmin; f <= kmax + 1; f++) {
            if (!need[f - kmin]) continue;
            D5 er[5], el[5];
            const Pt xf = face_pt(f);
            evolve(S, P.s, at(f - 2), at(f - 1), at(f), shift(xf, axis, -(dx * 0.5)), (D5*)nullptr, er);
            evolve(S, P.s, at(f - 1), at(f), at(f + 1), shift(xf, axis, dx * 0.5), el, (D5*)nullptr);
            force(S, P.s, er, el, xf, F[f - kmin]);
        }
    } else {  // each cell's evolution gives both its faces
        D5 A[7][5], B[7][5];  // cells kmin - 1 .. kmax + 1
        for (int k = kmin - 1; k <= kmax + 1; k++) {
            const bool left = k >= kmin && need[k - kmin], right = k + 1 <= kmax + 1 && need[k + 1 - kmin];
            if (!left && !right) continue;
            evolve(S, P.s, at(k - 1), at(k), at(k + 1), cell_pt(k), left ? A[k - kmin + 1] : (D5*)nullptr,
                   right ? B[k - kmin + 1] : (D5*)nullptr);
        }
        for (int f = kmin; f <= kmax + 1; f++)
            if (need[f - kmin]) force(S, P.s, B[f - kmin], A[f - kmin + 1], face_pt(f), F[f - kmin]);
    }
    double acc[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int q = 0; q < nk; q++) {
        const int k = kpos[q], cell = ghost(k, n, per);
        const size_t ok = base + (size_t)cell * step;
        if (!act[q]) {  // P'_k = P_k
            if (cell == me)
                for (int f = 0; f < 5; f++) acc[f] = acc[f] + P.pbar_out[f * P.fstride + ok];
            continue;
        }
        const Pt ck = cell_pt(cell);
        D5 u[5], nu[5], o[5];
        S.cons(at(k), ck, u);
        const double d = P.s.dt / dx;
        for (int f = 0; f < 5; f++) nu[f] = u[f] + (d * (F[k - kmin][f] - F[k + 1 - kmin][f]));
        S.prim(nu, ck, o);
        for (int f = 0; f < 5; f++) {
            const double pb = P.pbar_out[f * P.fstride + ok];
            for (int l = 0; l < 5; l++) acc[l] = acc[l] + (o[f].d[l] * pb);
        }
    }
    const size_t me_off = base + (size_t)me * step;
    for (int f = 0; f < 5; f++) P.pbar_in[f * P.fstride + me_off] = acc[f];
}

// ---- the black-hole RK source step, Solvers/BlackHoleEulerForcingSolver.cpp:3-250: classical RK4 on
// the source term with interleaved fractional evolutions on frozen neighbours
// (Solvers/BlackHoleEulerSolvers.cpp:159-232: face fluxes at xc -/+ dx, as written).
RADJ_HD void evolve_fraction(const GRSys& S, double frac, const D5* l, const D5* m, const D5* r, Pt xc, int axis,
                             double dx, double dt, double w, int lim, D5* out) {
    D5 ul[5], um[5], ur[5], sl[5];
    S.cons(l, shift(xc, axis, -dx), ul);
    S.cons(m, xc, um);
    S.cons(r, shift(xc, axis, dx), ur);
    slope_vector(ul, um, ur, w, lim, sl);
    D5 UL[5], UR[5], FL[5], FR[5];
    for (int k = 0; k < 5; k++) {
        UL[k] = um[k] - (0.5 * sl[k]);
        UR[k] = um[k] + (0.5 * sl[k]);
    }
    S.flux(UL, axis, shift(xc, axis, -dx), FL);
    S.flux(UR, axis, shift(xc, axis, dx), FR);
    const double s = frac * (dt / dx);
    D5 nu[5];
    for (int k = 0; k < 5; k++) nu[k] = um[k] + (s * (FL[k] - FR[k]));
    S.prim(nu, xc, out);
}
RADJ_HD void rk_cell(const GRSys& S, int dims, const D5* cl, const D5* cm, const D5* cr, const D5* ct, const D5* cb,
                     Pt q, double dx, double dt, double w, int lim, D5* out_cons) {
    D5 L[5], R[5], Tp[5], B[5], Mp[5], E1[5], E2[5], E[5];
    S.prim(cl, shift(q, 0, -dx), L);
    S.prim(cr, shift(q, 0, dx), R);
    if (dims == 2) {
        S.prim(ct, shift(q, 1, -dx), Tp);
        S.prim(cb, shift(q, 1, dx), B);
    }
    D5 k[4][5], st[5], c[5], sv[5];
    S.source(cm, q, sv);
    for (int i = 0; i < 5; i++) k[0][i] = dt * sv[i];
    const double fx1[3] = {0.5, 0.5, 1.0};                               // 1D fractions
    const double fx2[3] = {0.25, 0.25, 0.5}, fy2[3] = {0.5, 0.5, 1.0};  // 2D fractions
    for (int stage = 0; stage < 3; stage++) {
        for (int i = 0; i < 5; i++) st[i] = stage < 2 ? (cm[i] + (0.5 * k[stage][i])) : (cm[i] + k[stage][i]);
        S.prim(st, q, Mp);
        if (dims == 1) {
            evolve_fraction(S, fx1[stage], L, Mp, R, q, 0, dx, dt, w, lim, E);
        } else {
            evolve_fraction(S, fx2[stage], L, Mp, R, q, 0, dx, dt, w, lim, E1);
            evolve_fraction(S, fy2[stage], Tp, E1, B, q, 1, dx, dt, w, lim, E2);
            evolve_fraction(S, fx2[stage], L, E2, R, q, 0, dx, dt, w, lim, E);
        }
        S.cons(E, q, c);
        S.source(c, q, sv);
        for (int i = 0; i < 5; i++) k[stage + 1][i] = dt * sv[i];
    }
    for (int i = 0; i < 5; i++)
        out_cons[i] = cm[i] + ((1.0 / 6.0) * (k[0][i] + ((2.0 * k[1][i]) + ((2.0 * k[2][i]) + k[3][i]))));
}

// The input adjoint of cell c = i * nx + j for one RK source step (time step P.s.dt, slopes P.s.w and
// P.s.lim).  Output cell (i', j') reads itself and its 2 (1D) or 4 (2D) direct neighbours through a
// transmissive one-ghost copy (Solvers/BlackHoleEulerForcingSolver.cpp:187-250); an output whose
// point or a neighbour's lies in the excision region keeps its state.
RADJ_HD void rk_cell_adjoint(const Params& P, size_t c) {
    const GRSys S{P.gamma, KerrSchild{P.bh[0], P.bh[1], P.bh[2], P.bh[3], P.bh[4]}, P.dims, P.s.dx};
    const int i = (int)(c / (size_t)P.nx), j = (int)(c % (size_t)P.nx);
    const int dims = P.dims, ny = dims == 1 ? 1 : P.ny;
    const double dx = P.s.dx;
    auto active = [&](int ii, int jj) -> bool {
        const KerrSchild& b = S.bh;
        if (dims == 1) return !b.excised(jj * dx, 0.0, 0.0) && !b.excised((jj - 1) * dx, 0.0, 0.0) && !b.excised((jj + 1) * dx, 0.0, 0.0);
        return !b.excised(jj * dx, ii * dx, 0.0) && !b.excised((jj - 1) * dx, ii * dx, 0.0) &&
               !b.excised((jj + 1) * dx, ii * dx, 0.0) && !b.excised(jj * dx, (ii - 1) * dx, 0.0) &&
               !b.excised(jj * dx, (ii + 1) * dx, 0.0);
    };
    const int oi_[5] = {i, i, i, i - 1, i + 1}, oj_[5] = {j, j - 1, j + 1, j, j};
    double acc[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int q = 0; q < (dims == 1 ? 3 : 5); q++) {
        const int oi = oi_[q], oj = oj_[q];
        if (oi < 0 || oi >= ny || oj < 0 || oj >= P.nx) continue;
        const size_t ok = (size_t)oi * P.pitch + oj;
        if (!active(oi, oj)) {  // P'(i', j') = P(i', j')
            if (q == 0)
                for (int f = 0; f < 5; f++) acc[f] = acc[f] + P.pbar_out[f * P.fstride + ok];
            continue;
        }
        auto ld = [&](int ii, int jj, D5* p) {
            const int gi = ghost(ii, ny, false), gj = ghost(jj, P.nx, false);
            const size_t k = (size_t)gi * P.pitch + gj;
            for (int f = 0; f < 5; f++) p[f] = D5(P.state[f * P.fstride + k]);
            if (gi == i && gj == j)
                for (int f = 0; f < 5; f++) p[f].d[f] = 1.0;
        };
        const double y = dims == 1 ? 0.0 : oi * dx;
        const Pt pq{oj * dx, y, 0.0};
        D5 p[5], cl[5], cm[5], cr[5], ct[5], cb[5], nc[5], o[5];
        ld(oi, oj - 1, p);
        S.cons(p, Pt{(oj - 1) * dx, y, 0.0}, cl);
        ld(oi, oj, p);
        S.cons(p, pq, cm);
        ld(oi, oj + 1, p);
        S.cons(p, Pt{(oj + 1) * dx, y, 0.0}, cr);
        if (dims == 2) {
            ld(oi - 1, oj, p);
            S.cons(p, Pt{oj * dx, (oi - 1) * dx, 0.0}, ct);
            ld(oi + 1, oj, p);
            S.cons(p, Pt{oj * dx, (oi + 1) * dx, 0.0}, cb);
        }
        rk_cell(S, dims, cl, cm, cr, ct, cb, pq, dx, P.s.dt, P.s.w, P.s.lim, nc);
        S.prim(nc, pq, o);
        for (int f = 0; f < 5; f++) {
            const double pb = P.pbar_out[f * P.fstride + ok];
            for (int l = 0; l < 5; l++) acc[l] = acc[l] + (o[f].d[l] * pb);
        }
    }
    const size_t me = (size_t)i * P.pitch + j;
    for (int f = 0; f < 5; f++) P.pbar_in[f * P.fstride + me] = acc[f];
}

RADJ_HD void cell_adjoint(const Params& P, size_t c) {
    if (P.system == 2)
        cell_adjoint_sys(GRSys{P.gamma, KerrSchild{P.bh[0], P.bh[1], P.bh[2], P.bh[3], P.bh[4]}, P.dims, P.s.dx}, P, c);
    else
        cell_adjoint_sys(SRSys{P.gamma}, P, c);
}

}  // namespace radj
}  // namespace cg
