// Reference-exact device physics.  Every expression keeps the reference's evaluation order
// (left-to-right C++ semantics of the cited lines), so that a translation unit compiled with
// --fmad=false produces the reference's FP64 results bit for bit.  Used by the FP64 ("plain
// FP64") path; also instantiated in FP32 for the SR/GR bulk paths where noted.
#pragma once
#include "device_common.cuh"

namespace cg {

// ============================================================== slope limiters
// Solvers/SlopeLimiters.cpp:3-6
template <class T> CG_D T gradient_ratio(T r, T w) { return T(2.0) / ((T(1.0) - w) + ((T(1.0) + w) * r)); }

// Solvers/SlopeLimiters.cpp:8-69 (0 SuperBee, 1 van Leer, otherwise MinBee)
template <class T> CG_D T limiter_exact(T r, T w, int lim) {
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

// Solvers/SlopeLimiters.cpp:71-101 (numerator and denominator each clamped to +1e-5)
template <class T> CG_D void slope_exact(const T* ul, const T* uc, const T* ur, T w, int lim, T* s) {
    T dl[5], dr[5];
#pragma unroll
    for (int k = 0; k < 5; k++) { dl[k] = uc[k] - ul[k]; dr[k] = ur[k] - uc[k]; }
    const T a = T(0.5) * (T(1.0) + w), b = T(0.5) * (T(1.0) - w);
#pragma unroll
    for (int k = 0; k < 5; k++) s[k] = (a * dl[k]) + (b * dr[k]);
#pragma unroll
    for (int k = 0; k < 5; k++) {
        T num = dl[k], den = dr[k];
        if (fabs(num) < T(1e-5)) num = T(1e-5);
        if (fabs(den) < T(1e-5)) den = T(1e-5);
        s[k] = s[k] * limiter_exact(num / den, w, lim);
    }
}

// ============================================================== Newtonian Euler
template <class T> struct NewtonExact {
    T g;
    int* capped;  // unused (no iterative solve); keeps the policy interface uniform
    static constexpr bool kCoords = false;
    // Euler/EulerStateVector.cpp:55-66, computeTotalEnergy :129-134, EoS Euler/EulerEquationOfState.cpp:3-8
    CG_D void cons(const T* p, Pt, T* u) const {
        T rho = p[0], vx = p[1], vy = p[2], vz = p[3];
        u[0] = rho; u[1] = rho * vx; u[2] = rho * vy; u[3] = rho * vz;
        T v2 = ((vx * vx) + (vy * vy)) + (vz * vz);
        T e = p[4] / ((g - T(1.0)) * rho);
        u[4] = rho * ((T(0.5) * v2) + e);
    }
    // Euler/EulerStateVector.cpp:30-40, computePressure Euler/EulerEquationOfState.cpp:10-15
    CG_D void prim(const T* u, Pt, T* p) const {
        T rho = u[0];
        T vx = u[1] / rho, vy = u[2] / rho, vz = u[3] / rho;
        T v2 = ((vx * vx) + (vy * vy)) + (vz * vz);
        T e = (u[4] / rho) - (T(0.5) * v2);
        p[0] = rho; p[1] = vx; p[2] = vy; p[3] = vz; p[4] = (e * (g - T(1.0))) * rho;
    }
    // Euler/EulerStateVector.cpp:68-89 (x) and :96-117 (y)
    CG_D void flux(const T* u, int axis, Pt, T* f) const {
        T rho = u[0];
        T vx = u[1] / rho, vy = u[2] / rho, vz = u[3] / rho;
        T v2 = ((vx * vx) + (vy * vy)) + (vz * vz);
        T et = u[4] / rho;
        T pr = ((et - (T(0.5) * v2)) * (g - T(1.0))) * rho;
        if (axis == 0) {
            f[0] = rho * vx; f[1] = (rho * (vx * vx)) + pr; f[2] = rho * (vx * vy); f[3] = rho * (vx * vz);
            f[4] = (rho * (vx * et)) + (vx * pr);
        } else {
            f[0] = rho * vy; f[1] = rho * (vy * vx); f[2] = (rho * (vy * vy)) + pr; f[3] = rho * (vy * vz);
            f[4] = (rho * (vy * et)) + (vy * pr);
        }
    }
    // Solvers/EulerSolvers.cpp:87-128 with Euler/EulerEquationOfState.cpp:17-22;
    // 2D is max(|vx|, |vy| + c) exactly as written at :117-118.
    CG_D T wavespeed(const T* p, int dims, Pt) const {
        T c = fabs(sqrt((g * p[4]) / p[0]));
        if (dims == 1) return fabs(p[1]) + c;
        return mx(fabs(p[1]), fabs(p[2]) + c);
    }
};

// ============================================================== SR con2prim (FP64)
// RelativisticEuler/RelativisticEulerStateVector.cpp:30-101; the same solve appears in its flux
// functions (:138-309) and, on densitised variables, BlackHoleEuler/BlackHoleEulerStateVector.cpp
// (:30-103, :159-350 with tol 1e-10 in the x flux at :205, :359-430).  Newton from x = 1 on the
// quartic in x, stop when |x - x_new| < tol keeping the previous iterate, at most 1000 steps.
struct C2P { double rho, vx, vy, vz, p, W, h; };

CG_D C2P con2prim_exact(double D, double Sx, double Sy, double Sz, double tau, double g, double tol, int* capped) {
    double q = ((tau + D) * (tau + D)) - (((Sx * Sx) + (Sy * Sy)) + (Sz * Sz));
    double dc = D / sqrt(q);
    double ec = (D + tau) / sqrt(q);
    if (q < 1e-8) {
        dc = D / sqrt(1e-8);
        ec = (D + tau) / sqrt(1e-8);
    }
    double constant = -1.0 / (g * g);
    double linear = (-2.0 * dc) * ((g - 1.0) / (g * g));
    double quadratic = ((((g - 2.0) / g) * ((ec * ec) - 1.0)) + 1.0) - (((dc * dc) * ((g - 1.0) / g)) * ((g - 1.0) / g));
    double quartic = (ec * ec) - 1.0;
    double eta = (2.0 * dc) * ((g - 1.0) / g);
    double x = 1.0;
    int it = 0;
    bool conv = false;
    while (it < 1000) {
        double f = ((((quartic * ((x * x) * x)) * (x - eta)) + (quadratic * (x * x))) + (linear * x)) + constant;
        double fp = ((linear + ((2.0 * quadratic) * x)) + ((4.0 * quartic) * ((x * x) * x))) - (((3.0 * eta) * quartic) * (x * x));
        double nx = x - (f / fp);
        if (fabs(x - nx) < tol) { conv = true; break; }
        it += 1;
        x = nx;
    }
    if (!conv && capped) *capped = 1;
    C2P r;
    r.W = ((0.5 * ec) * x) * (1.0 + sqrt(1.0 + ((4.0 * ((g - 1.0) / g)) * ((1.0 - (dc * x)) / ((ec * ec) * (x * x))))));
    r.h = 1.0 / (dc * x);
    r.rho = D / r.W;
    double rhw = (r.rho * r.h) * (r.W * r.W);
    r.vx = Sx / rhw; r.vy = Sy / rhw; r.vz = Sz / rhw;
    r.p = (rhw - D) - tau;
    if (r.rho < 1e-8) r.rho = 1e-8;
    if (r.p < 1e-8) r.p = 1e-8;
    return r;
}

// RelativisticEuler/RelativisticEulerEquationOfState.cpp:3-18
CG_D double sr_enthalpy(double rho, double p, double g) { return 1.0 + ((p / rho) * (g / (g - 1.0))); }
CG_D double sr_sound(double rho, double p, double g) {
    double num = (g * p) / rho;
    double den = 1.0 + ((p / rho) * (g / (g - 1.0)));
    return sqrt(num / den);
}

// ============================================================== SR Euler (FP64)
struct SRExact {
    double g;
    int* capped;  // optional: set when a Newton solve hits its cap
    static constexpr bool kCoords = false;
    // RelativisticEuler/RelativisticEulerStateVector.cpp:116-136
    CG_D void cons(const double* p, Pt, double* u) const {
        double rho = p[0], vx = p[1], vy = p[2], vz = p[3], pr = p[4];
        double v2 = ((vx * vx) + (vy * vy)) + (vz * vz);
        double W = 1.0 / sqrt(1.0 - v2);
        if (v2 > 1.0 - 1e-8) W = 1.0 / sqrt(1.0 - 1e-8);
        double h = sr_enthalpy(rho, pr, g);
        double rhw = (rho * h) * (W * W);
        u[0] = rho * W; u[1] = rhw * vx; u[2] = rhw * vy; u[3] = rhw * vz;
        u[4] = (rhw - pr) - (rho * W);
    }
    CG_D void prim(const double* u, Pt, double* p) const {
        C2P c = con2prim_exact(u[0], u[1], u[2], u[3], u[4], g, 1e-8, capped);
        p[0] = c.rho; p[1] = c.vx; p[2] = c.vy; p[3] = c.vz; p[4] = c.p;
    }
    // RelativisticEuler/RelativisticEulerStateVector.cpp:138-220 (x), :227-309 (y)
    CG_D void flux(const double* u, int axis, Pt, double* f) const {
        C2P c = con2prim_exact(u[0], u[1], u[2], u[3], u[4], g, 1e-8, capped);
        double rhw = (c.rho * c.h) * (c.W * c.W);
        double vn = axis == 0 ? c.vx : c.vy;
        f[0] = (c.rho * c.W) * vn;
        if (axis == 0) {
            f[1] = (rhw * (c.vx * c.vx)) + c.p; f[2] = rhw * (c.vy * c.vx); f[3] = rhw * (c.vz * c.vx);
        } else {
            f[1] = rhw * (c.vx * c.vy); f[2] = (rhw * (c.vy * c.vy)) + c.p; f[3] = rhw * (c.vz * c.vy);
        }
        f[4] = (((rhw - c.p) - (c.rho * c.W)) * vn) + (c.p * vn);
    }
    // Solvers/RelativisticEulerSolvers.cpp:87-128 (2D: max(|vx|, |vy|) + c)
    CG_D double wavespeed(const double* p, int dims, Pt) const {
        double c = fabs(sr_sound(p[0], p[4], g));
        if (dims == 1) return fabs(p[1]) + c;
        return mx(fabs(p[1]), fabs(p[2])) + c;
    }
};

// ============================================================== Kerr-Schild spacetime (FP64)
struct BHExact {
    double M, a, bx, by, bz;
    // BlackHoleSpacetime.cpp:54-68
    CG_D double radius(double dx, double dy, double dz) const {
        double n2 = ((dx * dx) + (dy * dy)) + (dz * dz);
        double ma2 = (M * M) * (a * a);
        return sqrt(0.5 * ((n2 - ma2) + sqrt(((n2 - ma2) * (n2 - ma2)) + (4.0 * (ma2 * (dz * dz))))));
    }
    CG_D double H(double x, double y, double z) const {
        double dx = x - bx, dy = y - by, dz = z - bz;
        double r = radius(dx, dy, dz);
        double ma2 = (M * M) * (a * a);
        return -(M * ((r * r) * r)) / ((((r * r) * r) * r) + (ma2 * (dz * dz)));
    }
    // BlackHoleSpacetime.cpp:70-90
    CG_D void l(double x, double y, double z, double* o) const {
        double dx = x - bx, dy = y - by, dz = z - bz;
        double r = radius(dx, dy, dz);
        double ma2 = (M * M) * (a * a);
        o[0] = -((r * dx) + ((a * M) * dy)) / ((r * r) + ma2);
        o[1] = -((r * dy) - ((a * M) * dx)) / ((r * r) + ma2);
        o[2] = -dz / r;
    }
    // H and l together (same arithmetic as the two separate calls)
    CG_D void Hl(double x, double y, double z, double& h, double* o) const {
        double dx = x - bx, dy = y - by, dz = z - bz;
        double r = radius(dx, dy, dz);
        double ma2 = (M * M) * (a * a);
        h = -(M * ((r * r) * r)) / ((((r * r) * r) * r) + (ma2 * (dz * dz)));
        o[0] = -((r * dx) + ((a * M) * dy)) / ((r * r) + ma2);
        o[1] = -((r * dy) - ((a * M) * dx)) / ((r * r) + ma2);
        o[2] = -dz / r;
    }
    // BlackHoleSpacetime.cpp:92-113 with "r + (y - y_BH)" of :108 as written
    CG_D void L4(double x, double y, double z, double* o) const {
        double dx = x - bx, dy = y - by, dz = z - bz;
        double r = radius(dx, dy, dz);
        double ma2 = (M * M) * (a * a);
        o[0] = -1.0;
        o[1] = -((r * dx) + ((a * M) * dy)) / ((r * r) + ma2);
        o[2] = -((r + dy) - ((a * M) * dx)) / ((r * r) + ma2);
        o[3] = -dz / r;
    }
    // BlackHoleSpacetime.cpp:153-186
    CG_D void gamma(double x, double y, double z, double* m) const {
        double h, v[3];
        Hl(x, y, z, h, v);
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) m[3 * i + j] = (i == j ? 1.0 : 0.0) - (((2.0 * h) * v[i]) * v[j]);
    }
    // BlackHoleSpacetime.cpp:188-228
    CG_D void g4(double x, double y, double z, double* m) const {
        double h = H(x, y, z), v[4];
        L4(x, y, z, v);
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
            for (int j = 0; j < 4; j++) {
                double eta = (i == j) ? ((i == 0) ? -1.0 : 1.0) : 0.0;
                m[4 * i + j] = eta - (((2.0 * h) * v[i]) * v[j]);
            }
    }
    CG_D double lapse(double x, double y, double z) const { return 1.0 / sqrt(1.0 - (2.0 * H(x, y, z))); }
    CG_D void shiftv(double x, double y, double z, double* b) const {
        double h, v[3];
        Hl(x, y, z, h, v);
#pragma unroll
        for (int i = 0; i < 3; i++) b[i] = ((2.0 * h) / (1.0 - (2.0 * h))) * v[i];
    }
    // lapse and shift from one H/l evaluation (same arithmetic as the separate calls)
    CG_D void lapse_shift(double x, double y, double z, double& al, double* b) const {
        double h, v[3];
        Hl(x, y, z, h, v);
        al = 1.0 / sqrt(1.0 - (2.0 * h));
#pragma unroll
        for (int i = 0; i < 3; i++) b[i] = ((2.0 * h) / (1.0 - (2.0 * h))) * v[i];
    }
    // BlackHoleSpacetime.cpp:372-386
    CG_D bool excised(double x, double y, double z) const {
        double r = sqrt((((x - bx) * (x - bx)) + ((y - by) * (y - by))) + ((z - bz) * (z - bz)));
        return r <= (M * (1.0 + sqrt(1.0 - (a * a))));
    }
};

// Mathematics/MatrixAlgebra.cpp:106-149: cofactor expansion along row 0 down to 2x2.
CG_D double det2(double a00, double a01, double a10, double a11) { return (a00 * a11) - (a10 * a01); }
CG_D double det3(const double* m) {
    double d = 0.0;
    d = d + (m[0] * det2(m[4], m[5], m[7], m[8]));
    d = d - (m[1] * det2(m[3], m[5], m[6], m[8]));
    d = d + (m[2] * det2(m[3], m[4], m[6], m[7]));
    return d;
}
CG_D double det4(const double* m) {
    double d = 0.0;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        double c[9];
#pragma unroll
        for (int j = 0; j < 3; j++)
#pragma unroll
            for (int k = 0; k < 3; k++) c[3 * j + k] = (k < i) ? m[4 * (j + 1) + k] : m[4 * (j + 1) + k + 1];
        if (i % 2 == 0) d = d + (m[i] * det3(c));
        else d = d - (m[i] * det3(c));
    }
    return d;
}
template <int N> CG_D void matmul_n(const double* a, const double* b, double* c) {
#pragma unroll
    for (int i = 0; i < N; i++)
#pragma unroll
        for (int j = 0; j < N; j++) {
            double s = 0.0;
#pragma unroll
            for (int k = 0; k < N; k++) s = s + (a[N * i + k] * b[N * k + j]);
            c[N * i + j] = s;
        }
}
template <int N> CG_D double trace_n(const double* m) {
    double t = 0.0;
#pragma unroll
    for (int i = 0; i < N; i++) t = t + m[N * i + i];
    return t;
}
// Mathematics/MatrixAlgebra.cpp:151-194 (Cayley-Hamilton)
CG_D void inverse3(const double* m, double* o) {
    double d = det3(m), tr = trace_n<3>(m), m2[9];
    matmul_n<3>(m, m, m2);
    double tr2 = trace_n<3>(m2);
    double s = 0.5 * ((tr * tr) - tr2);
    double inv = 1.0 / d;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) o[3 * i + j] = inv * (((s * (i == j ? 1.0 : 0.0)) - (tr * m[3 * i + j])) + m2[3 * i + j]);
}
CG_D void inverse4(const double* m, double* o) {
    double d = det4(m), tr = trace_n<4>(m), m2[16], m3[16];
    matmul_n<4>(m, m, m2);
    matmul_n<4>(m2, m, m3);
    double tr2 = trace_n<4>(m2), tr3 = trace_n<4>(m3);
    double c0 = (1.0 / 6.0) * ((((tr * tr) * tr) - ((3.0 * tr) * tr2)) + (2.0 * tr3));
    double c1 = 0.5 * ((tr * tr) - tr2);
    double inv = 1.0 / d;
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
            o[4 * i + j] = inv * ((((c0 * (i == j ? 1.0 : 0.0)) - (c1 * m[4 * i + j])) + (tr * m2[4 * i + j])) - m3[4 * i + j]);
}

// ============================================================== GR Euler (FP64)
struct GRExact {
    double g;
    BHExact bh;
    double h;      // finite-difference spacing of the metric derivatives (the cell spacing)
    int* capped;
    static constexpr bool kCoords = true;

    CG_D double detg(Pt p) const { double m[9]; bh.gamma(p.x, p.y, p.z, m); return det3(m); }

    // BlackHoleEuler/BlackHoleEulerStateVector.cpp:118-157 (energy with W, not W^2, at :154)
    CG_D void cons(const double* p, Pt q, double* u) const {
        double m[9];
        bh.gamma(q.x, q.y, q.z, m);
        double dg = det3(m);
        double v[3] = {p[1], p[2], p[3]};
        double v2 = 0.0;
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) v2 = v2 + ((m[3 * i + j] * v[i]) * v[j]);
        double W = 1.0 / sqrt(1.0 - v2);
        if (v2 > 1.0 - 1e-8) W = 1.0 / sqrt(1.0 - 1e-8);
        double hh = sr_enthalpy(p[0], p[4], g);
        double sg = sqrt(dg);
        u[0] = (sg * p[0]) * W;
#pragma unroll
        for (int k = 0; k < 3; k++) u[1 + k] = (((sg * p[0]) * hh) * (W * W)) * v[k];
        u[4] = sg * ((((p[0] * hh) * W) - p[4]) - (p[0] * W));
    }
    CG_D C2P c2p(const double* u, double sg, double tol) const {
        return con2prim_exact(u[0] / sg, u[1] / sg, u[2] / sg, u[3] / sg, u[4] / sg, g, tol, capped);
    }
    // BlackHoleEuler/BlackHoleEulerStateVector.cpp:30-103
    CG_D void prim(const double* u, Pt q, double* p) const {
        C2P c = c2p(u, sqrt(detg(q)), 1e-8);
        p[0] = c.rho; p[1] = c.vx; p[2] = c.vy; p[3] = c.vz; p[4] = c.p;
    }
    // BlackHoleEuler/BlackHoleEulerStateVector.cpp:159-250 (x, tol 1e-10) and :259-350 (y)
    CG_D void flux(const double* u, int axis, Pt q, double* f) const {
        double sg = sqrt(detg(q));
        double al, be[3];
        bh.lapse_shift(q.x, q.y, q.z, al, be);
        C2P c = c2p(u, sg, axis == 0 ? 1e-10 : 1e-8);
        double as = al * sg;
        double rhw = (c.rho * c.h) * (c.W * c.W);
        double vn = axis == 0 ? c.vx : c.vy;
        double w = vn - ((axis == 0 ? be[0] : be[1]) / al);
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
    // ---- metric derivatives (BlackHoleSpacetime.cpp:115-151, :250-334), centred with spacing h
    CG_D Pt off(Pt q, int d, double s) const {
        if (d == 0) q.x = q.x + s; else if (d == 1) q.y = q.y + s; else q.z = q.z + s;
        return q;
    }
    // BlackHoleSpacetime.cpp:336-370
    CG_D void Kij(Pt q, double al, double* K) const {
        double Hs, v[3];
        bh.Hl(q.x, q.y, q.z, Hs, v);
        double dh[3], dv[9];
        const double hs = 0.5 * h;
#pragma unroll
        for (int d = 0; d < 3; d++) {
            Pt p1 = off(q, d, hs), p0 = off(q, d, -hs);
            double h1, h0, a1[3], a0[3];
            bh.Hl(p1.x, p1.y, p1.z, h1, a1);
            bh.Hl(p0.x, p0.y, p0.z, h0, a0);
            dh[d] = (h1 - h0) / h;
#pragma unroll
            for (int c = 0; c < 3; c++) dv[3 * d + c] = (1.0 / h) * (a1[c] - a0[c]);
        }
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) {
                double k = al * ((((-(v[i] * dh[j])) - (v[j] * dh[i])) - (Hs * dv[3 * j + i])) - (Hs * dv[3 * i + j]));
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    k = k + (((al * 2.0) * (Hs * Hs)) * (((v[i] * v[c]) * dv[3 * c + j]) + ((v[j] * v[c]) * dv[3 * c + i])));
                    k = k + ((((((al * 2.0) * Hs) * v[i]) * v[j]) * v[c]) * dh[c]);
                }
                K[3 * i + j] = k;
            }
    }
    // The metric part of the source term at q: inverse 4-metric, centred derivatives of the lapse,
    // shift and spatial metric (spacing h), extrinsic curvature (BlackHoleSpacetime.cpp:115-151,
    // :230-370).
    CG_D void source_metric(Pt q, double al, double* gi, double* da, double* db, double* dgm, double* K) const {
        double g4m[16];
        bh.g4(q.x, q.y, q.z, g4m);
        inverse4(g4m, gi);
        const double hs = 0.5 * h;
#pragma unroll
        for (int d = 0; d < 3; d++) {
            Pt p1 = off(q, d, hs), p0 = off(q, d, -hs);
            double a1, a0, b1[3], b0[3], g1[9], g0[9];
            bh.lapse_shift(p1.x, p1.y, p1.z, a1, b1);
            bh.lapse_shift(p0.x, p0.y, p0.z, a0, b0);
            bh.gamma(p1.x, p1.y, p1.z, g1);
            bh.gamma(p0.x, p0.y, p0.z, g0);
            da[d] = (a1 - a0) / h;
#pragma unroll
            for (int k = 0; k < 3; k++) db[3 * d + k] = (1.0 / h) * (b1[k] - b0[k]);
#pragma unroll
            for (int k = 0; k < 9; k++) dgm[9 * d + k] = (1.0 / h) * (g1[k] - g0[k]);
        }
        Kij(q, al, K);
    }
    // BlackHoleEuler/BlackHoleEulerStateVector.cpp:359-510
    CG_D void source(const double* u, Pt q, double* s) const {
        double gm[9];
        bh.gamma(q.x, q.y, q.z, gm);
        double dg = det3(gm);
        double al, be[3];
        bh.lapse_shift(q.x, q.y, q.z, al, be);
        C2P c = c2p(u, sqrt(dg), 1e-8);
        double gi[16], da[3], db[9], dgm[27], K[9];
        source_metric(q, al, gi, da, db, dgm, K);
        double uu[4];
        uu[0] = c.W / al;
        uu[1] = ((al * uu[0]) * c.vx) - (be[0] * uu[0]);
        uu[2] = ((al * uu[0]) * c.vy) - (be[1] * uu[0]);
        uu[3] = ((al * uu[0]) * c.vz) - (be[2] * uu[0]);
        double T[16];
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
            for (int j = 0; j < 4; j++) T[4 * i + j] = (((c.rho * c.h) * uu[i]) * uu[j]) + (c.p * gi[4 * i + j]);
        double S[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
        double vc[3];
#pragma unroll
        for (int i = 0; i < 3; i++) vc[i] = ((gm[3 * i + 0] * c.vx) + (gm[3 * i + 1] * c.vy)) + (gm[3 * i + 2] * c.vz);
        double rhw = (c.rho * c.h) * (c.W * c.W);
#pragma unroll
        for (int i = 0; i < 3; i++) {
#pragma unroll
            for (int j = 0; j < 3; j++) {
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    double dgijk = dgm[9 * i + 3 * j + k];
                    S[i + 1] = S[i + 1] + (T[0] * (((0.5 * be[j]) * be[k]) * dgijk));
                    S[i + 1] = S[i + 1] + ((T[j + 1] * be[k]) * dgijk);
                    S[i + 1] = S[i + 1] + (0.5 * (T[4 * (j + 1) + (k + 1)] * dgijk));
                }
                S[i + 1] = S[i + 1] + (((rhw * vc[j]) / al) * db[3 * i + j]);
            }
            S[i + 1] = S[i + 1] - ((T[0] * al) * da[i]);
        }
#pragma unroll
        for (int i = 0; i < 3; i++) {
#pragma unroll
            for (int j = 0; j < 3; j++) {
                S[4] = S[4] + (T[0] * ((be[i] * be[j]) * K[3 * i + j]));
                S[4] = S[4] + (T[i + 1] * ((2.0 * be[j]) * K[3 * i + j]));
                S[4] = S[4] + (T[4 * (i + 1) + (j + 1)] * K[3 * i + j]);
            }
            S[4] = S[4] - (T[0] * (be[i] * da[i]));
            S[4] = S[4] - (T[i + 1] * da[i]);
        }
        double f = al * sqrt(dg);
#pragma unroll
        for (int k = 0; k < 5; k++) s[k] = f * S[k];
    }
    // BlackHoleEuler/BlackHoleEulerStateVector.cpp:519-549, eigenvalues
    // BlackHoleEuler/BlackHoleEulerEigenvalues.cpp:3-96 (largest signed eigenvalue)
    CG_D double sound_speed(const double* p, Pt q) const {
        double al, be[3];
        bh.lapse_shift(q.x, q.y, q.z, al, be);
        double gm[9], gs[9];
        bh.gamma(q.x, q.y, q.z, gm);
        inverse3(gm, gs);
        double cs = sr_sound(p[0], p[4], g);
        double v[3] = {p[1], p[2], p[3]};
        double v2 = 0.0;
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) v2 = v2 + ((gm[3 * i + j] * v[i]) * v[j]);
        double s = 0.0;
#pragma unroll
        for (int i = 0; i < 3; i++) {
            double mat = (al * v[i]) - be[i];
            double rt = sqrt((1.0 - v2) * ((gs[3 * i + i] * (1.0 - (v2 * (cs * cs)))) - ((v[i] * v[i]) * (1.0 - (cs * cs)))));
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

// ============================================================== generic evolution pieces
// Half-step evolution (Solvers/EulerSolvers.cpp:174-223; SR Solvers/RelativisticEulerSolvers.cpp:148-199;
// GR Solvers/BlackHoleEulerSolvers.cpp:234-307).  Produces the left- and/or right-face state as
// primitives (the reference's evolved EulerStateVector).
template <class Sys, class T>
CG_D void evolve_half_exact(const Sys& S, const T* l, const T* m, const T* r, Pt xc, int axis, double dx, double dt,
                            T w, int lim, T* left_face, T* right_face) {
    T ul[5], um[5], ur[5], sl[5];
    S.cons(l, shift_pt(xc, axis, -dx), ul);
    S.cons(m, xc, um);
    S.cons(r, shift_pt(xc, axis, dx), ur);
    slope_exact(ul, um, ur, w, lim, sl);
    T UL[5], UR[5], FL[5], FR[5];
#pragma unroll
    for (int k = 0; k < 5; k++) { UL[k] = um[k] - (T(0.5) * sl[k]); UR[k] = um[k] + (T(0.5) * sl[k]); }
    S.flux(UL, axis, shift_pt(xc, axis, -(dx * 0.5)), FL);
    S.flux(UR, axis, shift_pt(xc, axis, dx * 0.5), FR);
    const T s = T(0.5) * (T(dt) / T(dx));
    T a[5], b[5];
#pragma unroll
    for (int k = 0; k < 5; k++) {
        T ev = s * (FL[k] - FR[k]);
        a[k] = UL[k] + ev;
        b[k] = UR[k] + ev;
    }
    if (left_face) S.prim(a, shift_pt(xc, axis, -(dx * 0.5)), left_face);
    if (right_face) S.prim(b, shift_pt(xc, axis, dx * 0.5), right_face);
}

// FORCE flux of two primitive states at interface xf (Solvers/EulerFirstOrderSolver.cpp:3-59;
// GR Solvers/BlackHoleEulerFirstOrderSolver.cpp:3-47).
template <class Sys, class T>
CG_D void force_exact(const Sys& S, const T* L, const T* R, Pt xf, int axis, double dx, double dt, T* F) {
    T uL[5], uR[5], fL[5], fR[5], us[5], fs[5];
    Pt pl = shift_pt(xf, axis, -(dx * 0.5)), pr = shift_pt(xf, axis, dx * 0.5);
    S.cons(L, pl, uL);
    S.cons(R, pr, uR);
    S.flux(uL, axis, pl, fL);
    S.flux(uR, axis, pr, fR);
    const T c = T(dx) / T(dt), d = T(dt) / T(dx);
#pragma unroll
    for (int k = 0; k < 5; k++) us[k] = T(0.5) * ((uL[k] + uR[k]) + (d * (fL[k] - fR[k])));
    S.flux(us, axis, xf, fs);
#pragma unroll
    for (int k = 0; k < 5; k++) {
        T lf = T(0.5) * ((fL[k] + fR[k]) + (c * (uL[k] - uR[k])));
        F[k] = T(0.5) * (lf + fs[k]);
    }
}

// ============================================================== GR source RK4 (FP64)
// Fractional evolution on frozen neighbours, Solvers/BlackHoleEulerSolvers.cpp:159-232: slopes
// from the neighbours at xc -/+ dx, face fluxes evaluated at xc -/+ dx (not dx/2), the middle
// state advanced by frac * dt/dx and converted back at xc.
CG_D void evolve_fraction_exact(const GRExact& S, double frac, const double* l, const double* m, const double* r,
                                Pt xc, int axis, double dx, double dt, double w, int lim, double* out) {
    double ul[5], um[5], ur[5], sl[5];
    S.cons(l, shift_pt(xc, axis, -dx), ul);
    S.cons(m, xc, um);
    S.cons(r, shift_pt(xc, axis, dx), ur);
    slope_exact(ul, um, ur, w, lim, sl);
    double UL[5], UR[5], FL[5], FR[5];
#pragma unroll
    for (int k = 0; k < 5; k++) { UL[k] = um[k] - (0.5 * sl[k]); UR[k] = um[k] + (0.5 * sl[k]); }
    S.flux(UL, axis, shift_pt(xc, axis, -dx), FL);
    S.flux(UR, axis, shift_pt(xc, axis, dx), FR);
    const double s = frac * (dt / dx);
    double nu[5];
#pragma unroll
    for (int k = 0; k < 5; k++) nu[k] = um[k] + (s * (FL[k] - FR[k]));
    S.prim(nu, xc, out);
}

// Classical RK4 on the source with interleaved fractional sweeps,
// Solvers/BlackHoleEulerForcingSolver.cpp:3-70 (1D: X fractions 1/2, 1/2, 1) and :72-185
// (2D: X 1/4, Y 1/2, X 1/4 for stages 1-2; X 1/2, Y 1, X 1/2 for stage 3).
// cl..cb are the conserved neighbours (cell-centred), q the cell's coordinate; returns the
// updated conserved state.
CG_D void rk_cell_exact(const GRExact& S, int dims, const double* cl, const double* cm, const double* cr,
                        const double* ct, const double* cb, Pt q, double dx, double dt, double w, int lim,
                        double* out) {
    double L[5], R[5], Tp[5], B[5];
    S.prim(cl, shift_pt(q, 0, -dx), L);
    S.prim(cr, shift_pt(q, 0, dx), R);
    if (dims == 2) {
        S.prim(ct, shift_pt(q, 1, -dx), Tp);
        S.prim(cb, shift_pt(q, 1, dx), B);
    }
    double k[4][5];
    {
        double s[5];
        S.source(cm, q, s);
#pragma unroll
        for (int i = 0; i < 5; i++) k[0][i] = dt * s[i];
    }
    for (int stage = 0; stage < 3; stage++) {
        double st[5], Mp[5], E[5], c[5], s[5];
#pragma unroll
        for (int i = 0; i < 5; i++) st[i] = stage < 2 ? (cm[i] + (0.5 * k[stage][i])) : (cm[i] + k[stage][i]);
        S.prim(st, q, Mp);
        if (dims == 1) {
            const double fx = stage < 2 ? 0.5 : 1.0;
            evolve_fraction_exact(S, fx, L, Mp, R, q, 0, dx, dt, w, lim, E);
        } else {
            const double fx = stage < 2 ? 0.25 : 0.5, fy = stage < 2 ? 0.5 : 1.0;
            double E1[5], E2[5];
            evolve_fraction_exact(S, fx, L, Mp, R, q, 0, dx, dt, w, lim, E1);
            evolve_fraction_exact(S, fy, Tp, E1, B, q, 1, dx, dt, w, lim, E2);
            evolve_fraction_exact(S, fx, L, E2, R, q, 0, dx, dt, w, lim, E);
        }
        S.cons(E, q, c);
        S.source(c, q, s);
#pragma unroll
        for (int i = 0; i < 5; i++) k[stage + 1][i] = dt * s[i];
    }
#pragma unroll
    for (int i = 0; i < 5; i++) out[i] = cm[i] + ((1.0 / 6.0) * (k[0][i] + ((2.0 * k[1][i]) + ((2.0 * k[2][i]) + k[3][i]))));
}

}  // namespace cg
