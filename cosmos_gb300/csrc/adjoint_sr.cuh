// Adjoint (vector-Jacobian product) of one special-relativistic SLIC sweep, FP64, gather form.
//
// Forward map of a sweep along a line of n cells (primitive states P, dt and dx fixed;
// Solvers/RelativisticEulerSecondOrderSolver.cpp:3-100 with the half-step evolution of
// Solvers/RelativisticEulerSolvers.cpp:148-199, the FORCE flux of Solvers/EulerFirstOrderSolver.cpp:3-59
// on RelativisticEulerStateVector's conversions and fluxes, RelativisticEulerStateVector.cpp:30-309,
// and the slope limiters of Solvers/SlopeLimiters.cpp:3-101):
//   A_k, B_k = the left- and right-face primitives of cell k's half-step evolution from P_{k-1..k+1}
//   F_f      = FORCE(B_{f-1}, A_f)
//   P'_k     = prim(cons(P_k) + (dt/dx) (F_k - F_{k+1}))
// so P'_k depends on P_{k-2} .. P_{k+2}, where positions outside the line read the interior cell
// they copy (transmissive mirror or periodic wrap).  Given the adjoint Pbar' of the output, the
// adjoint of input cell j is
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
#define SRA_HD __host__ __device__ inline
#else
#define SRA_HD inline
#endif

namespace cg {
namespace sra {

// ---- dual numbers: value and five tangent lanes; comparisons act on values
struct D5 {
    double v, d[5];
    SRA_HD D5() : v(0.0), d{0.0, 0.0, 0.0, 0.0, 0.0} {}
    SRA_HD D5(double x) : v(x), d{0.0, 0.0, 0.0, 0.0, 0.0} {}
};
SRA_HD D5 operator+(const D5& a, const D5& b) {
    D5 r(a.v + b.v);
    for (int i = 0; i < 5; i++) r.d[i] = a.d[i] + b.d[i];
    return r;
}
SRA_HD D5 operator-(const D5& a, const D5& b) {
    D5 r(a.v - b.v);
    for (int i = 0; i < 5; i++) r.d[i] = a.d[i] - b.d[i];
    return r;
}
SRA_HD D5 operator-(const D5& a) {
    D5 r(-a.v);
    for (int i = 0; i < 5; i++) r.d[i] = -a.d[i];
    return r;
}
SRA_HD D5 operator*(const D5& a, const D5& b) {
    D5 r(a.v * b.v);
    for (int i = 0; i < 5; i++) r.d[i] = (a.d[i] * b.v) + (a.v * b.d[i]);
    return r;
}
SRA_HD D5 operator/(const D5& a, const D5& b) {
    D5 r(a.v / b.v);
    for (int i = 0; i < 5; i++) r.d[i] = (a.d[i] - (r.v * b.d[i])) / b.v;
    return r;
}
SRA_HD D5 sqrt(const D5& a) {
    D5 r(::sqrt(a.v));
    for (int i = 0; i < 5; i++) r.d[i] = a.d[i] / (2.0 * r.v);
    return r;
}
SRA_HD D5 fabs(const D5& a) { return a.v < 0.0 ? -a : a; }
SRA_HD bool operator<(const D5& a, const D5& b) { return a.v < b.v; }
SRA_HD bool operator>(const D5& a, const D5& b) { return a.v > b.v; }
SRA_HD bool operator>=(const D5& a, const D5& b) { return a.v >= b.v; }

template <class T> SRA_HD T mn(const T& a, const T& b) { return (b < a) ? b : a; }

// ---- slope limiters, Solvers/SlopeLimiters.cpp:3-101 (0 = SuperBee, 1 = van Leer, else MinBee)
template <class T> SRA_HD T gradient_ratio(const T& r, double w) {
    return T(2.0) / (T(1.0 - w) + (T(1.0 + w) * r));
}
template <class T> SRA_HD T limiter(const T& r, double w, int lim) {
    if (r < T(0.0)) return T(0.0);
    if (lim == 0) {
        if (r < T(0.5)) return T(2.0) * r;
        if (r < T(1.0)) return T(1.0);
        return mn(mn(r, gradient_ratio(r, w)), T(2.0));
    }
    if (lim == 1) return mn((T(2.0) * r) / (T(1.0) + r), gradient_ratio(r, w));
    if (r < T(1.0)) return r;
    return mn(T(1.0), gradient_ratio(r, w));
}
template <class T> SRA_HD void slope_vector(const T* ul, const T* uc, const T* ur, double w, int lim, T* s) {
    const T a = T(0.5 * (1.0 + w)), b = T(0.5 * (1.0 - w));
    for (int k = 0; k < 5; k++) {
        const T dl = uc[k] - ul[k], dr = ur[k] - uc[k];
        s[k] = (a * dl) + (b * dr);
        T num = dl, den = dr;
        if (fabs(num) < T(1e-5)) num = T(1e-5);
        if (fabs(den) < T(1e-5)) den = T(1e-5);
        s[k] = s[k] * limiter(num / den, w, lim);
    }
}

// ---- the special-relativistic state, RelativisticEulerStateVector.cpp and
// RelativisticEulerEquationOfState.cpp:3-8 (h = 1 + (p / rho) gamma / (gamma - 1))
template <class T> struct Prim { T rho, vx, vy, vz, p, W, h; };

// Conserved -> primitive: the quartic in x = 1 / (h W) by Newton from x = 1, stopping when a step
// moves x by less than tol (RelativisticEulerStateVector.cpp:30-101), floors at 1e-8.
template <class T> SRA_HD Prim<T> con2prim(const T* u, double g, double tol) {
    const T D = u[0], Sx = u[1], Sy = u[2], Sz = u[3], tau = u[4];
    const T q = ((tau + D) * (tau + D)) - (((Sx * Sx) + (Sy * Sy)) + (Sz * Sz));
    T dc, ec;
    if (q < T(1e-8)) {
        dc = D / T(::sqrt(1e-8));
        ec = (D + tau) / T(::sqrt(1e-8));
    } else {
        dc = D / sqrt(q);
        ec = (D + tau) / sqrt(q);
    }
    const double gm = (g - 1.0) / g;
    const T cst = T(-1.0 / (g * g));
    const T lin = (T(-2.0) * dc) * T((g - 1.0) / (g * g));
    const T quad = ((T((g - 2.0) / g) * ((ec * ec) - T(1.0))) + T(1.0)) - (((dc * dc) * T(gm)) * T(gm));
    const T quart = (ec * ec) - T(1.0);
    const T eta = (T(2.0) * dc) * T(gm);
    T x = T(1.0);
    for (int it = 0; it < 1000; it++) {
        const T f = ((((quart * ((x * x) * x)) * (x - eta)) + (quad * (x * x))) + (lin * x)) + cst;
        const T fp = ((lin + ((T(2.0) * quad) * x)) + ((T(4.0) * quart) * ((x * x) * x))) -
                     (((T(3.0) * eta) * quart) * (x * x));
        const T nx = x - (f / fp);
        if (fabs(x - nx) < T(tol)) break;
        x = nx;
    }
    Prim<T> r;
    r.W = ((T(0.5) * ec) * x) *
          (T(1.0) + sqrt(T(1.0) + ((T(4.0) * T(gm)) * ((T(1.0) - (dc * x)) / ((ec * ec) * (x * x))))));
    r.h = T(1.0) / (dc * x);
    r.rho = D / r.W;
    const T rhw = (r.rho * r.h) * (r.W * r.W);
    r.vx = Sx / rhw;
    r.vy = Sy / rhw;
    r.vz = Sz / rhw;
    r.p = (rhw - D) - tau;
    if (r.rho < T(1e-8)) r.rho = T(1e-8);
    if (r.p < T(1e-8)) r.p = T(1e-8);
    return r;
}

// RelativisticEulerStateVector.cpp:116-136 (W capped where v^2 > 1 - 1e-8)
template <class T> SRA_HD void cons(const T* p, double g, T* u) {
    const T v2 = ((p[1] * p[1]) + (p[2] * p[2])) + (p[3] * p[3]);
    T W = T(1.0 / ::sqrt(1.0 - 1e-8));
    if (!(v2 > T(1.0 - 1e-8))) W = T(1.0) / sqrt(T(1.0) - v2);
    const T h = T(1.0) + ((p[4] / p[0]) * T(g / (g - 1.0)));
    const T rhw = (p[0] * h) * (W * W);
    u[0] = p[0] * W;
    u[1] = rhw * p[1];
    u[2] = rhw * p[2];
    u[3] = rhw * p[3];
    u[4] = (rhw - p[4]) - (p[0] * W);
}
template <class T> SRA_HD void prim(const T* u, double g, T* p) {
    const Prim<T> c = con2prim(u, g, 1e-8);
    p[0] = c.rho; p[1] = c.vx; p[2] = c.vy; p[3] = c.vz; p[4] = c.p;
}
// RelativisticEulerStateVector.cpp:138-220 (x) and :227-309 (y)
template <class T> SRA_HD void flux(const T* u, int axis, double g, T* f) {
    const Prim<T> c = con2prim(u, g, 1e-8);
    const T rhw = (c.rho * c.h) * (c.W * c.W);
    const T vn = axis == 0 ? c.vx : c.vy;
    f[0] = (c.rho * c.W) * vn;
    f[1] = (rhw * (c.vx * vn)) + (axis == 0 ? c.p : T(0.0));
    f[2] = (rhw * (c.vy * vn)) + (axis == 1 ? c.p : T(0.0));
    f[3] = rhw * (c.vz * vn);
    f[4] = (((rhw - c.p) - (c.rho * c.W)) * vn) + (c.p * vn);
}

struct Step {
    double g, dx, dt, w;
    int lim, axis;
};

// Half-step evolution of the middle cell to its two face primitives (either may be null).
template <class T> SRA_HD void evolve(const Step& s, const T* l, const T* m, const T* r, T* left, T* right) {
    T ul[5], um[5], ur[5], sl[5];
    cons(l, s.g, ul);
    cons(m, s.g, um);
    cons(r, s.g, ur);
    slope_vector(ul, um, ur, s.w, s.lim, sl);
    T UL[5], UR[5], FL[5], FR[5];
    for (int k = 0; k < 5; k++) {
        UL[k] = um[k] - (T(0.5) * sl[k]);
        UR[k] = um[k] + (T(0.5) * sl[k]);
    }
    flux(UL, s.axis, s.g, FL);
    flux(UR, s.axis, s.g, FR);
    const T hs = T(0.5 * (s.dt / s.dx));
    T a[5], b[5];
    for (int k = 0; k < 5; k++) {
        const T ev = hs * (FL[k] - FR[k]);
        a[k] = UL[k] + ev;
        b[k] = UR[k] + ev;
    }
    if (left) prim(a, s.g, left);
    if (right) prim(b, s.g, right);
}

// FORCE flux between two face primitives: the mean of the Lax-Friedrichs and Richtmyer fluxes.
template <class T> SRA_HD void force(const Step& s, const T* L, const T* R, T* F) {
    T uL[5], uR[5], fL[5], fR[5], us[5], fs[5];
    cons(L, s.g, uL);
    cons(R, s.g, uR);
    flux(uL, s.axis, s.g, fL);
    flux(uR, s.axis, s.g, fR);
    const T c = T(s.dx / s.dt), d = T(s.dt / s.dx);
    for (int k = 0; k < 5; k++) us[k] = T(0.5) * ((uL[k] + uR[k]) + (d * (fL[k] - fR[k])));
    flux(us, s.axis, s.g, fs);
    for (int k = 0; k < 5; k++) F[k] = T(0.5) * ((T(0.5) * ((fL[k] + fR[k]) + (c * (uL[k] - uR[k])))) + fs[k]);
}

// Position k of a line of n cells that a stencil position reads: transmissive mirror
// (g[-1] = c[0], g[-2] = c[1], g[n] = c[n-1], g[n+1] = c[n-2]) or periodic wrap.  n >= 2.
SRA_HD int ghost(int k, int n, bool periodic) {
    if (periodic) return ((k % n) + n) % n;
    if (k < 0) return -1 - k;
    if (k >= n) return 2 * n - 1 - k;
    return k;
}

// One sweep's adjoint over a grid in structure-of-arrays storage: field f of cell (i, j) at
// f * fstride + i * pitch + j, for the state (the sweep's input primitives), the output adjoint
// and the input adjoint alike.
struct Params {
    int nx, ny, pitch, axis, periodic;
    size_t fstride;
    Step s;
    const double* state;
    const double* pbar_out;
    double* pbar_in;
};

// The input adjoint of cell c = i * nx + j.
SRA_HD void cell_adjoint(const Params& P, size_t c) {
    const int i = (int)(c / (size_t)P.nx), j = (int)(c % (size_t)P.nx);
    const bool per = P.periodic != 0;
    const int n = P.axis == 0 ? P.nx : P.ny;
    const int me = P.axis == 0 ? j : i;
    // storage offset of line position k
    const size_t base = P.axis == 0 ? (size_t)i * P.pitch : (size_t)j;
    const size_t step = P.axis == 0 ? 1 : (size_t)P.pitch;
    int ks[5], nk = 0;
    for (int t = -2; t <= 2; t++) {
        int k = me + t;
        if (per) k = ghost(k, n, true);
        else if (k < 0 || k >= n) continue;
        bool dup = false;
        for (int q = 0; q < nk; q++) dup = dup || ks[q] == k;
        if (!dup) ks[nk++] = k;
    }
    double acc[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int q = 0; q < nk; q++) {
        const int k = ks[q];
        D5 win[5][5];
        bool hit = false;
        for (int p = 0; p < 5; p++) {
            const int src = ghost(k - 2 + p, n, per);
            const size_t off = base + (size_t)src * step;
            for (int f = 0; f < 5; f++) win[p][f] = D5(P.state[f * P.fstride + off]);
            if (src == me) {
                hit = true;
                for (int f = 0; f < 5; f++) win[p][f].d[f] = 1.0;
            }
        }
        if (!hit) continue;
        D5 Bm[5], A0[5], B0[5], A1[5], F0[5], F1[5];
        evolve(P.s, win[0], win[1], win[2], (D5*)nullptr, Bm);
        evolve(P.s, win[1], win[2], win[3], A0, B0);
        evolve(P.s, win[2], win[3], win[4], A1, (D5*)nullptr);
        force(P.s, Bm, A0, F0);
        force(P.s, B0, A1, F1);
        D5 u[5], nu[5], o[5];
        cons(win[2], P.s.g, u);
        const D5 d = D5(P.s.dt / P.s.dx);
        for (int f = 0; f < 5; f++) nu[f] = u[f] + (d * (F0[f] - F1[f]));
        prim(nu, P.s.g, o);
        const size_t ok = base + (size_t)k * step;
        for (int f = 0; f < 5; f++) {
            const double pb = P.pbar_out[f * P.fstride + ok];
            for (int l = 0; l < 5; l++) acc[l] = acc[l] + (o[f].d[l] * pb);
        }
    }
    const size_t me_off = base + (size_t)me * step;
    for (int f = 0; f < 5; f++) P.pbar_in[f * P.fstride + me_off] = acc[f];
}

}  // namespace sra
}  // namespace cg
