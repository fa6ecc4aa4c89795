// Hand-written adjoint (vector-Jacobian product) of one Newtonian SLIC sweep.
//
// Forward map of a sweep along a line of n cells (conserved variables U, dt and dx fixed;
// Solvers/EulerSecondOrderSolver.cpp:3-100, Solvers/EulerSolvers.cpp:174-223,
// Solvers/EulerFirstOrderSolver.cpp:3-101, Solvers/SlopeLimiters.cpp:3-147):
//   slope_i  = xi(r_i) * (a (U_i - U_{i-1}) + b (U_{i+1} - U_i)),  a,b = (1 +- w)/2,
//              r_i = num/den of the two differences, each replaced by +1e-5 when |.| < 1e-5
//   UL_i, UR_i = U_i -+ slope_i / 2;   e_i = (dt/dx)/2 (F(UL_i) - F(UR_i))
//   A_i = UL_i + e_i (left-face state),  B_i = UR_i + e_i (right-face state)
//   F_{j+1/2} = FORCE(B_j, A_{j+1}) = ((LF + F(U*)) / 2 with LF = (F(L)+F(R))/2 + (dx/dt)(L-R)/2,
//              U* = (L+R)/2 + (dt/dx)(F(L)-F(R))/2
//   U'_i = U_i + (dt/dx) (F_{i-1/2} - F_{i+1/2})
// Given the adjoint of the output, Ubar', the adjoint of the input is
//   Ubar_i = Ubar'_i + sum over the cells whose half-step stencil holds i of their evolve VJP,
// where the face adjoints Fbar_{j+1/2} = (dt/dx)(Ubar'_{j+1} - Ubar'_j) are pulled back through
// FORCE to (Bbar_j, Abar_{j+1}) and then through each cell's half-step evolution.  Ghost cells
// (transmissive mirror or periodic wrap) pass their adjoint to the interior cell they copy.
// The limiter is differentiated piecewise (its derivative on the branch the forward takes; the
// clamped differences carry no derivative), as a dual-number evaluation of the same code would.
//
// Line tiles: P positions along the sweep axis (P - 6 updated cells and a 3-cell halo on each side,
// 4 where a tile holds a line end: AdjTiles) times W lines; one thread per position, five
// barrier-separated phases in shared memory:
//   0 store state and Ubar' (loaded while the previous tile was computed)
//   1 half-step evolution (keeping each cell's slope and reverse factors)
//   2 FORCE reverse per face   3 half-step reverse per cell   4 gather per updated cell.
#pragma once
#include "device_common.cuh"
#include "physics_fast.cuh"
#include "sweep_kernels.cuh"

namespace cg {

// ---- lane types: float (one line per thread), f2 (two lines per thread on paired FP32
// instructions, physics_fast.cuh), double (the FP64 path; explicitly rounded like the others).
CG_D double vadd(double a, double b) { return __dadd_rn(a, b); }
CG_D double vsub(double a, double b) { return __dsub_rn(a, b); }
CG_D double vmul(double a, double b) { return __dmul_rn(a, b); }
CG_D double vfma(double a, double b, double c) { return __fma_rn(a, b, c); }
CG_D double vrcp(double a) { return 1.0 / a; }
CG_D double vmin(double a, double b) { return fmin(a, b); }
CG_D double vmax(double a, double b) { return fmax(a, b); }
CG_D double vabs(double a) { return fabs(a); }
CG_D double vsel_lt(double a, double b, double x, double y) { return a < b ? x : y; }

CG_D float adj_div(float a, float b) { return fdiv(a, b); }
CG_D double adj_div(double a, double b) { return a / b; }

template <class V> struct Lane;
template <> struct Lane<float> {
    using S = float;
    static constexpr int N = 1;
    static CG_D float bc(float s) { return s; }
};
template <> struct Lane<f2> {
    using S = float;
    static constexpr int N = 2;
    static CG_D f2 bc(float s) { return f2{make_float2(s, s)}; }
};
template <> struct Lane<double> {
    using S = double;
    static constexpr int N = 1;
    static CG_D double bc(double s) { return s; }
};
template <class V> CG_D V bcv(typename Lane<V>::S s) { return Lane<V>::bc(s); }

// Newtonian flux along axis AX of a conserved state, and its transposed Jacobian.
template <class V>
struct AdjFlux {
    V g1, ng1, ng1h;  // gamma - 1, -(gamma - 1), -(gamma - 1)/2
    template <int AX>
    CG_D void flux(const V* u, V* f) const {
        const V inv = vrcp(u[0]);
        const V vn = vmul(u[1 + AX], inv);
        const V q = vfma(u[1], u[1], vfma(u[2], u[2], vmul(u[3], u[3])));
        const V p = vfma(ng1h, vmul(q, inv), vmul(g1, u[4]));
        f[0] = u[1 + AX];
        f[1] = AX == 0 ? vfma(u[1], vn, p) : vmul(u[1], vn);
        f[2] = AX == 1 ? vfma(u[2], vn, p) : vmul(u[2], vn);
        f[3] = vmul(u[3], vn);
        f[4] = vmul(vadd(u[4], p), vn);
    }
    // ub += (dF/du)^T gb, with p = (gamma - 1)(E - rho |v|^2 / 2) and v = m / rho:
    //   pb = gb_n + gb_E v_n (everything p multiplies), vnb = sum_k gb_k m_k + gb_E (E + p)
    //   ub_rho += (gamma - 1) pb |v|^2 / 2 - vnb v_n / rho,  ub_mk += gb_k v_n - (gamma - 1) pb v_k,
    //   ub_mn += gb_rho + vnb / rho,  ub_E += gb_E v_n + (gamma - 1) pb
    template <int AX>
    CG_D void vjp(const V* u, const V* gb, V* ub) const {
        vjp_p<AX>(u, prep(u), gb, ub);
    }
    // The quantities flux and vjp share at one state: 1 / rho, the velocity, |v|^2 and p.
    struct Prep {
        V inv, v0, v1, v2, vv, p;
    };
    CG_D Prep prep(const V* u) const {
        Prep q;
        q.inv = vrcp(u[0]);
        q.v0 = vmul(u[1], q.inv);
        q.v1 = vmul(u[2], q.inv);
        q.v2 = vmul(u[3], q.inv);
        q.vv = vfma(q.v0, q.v0, vfma(q.v1, q.v1, vmul(q.v2, q.v2)));
        q.p = vfma(ng1h, vmul(u[0], q.vv), vmul(g1, u[4]));
        return q;
    }
    // flux from a state's prep (p from |v|^2: the same value as flux's to rounding)
    template <int AX>
    CG_D void flux_p(const V* u, const Prep& q, V* f) const {
        const V vn = AX == 0 ? q.v0 : q.v1;
        f[0] = u[1 + AX];
        f[1] = AX == 0 ? vfma(u[1], vn, q.p) : vmul(u[1], vn);
        f[2] = AX == 1 ? vfma(u[2], vn, q.p) : vmul(u[2], vn);
        f[3] = vmul(u[3], vn);
        f[4] = vmul(vadd(u[4], q.p), vn);
    }
    template <int AX>
    CG_D void vjp_p(const V* u, const Prep& q, const V* gb, V* ub) const {
        const V inv = q.inv, v0 = q.v0, v1 = q.v1, v2 = q.v2, vv = q.vv, p = q.p;
        const V vn = AX == 0 ? v0 : v1;
        const V pb = vfma(gb[4], vn, gb[1 + AX]);
        const V vnb = vfma(gb[4], vadd(u[4], p), vfma(gb[3], u[3], vfma(gb[2], u[2], vmul(gb[1], u[1]))));
        const V ngp = vmul(ng1, pb);    // -(gamma - 1) pb
        const V ngh = vmul(ng1h, pb);   // -(gamma - 1) pb / 2
        ub[0] = vsub(ub[0], vfma(ngh, vv, vmul(vmul(vnb, vn), inv)));
        ub[1] = vfma(gb[1], vn, vfma(ngp, v0, ub[1]));
        ub[2] = vfma(gb[2], vn, vfma(ngp, v1, ub[2]));
        ub[3] = vfma(gb[3], vn, vfma(ngp, v2, ub[3]));
        ub[1 + AX] = vfma(vnb, inv, vadd(ub[1 + AX], gb[0]));
        ub[4] = vfma(gb[4], vn, vsub(ub[4], ngp));
    }
};

// Slope factors of one sweep: ca = (1 + w)/2, cb = (1 - w)/2 and the gradient ratio's 1 -+ w.
template <class V>
struct AdjSlope {
    V ca, cb, w1m, w1p;
};

// Limiter value and derivative d(xi)/dr on the branch the forward evaluation takes
// (Solvers/SlopeLimiters.cpp:8-69; min(a, b) picks b only when b < a), as select chains.
template <class V, int LIM>
CG_D V limiter_d(const AdjSlope<V>& A, V r, V& d) {
    const V zero = bcv<V>(0), one = bcv<V>(1), two = bcv<V>(2);
    const V iden = vrcp(vfma(A.w1p, r, A.w1m));
    const V xr = vmul(two, iden);
    const V dxr = vmul(vmul(bcv<V>(-2), A.w1p), vmul(iden, iden));
    V val, der;
    if (LIM == 0) {  // SuperBee
        const V m1 = vsel_lt(xr, r, xr, r), d1 = vsel_lt(xr, r, dxr, one);
        const V m2 = vsel_lt(two, m1, two, m1), d2 = vsel_lt(two, m1, zero, d1);
        val = vsel_lt(r, bcv<V>(0.5), vmul(two, r), vsel_lt(r, one, one, m2));
        der = vsel_lt(r, bcv<V>(0.5), two, vsel_lt(r, one, zero, d2));
    } else if (LIM == 1) {  // van Leer
        const V iop = vrcp(vadd(one, r));
        const V vl = vmul(vmul(two, r), iop);
        val = vsel_lt(xr, vl, xr, vl);
        der = vsel_lt(xr, vl, dxr, vmul(two, vmul(iop, iop)));
    } else {  // MinBee: r below 1 (xr above 1), xr below 1 (r above 1); 0 for r < 0
        // value: max(min(r, xr), 0) is the same selection (xr >= 1 >= r for 0 <= r <= 1, xr < 1 < r
        // above); derivative on the branch taken: 1, dxr, or 0 (r < 0, and at r = 1, where the forward
        // takes the constant 1)
        d = vsel_lt(r, one, vsel_lt(r, zero, zero, one), vsel_lt(xr, one, dxr, zero));
        return vmax(vmin(r, xr), zero);
    }
    d = vsel_lt(r, zero, zero, der);
    return vsel_lt(r, zero, zero, val);
}

// Half-step evolution of one cell: A (left-face) and B (right-face) states, and per field the three
// numbers its reverse needs: the limited slope sl = xi(r) s and the factors P, Q with which the
// slope adjoint slb reaches the two differences, dlb = slb P and drb = slb Q:
//   P = a xi + s xi'(r) / den   (0 for the derivative term where |dl| < 1e-5: the clamped numerator)
//   Q = b xi - s xi'(r) r / den (0 for the derivative term where |dr| < 1e-5)
template <class V, int AX, int LIM>
CG_D void adj_evolve(const AdjFlux<V>& F, const AdjSlope<V>& Sl, const V* ul, const V* uc, const V* ur, V hs, V* A,
                     V* B, V* sl, V* Pf, V* Qf) {
    const V eps = bcv<V>(1e-5), zero = bcv<V>(0);
    V UL[5], UR[5];
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const V dl = vsub(uc[k], ul[k]), dr = vsub(ur[k], uc[k]);
        const V s = vfma(Sl.ca, dl, vmul(Sl.cb, dr));
        const V adl = vabs(dl), adr = vabs(dr);
        const V num = vsel_lt(adl, eps, eps, dl);
        const V iden = vrcp(vsel_lt(adr, eps, eps, dr));
        const V r = vmul(num, iden);
        V dxi;
        const V xi = limiter_d<V, LIM>(Sl, r, dxi);
        const V t = vmul(vmul(s, dxi), iden);
        sl[k] = vmul(s, xi);
        Pf[k] = vfma(Sl.ca, xi, vsel_lt(adl, eps, zero, t));
        Qf[k] = vsub(vmul(Sl.cb, xi), vsel_lt(adr, eps, zero, vmul(t, r)));
        UL[k] = vfma(bcv<V>(-0.5), sl[k], uc[k]);
        UR[k] = vfma(bcv<V>(0.5), sl[k], uc[k]);
    }
    V FL[5], FR[5];
    F.template flux<AX>(UL, FL);
    F.template flux<AX>(UR, FR);
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const V e = vmul(hs, vsub(FL[k], FR[k]));
        A[k] = vadd(UL[k], e);
        B[k] = vadd(UR[k], e);
    }
}

// Reverse of adj_evolve: given Abar, Bbar and the cell's (sl, P, Q), the contributions to the three
// stencil cells.
template <class V, int AX>
CG_D void adj_evolve_vjp(const AdjFlux<V>& F, const V* uc, const V* sl, const V* Pf, const V* Qf, V hs, const V* Ab,
                         const V* Bb, V* gl, V* gc, V* gr) {
    V UL[5], UR[5], ULb[5], URb[5], FLb[5], FRb[5];
#pragma unroll
    for (int k = 0; k < 5; k++) {
        UL[k] = vfma(bcv<V>(-0.5), sl[k], uc[k]);
        UR[k] = vfma(bcv<V>(0.5), sl[k], uc[k]);
        const V eb = vadd(Ab[k], Bb[k]);
        ULb[k] = Ab[k];
        URb[k] = Bb[k];
        FLb[k] = vmul(hs, eb);
        FRb[k] = vmul(bcv<V>(-1), FLb[k]);
    }
    F.template vjp<AX>(UL, FLb, ULb);
    F.template vjp<AX>(UR, FRb, URb);
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const V slb = vmul(bcv<V>(0.5), vsub(URb[k], ULb[k]));
        const V dlb = vmul(slb, Pf[k]), drb = vmul(slb, Qf[k]);
        gl[k] = vmul(bcv<V>(-1), dlb);
        gc[k] = vadd(vadd(ULb[k], URb[k]), vsub(dlb, drb));
        gr[k] = drb;
    }
}

// Reverse of the FORCE flux of (L, R): given Fbar, Lbar and Rbar.
template <class V, int AX>
CG_D void adj_force_vjp(const AdjFlux<V>& F, const V* L, const V* R, V c, V d, const V* Fb, V* Lb, V* Rb) {
    const V h = bcv<V>(0.5);
    V fL[5], fR[5], us[5];
    const typename AdjFlux<V>::Prep qL = F.prep(L), qR = F.prep(R);
    F.template flux_p<AX>(L, qL, fL);
    F.template flux_p<AX>(R, qR, fR);
#pragma unroll
    for (int k = 0; k < 5; k++) us[k] = vmul(h, vfma(d, vsub(fL[k], fR[k]), vadd(L[k], R[k])));
    V usb[5], fsb[5];
#pragma unroll
    for (int k = 0; k < 5; k++) {
        usb[k] = bcv<V>(0);
        fsb[k] = vmul(h, Fb[k]);
    }
    F.template vjp<AX>(us, fsb, usb);
    V fLb[5], fRb[5];
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const V lfb = vmul(h, Fb[k]);
        const V a = vmul(h, usb[k]), b = vmul(vmul(h, c), lfb), e = vmul(vmul(h, d), usb[k]), f = vmul(h, lfb);
        Lb[k] = vadd(a, b);
        Rb[k] = vsub(a, b);
        fLb[k] = vadd(e, f);
        fRb[k] = vsub(f, e);
    }
    F.template vjp_p<AX>(L, qL, fLb, Lb);
    F.template vjp_p<AX>(R, qR, fRb, Rb);
}

// Coefficients of one sweep in both precisions, formed once per sweep (on the host, or by
// adjoint_coef_kernel from the device's dts), not per thread: an FP64 divide per thread would
// dominate the FP32 kernel (GB300's FP64 rate is 1/64 of FP32).
template <class T>
struct AdjCoef {
    T g1, gam, w, d, c, hs;  // gamma - 1, gamma, bias, dt/dx, dx/dt, dt/(2 dx)
    T ca, cb, w1m, w1p;      // (1 + w)/2, (1 - w)/2, 1 - w, 1 + w
};
struct AdjCoefs {
    AdjCoef<float> f;
    AdjCoef<double> d;
};
CG_HD AdjCoefs adj_coefs(double dt, double dx, double gam, double w) {
    const AdjCoef<double> D{gam - 1.0,       gam,   w,       dt / dx, dx / dt, 0.5 * (dt / dx),
                            0.5 * (1.0 + w), 0.5 * (1.0 - w), 1.0 - w, 1.0 + w};
    const AdjCoef<float> F{(float)D.g1, (float)D.gam, (float)D.w,  (float)D.d,   (float)D.c,
                           (float)D.hs, (float)D.ca,  (float)D.cb, (float)D.w1m, (float)D.w1p};
    return AdjCoefs{F, D};
}
struct AdjSweepParams {
    Geom G;
    double dx, dt, bias, gamma;
    AdjCoef<float> cf;
    AdjCoef<double> cd;
    const AdjCoefs* coefp;  // non-null: the coefficients in device memory, in place of cf / cd
    const void* state;      // sweep input in storage precision (FP64 primitives or FP32 conserved)
    const void* ubar_out;   // adjoint of the sweep output (T, conserved SoA, same layout)
    void* ubar_in;          // adjoint of the sweep input (written)
};

// The coefficients of every sweep of `nsteps` steps from the forward pass's dts (device memory):
// sweep m of step s (m = 0..nsw - 1; dt/2 for the X sweeps of a 2D step) at out[s * nsw + m].
__global__ void adjoint_coef_kernel(const double* dts, int nsteps, int nsw, double dx, double gam, double w,
                                    AdjCoefs* out);

// Transmissive mirror (exact for up to two cells out) or periodic wrap, clamped into the line for
// the positions further out that only feed discarded halo work.
CG_D int adj_map(int i, int n, bool per) {
    if (per) {
        if (i >= 0 && i < n) return i;
        if (i < 0 && i >= -n) return i + n;
        if (i >= n && i < 2 * n) return i - n;
        return ((i % n) + n) % n;
    }
    int m = i < 0 ? -1 - i : (i >= n ? 2 * n - 1 - i : i);
    return m < 0 ? 0 : (m >= n ? n - 1 : m);
}

// Loads and stores of the lines a thread carries: one (float, double), or two (f2) -- adjacent rows
// (X sweep, two scalar accesses) or adjacent columns (Y sweep, one 8-byte access when both exist).
// q0/q1 are the offsets of the two lines; an incomplete pair repeats the first line and stores it once.
CG_D float ld_lanes(const float* p, size_t q0, size_t, bool, float) { return p[q0]; }
CG_D double ld_lanes(const double* p, size_t q0, size_t, bool, double) { return p[q0]; }
CG_D f2 ld_lanes(const float* p, size_t q0, size_t q1, bool vec, f2) {
    if (vec) return f2{*reinterpret_cast<const float2*>(p + q0)};
    return f2{make_float2(p[q0], p[q1])};
}
CG_D void st_lanes(float* p, size_t q0, size_t, bool, bool, float v) { p[q0] = v; }
CG_D void st_lanes(double* p, size_t q0, size_t, bool, bool, double v) { p[q0] = v; }
CG_D void st_lanes(float* p, size_t q0, size_t q1, bool vec, bool two, f2 v) {
    if (vec) {
        *reinterpret_cast<float2*>(p + q0) = v.v;
    } else {
        p[q0] = v.v.x;
        if (two) p[q1] = v.v.y;
    }
}

// Five-field vectors in shared memory, field f of slot x at arr[f * NW + x].  WIDE, for cell pairs
// (f2): fields 0-1 and 2-3 share one 16-byte word each instead (the first four field planes read
// as two float4 planes), so a vector moves in three shared-memory instructions instead of five;
// `arr` is then 16-byte aligned and NW even.
template <int NW, bool WIDE, class V>
CG_D void sv_st(V* arr, int x, const V* v) {
#pragma unroll
    for (int f = 0; f < 5; f++) arr[f * NW + x] = v[f];
}
template <int NW, bool WIDE, class V>
CG_D void sv_ld(const V* arr, int x, V* v) {
#pragma unroll
    for (int f = 0; f < 5; f++) v[f] = arr[f * NW + x];
}
template <int NW, bool WIDE>
CG_D void sv_st(f2* arr, int x, const f2* v) {
    if constexpr (WIDE) {
        static_assert(NW % 2 == 0, "16-byte planes");
        float4* a4 = reinterpret_cast<float4*>(arr);
        a4[x] = make_float4(v[0].v.x, v[0].v.y, v[1].v.x, v[1].v.y);
        a4[NW + x] = make_float4(v[2].v.x, v[2].v.y, v[3].v.x, v[3].v.y);
        arr[4 * NW + x] = v[4];
    } else {
#pragma unroll
        for (int f = 0; f < 5; f++) arr[f * NW + x] = v[f];
    }
}
template <int NW, bool WIDE>
CG_D void sv_ld(const f2* arr, int x, f2* v) {
    if constexpr (WIDE) {
        const float4* a4 = reinterpret_cast<const float4*>(arr);
        const float4 p = a4[x], q = a4[NW + x];
        v[0].v = make_float2(p.x, p.y);
        v[1].v = make_float2(p.z, p.w);
        v[2].v = make_float2(q.x, q.y);
        v[3].v = make_float2(q.z, q.w);
        v[4] = arr[4 * NW + x];
    } else {
#pragma unroll
        for (int f = 0; f < 5; f++) v[f] = arr[f * NW + x];
    }
}

// Tiles of P positions along a line of n cells.  An interior cell's adjoint gathers the
// contributions of its two neighbours, so a tile updates positions 3 .. P - 4 (P - 6 cells) and
// starts 3 cells before its first one; a cell within two of a line end also gathers from the ghost
// position two away, so it is updated only at positions 4 .. P - 5.  Tile 0 starts at cell -4;
// the tiles cover cells 0 .. n - 3 this way, and the last two cells join the last tile where they
// sit within its position P - 5, else one more tile (starting at cell n - 6) updates them.
struct AdjTiles {
    int n, P;
    CG_HD int first(int ts) const { return ts == 0 ? 0 : (P - 7) + (ts - 1) * (P - 6); }
    CG_HD int start(int ts) const { return ts == 0 ? -4 : first(ts) - 3; }
    CG_HD int regular() const {
        const int m = n - 2;
        return 1 + (m > P - 7 ? (m - (P - 7) + (P - 6) - 1) / (P - 6) : 0);
    }
    CG_HD bool extra() const { return n - 1 - start(regular() - 1) > P - 5; }
    CG_HD int count() const { return regular() + (extra() ? 1 : 0); }
    // the updated cells [lo, hi) and the start cell s (at position 0) of tile ts
    CG_HD void range(int ts, int& lo, int& hi, int& s) const {
        const int r = regular();
        if (ts < r) {
            lo = first(ts);
            s = start(ts);
            hi = ts < r - 1 ? first(ts + 1) : (extra() ? n - 2 : n);
        } else {
            lo = n - 2;
            hi = n;
            s = n - 6;
        }
    }
};

template <class V, class S, bool PRIM, int AX, int LIM, int P, int W>
__global__ void __launch_bounds__(P * W, (P * W >= 512 ? 1 : (Lane<V>::N == 2 ? 512 / (P * W) : (sizeof(V) == 4 ? 3 : 1))))
    adjoint_sweep_kernel(AdjSweepParams a) {
    using T = typename Lane<V>::S;
    constexpr int NL = Lane<V>::N;
    static_assert(!PRIM || NL == 1, "primitive storage is the FP64 one-line path");
    constexpr int NW = P * W;
    extern __shared__ __align__(16) unsigned char adj_smem[];
    static_assert(NW % 2 == 0, "every five-field array starts 16-byte aligned");  // (sv_st / sv_ld WIDE)
    V* sA = (V*)adj_smem;   // [5]  state
    V* sB = sA + 5 * NW;    // [5]  Ubar' (phase 0-2), then the contribution to the right neighbour
    V* sC = sB + 5 * NW;    // [10] A,B evolved states (1-2), then contributions to self and left neighbour
    V* sD = sC + 10 * NW;   // [10] Abar of the right state, Bbar of the left state per face
    // [15] X sweep: slope sl and reverse factors P, Q of each cell (phase 1 -> 3); the Y sweep keeps
    // them in the thread's registers (its blocks are bound by shared-memory instruction issue; in
    // the X sweep the registers spill)
    constexpr bool kRegSlope = AX == 1;
    // Y: five-field vectors in 16-byte shared-memory words (150.7 against 154 us per 2048^2 sweep);
    // in the X sweep the same measured slower (121.9 against 119 us)
    constexpr bool kWide = AX == 1;
    // X: the cell's right-face state, its adjoint and the contribution to the cell itself stay in
    // registers between the phases that write and read them (in the Y sweep, whose registers also
    // hold the slope factors, they spill)
    constexpr bool kRegOwn = AX == 0;
    // the adjoint of B, computed at the end of phase 2 and read at the start of phase 3, stays in
    // registers in both sweeps
    constexpr bool kRegLb = true;
    V* sE = sD + 10 * NW;
    const Geom& G = a.G;
    const int along = AX == 0 ? threadIdx.x : threadIdx.y;
    const int across = AX == 0 ? threadIdx.y : threadIdx.x;
    const int n = AX == 0 ? G.nx : G.ny;
    const int nl = AX == 0 ? G.ny : G.nx;
    const AdjTiles tiles{n, P};
    const int ntile_s = tiles.count();                 // tiles along the sweep axis
    const int ntiles = ntile_s * ((nl + W * NL - 1) / (W * NL));
    const bool per = G.bc == 1;
    // shared index of (across, position): positions contiguous for X, lines contiguous for Y
    auto si = [&](int pos) { return AX == 0 ? across * P + pos : pos * W + across; };
    auto gq = [&](int line, int pos) -> size_t {
        return AX == 0 ? (size_t)line * G.pitch + pos : (size_t)pos * G.pitch + line;
    };
    AdjCoef<T> K;
    if constexpr (sizeof(T) == 4) K = a.coefp ? a.coefp->f : a.cf;
    else K = a.coefp ? a.coefp->d : a.cd;
    const AdjFlux<V> F{bcv<V>(K.g1), bcv<V>(-K.g1), bcv<V>(T(-0.5) * K.g1)};
    const AdjSlope<V> Sl{bcv<V>(K.ca), bcv<V>(K.cb), bcv<V>(K.w1m), bcv<V>(K.w1p)};
    const V d = bcv<V>(K.d), c = bcv<V>(K.c), hs = bcv<V>(K.hs);
    const V zero = bcv<V>(0);
    const S* st = (const S*)a.state;
    const T* ubo = (const T*)a.ubar_out;
    const int me = si(along);

    // This thread's place in tile t: position k along the sweep, the tile's updated cells
    // [lo, hi), lines l0 and l1 (= l0 when the second lane has no line of its own).
    struct Place {
        int k, lo, hi, l0, l1;
        bool lok, two, vec;
    };
    auto place = [&](int t) {
        Place q;
        q.l0 = ((t / ntile_s) * W + across) * NL;
        q.lok = q.l0 < nl;
        q.two = NL == 2 && q.l0 + 1 < nl;
        q.vec = AX == 1 && q.two;  // adjacent columns: one 8-byte access
        q.l1 = q.two ? q.l0 + 1 : q.l0;
        int s0;
        tiles.range(t % ntile_s, q.lo, q.hi, s0);
        q.k = s0 + along;
        return q;
    };
    // Inputs at a place, as stored (FP64: primitives), fetched one tile ahead into registers.
    V ru[5], rb[5];
    auto fetch = [&](const Place& q) {
        ru[0] = ru[4] = bcv<V>(1);
        ru[1] = ru[2] = ru[3] = zero;
#pragma unroll
        for (int f = 0; f < 5; f++) rb[f] = zero;
        if (q.lok) {
            const int m = adj_map(q.k, n, per);
            const size_t q0 = gq(q.l0, m), q1 = gq(q.l1, m);
#pragma unroll
            for (int f = 0; f < 5; f++) ru[f] = ld_lanes(st + f * G.fstride, q0, q1, q.vec, V{});
            if (per || (q.k >= 0 && q.k < n)) {
#pragma unroll
                for (int f = 0; f < 5; f++) rb[f] = ld_lanes(ubo + f * G.fstride, q0, q1, q.vec, V{});
            }
        }
    };

    int t = blockIdx.x;
    if (t < ntiles) fetch(place(t));
    for (; t < ntiles; t += gridDim.x) {
        const Place q = place(t);
        const int k = q.k;
        const bool lok = q.lok;
        // ---- 0: state and Ubar' at this position
        V ub_own[5];
        {
            V u[5];
            if constexpr (PRIM) {  // Euler/EulerStateVector.cpp:55-66
                const T* v = ru;
                u[0] = v[0];
                u[1] = v[0] * v[1];
                u[2] = v[0] * v[2];
                u[3] = v[0] * v[3];
                u[4] = v[0] * (T(0.5) * ((v[1] * v[1] + v[2] * v[2]) + v[3] * v[3]) + v[4] / (K.g1 * v[0]));
            } else {
#pragma unroll
                for (int f = 0; f < 5; f++) u[f] = ru[f];
            }
            sv_st<NW, kWide>(sA, me, u);
            sv_st<NW, kWide>(sB, me, rb);
#pragma unroll
            for (int f = 0; f < 5; f++) ub_own[f] = rb[f];
        }
        __syncthreads();
        // the next tile's inputs load while this one is computed (Y: from phase 3 on, so that the
        // registers they occupy are free during the flux reverse of phase 2: spills 52 -> 20 bytes,
        // 150.3 -> 149.2 us per 2048^2 sweep)
        constexpr bool kLateFetch = AX == 1;
        if (!kLateFetch && t + (int)gridDim.x < ntiles) fetch(place(t + gridDim.x));
        auto ld = [&](const V* arr, int pos, V* out) { sv_ld<NW, kWide>(arr, si(pos), out); };
        // ---- 1: half-step evolution of every cell with both neighbours in the tile.  kRegOwn: values
        // that only this thread reads in the next phase stay in its registers -- the cell's
        // right-face state B (phase 2), the adjoint of B (phase 3), the contribution to the cell
        // itself (phase 4; also stored, for the gather at line ends)
        V sl[5], Pf[5], Qf[5], B[5], Lb[5], gc[5];
        if (lok && along >= 1 && along < P - 1) {
            V ul[5], uc[5], ur[5], A[5];
            ld(sA, along - 1, ul);
            ld(sA, along, uc);
            ld(sA, along + 1, ur);
            adj_evolve<V, AX, LIM>(F, Sl, ul, uc, ur, hs, A, B, sl, Pf, Qf);
            sv_st<NW, kWide>(sC, me, A);
            if (!kRegOwn) sv_st<NW, kWide>(sC + 5 * NW, me, B);
            if (!kRegSlope) {
                sv_st<NW, kWide>(sE, me, sl);
                sv_st<NW, kWide>(sE + 5 * NW, me, Pf);
                sv_st<NW, kWide>(sE + 10 * NW, me, Qf);
            }
        }
        __syncthreads();
        // ---- 2: FORCE reverse at the face between this cell (k) and the next (k + 1)
        if (along >= 1 && along < P - 2) {
            V Rb[5] = {zero, zero, zero, zero, zero};
#pragma unroll
            for (int f = 0; f < 5; f++) Lb[f] = zero;
            if (lok && (per || (k >= -1 && k <= n - 1))) {
                V R[5], Fb[5], bn[5], bm[5];
                const int nx1 = si(along + 1);
                if (!kRegOwn) sv_ld<NW, kWide>(sC + 5 * NW, me, B);
                sv_ld<NW, kWide>(sC, nx1, R);
                sv_ld<NW, kWide>(sB, nx1, bn);
                sv_ld<NW, kWide>(sB, me, bm);
#pragma unroll
                for (int f = 0; f < 5; f++) Fb[f] = vmul(d, vsub(bn[f], bm[f]));
                adj_force_vjp<V, AX>(F, B, R, c, d, Fb, Lb, Rb);
            }
            if (!kRegLb) sv_st<NW, kWide>(sD, me, Lb);  // adjoint of B_k
            sv_st<NW, kWide>(sD + 5 * NW, me, Rb);        // adjoint of A_{k+1}
        }
        __syncthreads();
        if (kLateFetch && t + (int)gridDim.x < ntiles) fetch(place(t + gridDim.x));
        // ---- 3: half-step reverse of this cell; neither sB nor sC is read in this phase
        if (along >= 2 && along < P - 2) {
            V gl[5] = {zero, zero, zero, zero, zero}, gr[5] = {zero, zero, zero, zero, zero};
#pragma unroll
            for (int f = 0; f < 5; f++) gc[f] = zero;
            if (lok && (per || (k >= -1 && k <= n))) {
                V uc[5], Ab[5];
                ld(sA, along, uc);
                if (!kRegSlope) {
                    ld(sE, along, sl);
                    ld(sE + 5 * NW, along, Pf);
                    ld(sE + 10 * NW, along, Qf);
                }
                if (!kRegLb) sv_ld<NW, kWide>(sD, me, Lb);
                sv_ld<NW, kWide>(sD + 5 * NW, si(along - 1), Ab);
                adj_evolve_vjp<V, AX>(F, uc, sl, Pf, Qf, hs, Ab, Lb, gl, gc, gr);
            }
            sv_st<NW, kWide>(sC, me, gc);
            sv_st<NW, kWide>(sC + 5 * NW, me, gl);
            sv_st<NW, kWide>(sB, me, gr);
        }
        __syncthreads();
        // ---- 4: gather for the updated cells
        if (lok && k >= q.lo && k < q.hi) {
            V acc[5];
#pragma unroll
            for (int f = 0; f < 5; f++) acc[f] = ub_own[f];
            if (k >= 2 && k <= n - 3) {
                // interior (n >= 5): the right neighbour of k - 1, k itself, the left neighbour of k + 1
                V gr_l[5], gl_r[5];
                if (!kRegOwn) sv_ld<NW, kWide>(sC, me, gc);
                sv_ld<NW, kWide>(sB, si(along - 1), gr_l);
                sv_ld<NW, kWide>(sC + 5 * NW, si(along + 1), gl_r);
#pragma unroll
                for (int f = 0; f < 5; f++) acc[f] = vadd(acc[f], vadd(vadd(gr_l[f], gc[f]), gl_r[f]));
            } else
#pragma unroll
            for (int dd = -2; dd <= 2; dd++) {
                const int i = k + dd;
                if (!per && (i < -1 || i > n)) continue;
                if (per && dd - n >= -2) continue;  // same physical cell as an earlier dd (n <= 4)
                const int x = si(along + dd);
#pragma unroll
                for (int q = -1; q <= 1; q++) {
                    const int tgt = per ? ((i + q) % n + n) % n : (i + q < 0 ? -1 - (i + q) : (i + q >= n ? 2 * n - 1 - (i + q) : i + q));
                    if (tgt != k) continue;
                    const V* src = q == -1 ? sC + 5 * NW : (q == 0 ? sC : sB);
                    V g[5];
                    sv_ld<NW, kWide>(src, x, g);
#pragma unroll
                    for (int f = 0; f < 5; f++) acc[f] = vadd(acc[f], g[f]);
                }
            }
            T* ubi = (T*)a.ubar_in;
            const size_t q0 = gq(q.l0, k), q1 = gq(q.l1, k);
#pragma unroll
            for (int f = 0; f < 5; f++) st_lanes(ubi + f * G.fstride, q0, q1, q.vec, q.two, acc[f]);
        }
        __syncthreads();  // phase 4 reads sB and sC, which the next tile's phases 0 and 1 overwrite
    }
}

// Loss L = 1/2 sum (rho - target)^2 over the grid, seed Ubar = (rho - target, 0, 0, 0, 0).
// One block per row; the row sums are added in row order by adjoint_loss_final_kernel.
template <class T, class S>
__global__ void __launch_bounds__(256) adjoint_loss_kernel(Geom G, const S* state, const double* target, T* ubar,
                                                           double* row_sums) {
    const int i = blockIdx.x;
    double acc = 0.0;
    for (int j = threadIdx.x; j < G.nx; j += 256) {
        const size_t q = (size_t)i * G.pitch + j;
        const double e = (double)state[q] - target[(size_t)i * G.nx + j];
        acc += 0.5 * e * e;
        ubar[q] = T(e);
#pragma unroll
        for (int f = 1; f < 5; f++) ubar[f * G.fstride + q] = T(0);
    }
    __shared__ double red[256];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) row_sums[i] = red[0];
}

// Fixed-order sum of the row sums: lane l adds rows l, l + 32, ... in order, then a fixed shuffle tree.
static __global__ void __launch_bounds__(32) adjoint_loss_final_kernel(const double* row_sums, int n, double* loss) {
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += 32) s += row_sums[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) *loss = s;
}

// Gradient with respect to the initial primitives: Pbar = (dU/dP)^T Ubar at the initial state,
// written as AoS doubles (the layout of cosmos_grid_set_prim), evaluated in the adjoint's precision T
// (1/(gamma - 1) formed on the host for FP32).
template <class T, class S, bool PRIM>
__global__ void adjoint_grad_kernel(Geom G, double gamma, T ig1, const S* state, const T* ubar, double* grad) {
    const size_t ncell = (size_t)G.nx * G.ny;
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < ncell; c += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(c / G.nx), j = (int)(c % G.nx);
        const size_t q = (size_t)i * G.pitch + j;
        T v[5], u[5];
#pragma unroll
        for (int f = 0; f < 5; f++) {
            v[f] = (T)state[f * G.fstride + q];
            u[f] = ubar[f * G.fstride + q];
        }
        T rho, vx, vy, vz;
        if (PRIM) {
            rho = v[0]; vx = v[1]; vy = v[2]; vz = v[3];
        } else {
            rho = v[0];
            const T ir = adj_div(T(1), rho);
            vx = v[1] * ir; vy = v[2] * ir; vz = v[3] * ir;
        }
        const T vv = vx * vx + vy * vy + vz * vz;
        double* o = grad + 5 * c;
        o[0] = (double)(u[0] + u[1] * vx + u[2] * vy + u[3] * vz + u[4] * T(0.5) * vv);
        o[1] = (double)(rho * (u[1] + u[4] * vx));
        o[2] = (double)(rho * (u[2] + u[4] * vy));
        o[3] = (double)(rho * (u[3] + u[4] * vz));
        o[4] = sizeof(T) == 8 ? (double)u[4] / (gamma - 1.0) : (double)(u[4] * ig1);
    }
}

}  // namespace cg

namespace cg {

// Launch the sweep adjoint for one axis.  X tiles: lines of 128 positions (120 updated cells; 128
// threads, four blocks per SM: smaller blocks wait less at the phase barriers) in FP32, of 256 in
// FP64; Y tiles: 64 positions (56 cells) x 4 threads across (256 threads; four column pairs keep
// each row access a whole 32-byte sector).  FP32 carries two lines per thread (f2: two rows for X,
// two adjacent columns for Y), FP64 one.  Persistent: as many blocks as
// stay resident, each walking tiles t, t + gridDim.x, ... with the next tile's inputs in flight.
template <class V, class S, bool PRIM, int AX, int LIM>
cudaError_t launch_adjoint_sweep_t(const AdjSweepParams& a, cudaStream_t st) {
    constexpr int P = AX == 0 ? (Lane<V>::N == 2 ? 128 : 256) : 64;
    constexpr int W = AX == 0 ? 1 : 4;
    constexpr int LB = W * Lane<V>::N;  // lines per block
    const size_t smem = (size_t)(AX == 1 ? 30 : 45) * P * W * sizeof(V);
    auto kern = adjoint_sweep_kernel<V, S, PRIM, AX, LIM, P, W>;
    // per instantiation: the attribute and the resident-block count (one GPU model per process)
    static int resident = 0;
    if (!resident) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        int dev = 0, sms = 0, per = 0;
        if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
        if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
        if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, P * W, smem)) != cudaSuccess) return e;
        resident = sms * std::max(per, 1);
    }
    const Geom& G = a.G;
    const int n = AX == 0 ? G.nx : G.ny, nl = AX == 0 ? G.ny : G.nx;
    const long long ntiles = (long long)AdjTiles{n, P}.count() * ((nl + LB - 1) / LB);
    const int blocks = (int)std::min<long long>(ntiles, resident);
    dim3 block = AX == 0 ? dim3(P, W) : dim3(W, P);
    kern<<<blocks, block, smem, st>>>(a);
    return cudaGetLastError();
}

template <class V, class S, bool PRIM>
cudaError_t launch_adjoint_sweep_any(const AdjSweepParams& a, int lim, cudaStream_t st) {
    const int ax = a.G.axis;
    if (ax == 0) {
        if (lim == 0) return launch_adjoint_sweep_t<V, S, PRIM, 0, 0>(a, st);
        if (lim == 1) return launch_adjoint_sweep_t<V, S, PRIM, 0, 1>(a, st);
        return launch_adjoint_sweep_t<V, S, PRIM, 0, 2>(a, st);
    }
    if (lim == 0) return launch_adjoint_sweep_t<V, S, PRIM, 1, 0>(a, st);
    if (lim == 1) return launch_adjoint_sweep_t<V, S, PRIM, 1, 1>(a, st);
    return launch_adjoint_sweep_t<V, S, PRIM, 1, 2>(a, st);
}

template <class T, class S, bool PRIM>
cudaError_t launch_adjoint_loss_t(const Geom& G, const void* state, const double* target, void* ubar, double* row_sums,
                                  double* loss, cudaStream_t st) {
    adjoint_loss_kernel<T, S><<<G.ny, 256, 0, st>>>(G, (const S*)state, target, (T*)ubar, row_sums);
    adjoint_loss_final_kernel<<<1, 32, 0, st>>>(row_sums, G.ny, loss);
    return cudaGetLastError();
}

template <class T, class S, bool PRIM>
cudaError_t launch_adjoint_grad_t(const Geom& G, double gamma, const void* state, const void* ubar, double* grad,
                                  cudaStream_t st) {
    const size_t ncell = (size_t)G.nx * G.ny;
    const int blocks = (int)std::min<size_t>((ncell + 255) / 256, (size_t)device_sm_count() * 16);
    adjoint_grad_kernel<T, S, PRIM>
        <<<blocks, 256, 0, st>>>(G, gamma, T(1.0 / (gamma - 1.0)), (const S*)state, (const T*)ubar, grad);
    return cudaGetLastError();
}

}  // namespace cg
