// FP32 bulk physics for the special-relativistic system: conserved FP32 storage (D, Sx, Sy, Sz,
// tau), FP32 slopes, half-step evolution, FORCE flux and update, and a conserved-to-primitive solve
// whose Newton iterations finish in FP64.
//
// The primitive recovery is the reference's (RelativisticEuler/RelativisticEulerStateVector.cpp:
// 30-101): the quartic in xi built from dc = D / sqrt(q) and ec = (D + tau) / sqrt(q),
// q = (tau + D)^2 - |S|^2 (guarded at 1e-8), solved by Newton from xi = 1, then W, h, rho, v, p,
// with rho and p floored at 1e-8.  Here the iteration runs in FP32 to FP32 accuracy first; FP64
// Newton steps from that root follow (the coefficients formed again in FP64; square root and
// division as refined FP32 estimates) until a step is below 1e-7, after which quadratic
// convergence has put the root within 1e-14 -- the reference's |step| < 1e-8 criterion holds on
// the next step.  The FP64 stage runs for every solve when
// c2p64_above <= 0; otherwise only for states whose FP32 Lorentz factor exceeds c2p64_above (or
// whose FP32 iteration did not converge).  Primitives are then formed in FP32.  The iteration caps
// are 40 (FP32, from xi = 1; physical states converge in well under 20) and 8 (FP64, from the FP32
// iterate) instead of the reference's 1000: beyond them the state has no physical root (on GB300
// one FP64 iteration costs as much as a whole FP32 recovery), and the result is the last iterate
// as in the reference, flagged in the status word.
//
// A sweep costs five primitive recoveries per cell (the two extrapolated states of the cell, the
// two face states and the Richtmyer state of one face), against about two dozen in the reference,
// which converts every intermediate state back and forth.
#pragma once
#include "device_common.cuh"
#include "physics_fast.cuh"

namespace cg {

struct SRFastParams {
    float wa, wb, hom, hop;  // bias factors as in NewtonFastParams
    float gf;                // gamma
    double g;                // gamma (FP64 stage)
    float w64;               // Lorentz factor above which the FP64 stage runs (0: always)
    // constants of gamma, formed on the host (sr_fast_constants): (g-1)/g, -1/g^2, (g-1)/g^2,
    // (g-2)/g, g/(g-1), in FP32 and for the FP64 stage
    float gr, c0, grg, g2g, hfac;
    double grd, k0d, grgd, g2gd;
};

inline void sr_fast_constants(SRFastParams& P, double g) {
    P.gf = (float)g;
    P.g = g;
    P.grd = (g - 1.0) / g;
    P.k0d = -1.0 / (g * g);
    P.grgd = P.grd / g;
    P.g2gd = (g - 2.0) / g;
    P.gr = (float)P.grd;
    P.c0 = (float)P.k0d;
    P.grg = (float)P.grgd;
    P.g2g = (float)P.g2gd;
    P.hfac = (float)(g / (g - 1.0));
}

struct SRPrim32 {
    float rho, vx, vy, vz, p, W, h;
};

// FP64 helpers of the recovery's FP64 stage: within FP32's normal range an FP32 estimate refined
// by one FP64 Newton step (relative error about 1e-14; no FP64 division or square root -- on
// GB300 the FP64 rate is 1/64 of FP32); outside it (states far beyond any physical range) IEEE.
CG_D double rcp64(double a) {
    const double m = fabs(a);
    if (m > 1e-30 && m < 1e30) {
        const double r = (double)frcp((float)a);
        return r * fma(-a, r, 2.0);
    }
    return 1.0 / a;
}
CG_D double rsqrt64(double a) {
    if (a > 1e-30 && a < 1e30) {
        const double r = (double)frsqrt((float)a);
        return r * fma(-0.5 * a * r, r, 1.5);
    }
    return 1.0 / sqrt(a);
}

struct SRStage64 {
    float x;
    bool conv;
};

// The recovery's FP64 stage: Newton on the quartic with coefficients in FP64 (they cancel at high
// Lorentz factor) from x0 (the FP32 iterate, or the reference's start 1), 1/sqrt(q) and each
// step's 1/f' through rcp64 / rsqrt64.  Out of line: kernels call the recovery at dozens of sites
// (39 per GR source step) and this rarely taken stage would otherwise be inlined at each; it is
// kept small because its registers add to those live at every call site.
static __device__ __noinline__ SRStage64 sr_c2p_stage64(double grd, double k0, double grgd, double g2gd, float D,
                                                        float Sx, float Sy, float Sz, float tau, float x0) {
    const double Dd = D, td = tau;
    double qd = (td + Dd) * (td + Dd) - ((double)Sx * Sx + (double)Sy * Sy + (double)Sz * Sz);
    qd = qd < 1e-8 ? 1e-8 : qd;
    const double iqd = rsqrt64(qd);
    const double dcd = Dd * iqd, ecd = (Dd + td) * iqd;
    const double k1 = -2.0 * dcd * grgd;
    const double k2 = g2gd * (ecd * ecd - 1.0) + 1.0 - dcd * dcd * grd * grd;
    const double k4 = ecd * ecd - 1.0;
    const double et = 2.0 * dcd * grd;
    double xd = x0;
    // from the FP32 iterate a solvable state converges in one to three steps; a state without a
    // physical root gives up after 8 (reported through the status word)
    for (int it = 0; it < 8; it++) {
        const double x2 = xd * xd;
        const double f = k4 * x2 * xd * (xd - et) + k2 * x2 + k1 * xd + k0;
        const double fp = k1 + 2.0 * k2 * xd + 4.0 * k4 * x2 * xd - 3.0 * et * k4 * x2;
        const double step = f * rcp64(fp);
        xd -= step;
        if (fabs(step) < 1e-7) return SRStage64{(float)xd, true};
    }
    return SRStage64{(float)xd, false};
}

// Primitive recovery of one FP32 conserved state; sets bit 0 of *flags when neither stage converged.
// Near the horizon the reference's recovery meets states without a physical root, whose garbage
// primitives grow through the W cap and the fluxes to magnitudes beyond FP32's range (|S| ~ 1e30;
// the reference's FP64 holds them, with garbage values of its own): where the coefficients or the
// result leave FP32's range, the result is the floor state (rho = p = 1e-8 at rest).
CG_D SRPrim32 sr_c2p_fast(const SRFastParams& P, const float* u, int* flags) {
    const float D = u[0], Sx = u[1], Sy = u[2], Sz = u[3], tau = u[4];
    const float gr = P.gr;
    float q = (tau + D) * (tau + D) - (Sx * Sx + Sy * Sy + Sz * Sz);
    q = q < 1e-8f ? 1e-8f : q;
    const float iq = frsqrt(q);
    const float dc = D * iq, ec = (D + tau) * iq;
    const float c0 = P.c0;
    const float c1 = -2.0f * dc * P.grg;
    const float c2 = P.g2g * (ec * ec - 1.0f) + 1.0f - dc * dc * gr * gr;
    const float c4 = ec * ec - 1.0f;
    const float eta = 2.0f * dc * gr;
    // coefficients beyond FP32's range (or a non-finite state): no iteration, the floor state below
    const bool inrange = fabsf(c4) + fabsf(c2) + fabsf(c1) < 1e30f;
    float x = inrange ? 1.0f : 0.0f;
    bool conv = false;
    for (int it = 0; inrange && it < 40; it++) {
        const float x2 = x * x;
        const float f = c4 * x2 * x * (x - eta) + c2 * x2 + c1 * x + c0;
        const float fp = c1 + 2.0f * c2 * x + 4.0f * c4 * x2 * x - 3.0f * eta * c4 * x2;
        const float nx = x - fdiv(f, fp);
        const bool done = fabsf(nx - x) <= 1e-6f * fabsf(x);
        x = nx;
        if (done) { conv = true; break; }
    }
    float W = 0.5f * ec * x * (1.0f + fsqrt(1.0f + fdiv(4.0f * gr * (1.0f - dc * x), ec * ec * x * x)));
    if (inrange && (!conv || !(W <= P.w64))) {  // also a non-finite iterate
        // from the FP32 iterate unless it ran off (then from the reference's start, 1)
        const SRStage64 r = sr_c2p_stage64(P.grd, P.k0d, P.grgd, P.g2gd, D, Sx, Sy, Sz, tau, fabsf(x) < 1e3f ? x : 1.0f);
        conv = r.conv;
        x = r.x;
        W = 0.5f * ec * x * (1.0f + fsqrt(1.0f + fdiv(4.0f * gr * (1.0f - dc * x), ec * ec * x * x)));
    }
    SRPrim32 r;
    r.W = W;
    r.h = frcp(dc * x);
    r.rho = fdiv(D, W);
    const float rhw = r.rho * r.h * W * W;
    const float irhw = frcp(rhw);
    r.vx = Sx * irhw;
    r.vy = Sy * irhw;
    r.vz = Sz * irhw;
    r.p = (rhw - D) - tau;
    r.rho = r.rho < 1e-8f ? 1e-8f : r.rho;
    r.p = r.p < 1e-8f ? 1e-8f : r.p;
    // one test for every output: non-finite or beyond 1e30 (a NaN or an infinity carries through the sum)
    if (!(fabsf(W) + fabsf(r.h) + r.rho + r.p + fabsf(r.vx) + fabsf(r.vy) + fabsf(r.vz) < 1e30f)) {
        conv = false;
        r.rho = r.p = 1e-8f;
        r.vx = r.vy = r.vz = 0.0f;
        r.W = 1.0f;
        r.h = 1.0f + P.hfac;  // 1 + (p / rho) gamma / (gamma - 1) at the floors
    }
    if (!conv && flags) *flags |= 1;
    return r;
}

// RelativisticEuler/RelativisticEulerStateVector.cpp:138-220 (x) / :227-309 (y) from primitives
template <int AXIS>
CG_D void sr_flux_prim(const SRPrim32& c, float* f) {
    const float rhw = c.rho * c.h * c.W * c.W;
    const float vn = AXIS == 0 ? c.vx : c.vy;
    f[0] = c.rho * c.W * vn;
    f[1] = rhw * c.vx * vn + (AXIS == 0 ? c.p : 0.0f);
    f[2] = rhw * c.vy * vn + (AXIS == 1 ? c.p : 0.0f);
    f[3] = rhw * c.vz * vn;
    f[4] = ((rhw - c.p) - c.rho * c.W) * vn + c.p * vn;
}

// Flux of a conserved state: primitive recovery (with its floors), then the flux of the primitives
template <int AXIS>
CG_D void sr_flux_fast(const SRFastParams& P, const float* u, float* f, int* flags) {
    sr_flux_prim<AXIS>(sr_c2p_fast(P, u, flags), f);
}

// Conserved state of primitives (RelativisticEuler/RelativisticEulerStateVector.cpp:116-136): W from
// v (clamped where v^2 > 1 - 1e-8), h from rho and p (RelativisticEulerEquationOfState.cpp:3-8)
CG_D void sr_cons_of(const SRFastParams& P, const SRPrim32& c, float* u) {
    const float v2 = c.vx * c.vx + c.vy * c.vy + c.vz * c.vz;
    // the reference's clamp of v^2 to 1 - 1e-8 (W <= 1e4), applied to 1 - v^2: in FP32, 1 - 1e-8
    // rounds to 1, which would make W infinite
    const float omv = 1.0f - v2;
    const float W = frsqrt(omv < 1e-8f ? 1e-8f : omv);
    const float h = 1.0f + fdiv(c.p, c.rho) * P.hfac;
    const float rhw = c.rho * h * W * W;
    u[0] = c.rho * W;
    u[1] = rhw * c.vx;
    u[2] = rhw * c.vy;
    u[3] = rhw * c.vz;
    u[4] = (rhw - c.p) - c.rho * W;
}

// Half-step evolution (Solvers/RelativisticEulerSolvers.cpp:148-199) of the two extrapolated states
template <int AXIS, int LIM>
CG_D void sr_recon_fast(const SRFastParams& P, const NewtonFastParams& NP, const float* ul, const float* um,
                        const float* ur, float half_dtdx, float* fl, float* fr, int* flags) {
    float s[5], a[5], b[5], Fa[5], Fb[5];
    nf_slope<LIM>(NP, ul, um, ur, s);
#pragma unroll
    for (int k = 0; k < 5; k++) { a[k] = fmaf(-0.5f, s[k], um[k]); b[k] = fmaf(0.5f, s[k], um[k]); }
    sr_flux_fast<AXIS>(P, a, Fa, flags);
    sr_flux_fast<AXIS>(P, b, Fb, flags);
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const float ev = half_dtdx * (Fa[k] - Fb[k]);
        fl[k] = a[k] + ev;
        fr[k] = b[k] + ev;
    }
}

// FORCE flux (Solvers/RelativisticEulerFirstOrderSolver.cpp:3-60).  The reference hands FORCE the
// evolved face states as primitives (with the recovery's floors applied) and converts them back,
// so the face states here are rebuilt from their recovered primitives before use.
template <int AXIS>
CG_D void sr_force_fast(const SRFastParams& P, const float* L, const float* R, float half_dtdx, float q_dxdt, float* F,
                        int* flags) {
    float uL[5], uR[5], fL[5], fR[5], us[5], fs[5];
    const SRPrim32 pL = sr_c2p_fast(P, L, flags), pR = sr_c2p_fast(P, R, flags);
    sr_cons_of(P, pL, uL);
    sr_cons_of(P, pR, uR);
    sr_flux_prim<AXIS>(pL, fL);
    sr_flux_prim<AXIS>(pR, fR);
#pragma unroll
    for (int k = 0; k < 5; k++) us[k] = fmaf(0.5f, uL[k] + uR[k], half_dtdx * (fL[k] - fR[k]));
    sr_flux_fast<AXIS>(P, us, fs, flags);
#pragma unroll
    for (int k = 0; k < 5; k++) F[k] = fmaf(0.25f, fL[k] + fR[k], fmaf(q_dxdt, uL[k] - uR[k], 0.5f * fs[k]));
}

// Solvers/RelativisticEulerSolvers.cpp:87-128 (2D: max(|vx|, |vy|) + c), c from
// RelativisticEuler/RelativisticEulerEquationOfState.cpp:3-18
CG_D float sr_wavespeed_fast(const SRFastParams& P, const float* u, int dims, int* flags) {
    const SRPrim32 c = sr_c2p_fast(P, u, flags);
    const float cs = fsqrt(fdiv(P.gf * c.p, c.rho * c.h));
    if (dims == 1) return speed_or_inf(u[0], u[4], fabsf(c.vx) + cs);
    return speed_or_inf(u[0], u[4], fmaxf(fabsf(c.vx), fabsf(c.vy)) + cs);
}

}  // namespace cg
