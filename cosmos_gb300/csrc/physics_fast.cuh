// FP32 bulk physics for the Newtonian system.  The algorithm is the reference's SLIC/FORCE step
// (same limiter formula with the +1e-5 clamps, same half-step evolution, same FORCE flux), with
// reformulations that are identities in exact arithmetic:
//  * the state stays conserved between operations -- the reference converts every evolved and
//    updated state to primitives and back (Euler/EulerStateVector.cpp:30-66, :91-94);
//  * divisions use one approximate reciprocal each (rho, the limiter ratio, the limiter bound);
//  * the limiters are written as min/max/select chains instead of branches;
//  * constants are folded (0.5 factors, the gradient-ratio 2).
// The sweep axis and the limiter are template parameters, so no run-time switch remains in the
// per-cell code.
#pragma once
#include "device_common.cuh"

namespace cg {

CG_D float frcp(float x) { return __fdividef(1.0f, x); }

struct NewtonFastParams {
    float g1;        // gamma - 1
    float hg1;       // (gamma - 1) / 2
    float gam;       // gamma
    float wa, wb;    // 0.5 (1 + bias), 0.5 (1 - bias)
    float hom, hop;  // (1 - bias) / 2, (1 + bias) / 2  (gradient ratio 2 / (om + op r) = 1 / (hom + hop r))
};

// Euler/EulerStateVector.cpp:68-89 (x) / :96-117 (y) on a conserved state
template <int AXIS>
CG_D void nf_flux(const NewtonFastParams& P, const float* u, float* f) {
    const float ir = frcp(u[0]);
    const float vn = (AXIS == 0 ? u[1] : u[2]) * ir;
    const float q = u[1] * u[1] + u[2] * u[2] + u[3] * u[3];
    const float p = P.g1 * u[4] - P.hg1 * q * ir;
    f[0] = AXIS == 0 ? u[1] : u[2];
    f[1] = AXIS == 0 ? u[1] * vn + p : u[1] * vn;
    f[2] = AXIS == 1 ? u[2] * vn + p : u[2] * vn;
    f[3] = u[3] * vn;
    f[4] = (u[4] + p) * vn;
}

// Solvers/SlopeLimiters.cpp:8-69 as select chains; `xi` = 2 / ((1-w) + (1+w) r)
template <int LIM>
CG_D float nf_limiter(const NewtonFastParams& P, float r) {
    const float xi = frcp(P.hom + P.hop * r);
    if (LIM == 0) {  // SuperBee
        const float hi = fminf(fminf(r, xi), 2.0f);
        const float v = r < 0.5f ? 2.0f * r : (r < 1.0f ? 1.0f : hi);
        return r < 0.0f ? 0.0f : v;
    } else if (LIM == 1) {  // van Leer
        const float v = fminf(__fdividef(2.0f * r, 1.0f + r), xi);
        return r < 0.0f ? 0.0f : v;
    }
    // MinBee: r for 0 <= r < 1, min(1, xi) above (xi > 1 > r whenever r < 1)
    return fmaxf(fminf(fminf(r, 1.0f), xi), 0.0f);
}

// Solvers/SlopeLimiters.cpp:71-101 with the +1e-5 clamps of numerator and denominator
template <int LIM>
CG_D void nf_slope(const NewtonFastParams& P, const float* ul, const float* uc, const float* ur, float* s) {
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const float dl = uc[k] - ul[k], dr = ur[k] - uc[k];
        const float num = fabsf(dl) < 1e-5f ? 1e-5f : dl;
        const float den = fabsf(dr) < 1e-5f ? 1e-5f : dr;
        s[k] = (P.wa * dl + P.wb * dr) * nf_limiter<LIM>(P, num * frcp(den));
    }
}

// Half-step evolution of a cell's extrapolated states (Solvers/EulerSolvers.cpp:163-223).
// half_dtdx = 0.5 dt/dx.  fl/fr receive the evolved left/right face states (conserved).
template <int AXIS, int LIM>
CG_D void nf_recon(const NewtonFastParams& P, const float* ul, const float* um, const float* ur, float half_dtdx,
                   float* fl, float* fr) {
    float s[5], a[5], b[5], Fa[5], Fb[5];
    nf_slope<LIM>(P, ul, um, ur, s);
#pragma unroll
    for (int k = 0; k < 5; k++) { a[k] = fmaf(-0.5f, s[k], um[k]); b[k] = fmaf(0.5f, s[k], um[k]); }
    nf_flux<AXIS>(P, a, Fa);
    nf_flux<AXIS>(P, b, Fb);
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const float ev = half_dtdx * (Fa[k] - Fb[k]);
        fl[k] = a[k] + ev;
        fr[k] = b[k] + ev;
    }
}

// FORCE flux (Solvers/EulerFirstOrderSolver.cpp:3-24) of conserved states L | R:
// 0.5 (LF + RI) with LF = 0.5 (fL + fR) + 0.5 (dx/dt)(L - R), RI = F(0.5 (L + R) + 0.5 (dt/dx)(fL - fR)).
template <int AXIS>
CG_D void nf_force(const NewtonFastParams& P, const float* L, const float* R, float half_dtdx, float q_dxdt,
                   float* F) {
    float fL[5], fR[5], us[5], fs[5];
    nf_flux<AXIS>(P, L, fL);
    nf_flux<AXIS>(P, R, fR);
#pragma unroll
    for (int k = 0; k < 5; k++) us[k] = fmaf(0.5f, L[k] + R[k], half_dtdx * (fL[k] - fR[k]));
    nf_flux<AXIS>(P, us, fs);
#pragma unroll
    for (int k = 0; k < 5; k++) F[k] = fmaf(0.25f, fL[k] + fR[k], fmaf(q_dxdt, L[k] - R[k], 0.5f * fs[k]));
}

// Solvers/EulerSolvers.cpp:87-128 (2D: max(|vx|, |vy| + c) as written in the reference)
CG_D float nf_wavespeed(const NewtonFastParams& P, const float* u, int dims) {
    const float ir = frcp(u[0]);
    const float vx = u[1] * ir, vy = u[2] * ir;
    const float p = P.g1 * u[4] - P.hg1 * (u[1] * u[1] + u[2] * u[2] + u[3] * u[3]) * ir;
    const float c = sqrtf(P.gam * p * ir);  // NaN for p < 0 is dropped by the max, as in the reference
    if (dims == 1) return fabsf(vx) + c;
    return fmaxf(fabsf(vx), fabsf(vy) + c);
}

}  // namespace cg
