// FP32 bulk physics for the Newtonian system.  The algorithm is the reference's SLIC/FORCE step
// (same limiter formula with the +1e-5 clamps, same half-step evolution, same FORCE flux), with
// two reformulations that are identities in exact arithmetic:
//  * the state stays conserved between operations -- the reference converts every evolved and
//    updated state to primitives and back (Euler/EulerStateVector.cpp:30-66, :91-94);
//  * divisions by the density use one reciprocal per state.
#pragma once
#include "device_common.cuh"

namespace cg {

CG_D float frcp(float x) { return __fdividef(1.0f, x); }

struct NewtonFastParams {
    float g1;        // gamma - 1
    float gam;       // gamma
    float wa, wb;    // 0.5 (1 + bias), 0.5 (1 - bias)
    float om, op;    // 1 - bias, 1 + bias (gradient ratio)
    int lim;
};

// Euler/EulerStateVector.cpp:68-89 / :96-117 on a conserved state
CG_D void nf_flux(const NewtonFastParams& P, const float* u, int axis, float* f) {
    const float ir = frcp(u[0]);
    const float vx = u[1] * ir, vy = u[2] * ir, vz = u[3] * ir;
    const float ke = 0.5f * (u[1] * vx + u[2] * vy + u[3] * vz);
    const float p = P.g1 * (u[4] - ke);
    const float vn = axis == 0 ? vx : vy;
    f[0] = axis == 0 ? u[1] : u[2];  // select, not an indexed register array
    f[1] = u[1] * vn + (axis == 0 ? p : 0.0f);
    f[2] = u[2] * vn + (axis == 1 ? p : 0.0f);
    f[3] = u[3] * vn;
    f[4] = (u[4] + p) * vn;
}

// Solvers/SlopeLimiters.cpp:3-101
CG_D float nf_limiter(const NewtonFastParams& P, float r) {
    if (r < 0.0f) return 0.0f;
    const float xi = __fdividef(2.0f, P.om + P.op * r);
    if (P.lim == 0) {
        if (r < 0.5f) return 2.0f * r;
        if (r < 1.0f) return 1.0f;
        return fminf(fminf(r, xi), 2.0f);
    } else if (P.lim == 1) {
        return fminf(__fdividef(2.0f * r, 1.0f + r), xi);
    }
    if (r < 1.0f) return r;
    return fminf(1.0f, xi);
}

CG_D void nf_slope(const NewtonFastParams& P, const float* ul, const float* uc, const float* ur, float* s) {
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const float dl = uc[k] - ul[k], dr = ur[k] - uc[k];
        float num = dl, den = dr;
        if (fabsf(num) < 1e-5f) num = 1e-5f;
        if (fabsf(den) < 1e-5f) den = 1e-5f;
        s[k] = (P.wa * dl + P.wb * dr) * nf_limiter(P, __fdividef(num, den));
    }
}

// Half-step evolution of a cell's extrapolated states (Solvers/EulerSolvers.cpp:163-223).
// half_dtdx = 0.5 dt/dx.  fl/fr receive the evolved left/right face states (conserved).
CG_D void nf_recon(const NewtonFastParams& P, const float* ul, const float* um, const float* ur, int axis,
                   float half_dtdx, float* fl, float* fr) {
    float s[5], a[5], b[5], Fa[5], Fb[5];
    nf_slope(P, ul, um, ur, s);
#pragma unroll
    for (int k = 0; k < 5; k++) { a[k] = um[k] - 0.5f * s[k]; b[k] = um[k] + 0.5f * s[k]; }
    nf_flux(P, a, axis, Fa);
    nf_flux(P, b, axis, Fb);
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const float ev = half_dtdx * (Fa[k] - Fb[k]);
        fl[k] = a[k] + ev;
        fr[k] = b[k] + ev;
    }
}

// FORCE flux (Solvers/EulerFirstOrderSolver.cpp:3-24) of conserved states L | R.
CG_D void nf_force(const NewtonFastParams& P, const float* L, const float* R, int axis, float dtdx, float dxdt,
                   float* F) {
    float fL[5], fR[5], us[5], fs[5];
    nf_flux(P, L, axis, fL);
    nf_flux(P, R, axis, fR);
#pragma unroll
    for (int k = 0; k < 5; k++) us[k] = 0.5f * ((L[k] + R[k]) + dtdx * (fL[k] - fR[k]));
    nf_flux(P, us, axis, fs);
#pragma unroll
    for (int k = 0; k < 5; k++) F[k] = 0.25f * ((fL[k] + fR[k]) + dxdt * (L[k] - R[k])) + 0.5f * fs[k];
}

// Solvers/EulerSolvers.cpp:87-128 (2D: max(|vx|, |vy| + c) as written in the reference)
CG_D float nf_wavespeed(const NewtonFastParams& P, const float* u, int dims) {
    const float ir = frcp(u[0]);
    const float vx = u[1] * ir, vy = u[2] * ir, vz = u[3] * ir;
    const float p = P.g1 * (u[4] - 0.5f * (u[1] * vx + u[2] * vy + u[3] * vz));
    const float c = sqrtf(P.gam * p * ir);  // NaN for p < 0 is dropped by the max, as in the reference
    if (dims == 1) return fabsf(vx) + c;
    return fmaxf(fabsf(vx), fabsf(vy) + c);
}

}  // namespace cg
