// FP32 bulk physics for the Newtonian system.  The algorithm is the reference's SLIC/FORCE step
// (same limiter formula with the +1e-5 clamps, same half-step evolution, same FORCE flux), with
// reformulations that are identities in exact arithmetic:
//  * the state stays conserved between operations -- the reference converts every evolved and
//    updated state to primitives and back (Euler/EulerStateVector.cpp:30-66, :91-94);
//  * divisions use one approximate reciprocal each (rho, the limiter ratio, the limiter bound);
//  * the limiters are written as min/max/select chains instead of branches;
//  * constants are folded (0.5 factors, the gradient-ratio 2).
// Every function is generic over the lane type V: `float` (one cell per thread) or `f2` (two
// cells per thread on Blackwell's paired FP32 instructions).  All arithmetic goes through the
// explicitly rounded helpers below, so both lane types evaluate the same operation sequence and
// agree to FP32 rounding.
// The sweep axis and the limiter are template parameters, so no run-time switch remains in the
// per-cell code.
#pragma once
#include "device_common.cuh"

namespace cg {

// Single-instruction approximations used by every FP32 path: PTX rcp / sqrt / rsqrt .approx.ftz,
// one MUFU operation each, within about 2 ulp of the rounded result; subnormal inputs and results
// flush to zero, a range that physical states do not reach.  (Measured on GB300: a reciprocal
// written as __fdividef(1, x) executes five instructions per lane; this form executes one.)
CG_D float frcp(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
CG_D float fsqrt(float x) {
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
CG_D float frsqrt(float x) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
CG_D float fdiv(float a, float b) { return __fmul_rn(a, frcp(b)); }

// ---- lane types and their arithmetic
struct f2 {
    float2 v;
};
CG_D float splat(float s, float) { return s; }
CG_D f2 splat(float s, f2) { return f2{make_float2(s, s)}; }
template <class V> CG_D V splat_v(float s) { return splat(s, V{}); }

CG_D float vadd(float a, float b) { return __fadd_rn(a, b); }
CG_D float vsub(float a, float b) { return __fsub_rn(a, b); }
CG_D float vmul(float a, float b) { return __fmul_rn(a, b); }
CG_D float vfma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
CG_D float vrcp(float a) { return frcp(a); }
CG_D float vdiv(float a, float b) { return fdiv(a, b); }
CG_D float vmin(float a, float b) { return fminf(a, b); }
CG_D float vmax(float a, float b) { return fmaxf(a, b); }
CG_D float vabs(float a) { return fabsf(a); }
CG_D float vsqrt(float a) { return fsqrt(a); }
CG_D float vsel_lt(float a, float b, float x, float y) { return a < b ? x : y; }  // a < b ? x : y

CG_D f2 vadd(f2 a, f2 b) { return f2{__fadd2_rn(a.v, b.v)}; }
CG_D f2 vsub(f2 a, f2 b) { return f2{__ffma2_rn(b.v, make_float2(-1.0f, -1.0f), a.v)}; }
CG_D f2 vmul(f2 a, f2 b) { return f2{__fmul2_rn(a.v, b.v)}; }
CG_D f2 vfma(f2 a, f2 b, f2 c) { return f2{__ffma2_rn(a.v, b.v, c.v)}; }
CG_D f2 vrcp(f2 a) { return f2{make_float2(frcp(a.v.x), frcp(a.v.y))}; }
CG_D f2 vdiv(f2 a, f2 b) { return vmul(a, vrcp(b)); }
CG_D f2 vmin(f2 a, f2 b) { return f2{make_float2(fminf(a.v.x, b.v.x), fminf(a.v.y, b.v.y))}; }
CG_D f2 vmax(f2 a, f2 b) { return f2{make_float2(fmaxf(a.v.x, b.v.x), fmaxf(a.v.y, b.v.y))}; }
CG_D f2 vabs(f2 a) { return f2{make_float2(fabsf(a.v.x), fabsf(a.v.y))}; }
CG_D f2 vsqrt(f2 a) { return f2{make_float2(fsqrt(a.v.x), fsqrt(a.v.y))}; }
CG_D f2 vsel_lt(f2 a, f2 b, f2 x, f2 y) {
    return f2{make_float2(a.v.x < b.v.x ? x.v.x : y.v.x, a.v.y < b.v.y ? x.v.y : y.v.y)};
}

struct NewtonFastParams {
    float g1;        // gamma - 1
    float hg1;       // (gamma - 1) / 2
    float gam;       // gamma
    float wa, wb;    // 0.5 (1 + bias), 0.5 (1 - bias)
    float hom, hop;  // (1 - bias) / 2, (1 + bias) / 2  (gradient ratio 2 / (om + op r) = 1 / (hom + hop r))
};

// Euler/EulerStateVector.cpp:68-89 (x) / :96-117 (y) on a conserved state
template <int AXIS, class V>
CG_D void nf_flux(const NewtonFastParams& P, const V* u, V* f) {
    const V ir = vrcp(u[0]);
    const V vn = vmul(AXIS == 0 ? u[1] : u[2], ir);
    const V q = vfma(u[1], u[1], vfma(u[2], u[2], vmul(u[3], u[3])));
    const V p = vfma(splat_v<V>(P.g1), u[4], vmul(splat_v<V>(-P.hg1), vmul(q, ir)));
    f[0] = AXIS == 0 ? u[1] : u[2];
    f[1] = AXIS == 0 ? vfma(u[1], vn, p) : vmul(u[1], vn);
    f[2] = AXIS == 1 ? vfma(u[2], vn, p) : vmul(u[2], vn);
    f[3] = vmul(u[3], vn);
    f[4] = vmul(vadd(u[4], p), vn);
}

// Solvers/SlopeLimiters.cpp:8-69 as select chains; `xi` = 2 / ((1-w) + (1+w) r)
template <int LIM, class V>
CG_D V nf_limiter(const NewtonFastParams& P, V r) {
    const V zero = splat_v<V>(0.0f), one = splat_v<V>(1.0f), two = splat_v<V>(2.0f);
    const V xi = vrcp(vfma(splat_v<V>(P.hop), r, splat_v<V>(P.hom)));
    if (LIM == 0) {  // SuperBee
        const V hi = vmin(vmin(r, xi), two);
        const V v = vsel_lt(r, splat_v<V>(0.5f), vmul(two, r), vsel_lt(r, one, one, hi));
        return vsel_lt(r, zero, zero, v);
    } else if (LIM == 1) {  // van Leer
        const V v = vmin(vdiv(vmul(two, r), vadd(one, r)), xi);
        return vsel_lt(r, zero, zero, v);
    }
    // MinBee: r for 0 <= r <= 1, min(1, xi) = xi above; min(r, xi) is both (xi >= 1 >= r below
    // r = 1, xi < 1 < r above)
    return vmax(vmin(r, xi), zero);
}

// Solvers/SlopeLimiters.cpp:71-101 with the +1e-5 clamps of numerator and denominator
template <int LIM, class V>
CG_D void nf_slope(const NewtonFastParams& P, const V* ul, const V* uc, const V* ur, V* s) {
    const V eps = splat_v<V>(1e-5f);
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const V dl = vsub(uc[k], ul[k]), dr = vsub(ur[k], uc[k]);
        const V num = vsel_lt(vabs(dl), eps, eps, dl);
        const V den = vsel_lt(vabs(dr), eps, eps, dr);
        s[k] = vmul(vfma(splat_v<V>(P.wa), dl, vmul(splat_v<V>(P.wb), dr)),
                    nf_limiter<LIM>(P, vmul(num, vrcp(den))));
    }
}

// Half-step evolution of a cell's extrapolated states (Solvers/EulerSolvers.cpp:163-223).
// half_dtdx = 0.5 dt/dx.  fl/fr receive the evolved left/right face states (conserved).
template <int AXIS, int LIM, class V>
CG_D void nf_recon(const NewtonFastParams& P, const V* ul, const V* um, const V* ur, float half_dtdx, V* fl, V* fr) {
    V s[5], a[5], b[5], Fa[5], Fb[5];
    nf_slope<LIM>(P, ul, um, ur, s);
#pragma unroll
    for (int k = 0; k < 5; k++) {
        a[k] = vfma(splat_v<V>(-0.5f), s[k], um[k]);
        b[k] = vfma(splat_v<V>(0.5f), s[k], um[k]);
    }
    nf_flux<AXIS>(P, a, Fa);
    nf_flux<AXIS>(P, b, Fb);
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const V d = vsub(Fa[k], Fb[k]);
        fl[k] = vfma(splat_v<V>(half_dtdx), d, a[k]);
        fr[k] = vfma(splat_v<V>(half_dtdx), d, b[k]);
    }
}

// FORCE flux (Solvers/EulerFirstOrderSolver.cpp:3-24) of conserved states L | R:
// 0.5 (LF + RI) with LF = 0.5 (fL + fR) + 0.5 (dx/dt)(L - R), RI = F(0.5 (L + R) + 0.5 (dt/dx)(fL - fR)).
template <int AXIS, class V>
CG_D void nf_force(const NewtonFastParams& P, const V* L, const V* R, float half_dtdx, float q_dxdt, V* F) {
    V fL[5], fR[5], us[5], fs[5];
    nf_flux<AXIS>(P, L, fL);
    nf_flux<AXIS>(P, R, fR);
#pragma unroll
    for (int k = 0; k < 5; k++)
        us[k] = vfma(splat_v<V>(0.5f), vadd(L[k], R[k]), vmul(splat_v<V>(half_dtdx), vsub(fL[k], fR[k])));
    nf_flux<AXIS>(P, us, fs);
#pragma unroll
    for (int k = 0; k < 5; k++)
        F[k] = vfma(splat_v<V>(0.25f), vadd(fL[k], fR[k]),
                    vfma(splat_v<V>(q_dxdt), vsub(L[k], R[k]), vmul(splat_v<V>(0.5f), fs[k])));
}

// Four times the FORCE flux, from the flux's homogeneity F(2u) = 2 F(u) (exact in floating point:
// doubling is exact): 4F = (fL + fR) + (dx/dt)(L - R) + F((L + R) + (dt/dx)(fL - fR)) -- two
// operations per field fewer than nf_force.  Callers update with nf_update and dt/(4 dx).
template <int AXIS, class V>
CG_D void nf_force4(const NewtonFastParams& P, const V* L, const V* R, float dtdx, float dxdt, V* F4) {
    V fL[5], fR[5], us[5], fs[5];
    nf_flux<AXIS>(P, L, fL);
    nf_flux<AXIS>(P, R, fR);
#pragma unroll
    for (int k = 0; k < 5; k++) us[k] = vfma(splat_v<V>(dtdx), vsub(fL[k], fR[k]), vadd(L[k], R[k]));
    nf_flux<AXIS>(P, us, fs);
#pragma unroll
    for (int k = 0; k < 5; k++) F4[k] = vfma(splat_v<V>(dxdt), vsub(L[k], R[k]), vadd(vadd(fL[k], fR[k]), fs[k]));
}

// The coefficients nf_force4 and its update take: dt/dx, dx/dt, dt/(4 dx) (exact scalings of the
// step's FP32 coefficients), and 0.5 dt/dx for the half-step evolution.
struct Force4Coef {
    float half_dtdx, dtdx, dxdt, q_dtdx;
};
CG_D Force4Coef force4_coef(const FastCoef& c) { return Force4Coef{c.half_dtdx, c.dtdx, 4.0f * c.q_dxdt, 0.25f * c.dtdx}; }

// Conservative update U + (dt/dx)(F_left - F_right)
template <class V>
CG_D void nf_update(float dtdx, const V* c, const V* FL, const V* FR, V* o) {
#pragma unroll
    for (int f = 0; f < 5; f++) o[f] = vfma(splat_v<V>(dtdx), vsub(FL[f], FR[f]), c[f]);
}

// speed_or_inf (device_common.cuh) per lane
CG_D float nf_speed_or_inf(float a, float b, float s) { return speed_or_inf(a, b, s); }
CG_D f2 nf_speed_or_inf(f2 a, f2 b, f2 s) {
    return f2{make_float2(speed_or_inf(a.v.x, b.v.x, s.v.x), speed_or_inf(a.v.y, b.v.y, s.v.y))};
}

// Solvers/EulerSolvers.cpp:87-128 (2D: max(|vx|, |vy| + c) as written in the reference)
template <class V>
CG_D V nf_wavespeed(const NewtonFastParams& P, const V* u, int dims) {
    const V ir = vrcp(u[0]);
    const V vx = vmul(u[1], ir), vy = vmul(u[2], ir);
    const V q = vfma(u[1], u[1], vfma(u[2], u[2], vmul(u[3], u[3])));
    const V p = vfma(splat_v<V>(P.g1), u[4], vmul(splat_v<V>(-P.hg1), vmul(q, ir)));
    const V c = vsqrt(vmul(vmul(splat_v<V>(P.gam), p), ir));  // NaN for p < 0 is dropped by the max, as in the reference
    const V s = dims == 1 ? vadd(vabs(vx), c) : vmax(vabs(vx), vadd(vabs(vy), c));
    return nf_speed_or_inf(u[0], u[4], s);
}

}  // namespace cg
