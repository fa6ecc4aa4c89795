// FP32 bulk physics for the black-hole (3+1 Kerr-Schild) system: primitive FP32 storage (as the
// reference's grids), FP32 slopes, fluxes, FORCE, RK4 source and sums, with every metric quantity
// taken from
// tables evaluated once in FP64 (the spacetime is static), and the primitive recovery of
// physics_sr_fast.cuh (FP32 Newton iterations, finished in FP64 above a Lorentz factor) applied to
// u / sqrt(gamma) -- the reference's GR recovery is its SR recovery of the de-densitised state
// (BlackHoleEuler/BlackHoleEulerStateVector.cpp:30-103).
//
// Structure kept from the reference (Solvers/BlackHoleEulerSolvers.cpp, Solvers/BlackHoleEuler
// SecondOrderSolver.cpp, Solvers/BlackHoleEulerForcingSolver.cpp):
//  * half-step evolution at the cell centre with the extrapolated states' fluxes at the faces;
//    the evolved face states are recovered at the face and re-densitised at the neighbouring cell
//    centres inside FORCE, whose Richtmyer flux is taken at the face;
//  * the forcing step's fractional sweeps take their neighbour fluxes at the neighbour centres;
//  * excision masks (stencil reach 2 along both axes for the sweeps, 1 for the source step) and the
//    CFL speed's 1/N coordinates with x and y swapped in 2D.
// Every conversion between primitive and conserved states sits where the reference's does: with the
// W-for-W^2 energy of BlackHoleEuler/BlackHoleEulerStateVector.cpp:154 the two are not inverse,
// so the round trips are part of the algorithm.  Differences (FP32 path only): points are exact
// geometric positions (the reference's separately rounded face coordinates differ in the last
// bits), and each cell is evolved once for both faces.
#pragma once
#include "device_common.cuh"
#include "physics_fast.cuh"
#include "physics_sr_fast.cuh"

namespace cg {

// Metric at one point (FP32 copies of FP64 values): gamma_ij (xx xy xz yy yz zz), sqrt(det gamma),
// lapse, shift.
constexpr int kMetFields = 11;
struct GRMet {
    float g[6];
    float sg, al, be[3];
};
// Source-term data at a cell centre: g^{mu nu} (00 01 02 03 11 12 13 22 23 33), d_i alpha,
// d_i beta^k (3x3, [i][k]), d_i gamma_jk (i major; jk as in GRMet), K_ij (as in GRMet).
constexpr int kSrcFields = 10 + 3 + 9 + 18 + 6;
struct GRSrc {
    float gi[10], da[3], db[9], dg[18], K[6];
};
// CFL data at the reference's wavespeed point: lapse, shift, gamma_ij, diagonal of gamma^ij.
constexpr int kWsFields = 1 + 3 + 6 + 3;

// Structure-of-arrays table: field q of point k at p[q * stride + k].
struct GRTab {
    const float* p;
    size_t stride;
    CG_D float at(int q, size_t k) const { return p[q * stride + k]; }
};

CG_D void load_met(const GRTab& T, size_t k, GRMet& m) {
#pragma unroll
    for (int q = 0; q < 6; q++) m.g[q] = T.at(q, k);
    m.sg = T.at(6, k);
    m.al = T.at(7, k);
#pragma unroll
    for (int q = 0; q < 3; q++) m.be[q] = T.at(8 + q, k);
}
CG_D void load_src(const GRTab& T, size_t k, GRSrc& s) {
    float* d = s.gi;  // the struct's fields are contiguous floats
#pragma unroll
    for (int q = 0; q < kSrcFields; q++) d[q] = T.at(q, k);
}

// index of gamma_ij in GRMet::g
CG_D int gsym(int i, int j) {
    const int a = i < j ? i : j, b = i < j ? j : i;
    return a == 0 ? b : (a == 1 ? 2 + b : 5);
}
// index of g^{mu nu} in GRSrc::gi
CG_D int g4sym(int m, int n) {
    const int a = m < n ? m : n, b = m < n ? n : m;
    return a == 0 ? b : (a == 1 ? 3 + b : (a == 2 ? 5 + b : 9));
}

// ---- state conversions and fluxes.  Primitives travel as float[5] (rho, vx, vy, vz, p), the
// reference's stored state; conserved states are densitised.
CG_D SRPrim32 gr_c2p_fast(const SRFastParams& P, const float* u, const GRMet& M, int* flags) {
    const float is = frcp(M.sg);
    float v[5];
#pragma unroll
    for (int k = 0; k < 5; k++) v[k] = u[k] * is;
    return sr_c2p_fast(P, v, flags);
}
CG_D void gr_prim_fast(const SRFastParams& P, const float* u, const GRMet& M, float* p, int* flags) {
    const SRPrim32 c = gr_c2p_fast(P, u, M, flags);
    p[0] = c.rho;
    p[1] = c.vx;
    p[2] = c.vy;
    p[3] = c.vz;
    p[4] = c.p;
}

// BlackHoleEuler/BlackHoleEulerStateVector.cpp:118-157 (energy with W, not W^2, at :154): W from
// gamma_ij v^i v^j, h from rho and p
CG_D void gr_cons_fast(const SRFastParams& P, const float* p, const GRMet& M, float* u) {
    const float v[3] = {p[1], p[2], p[3]};
    float v2 = 0.0f;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) v2 = fmaf(M.g[gsym(i, j)] * v[i], v[j], v2);
    // the reference's clamp of v^2 to 1 - 1e-8 (W <= 1e4), applied to 1 - v^2: in FP32, 1 - 1e-8
    // rounds to 1, which would make W infinite
    const float omv = 1.0f - v2;
    const float W = frsqrt(omv < 1e-8f ? 1e-8f : omv);
    const float h = 1.0f + fdiv(p[4], p[0]) * P.hfac;
    const float sr = M.sg * p[0];
    u[0] = sr * W;
    const float m = sr * h * W * W;
    u[1] = m * v[0];
    u[2] = m * v[1];
    u[3] = m * v[2];
    u[4] = M.sg * ((p[0] * h * W - p[4]) - p[0] * W);
}

// BlackHoleEuler/BlackHoleEulerStateVector.cpp:159-250 (x) and :259-350 (y): the flux of a
// conserved state, through its primitive recovery
template <int AXIS>
CG_D void gr_flux_fast(const SRFastParams& P, const float* u, const GRMet& M, float* f, int* flags) {
    const SRPrim32 c = gr_c2p_fast(P, u, M, flags);
    const float as = M.al * M.sg;
    const float rhw = c.rho * c.h * c.W * c.W;
    const float vn = AXIS == 0 ? c.vx : c.vy;
    const float w = vn - fdiv(M.be[AXIS], M.al);
    f[0] = as * (c.rho * c.W * w);
    f[1] = as * (rhw * c.vx * w + (AXIS == 0 ? c.p : 0.0f));
    f[2] = as * (rhw * c.vy * w + (AXIS == 1 ? c.p : 0.0f));
    f[3] = as * (rhw * c.vz * w);
    f[4] = as * (((rhw - c.p) - c.rho * c.W) * w + c.p * vn);
}

// Half-step evolution (Solvers/BlackHoleEulerSolvers.cpp:234-307) of the cell with primitive
// neighbours l | r: slopes of the conserved states at their own centres (Ml, Mc, Mr), the
// extrapolated states' fluxes at the cell's faces (FL, FR); A / B receive the evolved left / right
// face states as primitives recovered at those faces.
template <int AXIS, int LIM>
CG_D void gr_evolve_fast(const SRFastParams& P, const NewtonFastParams& NP, const float* l, const float* m,
                         const float* r, const GRMet& Ml, const GRMet& Mc, const GRMet& Mr, const GRMet& FL,
                         const GRMet& FR, float half_dtdx, float* A, float* B, int* flags) {
    float ul[5], um[5], ur[5], s[5], a[5], b[5], Fa[5], Fb[5];
    gr_cons_fast(P, l, Ml, ul);
    gr_cons_fast(P, m, Mc, um);
    gr_cons_fast(P, r, Mr, ur);
    nf_slope<LIM>(NP, ul, um, ur, s);
#pragma unroll
    for (int k = 0; k < 5; k++) { a[k] = fmaf(-0.5f, s[k], um[k]); b[k] = fmaf(0.5f, s[k], um[k]); }
    gr_flux_fast<AXIS>(P, a, FL, Fa, flags);
    gr_flux_fast<AXIS>(P, b, FR, Fb, flags);
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const float ev = half_dtdx * (Fa[k] - Fb[k]);
        a[k] = a[k] + ev;
        b[k] = b[k] + ev;
    }
    gr_prim_fast(P, a, FL, A, flags);
    gr_prim_fast(P, b, FR, B, flags);
}

// FORCE flux at a face (Solvers/BlackHoleEulerFirstOrderSolver.cpp:3-47): the primitive face
// states L (left cell) and R (right cell) become conserved states at the left / right cell
// centres (MCL, MCR), where their fluxes are also taken; the Richtmyer state's flux is taken at
// the face (MF).
template <int AXIS>
CG_D void gr_force_fast(const SRFastParams& P, const float* L, const float* R, const GRMet& MCL, const GRMet& MF,
                        const GRMet& MCR, float half_dtdx, float q_dxdt, float* F, int* flags) {
    float uL[5], uR[5], fL[5], fR[5], us[5], fs[5];
    gr_cons_fast(P, L, MCL, uL);
    gr_cons_fast(P, R, MCR, uR);
    gr_flux_fast<AXIS>(P, uL, MCL, fL, flags);
    gr_flux_fast<AXIS>(P, uR, MCR, fR, flags);
#pragma unroll
    for (int k = 0; k < 5; k++) us[k] = fmaf(0.5f, uL[k] + uR[k], half_dtdx * (fL[k] - fR[k]));
    gr_flux_fast<AXIS>(P, us, MF, fs, flags);
#pragma unroll
    for (int k = 0; k < 5; k++) F[k] = fmaf(0.25f, fL[k] + fR[k], fmaf(q_dxdt, uL[k] - uR[k], 0.5f * fs[k]));
}

// Conservative update of a primitive cell at its centre (computeFORCEUpdate, then the recovery of
// the stored primitives)
CG_D void gr_update_fast(const SRFastParams& P, const float* c, const float* FL, const float* FR, const GRMet& M,
                         float dtdx, float* o, int* flags) {
    float u[5];
    gr_cons_fast(P, c, M, u);
#pragma unroll
    for (int f = 0; f < 5; f++) u[f] = fmaf(dtdx, FL[f] - FR[f], u[f]);
    gr_prim_fast(P, u, M, o, flags);
}

// Source term (BlackHoleEuler/BlackHoleEulerStateVector.cpp:359-510) of a densitised state at a
// cell centre, from the cell's metric and source tables.
CG_D void gr_source_fast(const SRFastParams& P, const float* u, const GRMet& M, const GRSrc& X, float* s, int* flags) {
    const SRPrim32 c = gr_c2p_fast(P, u, M, flags);
    float uu[4];
    uu[0] = fdiv(c.W, M.al);
    uu[1] = (M.al * uu[0]) * c.vx - M.be[0] * uu[0];
    uu[2] = (M.al * uu[0]) * c.vy - M.be[1] * uu[0];
    uu[3] = (M.al * uu[0]) * c.vz - M.be[2] * uu[0];
    const float rh = c.rho * c.h;
    auto T = [&](int m, int n) { return rh * uu[m] * uu[n] + c.p * X.gi[g4sym(m, n)]; };
    float S[5] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    const float v[3] = {c.vx, c.vy, c.vz};
    float vc[3];
#pragma unroll
    for (int i = 0; i < 3; i++) vc[i] = M.g[gsym(i, 0)] * v[0] + M.g[gsym(i, 1)] * v[1] + M.g[gsym(i, 2)] * v[2];
    const float rhw = rh * c.W * c.W;
    const float T00 = T(0, 0);
    const float ial = frcp(M.al);
#pragma unroll
    for (int i = 0; i < 3; i++) {
#pragma unroll
        for (int j = 0; j < 3; j++) {
#pragma unroll
            for (int k = 0; k < 3; k++) {
                const float dgijk = X.dg[6 * i + gsym(j, k)];
                S[i + 1] += T00 * (0.5f * M.be[j] * M.be[k] * dgijk) + T(0, j + 1) * M.be[k] * dgijk +
                            0.5f * T(j + 1, k + 1) * dgijk;
            }
            S[i + 1] += rhw * vc[j] * ial * X.db[3 * i + j];
        }
        S[i + 1] -= T00 * M.al * X.da[i];
    }
#pragma unroll
    for (int i = 0; i < 3; i++) {
#pragma unroll
        for (int j = 0; j < 3; j++) {
            const float K = X.K[gsym(i, j)];
            S[4] += T00 * (M.be[i] * M.be[j] * K) + T(0, i + 1) * (2.0f * M.be[j] * K) + T(i + 1, j + 1) * K;
        }
        S[4] -= T00 * M.be[i] * X.da[i] + T(0, i + 1) * X.da[i];
    }
    const float f = M.al * M.sg;
#pragma unroll
    for (int k = 0; k < 5; k++) s[k] = f * S[k];
}

// Fractional evolution on frozen neighbours (Solvers/BlackHoleEulerSolvers.cpp:159-232): primitive
// neighbours l | r with centres Ml, Mr (where their extrapolated fluxes are also taken), the cell's
// primitives m; o receives the cell's primitives after frac * dt.
template <int AXIS, int LIM>
CG_D void gr_fraction_fast(const SRFastParams& P, const NewtonFastParams& NP, float frac, const float* l,
                           const float* m, const float* r, const GRMet& Ml, const GRMet& Mc, const GRMet& Mr,
                           float dtdx, float* o, int* flags) {
    float ul[5], um[5], ur[5], sl[5], a[5], b[5], Fa[5], Fb[5], nu[5];
    gr_cons_fast(P, l, Ml, ul);
    gr_cons_fast(P, m, Mc, um);
    gr_cons_fast(P, r, Mr, ur);
    nf_slope<LIM>(NP, ul, um, ur, sl);
#pragma unroll
    for (int k = 0; k < 5; k++) { a[k] = fmaf(-0.5f, sl[k], um[k]); b[k] = fmaf(0.5f, sl[k], um[k]); }
    gr_flux_fast<AXIS>(P, a, Ml, Fa, flags);
    gr_flux_fast<AXIS>(P, b, Mr, Fb, flags);
    const float s = frac * dtdx;
#pragma unroll
    for (int k = 0; k < 5; k++) nu[k] = fmaf(s, Fa[k] - Fb[k], um[k]);
    gr_prim_fast(P, nu, Mc, o, flags);
}

// Classical RK4 on the source with interleaved fractional sweeps
// (Solvers/BlackHoleEulerForcingSolver.cpp:3-185; the solvers call it with bias 0 and limiter 1,
// Solvers/BlackHoleEulerSecondOrderSolver.cpp:195-209).  cl..cb: the neighbours' and the cell's
// conserved states at their centres (l, r along x; t, b along y); out: the cell's primitives.
template <int LIM>
CG_D void gr_rk_fast(const SRFastParams& P, const NewtonFastParams& NP, int dims, const float* cl, const float* cm,
                     const float* cr, const float* ct, const float* cb, const GRMet& Ml, const GRMet& Mc,
                     const GRMet& Mr, const GRMet& Mt, const GRMet& Mb, const GRSrc& X, float dt, float dtdx,
                     float* out, int* flags) {
    float L[5], R[5], Tp[5], B[5];
    gr_prim_fast(P, cl, Ml, L, flags);
    gr_prim_fast(P, cr, Mr, R, flags);
    if (dims == 2) {
        gr_prim_fast(P, ct, Mt, Tp, flags);
        gr_prim_fast(P, cb, Mb, B, flags);
    }
    float k[4][5];
    {
        float s[5];
        gr_source_fast(P, cm, Mc, X, s, flags);
#pragma unroll
        for (int i = 0; i < 5; i++) k[0][i] = dt * s[i];
    }
#pragma unroll 1
    for (int stage = 0; stage < 3; stage++) {
        float st[5], Mp[5], E[5], c[5], s[5];
        const float h = stage < 2 ? 0.5f : 1.0f;
#pragma unroll
        for (int i = 0; i < 5; i++) st[i] = fmaf(h, k[stage][i], cm[i]);
        gr_prim_fast(P, st, Mc, Mp, flags);
        if (dims == 1) {
            gr_fraction_fast<0, LIM>(P, NP, stage < 2 ? 0.5f : 1.0f, L, Mp, R, Ml, Mc, Mr, dtdx, E, flags);
        } else {
            const float fx = stage < 2 ? 0.25f : 0.5f, fy = stage < 2 ? 0.5f : 1.0f;
            float E1[5], E2[5];
            gr_fraction_fast<0, LIM>(P, NP, fx, L, Mp, R, Ml, Mc, Mr, dtdx, E1, flags);
            gr_fraction_fast<1, LIM>(P, NP, fy, Tp, E1, B, Mt, Mc, Mb, dtdx, E2, flags);
            gr_fraction_fast<0, LIM>(P, NP, fx, L, E2, R, Ml, Mc, Mr, dtdx, E, flags);
        }
        gr_cons_fast(P, E, Mc, c);
        gr_source_fast(P, c, Mc, X, s, flags);
#pragma unroll
        for (int i = 0; i < 5; i++) k[stage + 1][i] = dt * s[i];
    }
    float nc[5];
#pragma unroll
    for (int i = 0; i < 5; i++) nc[i] = cm[i] + (1.0f / 6.0f) * (k[0][i] + 2.0f * k[1][i] + 2.0f * k[2][i] + k[3][i]);
    gr_prim_fast(P, nc, Mc, out, flags);
}

// Largest signed characteristic speed (BlackHoleEuler/BlackHoleEulerStateVector.cpp:519-549,
// BlackHoleEuler/BlackHoleEulerEigenvalues.cpp:3-96) of primitives c at a CFL point whose data are
// w[0] lapse, w[1..3] shift, w[4..9] gamma_ij, w[10..12] diagonal of gamma^ij (sound speed from
// RelativisticEuler/RelativisticEulerEquationOfState.cpp:3-18).
// The same in FP64 (IEEE square roots and divisions), for the garbage states the recovery leaves at
// the density floor near the horizon (velocities far above 1): their products overflow FP32, where
// the reference's FP64 gives large finite speeds that limit the time step.
static __device__ __noinline__ float gr_speed64(double gf, double hfac, const float* p, const float* w) {
    const double al = w[0];
    const double h = 1.0 + (double)p[4] / (double)p[0] * hfac;
    const double cs2 = gf * p[4] / ((double)p[0] * h);
    const double cs = sqrt(cs2);
    const double v[3] = {p[1], p[2], p[3]};
    double v2 = 0.0;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) v2 += (double)w[4 + gsym(i, j)] * v[i] * v[j];
    double s = 0.0;
    for (int i = 0; i < 3; i++) {
        const double be = w[1 + i];
        const double mat = al * v[i] - be;
        const double rt = sqrt((1.0 - v2) * (w[10 + i] * (1.0 - v2 * cs2) - v[i] * v[i] * (1.0 - cs2)));
        const double pre = al / (1.0 - v2 * cs2);
        const double fast = pre * (v[i] * (1.0 - cs2) + cs * rt) - be;
        const double slow = pre * (v[i] * (1.0 - cs2) - cs * rt) - be;
        s = mat > s ? mat : s;
        s = fast > s ? fast : s;
        s = slow > s ? slow : s;
    }
    return (float)fabs(s);
}

CG_D float gr_speed_fast(const SRFastParams& P, const float* p, const float* w) {
    if (!(fabsf(p[1]) < 1e6f && fabsf(p[2]) < 1e6f && fabsf(p[3]) < 1e6f)) return gr_speed64(P.g, 1.0 / P.grd, p, w);
    const float al = w[0];
    const float h = 1.0f + fdiv(p[4], p[0]) * P.hfac;
    const float cs2 = fdiv(P.gf * p[4], p[0] * h);
    const float cs = fsqrt(cs2);
    const float v[3] = {p[1], p[2], p[3]};
    float v2 = 0.0f;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) v2 = fmaf(w[4 + gsym(i, j)] * v[i], v[j], v2);
    float s = 0.0f;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const float be = w[1 + i];
        const float mat = al * v[i] - be;
        const float rt = fsqrt((1.0f - v2) * (w[10 + i] * (1.0f - v2 * cs2) - v[i] * v[i] * (1.0f - cs2)));
        const float pre = fdiv(al, 1.0f - v2 * cs2);
        const float fast = pre * (v[i] * (1.0f - cs2) + cs * rt) - be;
        const float slow = pre * (v[i] * (1.0f - cs2) - cs * rt) - be;
        s = mat > s ? mat : s;
        s = fast > s ? fast : s;
        s = slow > s ? slow : s;
    }
    return fabsf(s);
}

}  // namespace cg
