// Physics policies plugged into the generic sweep kernels (sweep_kernels.cuh).
#pragma once
#include "physics_exact.cuh"
#include "physics_fast.cuh"
#include "physics_sr_fast.cuh"
#include "sweep_kernels.cuh"

namespace cg {

// Cell position helpers shared by the policies.  A sweep line is a row (axis 0) or a column
// (axis 1); k indexes cells along it.  Cell (i, j) sits at (x, y) = (j dx, i dx)
// (Solvers/BlackHoleEulerSecondOrderSolver.cpp:88-100); 1D grids are row i = 0, so y = 0 as in
// the reference's 1D solvers.
struct LineMap {
    int axis, nx;
    CG_D void ij(int line, int k, int& i, int& j) const {
        if (axis == 0) { i = line; j = k; } else { i = k; j = line; }
    }
    CG_D bool mask_on(const unsigned char* mask, int line, int k) const {
        if (!mask) return true;
        int i, j;
        ij(line, k, i, j);
        return mask[(size_t)i * nx + j] != 0;
    }
};

// ------------------------------------------------------------------ reference-exact, FP64
// Primitive storage exactly like the reference's grids.  Sys = NewtonExact<double>, SRExact or
// GRExact.  Coordinate-free systems share one half-step evolution per cell (both faces);
// GR evolves each face at its own, separately rounded, coordinate.
template <class Sys>
struct ExactPolicy {
    using S = double;
    using X = double;
    using W = double;  // wavespeed reduction type
    using Cell = V5<double>;
    using Face = V5<double>;
    struct Coef { double dt; };
    static constexpr bool kShared = !Sys::kCoords;
    static constexpr bool kMasked = true;
    static constexpr bool kHasDx = true;
    Sys sys;
    LineMap lm;
    int dims, order, ny;
    double dx, dt, w;
    int lim;
    int capped;

    CG_D Coef make_coef(const DtSrc&, double d) const { return Coef{d}; }
    CG_D void use_coef(const Coef& c) { dt = c.dt; capped = 0; sys.capped = &capped; }
    CG_D Pt cell_pt(int line, int k) const {
        int i, j;
        lm.ij(line, k, i, j);
        return Pt{j * dx, i * dx, 0.0};
    }
    // interface between cells f-1 and f: (f - 0.5) dx along the sweep axis
    CG_D Pt face_pt(int line, int f) const {
        if (lm.axis == 0) return Pt{(f - 0.5) * dx, line * dx, 0.0};
        return Pt{line * dx, (f - 0.5) * dx, 0.0};
    }
    CG_D void recon(const Cell& l, const Cell& m, const Cell& r, int, int, Face& L, Face& R) const {
        evolve_half_exact(sys, l.v, m.v, r.v, Pt{0.0, 0.0, 0.0}, lm.axis, dx, dt, w, lim, L.v, R.v);
    }
    // GR: the left cell of interface f evolves at xf - dx/2, the right cell at xf + dx/2
    // (Solvers/BlackHoleEulerSecondOrderSolver.cpp:3-37)
    CG_D void recon_side(const Cell& l, const Cell& m, const Cell& r, int line, int k, int side, Face& o) const {
        if (side == 1) {
            Pt xc = shift_pt(face_pt(line, k + 1), lm.axis, -(dx * 0.5));
            evolve_half_exact(sys, l.v, m.v, r.v, xc, lm.axis, dx, dt, w, lim, (double*)nullptr, o.v);
        } else {
            Pt xc = shift_pt(face_pt(line, k), lm.axis, dx * 0.5);
            evolve_half_exact(sys, l.v, m.v, r.v, xc, lm.axis, dx, dt, w, lim, o.v, (double*)nullptr);
        }
    }
    CG_D void face_of(const Cell& c, Face& f) const { f = c; }
    CG_D void flux(const Face& L, const Face& R, int line, int f, V5<double>& F) const {
        force_exact(sys, L.v, R.v, face_pt(line, f), lm.axis, dx, dt, F.v);
    }
    // computeFORCEUpdate, Solvers/EulerFirstOrderSolver.cpp:96-101, then setConservedVariableVector
    CG_D Cell update(const Cell& c, const V5<double>& FL, const V5<double>& FR, int line, int k) const {
        Pt q = cell_pt(line, k);
        double u[5], nu[5];
        sys.cons(c.v, q, u);
        const double d = dt / dx;
#pragma unroll
        for (int f = 0; f < 5; f++) nu[f] = u[f] + (d * (FL.v[f] - FR.v[f]));
        Cell o;
        sys.prim(nu, q, o.v);
        return o;
    }
    CG_D bool excised_stencil(int line, int k) const;
    CG_D bool active(int line, int k, const unsigned char* mask) const {
        if (!lm.mask_on(mask, line, k)) return false;
        if (Sys::kCoords) return !excised_stencil(line, k);
        return true;
    }
    CG_D double wavespeed(const Cell& c, int line, int k) const;
    CG_D void flush_status(int* st) const {
        if (st && capped) atomicOr(st, ST_NEWTON_CAP);
    }
};

template <class Sys>
CG_D bool ExactPolicy<Sys>::excised_stencil(int, int) const { return false; }
template <class Sys>
CG_D double ExactPolicy<Sys>::wavespeed(const Cell& c, int, int) const {
    return speed_or_inf(c.v[0], c.v[4], sys.wavespeed(c.v, dims, Pt{0, 0, 0}));
}

// GR excision: the updated cell and its stencil along both axes must lie outside the horizon
// (Solvers/BlackHoleEulerSecondOrderSolver.cpp:44-46 in 1D, :81-85 in 2D; reach 1 for FORCE,
// Solvers/BlackHoleEulerFirstOrderSolver.cpp:94-95, :131-133).
template <>
CG_D bool ExactPolicy<GRExact>::excised_stencil(int line, int k) const {
    int i, j;
    lm.ij(line, k, i, j);
    const int reach = order == 2 ? 2 : 1;
    const BHExact& b = sys.bh;
    if (dims == 1) {
        for (int d = -reach; d <= reach; d++)
            if (b.excised((j + d) * dx, 0.0, 0.0)) return true;
        return false;
    }
    if (b.excised(j * dx, i * dx, 0.0)) return true;
    for (int d = 1; d <= reach; d++) {
        if (b.excised((j - d) * dx, i * dx, 0.0) || b.excised((j + d) * dx, i * dx, 0.0) ||
            b.excised(j * dx, (i - d) * dx, 0.0) || b.excised(j * dx, (i + d) * dx, 0.0))
            return true;
    }
    return false;
}

// GR CFL speed, Solvers/BlackHoleEulerSolvers.cpp:87-131: coordinates use spacing 1/N, and in 2D
// the excision test reads (j/ncol, i/nrow) while the speed is evaluated at (i/nrow, j/ncol).
template <>
CG_D double ExactPolicy<GRExact>::wavespeed(const Cell& c, int line, int k) const {
    int i, j;
    lm.ij(line, k, i, j);
    if (dims == 1) {
        const double cs = 1.0 / lm.nx;
        if (sys.bh.excised(j * cs, 0.0, 0.0)) return 0.0;
        return speed_or_inf(c.v[0], c.v[4], fabs(sys.sound_speed(c.v, Pt{j * cs, 0.0, 0.0})));
    }
    const double rs = 1.0 / ny, cs = 1.0 / lm.nx;
    if (sys.bh.excised(j * cs, i * rs, 0.0)) return 0.0;
    return speed_or_inf(c.v[0], c.v[4], fabs(sys.sound_speed(c.v, Pt{i * rs, j * cs, 0.0})));
}

// ------------------------------------------------------------------ Newtonian FP32 bulk
// Conserved FP32 storage; see physics_fast.cuh for the reformulations.  AXIS and LIM are fixed at
// compile time; MASKED selects whether the AMR update mask is consulted at all.
template <int AXIS, int LIM, bool MASKED>
struct NewtonFastPolicy {
    using S = float;
    using X = float;
    using W = float;
    using Cell = V5<float>;
    using Face = V5<float>;
    using Coef = FastCoef;
    static constexpr bool kShared = true;
    static constexpr bool kMasked = MASKED;
    static constexpr bool kHasDx = false;  // dx enters through the precomputed coefficients
    NewtonFastParams P;
    LineMap lm;
    int dims;
    float dtdx, half_dtdx, q_dxdt;

    // FP32 coefficients come precomputed (device step controller or host), so no FP64
    // instruction runs in the FP32 sweeps
    CG_D Coef make_coef(const DtSrc& ds, double) const { return ds.fast_coef(); }
    CG_D void use_coef(const Coef& c) {
        dtdx = c.dtdx;
        half_dtdx = c.half_dtdx;
        q_dxdt = c.q_dxdt;
    }
    CG_D void recon(const Cell& l, const Cell& m, const Cell& r, int, int, Face& L, Face& R) const {
        nf_recon<AXIS, LIM>(P, l.v, m.v, r.v, half_dtdx, L.v, R.v);
    }
    CG_D void recon_side(const Cell&, const Cell&, const Cell&, int, int, int, Face&) const {}
    CG_D void face_of(const Cell& c, Face& f) const { f = c; }
    CG_D void flux(const Face& L, const Face& R, int, int, V5<float>& F) const {
        nf_force<AXIS>(P, L.v, R.v, half_dtdx, q_dxdt, F.v);
    }
    CG_D Cell update(const Cell& c, const V5<float>& FL, const V5<float>& FR, int, int) const {
        Cell o;
        nf_update(dtdx, c.v, FL.v, FR.v, o.v);
        return o;
    }
    CG_D bool active(int line, int k, const unsigned char* mask) const {
        return MASKED ? lm.mask_on(mask, line, k) : true;
    }
    CG_D float wavespeed(const Cell& c, int, int) const { return nf_wavespeed(P, c.v, dims); }
    CG_D void flush_status(int*) const {}
};

// FP32 bulk policy of the special-relativistic system (physics_sr_fast.cuh): the sweep structure
// of NewtonFastPolicy with the relativistic flux, whose primitive recovery ends in FP64.
template <int AXIS, int LIM, bool MASKED>
struct SRFastPolicy {
    using S = float;
    using X = float;
    using W = float;
    using Cell = V5<float>;
    using Face = V5<float>;
    using Coef = FastCoef;
    static constexpr bool kShared = true;
    static constexpr bool kMasked = MASKED;
    static constexpr bool kHasDx = false;
    NewtonFastParams NP;  // limiter and bias factors
    SRFastParams P;
    LineMap lm;
    int dims;
    float dtdx, half_dtdx, q_dxdt;
    int flags;  // bit 0: a primitive recovery did not converge

    CG_D Coef make_coef(const DtSrc& ds, double) const { return ds.fast_coef(); }
    CG_D void use_coef(const Coef& c) {
        dtdx = c.dtdx;
        half_dtdx = c.half_dtdx;
        q_dxdt = c.q_dxdt;
    }
    CG_D void recon(const Cell& l, const Cell& m, const Cell& r, int, int, Face& L, Face& R) {
        sr_recon_fast<AXIS, LIM>(P, NP, l.v, m.v, r.v, half_dtdx, L.v, R.v, &flags);
    }
    CG_D void recon_side(const Cell&, const Cell&, const Cell&, int, int, int, Face&) const {}
    CG_D void face_of(const Cell& c, Face& f) const { f = c; }
    CG_D void flux(const Face& L, const Face& R, int, int, V5<float>& F) {
        sr_force_fast<AXIS>(P, L.v, R.v, half_dtdx, q_dxdt, F.v, &flags);
    }
    CG_D Cell update(const Cell& c, const V5<float>& FL, const V5<float>& FR, int, int) const {
        Cell o;
#pragma unroll
        for (int f = 0; f < 5; f++) o.v[f] = fmaf(dtdx, FL.v[f] - FR.v[f], c.v[f]);
        return o;
    }
    CG_D bool active(int line, int k, const unsigned char* mask) const {
        return MASKED ? lm.mask_on(mask, line, k) : true;
    }
    CG_D float wavespeed(const Cell& c, int, int) { return sr_wavespeed_fast(P, c.v, dims, &flags); }
    CG_D void flush_status(int* st) const {
        if (st && flags) atomicOr(st, ST_NEWTON_CAP);
    }
};

template <int AXIS, int LIM, bool MASKED>
inline SRFastPolicy<AXIS, LIM, MASKED> make_sr_fast(double gamma, double bias, int nx, int dims, double c2p64_above) {
    SRFastPolicy<AXIS, LIM, MASKED> p;
    const float w = (float)bias;
    p.NP.g1 = p.NP.hg1 = p.NP.gam = 0.0f;
    p.NP.wa = 0.5f * (1.0f + w);
    p.NP.wb = 0.5f * (1.0f - w);
    p.NP.hom = 0.5f * (1.0f - w);
    p.NP.hop = 0.5f * (1.0f + w);
    p.P.wa = p.NP.wa;
    p.P.wb = p.NP.wb;
    p.P.hom = p.NP.hom;
    p.P.hop = p.NP.hop;
    sr_fast_constants(p.P, gamma);
    p.P.w64 = c2p64_above > 0.0 ? (float)c2p64_above : 0.0f;  // W >= 1 > 0: threshold 0 always runs FP64
    p.lm.axis = AXIS;
    p.lm.nx = nx;
    p.dims = dims;
    p.dtdx = p.half_dtdx = p.q_dxdt = 0.0f;
    p.flags = 0;
    return p;
}

template <int AXIS, int LIM, bool MASKED>
inline NewtonFastPolicy<AXIS, LIM, MASKED> make_newton_fast(double gamma, double bias, int nx, int dims) {
    NewtonFastPolicy<AXIS, LIM, MASKED> p;
    const float g = (float)gamma, w = (float)bias;
    p.P.g1 = g - 1.0f;
    p.P.hg1 = 0.5f * (g - 1.0f);
    p.P.gam = g;
    p.P.wa = 0.5f * (1.0f + w);
    p.P.wb = 0.5f * (1.0f - w);
    p.P.hom = 0.5f * (1.0f - w);
    p.P.hop = 0.5f * (1.0f + w);
    p.lm.axis = AXIS;
    p.lm.nx = nx;
    p.dims = dims;
    p.dtdx = p.half_dtdx = p.q_dxdt = 0.0f;
    return p;
}

}  // namespace cg
