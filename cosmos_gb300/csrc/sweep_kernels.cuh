// Generic dimensional-sweep kernels (SLIC order 2 / FORCE order 1) over a physics policy.
//
// Reference loop being replaced: Solvers/EulerSecondOrderSolver.cpp:27-100 (and the FORCE,
// SR and GR twins): for every cell, two interface fluxes from a 4-cell stencil, then the
// conservative update.  Here every interface flux is computed once per tile and shared by its
// two cells; every half-step evolution once per cell (for coordinate-free systems).
//
// Layout: structure of arrays, field f of cell (i, j) at base[f * fstride + i * pitch + j].
// Sweeps are out of place (src -> dst): neighbours must see the pre-sweep state.
#pragma once
#include "device_common.cuh"

namespace cg {

struct Geom {
    int nx, ny, pitch, dims, axis, bc;
    size_t fstride;
};

// Where a sweep gets its time step: a fixed value (the per-sweep API) or the device step
// controller (graph-replayed runs; scale 1 or 0.5, or 0.5 * (dt / nsub) for the GR source).
struct DtSrc {
    const StepCtl* ctl;
    double fixed;
    double scale;
    int nsub;        // > 0 selects 0.5 * (dt / nsub)
    int fsel;        // FP32 coefficients: controller slot (0: dt, 1: dt/2)
    FastCoef ffix;   // FP32 coefficients of `fixed`, formed on the host
    CG_D bool get(double& dt) const {
        if (!ctl) { dt = fixed; return true; }
        if (!ctl->active) return false;
        dt = nsub > 0 ? 0.5 * (ctl->dt / nsub) : ctl->dt * scale;
        return true;
    }
    CG_D FastCoef fast_coef() const { return ctl ? ctl->fc[fsel] : ffix; }
};

// Output side of a sweep: fused wavespeed maximum (for the next step's dt) and status bits.
struct SweepOut {
    unsigned long long* smax;  // non-null: reduce the updated cells' wavespeed into it
    StepCtl* ws_ctl;           // non-null: reduce into ws_ctl->smax[ws_ctl->it & 1] instead
    int* status;               // non-null: OR status bits into it
    const unsigned char* mask; // optional per-cell update mask (AMR masked steps)
    CG_D unsigned long long* slot() const { return ws_ctl ? &ws_ctl->smax[ws_ctl->it & 1] : smax; }
    CG_HD bool slot_set() const { return ws_ctl != nullptr || smax != nullptr; }  // a reduction is wanted
};

template <class Pol>
CG_D void load_cell(const Pol& pol, const typename Pol::S* src, const Geom& G, int i, int j, typename Pol::Cell& c) {
    const size_t idx = (size_t)i * G.pitch + j;
#pragma unroll
    for (int f = 0; f < 5; f++) c.v[f] = (typename Pol::X)src[f * G.fstride + idx];
}
template <class Pol>
CG_D void store_cell(const typename Pol::Cell& c, typename Pol::S* dst, const Geom& G, int i, int j) {
    const size_t idx = (size_t)i * G.pitch + j;
#pragma unroll
    for (int f = 0; f < 5; f++) dst[f * G.fstride + idx] = (typename Pol::S)c.v[f];
}

// ------------------------------------------------------------------ X sweep: one row tile
// NT threads; cells s0-2 .. s0+NT-1 staged in shared memory; NT half-step evolutions,
// NT-1 interface fluxes, NT-2 updates per block.
template <class Pol, int ORDER, int NT>
__global__ void __launch_bounds__(NT) sweep_x_kernel(Pol pol, Geom G, const typename Pol::S* __restrict__ src,
                                                     typename Pol::S* __restrict__ dst, DtSrc ds, SweepOut out) {
    using X = typename Pol::X;
    constexpr int TS = NT - 2;
    __shared__ X sc[5][NT + 2];
    __shared__ X sl[5][NT];
    __shared__ X sr[5][NT];
    __shared__ X sf[5][NT];
    const int t = threadIdx.x;
    const int row = blockIdx.y;
    const int s0 = blockIdx.x * TS;
    const int n = G.nx;
    const int send = min(s0 + TS, n);  // one past the last updated cell
    // the step's coefficients are formed once per block (FP64 work is 1/64 rate on GB300)
    __shared__ typename Pol::Coef s_coef;
    __shared__ int s_act;
    if (t == 0) {
        double dt;
        s_act = ds.get(dt);
        if (s_act) s_coef = pol.make_coef(ds, dt);
    }
    __syncthreads();
    const bool act = s_act != 0;
    if (!act) {  // inactive step: keep the ping-pong buffers consistent
        if (s0 + t < send) {
            typename Pol::Cell c;
            load_cell(pol, src, G, row, s0 + t, c);
            store_cell<Pol>(c, dst, G, row, s0 + t);
        }
        return;
    }
    pol.use_coef(s_coef);
    // stage cells s0-2+t (and two more) with ghost mapping along x
    for (int q = t; q < NT + 2; q += NT) {
        const int k = s0 - 2 + q;
        if (k <= send + 1) {
            typename Pol::Cell c;
            load_cell(pol, src, G, row, ghost_index(k, n, G.bc), c);
#pragma unroll
            for (int f = 0; f < 5; f++) sc[f][q] = c.v[f];
        }
    }
    __syncthreads();
    auto cell_at = [&](int q, typename Pol::Cell& c) {
#pragma unroll
        for (int f = 0; f < 5; f++) c.v[f] = sc[f][q];
    };
    // interface s0+t lies between cells s0+t-1 and s0+t; needed when either side updates
    auto iface_needed = [&](int fi) {
        if (fi < s0 || fi > send) return false;
        const bool a = fi - 1 >= s0 && pol.active(row, fi - 1, out.mask);
        const bool b = fi < send && pol.active(row, fi, out.mask);
        return a || b;
    };
    if (ORDER == 2 && Pol::kShared) {
        // half-step evolution of cell s0-1+t from smem cells t, t+1, t+2
        const int k = s0 - 1 + t;
        if (k <= send && (iface_needed(k) || iface_needed(k + 1))) {
            typename Pol::Cell a, b, c;
            typename Pol::Face L, R;
            cell_at(t, a); cell_at(t + 1, b); cell_at(t + 2, c);
            pol.recon(a, b, c, row, k, L, R);
#pragma unroll
            for (int f = 0; f < 5; f++) { sl[f][t] = L.v[f]; sr[f][t] = R.v[f]; }
        }
        __syncthreads();
    }
    {
        const int fi = s0 + t;
        if (t < NT - 1 && iface_needed(fi)) {
            typename Pol::Face L, R;
            if (ORDER == 1) {
                typename Pol::Cell a, b;
                cell_at(t + 1, a); cell_at(t + 2, b);
                pol.face_of(a, L); pol.face_of(b, R);
            } else if (Pol::kShared) {
#pragma unroll
                for (int f = 0; f < 5; f++) { L.v[f] = sr[f][t]; R.v[f] = sl[f][t + 1]; }
            } else {
                typename Pol::Cell a, b, c, d;
                cell_at(t, a); cell_at(t + 1, b); cell_at(t + 2, c); cell_at(t + 3, d);
                pol.recon_side(a, b, c, row, fi - 1, 1, L);
                pol.recon_side(b, c, d, row, fi, 0, R);
            }
            V5<X> F;
            pol.flux(L, R, row, fi, F);
#pragma unroll
            for (int f = 0; f < 5; f++) sf[f][t] = F.v[f];
        }
    }
    __syncthreads();
    typename Pol::W w = 0;
    unsigned long long* const wslot = out.slot();
    const int k = s0 + t;
    if (t < TS && k < send) {
        typename Pol::Cell c, nc;
        cell_at(t + 2, c);
        if (pol.active(row, k, out.mask)) {
            V5<X> FL, FR;
#pragma unroll
            for (int f = 0; f < 5; f++) { FL.v[f] = sf[f][t]; FR.v[f] = sf[f][t + 1]; }
            nc = pol.update(c, FL, FR, row, k);
        } else {
            nc = c;
        }
        store_cell<Pol>(nc, dst, G, row, k);
        if (wslot) w = pol.wavespeed(nc, row, k);
    }
    if (wslot) block_max_to<NT>(wslot, w);
    pol.flush_status(out.status);
}

// ------------------------------------------------------------------ X sweep, cell ownership
// For policies whose half-step evolution gives both faces of a cell (coordinate-free systems).
// Thread t owns cell c = s0 - 1 + t for the whole sweep: it evolves c (both faces stay in
// registers), computes the flux at c's right interface, and updates c with that flux and its
// left neighbour's.  Shared memory carries only what crosses threads: the cells (stencil
// neighbours), the left faces and the fluxes.  NT threads update NT - 2 cells.
template <class X, int NT>
struct XTileSmem {
    X sc[5][NT + 2];  // cells s0-2 .. s0+NT-1 (own cell of thread t at t+1)
    X sl[5][NT];      // left face of the cell owned by thread t
    X sf[5][NT];      // flux at the right interface of the cell owned by thread t
    unsigned char sa[NT + 1];  // masked sweeps: whether the cell owned by thread t updates
};

// One X tile: updates cells s0 .. min(s0 + NT - 2, nx) - 1 of `row`.  `act` and the policy's
// coefficients are block-uniform and already set; all NT threads call this together, and may call
// it again at once for another tile (every shared array is last read before a barrier that the
// next tile's writes to it follow).  Returns the thread's wavespeed maximum over its updated cell
// when want_w (0 otherwise); the caller reduces it.
template <class Pol, int ORDER, int NT>
CG_D typename Pol::W x_own_tile(Pol& pol, const Geom& G, const typename Pol::S* __restrict__ src,
                                typename Pol::S* __restrict__ dst, int row, int s0, bool act, const SweepOut& out,
                                bool want_w, XTileSmem<typename Pol::X, NT>& sm) {
    using X = typename Pol::X;
    using Cell = typename Pol::Cell;
    using Face = typename Pol::Face;
    constexpr int TS = NT - 2;
    auto& sc = sm.sc;
    auto& sl = sm.sl;
    auto& sf = sm.sf;
    const int t = threadIdx.x;
    const int n = G.nx;
    const int send = min(s0 + TS, n);
    const int c = s0 - 1 + t;  // owned cell (may be a ghost position)
    // own cell and, for the two edge threads, the extra stencil cell
    const bool live = c <= send;  // cells beyond send neither update nor feed an interface
    Cell own;
    if (live) {
        load_cell(pol, src, G, row, ghost_index(c, n, G.bc), own);
#pragma unroll
        for (int f = 0; f < 5; f++) sc[f][t + 1] = own.v[f];
    }
    if (t == 0) {
        Cell e;
        load_cell(pol, src, G, row, ghost_index(s0 - 2, n, G.bc), e);
#pragma unroll
        for (int f = 0; f < 5; f++) sc[f][0] = e.v[f];
    }
    if ((t == NT - 1 && live) || c == send) {  // c + 1 <= send + 1 <= n + 1: a valid ghost
        Cell e;
        load_cell(pol, src, G, row, ghost_index(c + 1, n, G.bc), e);
#pragma unroll
        for (int f = 0; f < 5; f++) sc[f][t + 2] = e.v[f];
    }
    // Masked sweeps (AMR levels) reconstruct only cells next to an updating cell and evaluate only
    // the interfaces of updating cells; the skipped values are never read.
    const bool msk = Pol::kMasked && out.mask != nullptr;
    bool my_act = false;
    if (msk) {
        my_act = act && t >= 1 && c < send && pol.active(row, c, out.mask);
        sm.sa[t] = my_act ? 1 : 0;
        if (t == NT - 1) sm.sa[NT] = 0;  // cell s0 + NT - 1 belongs to the next tile
    }
    __syncthreads();
    if (!act) {  // inactive step: keep the ping-pong buffers consistent
        if (t >= 1 && c < send) store_cell<Pol>(own, dst, G, row, c);
        return typename Pol::W(0);
    }
    const bool need_recon = !msk || my_act || sm.sa[t + 1] || (t >= 1 && sm.sa[t - 1]);
    const bool need_flux = !msk || my_act || sm.sa[t + 1];  // interface between c and c + 1
    Face L, R;
    if (live && need_recon) {
        if (ORDER == 2) {
            Cell a, b;
#pragma unroll
            for (int f = 0; f < 5; f++) { a.v[f] = sc[f][t]; b.v[f] = sc[f][t + 2]; }
            pol.recon(a, own, b, row, c, L, R);
        } else {
            pol.face_of(own, L);
            pol.face_of(own, R);
        }
#pragma unroll
        for (int f = 0; f < 5; f++) sl[f][t] = L.v[f];
    }
    __syncthreads();
    V5<X> Fr;
    if (live && c < send && t < NT - 1 && need_flux) {  // right interface of c, between c and c + 1
        Face Rn;
        if (ORDER == 2) {
#pragma unroll
            for (int f = 0; f < 5; f++) Rn.v[f] = sl[f][t + 1];
        } else {
            Cell b;
#pragma unroll
            for (int f = 0; f < 5; f++) b.v[f] = sc[f][t + 2];
            pol.face_of(b, Rn);
        }
        pol.flux(R, Rn, row, c + 1, Fr);
#pragma unroll
        for (int f = 0; f < 5; f++) sf[f][t] = Fr.v[f];
    }
    __syncthreads();
    typename Pol::W w = 0;
    if (t >= 1 && c < send) {
        Cell nc = own;
        if (msk ? my_act : pol.active(row, c, out.mask)) {
            V5<X> Fl;
#pragma unroll
            for (int f = 0; f < 5; f++) Fl.v[f] = sf[f][t - 1];
            nc = pol.update(own, Fl, Fr, row, c);
        }
        store_cell<Pol>(nc, dst, G, row, c);
        if (want_w) w = pol.wavespeed(nc, row, c);
    }
    pol.flush_status(out.status);
    return w;
}

template <class Pol, int ORDER, int NT>
__global__ void __launch_bounds__(NT) sweep_x_own_kernel(Pol pol, Geom G, const typename Pol::S* __restrict__ src,
                                                         typename Pol::S* __restrict__ dst, DtSrc ds, SweepOut out) {
    __shared__ XTileSmem<typename Pol::X, NT> sm;
    __shared__ typename Pol::Coef s_coef;
    __shared__ int s_act;
    if (threadIdx.x == 0) {
        double dt;
        s_act = ds.get(dt);
        if (s_act) s_coef = pol.make_coef(ds, dt);
    }
    __syncthreads();
    const bool act = s_act != 0;
    if (act) pol.use_coef(s_coef);
    unsigned long long* wslot = out.slot();
    const auto w = x_own_tile<Pol, ORDER, NT>(pol, G, src, dst, blockIdx.y, blockIdx.x * (NT - 2), act, out,
                                              wslot != nullptr, sm);
    if (wslot) block_max_to<NT>(wslot, w);
}

// ------------------------------------------------------------------ Y sweep: column march
// One thread per column marches SEG rows keeping the stencil in registers.
// One Y segment: columns j0 .. j0 + NT - 1, rows y0 .. y1 - 1 (y1 <= ny).  `act` and the
// policy's coefficients are block-uniform and already set.  Returns the thread's wavespeed
// maximum over its updated cells when want_w (0 otherwise); the caller reduces it.
template <class Pol, int ORDER, int NT>
CG_D typename Pol::W y_march_seg(Pol& pol, const Geom& G, const typename Pol::S* __restrict__ src,
                                 typename Pol::S* __restrict__ dst, int j0, int y0, int y1, bool act,
                                 const SweepOut& out, bool want_w) {
    using X = typename Pol::X;
    using Cell = typename Pol::Cell;
    using Face = typename Pol::Face;
    const int j = j0 + threadIdx.x;
    const int n = G.ny;
    const bool col_ok = j < G.nx;
    if (!act) {
        if (col_ok)
            for (int y = y0; y < y1; y++) {
                Cell c;
                load_cell(pol, src, G, y, j, c);
                store_cell<Pol>(c, dst, G, y, j);
            }
        return typename Pol::W(0);
    }
    typename Pol::W w = 0;
    if (col_ok) {
        auto ld = [&](int y, Cell& c) { load_cell(pol, src, G, ghost_index(y, n, G.bc), j, c); };
        auto need = [&](int fi) {  // interface between fi-1 and fi
            if (!Pol::kMasked) return true;  // unmasked: every interface in the segment is used
            const bool a = fi - 1 >= y0 && fi - 1 < y1 && pol.active(j, fi - 1, out.mask);
            const bool b = fi >= y0 && fi < y1 && pol.active(j, fi, out.mask);
            return a || b;
        };
        // Masked sweeps (AMR levels) reconstruct a cell only when one of its two interfaces is
        // needed; nf_next carries the next interface's need so each is evaluated once.
        const bool msk = Pol::kMasked && out.mask != nullptr;
        // window: cm1 = y-1, c0 = y, c1 = y+1, c2 = y+2
        Cell cm2, cm1, c0, c1, c2;
        ld(y0 - 2, cm2); ld(y0 - 1, cm1); ld(y0, c0); ld(y0 + 1, c1);
        V5<X> Fp, Fn;
        Face R0;  // right face of the current cell (shared recon)
        bool nf_next = msk ? need(y0 + 1) : true;
        if (ORDER == 1) {
            if (need(y0)) { Face L, R; pol.face_of(cm1, L); pol.face_of(c0, R); pol.flux(L, R, j, y0, Fp); }
        } else if (Pol::kShared) {
            Face Lm1, Rm1, L0;
            if (need(y0)) {
                pol.recon(cm2, cm1, c0, j, y0 - 1, Lm1, Rm1);
                pol.recon(cm1, c0, c1, j, y0, L0, R0);
                pol.flux(Rm1, L0, j, y0, Fp);
            } else if (nf_next) {
                pol.recon(cm1, c0, c1, j, y0, L0, R0);
            }
        } else {
            if (need(y0)) {
                Face L, R;
                pol.recon_side(cm2, cm1, c0, j, y0 - 1, 1, L);
                pol.recon_side(cm1, c0, c1, j, y0, 0, R);
                pol.flux(L, R, j, y0, Fp);
            }
        }
        for (int y = y0; y < y1; y++) {
            ld(y + 2, c2);
            const bool nf = msk ? nf_next : need(y + 1);
            if (msk) nf_next = need(y + 2);
            if (ORDER == 1) {
                if (nf) { Face L, R; pol.face_of(c0, L); pol.face_of(c1, R); pol.flux(L, R, j, y + 1, Fn); }
            } else if (Pol::kShared) {
                Face L1, R1;
                if (nf || nf_next) pol.recon(c0, c1, c2, j, y + 1, L1, R1);  // R1 is read only if nf_next
                if (nf) pol.flux(R0, L1, j, y + 1, Fn);
                R0 = R1;
            } else {
                if (nf) {
                    Face L, R;
                    pol.recon_side(cm1, c0, c1, j, y, 1, L);
                    pol.recon_side(c0, c1, c2, j, y + 1, 0, R);
                    pol.flux(L, R, j, y + 1, Fn);
                }
            }
            Cell nc = c0;
            if (pol.active(j, y, out.mask)) nc = pol.update(c0, Fp, Fn, j, y);
            store_cell<Pol>(nc, dst, G, y, j);
            if (want_w) { const typename Pol::W ws = pol.wavespeed(nc, j, y); w = (ws > w) ? ws : w; }
            Fp = Fn;
            cm1 = c0; c0 = c1; c1 = c2;
        }
    }
    pol.flush_status(out.status);
    return w;
}

template <class Pol, int ORDER, int NT, int SEG>
__global__ void __launch_bounds__(NT) sweep_y_kernel(Pol pol, Geom G, const typename Pol::S* __restrict__ src,
                                                     typename Pol::S* __restrict__ dst, DtSrc ds, SweepOut out) {
    __shared__ typename Pol::Coef s_coef;
    __shared__ int s_act;
    if (threadIdx.x == 0) {
        double dt;
        s_act = ds.get(dt);
        if (s_act) s_coef = pol.make_coef(ds, dt);
    }
    __syncthreads();
    const bool act = s_act != 0;
    if (act) pol.use_coef(s_coef);
    unsigned long long* wslot = out.slot();
    const int y0 = blockIdx.y * SEG;
    const auto w = y_march_seg<Pol, ORDER, NT>(pol, G, src, dst, blockIdx.x * NT, y0, min(y0 + SEG, G.ny), act, out,
                                               wslot != nullptr);
    if (wslot) block_max_to<NT>(wslot, w);
}

// ------------------------------------------------------------------ helpers
template <class Pol, int NT>
__global__ void __launch_bounds__(NT) wavespeed_kernel(Pol pol, Geom G, const typename Pol::S* __restrict__ src,
                                                       SweepOut out) {
    typename Pol::W w = 0;
    const size_t ncell = (size_t)G.nx * G.ny;
    for (size_t c = (size_t)blockIdx.x * NT + threadIdx.x; c < ncell; c += (size_t)gridDim.x * NT) {
        const int i = (int)(c / G.nx), j = (int)(c % G.nx);
        typename Pol::Cell cc;
        load_cell(pol, src, G, i, j, cc);
        // wavespeed takes (line, k) in the X-sweep convention: line = row i, k = column j
        const typename Pol::W ws = pol.wavespeed(cc, i, j);
        w = (ws > w) ? ws : w;
    }
    block_max_to<NT>(out.slot(), w);
    pol.flush_status(out.status);
}

}  // namespace cg
