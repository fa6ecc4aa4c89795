// FP64 reference-exact kernels.  Compiled with --fmad=false so that every double operation is
// rounded exactly as the reference's (built with -ffp-contract=off) -- results are bit-identical.
#include "launch.h"
#include "policies.cuh"

namespace cg {

namespace {

constexpr int kXThreads = 128;  // X sweep tile: 128 evolutions, 127 fluxes, 126 updates
constexpr int kYThreads = 64;   // Y sweep: columns per block
constexpr int kYSeg = 16;       // Y sweep: rows marched per thread

template <class Sys>
ExactPolicy<Sys> make_policy(const SweepArgs& a, const Sys& sys) {
    ExactPolicy<Sys> p;
    p.sys = sys;
    p.lm.axis = a.G.axis;
    p.lm.nx = a.G.nx;
    p.dims = a.G.dims;
    p.order = a.order;
    p.ny = a.G.ny;
    p.dx = a.dx;
    p.dt = 0.0;
    p.w = a.bias;
    p.lim = a.lim;
    p.capped = 0;
    return p;
}

template <class Pol>
cudaError_t run_sweep(const Pol& pol, const SweepArgs& a) {
    const Geom& G = a.G;
    const double* src = (const double*)a.src;
    double* dst = (double*)a.dst;
    if (G.axis == 0) {
        dim3 grid((G.nx + kXThreads - 3) / (kXThreads - 2), G.ny);
        if constexpr (Pol::kShared) {
            if (a.order == 2) sweep_x_own_kernel<Pol, 2, kXThreads><<<grid, kXThreads, 0, a.stream>>>(pol, G, src, dst, a.ds, a.out);
            else sweep_x_own_kernel<Pol, 1, kXThreads><<<grid, kXThreads, 0, a.stream>>>(pol, G, src, dst, a.ds, a.out);
        } else {
            if (a.order == 2) sweep_x_kernel<Pol, 2, kXThreads><<<grid, kXThreads, 0, a.stream>>>(pol, G, src, dst, a.ds, a.out);
            else sweep_x_kernel<Pol, 1, kXThreads><<<grid, kXThreads, 0, a.stream>>>(pol, G, src, dst, a.ds, a.out);
        }
    } else {
        dim3 grid((G.nx + kYThreads - 1) / kYThreads, (G.ny + kYSeg - 1) / kYSeg);
        if (a.order == 2) sweep_y_kernel<Pol, 2, kYThreads, kYSeg><<<grid, kYThreads, 0, a.stream>>>(pol, G, src, dst, a.ds, a.out);
        else sweep_y_kernel<Pol, 1, kYThreads, kYSeg><<<grid, kYThreads, 0, a.stream>>>(pol, G, src, dst, a.ds, a.out);
    }
    count_launch();
    return cudaGetLastError();
}

GRExact make_gr(const SweepArgs& a) {
    GRExact s;
    s.g = a.gamma;
    s.bh = BHExact{a.bh[0], a.bh[1], a.bh[2], a.bh[3], a.bh[4]};
    s.h = a.dx;
    s.capped = nullptr;
    return s;
}

}  // namespace

cudaError_t launch_sweep_exact(const SweepArgs& a) {
    if (a.system == 0) return run_sweep(make_policy(a, NewtonExact<double>{a.gamma}), a);
    if (a.system == 1) return run_sweep(make_policy(a, SRExact{a.gamma, nullptr}), a);
    return run_sweep(make_policy(a, make_gr(a)), a);
}

cudaError_t launch_wavespeed_exact(const SweepArgs& a, unsigned long long* slot) {
    constexpr int NT = 256;
    Geom G = a.G;
    SweepArgs b = a;
    b.G.axis = 0;
    SweepOut o = a.out;
    if (slot) { o.smax = slot; o.ws_ctl = nullptr; }
    const size_t n = (size_t)G.nx * G.ny;
    int blocks = (int)((n + NT - 1) / NT);
    if (blocks > device_sm_count() * 16) blocks = device_sm_count() * 16;
    const double* src = (const double*)a.src;
    if (a.system == 0) wavespeed_kernel<ExactPolicy<NewtonExact<double>>, NT><<<blocks, NT, 0, a.stream>>>(make_policy(b, NewtonExact<double>{a.gamma}), b.G, src, o);
    else if (a.system == 1) wavespeed_kernel<ExactPolicy<SRExact>, NT><<<blocks, NT, 0, a.stream>>>(make_policy(b, SRExact{a.gamma, nullptr}), b.G, src, o);
    else wavespeed_kernel<ExactPolicy<GRExact>, NT><<<blocks, NT, 0, a.stream>>>(make_policy(b, make_gr(a)), b.G, src, o);
    count_launch();
    return cudaGetLastError();
}

// ------------------------------------------------------------------ GR RK4 source step
// Solvers/BlackHoleEulerForcingSolver.cpp:187-250: per cell away from the horizon (cell and its
// 2 (1D) or 4 (2D) neighbours outside), conserved neighbours from a 1-ghost transmissive copy,
// classical RK4 with interleaved fractional sweeps, converted back at the cell.
__global__ void __launch_bounds__(128) rk_source_kernel(GRExact sys, Geom G, double dx, double w, int lim,
                                                        const double* __restrict__ src, double* __restrict__ dst,
                                                        DtSrc ds, int* status) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;
    if (j >= G.nx) return;
    const size_t idx = (size_t)i * G.pitch + j;
    double dt;
    int capped = 0;
    sys.capped = &capped;
    bool on = ds.get(dt);
    const BHExact& b = sys.bh;
    if (on) {
        if (G.dims == 1)
            on = !b.excised(j * dx, 0.0, 0.0) && !b.excised((j - 1) * dx, 0.0, 0.0) && !b.excised((j + 1) * dx, 0.0, 0.0);
        else
            on = !b.excised(j * dx, i * dx, 0.0) && !b.excised((j - 1) * dx, i * dx, 0.0) &&
                 !b.excised((j + 1) * dx, i * dx, 0.0) && !b.excised(j * dx, (i - 1) * dx, 0.0) &&
                 !b.excised(j * dx, (i + 1) * dx, 0.0);
    }
    if (!on) {
#pragma unroll
        for (int f = 0; f < 5; f++) dst[f * G.fstride + idx] = src[f * G.fstride + idx];
        return;
    }
    auto ld = [&](int ii, int jj, double* p) {
        const size_t k = (size_t)ghost_index(ii, G.ny, 0) * G.pitch + ghost_index(jj, G.nx, 0);
#pragma unroll
        for (int f = 0; f < 5; f++) p[f] = src[f * G.fstride + k];
    };
    double p[5], cl[5], cm[5], cr[5], ct[5], cb[5], nc[5];
    const double y = G.dims == 1 ? 0.0 : i * dx;
    const Pt q{j * dx, y, 0.0};
    ld(i, j - 1, p); sys.cons(p, Pt{(j - 1) * dx, y, 0.0}, cl);
    ld(i, j, p); sys.cons(p, q, cm);
    ld(i, j + 1, p); sys.cons(p, Pt{(j + 1) * dx, y, 0.0}, cr);
    if (G.dims == 2) {
        ld(i - 1, j, p); sys.cons(p, Pt{j * dx, (i - 1) * dx, 0.0}, ct);
        ld(i + 1, j, p); sys.cons(p, Pt{j * dx, (i + 1) * dx, 0.0}, cb);
    }
    rk_cell_exact(sys, G.dims, cl, cm, cr, ct, cb, q, dx, dt, w, lim, nc);
    sys.prim(nc, q, p);
#pragma unroll
    for (int f = 0; f < 5; f++) dst[f * G.fstride + idx] = p[f];
    if (capped && status) atomicOr(status, ST_NEWTON_CAP);
}

cudaError_t launch_rk_source_exact(const SweepArgs& a) {
    dim3 grid((a.G.nx + 127) / 128, a.G.ny);
    rk_source_kernel<<<grid, 128, 0, a.stream>>>(make_gr(a), a.G, a.dx, a.bias, a.lim, (const double*)a.src,
                                                 (double*)a.dst, a.ds, a.out.status);
    count_launch();
    return cudaGetLastError();
}

// ------------------------------------------------------------------ conversions
__global__ void prim_in_exact_kernel(const double* __restrict__ aos, double* __restrict__ soa, Geom G) {
    const size_t n = (size_t)G.nx * G.ny;
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
        const size_t i = c / G.nx, j = c % G.nx;
#pragma unroll
        for (int f = 0; f < 5; f++) soa[f * G.fstride + i * G.pitch + j] = aos[5 * c + f];
    }
}
__global__ void prim_out_exact_kernel(const double* __restrict__ soa, double* __restrict__ aos, Geom G) {
    const size_t n = (size_t)G.nx * G.ny;
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
        const size_t i = c / G.nx, j = c % G.nx;
#pragma unroll
        for (int f = 0; f < 5; f++) aos[5 * c + f] = soa[f * G.fstride + i * G.pitch + j];
    }
}
static int grid_for(size_t n) {
    size_t b = (n + 255) / 256;
    return (int)(b > device_sm_count() * 32 ? device_sm_count() * 32 : (b ? b : 1));
}
cudaError_t launch_prim_in_exact(const double* aos, void* soa, const Geom& G, cudaStream_t st) {
    prim_in_exact_kernel<<<grid_for((size_t)G.nx * G.ny), 256, 0, st>>>(aos, (double*)soa, G);
    count_launch();
    return cudaGetLastError();
}
cudaError_t launch_prim_out_exact(const void* soa, double* aos, const Geom& G, cudaStream_t st) {
    prim_out_exact_kernel<<<grid_for((size_t)G.nx * G.ny), 256, 0, st>>>((const double*)soa, aos, G);
    count_launch();
    return cudaGetLastError();
}

// ------------------------------------------------------------------ step controller
// Solvers/EulerSolvers.cpp:130-161: dt = CFL * (dx / s_max); x0.2 while it <= 5; clamped so
// that t + dt does not pass t_final.  The solver loop `while (t < t_final)` becomes `active`.
__global__ void dt_kernel(StepCtl* c) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    if (!(c->t < c->t_final) || c->it >= c->it_limit) {
        c->active = 0;
        c->dt = 0.0;
        return;
    }
    double dt;
    if (c->dt_fixed) {
        dt = c->dt_fixed[c->it];
    } else {
        const double smax = __longlong_as_double((long long)c->smax[c->it & 1]);
        dt = c->cfl * (c->dx / smax);
        if (c->it <= 5) dt = dt * 0.2;
        if ((c->t + dt) > c->t_final) dt = c->t_final - c->t;
    }
    if (!(dt > 0.0) || !isfinite(dt)) c->status |= ST_NONFINITE;
    if (c->dt_log) c->dt_log[c->it] = dt;
    c->dt = dt;
    c->fc[0] = make_fast_coef(dt, c->dx);
    c->fc[1] = make_fast_coef(dt * 0.5, c->dx);
    c->active = 1;
    c->smax[(c->it + 1) & 1] = 0ull;
    c->t = c->t + dt;
    c->it = c->it + 1;
}
cudaError_t launch_dt_kernel(StepCtl* ctl, cudaStream_t st) {
    dt_kernel<<<1, 32, 0, st>>>(ctl);
    count_launch();
    return cudaGetLastError();
}

// ------------------------------------------------------------------ AMR flagging
// Conserved state of a cell for the flag passes: FP64 storage and the FP32 black-hole storage hold
// primitives (converted with the system's exact cons), FP32 Newtonian and SR storage holds
// conserved values already.
struct ConsLoader {
    int system, precision;
    Geom G;
    const void* state;
    NewtonExact<double> nw;
    SRExact sr;
    GRExact gr;
    CG_D void get(int i, int j, Pt q, double* u) const {
        const size_t k = (size_t)ghost_index(i, G.ny, 0) * G.pitch + ghost_index(j, G.nx, 0);
        if (precision == 1 && system != 2) {  // FP32 Newtonian / SR storage is conserved
            const float* s = (const float*)state;
#pragma unroll
            for (int f = 0; f < 5; f++) u[f] = (double)s[f * G.fstride + k];
            return;
        }
        // primitives: FP64 storage, and the FP32 black-hole storage
        double p[5];
#pragma unroll
        for (int f = 0; f < 5; f++)
            p[f] = precision == 1 ? (double)((const float*)state)[f * G.fstride + k]
                                  : ((const double*)state)[f * G.fstride + k];
        cons_of(p, q, u);
    }
    CG_D void cons_of(const double* p, Pt q, double* u) const {
        if (system == 0) nw.cons(p, q, u);
        else if (system == 1) sr.cons(p, q, u);
        else gr.cons(p, q, u);
    }
};

// Refinement pass, AMR/EulerAMR.cpp:207-229 (1D) and :400-431 (2D); the SR and GR Level-1 drivers
// read the bottom neighbour at [i+2][j+2] (AMR/RelativisticEulerAMR.cpp:422,
// AMR/BlackHoleEulerAMR.cpp:490), whose corner ghost keeps the default state (1,0,0,0,1).
// The Level-2 drivers' passes (AMR/EulerAMR.cpp:643-664 coarse, :699-722 intermediate, and the SR
// twins, whose coarse pass reads [i+2][j+1], AMR/RelativisticEulerAMR.cpp:1008) use `plain` (the
// Newtonian neighbours for every system), a threshold other than the tolerance, the coarse spacing
// as the divisor on a finer grid (`div`) and, for the intermediate pass, `need_on` (only cells
// whose own flag is on are tested).  dx places the cells (black-hole coordinates).
__global__ void amr_flags_kernel(ConsLoader L, double dx, double tol, double div, int plain, int need_on,
                                 unsigned char* coarse, unsigned char* fine) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;
    const Geom& G = L.G;
    if (j >= G.nx) return;
    if (need_on && !coarse[(size_t)i * G.nx + j]) return;
    double c[5], l[5], r[5], t[5], b[5];
    bool hit = false;
    if (G.dims == 1) {
        L.get(0, j - 1, Pt{(j - 1) * dx, 0.0, 0.0}, l);
        L.get(0, j, Pt{j * dx, 0.0, 0.0}, c);
        L.get(0, j + 1, Pt{(j + 1) * dx, 0.0, 0.0}, r);
#pragma unroll
        for (int k = 0; k < 5; k++)
            if (fabs((c[k] - l[k]) / div) >= tol || fabs((r[k] - c[k]) / div) >= tol) hit = true;
    } else {
        L.get(i - 1, j, Pt{j * dx, (i - 1) * dx, 0.0}, t);
        L.get(i, j - 1, Pt{(j - 1) * dx, i * dx, 0.0}, l);
        L.get(i, j, Pt{j * dx, i * dx, 0.0}, c);
        L.get(i, j + 1, Pt{(j + 1) * dx, i * dx, 0.0}, r);
        if (L.system == 0 || plain) L.get(i + 1, j, Pt{j * dx, (i + 1) * dx, 0.0}, b);
        else if (i == G.ny - 1 && j == G.nx - 1) {
            const double dflt[5] = {1.0, 0.0, 0.0, 0.0, 1.0};
            if (L.precision == 1) {
                // FP32 grids hold conserved values; the default state in conserved form
                L.cons_of(dflt, Pt{(j + 1) * dx, (i + 1) * dx, 0.0}, b);
            } else {
                L.cons_of(dflt, Pt{(j + 1) * dx, (i + 1) * dx, 0.0}, b);
            }
        } else L.get(i + 1, j + 1, Pt{(j + 1) * dx, (i + 1) * dx, 0.0}, b);
#pragma unroll
        for (int k = 0; k < 5; k++)
            if (fabs((c[k] - t[k]) / div) >= tol || fabs((b[k] - c[k]) / div) >= tol ||
                fabs((c[k] - l[k]) / div) >= tol || fabs((r[k] - c[k]) / div) >= tol)
                hit = true;
    }
    if (!hit) return;
    if (G.dims == 1) {
        coarse[j] = 0;
        fine[2 * j] = 1;
        fine[2 * j + 1] = 1;
    } else {
        coarse[(size_t)i * G.nx + j] = 0;
        const size_t fw = 2 * (size_t)G.nx;
        fine[(2 * i) * fw + 2 * j] = 1;
        fine[(2 * i) * fw + 2 * j + 1] = 1;
        fine[(2 * i + 1) * fw + 2 * j] = 1;
        fine[(2 * i + 1) * fw + 2 * j + 1] = 1;
    }
}

static ConsLoader make_loader(const SweepArgs& a, int precision, const void* state, const Geom& G) {
    ConsLoader L;
    L.system = a.system;
    L.precision = precision;
    L.G = G;
    L.state = state;
    L.nw = NewtonExact<double>{a.gamma};
    L.sr = SRExact{a.gamma, nullptr};
    L.gr = make_gr(a);
    return L;
}

cudaError_t launch_amr_flags(const SweepArgs& a, int precision, double tol, unsigned char* coarse, unsigned char* fine) {
    return launch_amr_flags_ex(a, precision, tol, a.dx, false, false, coarse, fine);
}
cudaError_t launch_amr_flags_ex(const SweepArgs& a, int precision, double thr, double div, bool plain, bool need_on,
                                unsigned char* coarse, unsigned char* fine) {
    dim3 grid((a.G.nx + 127) / 128, a.G.ny);
    amr_flags_kernel<<<grid, 128, 0, a.stream>>>(make_loader(a, precision, a.src, a.G), a.dx, thr, div, plain ? 1 : 0,
                                                 need_on ? 1 : 0, coarse, fine);
    count_launch();
    return cudaGetLastError();
}

// Derefinement pass, AMR/EulerAMR.cpp:310-345 (1D) and :538-586 (2D); GR coordinates
// AMR/BlackHoleEulerAMR.cpp:388-421 (1D fine cells read one fine cell to the left) and :632-686.
// Restriction writes the coarse state (FP64 storage only holds primitives, converted with the
// system's exact prim; FP32 storage receives the averaged conserved state).
// The Level-2 drivers' passes (AMR/EulerAMR.cpp:804-838 on the fine grid, :875-911 on the
// intermediate grid) take other thresholds and the coarse spacing as divisor (`div`), and are
// `strict`: they derefine only where every child is flagged (Level-1 tests the first child).
__global__ void amr_derefine_kernel(ConsLoader F, Geom CG, double dx, double half, double div, int strict,
                                    unsigned char* coarse, unsigned char* fine, void* coarse_state) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;
    if (j >= CG.nx) return;
    const double fdx = dx * 0.5;
    bool marked = false;
    double c[5], l[5], r[5], t[5], b[5], avg[5];
    Pt qc;
    if (CG.dims == 1) {
        F.get(0, 2 * j, Pt{((j * 2) - 1) * fdx, 0.0, 0.0}, l);
        F.get(0, 2 * j + 1, Pt{(j * 2) * fdx, 0.0, 0.0}, c);
        F.get(0, 2 * j + 2, Pt{((j * 2) + 1) * fdx, 0.0, 0.0}, r);
#pragma unroll
        for (int k = 0; k < 5; k++)
            if (fabs((c[k] - l[k]) / div) >= half || fabs((r[k] - c[k]) / div) >= half) marked = true;
        if (marked || !fine[2 * j] || (strict && !fine[2 * j + 1])) return;
        fine[2 * j] = 0;
        fine[2 * j + 1] = 0;
        coarse[j] = 1;
        double u0[5], u1[5];
        F.get(0, 2 * j, Pt{(j * 2) * fdx, 0.0, 0.0}, u0);
        F.get(0, 2 * j + 1, Pt{((j * 2) + 1) * fdx, 0.0, 0.0}, u1);
#pragma unroll
        for (int k = 0; k < 5; k++) avg[k] = 0.5 * (u0[k] + u1[k]);
        qc = Pt{j * dx, 0.0, 0.0};
    } else {
        F.get(2 * i, 2 * j + 1, Pt{((j * 2) + 1) * fdx, (i * 2) * fdx, 0.0}, t);
        F.get(2 * i + 1, 2 * j, Pt{(j * 2) * fdx, ((i * 2) + 1) * fdx, 0.0}, l);
        F.get(2 * i + 1, 2 * j + 1, Pt{((j * 2) + 1) * fdx, ((i * 2) + 1) * fdx, 0.0}, c);
        F.get(2 * i + 1, 2 * j + 2, Pt{((j * 2) + 2) * fdx, ((i * 2) + 1) * fdx, 0.0}, r);
        F.get(2 * i + 2, 2 * j + 1, Pt{((j * 2) + 1) * fdx, ((i * 2) + 2) * fdx, 0.0}, b);
#pragma unroll
        for (int k = 0; k < 5; k++)
            if (fabs((c[k] - t[k]) / div) >= half || fabs((b[k] - c[k]) / div) >= half ||
                fabs((c[k] - l[k]) / div) >= half || fabs((r[k] - c[k]) / div) >= half)
                marked = true;
        const size_t fw = 2 * (size_t)CG.nx;
        if (marked || !fine[(2 * i) * fw + 2 * j]) return;
        if (strict && !(fine[(2 * i) * fw + 2 * j + 1] && fine[(2 * i + 1) * fw + 2 * j] &&
                        fine[(2 * i + 1) * fw + 2 * j + 1]))
            return;
        fine[(2 * i) * fw + 2 * j] = 0;
        fine[(2 * i) * fw + 2 * j + 1] = 0;
        fine[(2 * i + 1) * fw + 2 * j] = 0;
        fine[(2 * i + 1) * fw + 2 * j + 1] = 0;
        coarse[(size_t)i * CG.nx + j] = 1;
        double u0[5], u1[5], u2[5], u3[5];
        F.get(2 * i, 2 * j, Pt{(j * 2) * fdx, (i * 2) * fdx, 0.0}, u0);
        F.get(2 * i, 2 * j + 1, Pt{((j * 2) + 1) * fdx, (i * 2) * fdx, 0.0}, u1);
        F.get(2 * i + 1, 2 * j, Pt{(j * 2) * fdx, ((i * 2) + 1) * fdx, 0.0}, u2);
        F.get(2 * i + 1, 2 * j + 1, Pt{((j * 2) + 1) * fdx, ((i * 2) + 1) * fdx, 0.0}, u3);
#pragma unroll
        for (int k = 0; k < 5; k++) avg[k] = 0.25 * (((u0[k] + u1[k]) + u2[k]) + u3[k]);
        qc = Pt{j * dx, i * dx, 0.0};
    }
    if (!coarse_state) return;
    const size_t idx = (size_t)i * CG.pitch + j;
    if (F.precision == 1) {
        float* s = (float*)coarse_state;
#pragma unroll
        for (int k = 0; k < 5; k++) s[k * CG.fstride + idx] = (float)avg[k];
    } else {
        double p[5];
        if (F.system == 0) F.nw.prim(avg, qc, p);
        else if (F.system == 1) F.sr.prim(avg, qc, p);
        else F.gr.prim(avg, qc, p);
        double* s = (double*)coarse_state;
#pragma unroll
        for (int k = 0; k < 5; k++) s[k * CG.fstride + idx] = p[k];
    }
}

cudaError_t launch_amr_derefine(const SweepArgs& a, int precision, const void* fine_state, const Geom& FG, double tol,
                                unsigned char* coarse, unsigned char* fine, void* coarse_state) {
    return launch_amr_derefine_ex(a, precision, fine_state, FG, tol * 0.5, a.dx, false, coarse, fine, coarse_state);
}
cudaError_t launch_amr_derefine_ex(const SweepArgs& a, int precision, const void* fine_state, const Geom& FG, double thr,
                                   double div, bool strict, unsigned char* coarse, unsigned char* fine,
                                   void* coarse_state) {
    dim3 grid((a.G.nx + 127) / 128, a.G.ny);
    amr_derefine_kernel<<<grid, 128, 0, a.stream>>>(make_loader(a, precision, fine_state, FG), a.G, a.dx, thr, div,
                                                    strict ? 1 : 0, coarse, fine, coarse_state);
    count_launch();
    return cudaGetLastError();
}

// End-of-step level exchange of the Level-1 drivers, AMR/EulerAMR.cpp:287-307 (1D) and :500-546
// (2D): a coarse cell whose flag is off takes the conserved average of its fine children
// (0.5 (a + b) in 1D, 0.25 (((a + b) + c) + d) in 2D, then the system's prim), and every fine
// child whose flag is off takes its parent's state.  One thread per coarse cell touches only
// that cell and its own children, in the reference's order (restriction, then injection).  The
// Level-2 drivers' exchange between the intermediate and fine levels (AMR/EulerAMR.cpp:780-801) is
// `strict`: restriction only where every child is flagged, injection only under a flagged parent.
// FP64 storage holds primitives; FP32 Newtonian/SR storage holds conserved values, which are
// averaged in FP64 and copied as stored.
__global__ void amr_sync_kernel(ConsLoader F, Geom CG, void* coarse_state, void* fine_state,
                                const unsigned char* coarse, const unsigned char* fine, int strict) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;
    if (j >= CG.nx) return;
    const Geom& FG = F.G;
    const int nk = CG.dims == 1 ? 2 : 4;
    int ki[4], kj[4];
    for (int q = 0; q < nk; q++) {
        ki[q] = CG.dims == 1 ? 0 : 2 * i + (q >> 1);
        kj[q] = 2 * j + (q & 1);
    }
    const size_t cidx = (size_t)i * CG.pitch + j;
    const bool fp32 = F.precision == 1;
    const bool on = coarse[(size_t)i * CG.nx + j] != 0;
    bool all = true;
    for (int q = 0; q < nk; q++) all = all && fine[(size_t)ki[q] * FG.nx + kj[q]];
    if (!on && (!strict || all)) {
        double u[4][5], avg[5];
        for (int q = 0; q < nk; q++) F.get(ki[q], kj[q], Pt{0.0, 0.0, 0.0}, u[q]);
#pragma unroll
        for (int k = 0; k < 5; k++)
            avg[k] = nk == 2 ? 0.5 * (u[0][k] + u[1][k]) : 0.25 * (((u[0][k] + u[1][k]) + u[2][k]) + u[3][k]);
        if (fp32) {
#pragma unroll
            for (int k = 0; k < 5; k++) ((float*)coarse_state)[k * CG.fstride + cidx] = (float)avg[k];
        } else {
            double p[5];
            if (F.system == 0) F.nw.prim(avg, Pt{0.0, 0.0, 0.0}, p);
            else F.sr.prim(avg, Pt{0.0, 0.0, 0.0}, p);
#pragma unroll
            for (int k = 0; k < 5; k++) ((double*)coarse_state)[k * CG.fstride + cidx] = p[k];
        }
    }
    for (int q = 0; q < nk; q++) {
        if (fine[(size_t)ki[q] * FG.nx + kj[q]] || (strict && !on)) continue;
        const size_t fidx = (size_t)ki[q] * FG.pitch + kj[q];
        if (fp32) {
#pragma unroll
            for (int k = 0; k < 5; k++)
                ((float*)fine_state)[k * FG.fstride + fidx] = ((const float*)coarse_state)[k * CG.fstride + cidx];
        } else {
#pragma unroll
            for (int k = 0; k < 5; k++)
                ((double*)fine_state)[k * FG.fstride + fidx] = ((const double*)coarse_state)[k * CG.fstride + cidx];
        }
    }
}

cudaError_t launch_amr_sync(const SweepArgs& a, int precision, void* coarse_state, void* fine_state, const Geom& FG,
                            const unsigned char* coarse, const unsigned char* fine, bool strict) {
    if (a.system == 2) return cudaErrorNotSupported;
    dim3 grid((a.G.nx + 127) / 128, a.G.ny);
    amr_sync_kernel<<<grid, 128, 0, a.stream>>>(make_loader(a, precision, fine_state, FG), a.G, coarse_state,
                                                fine_state, coarse, fine, strict ? 1 : 0);
    count_launch();
    return cudaGetLastError();
}

// Whether any of n flag bytes is set (the drivers' `refined` test, AMR/EulerAMR.cpp:241-249):
// ORs 1 into *out, which the caller zeroes first.
__global__ void amr_any_kernel(const unsigned char* __restrict__ f, size_t n, unsigned long long* out) {
    int hit = 0;
    for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
        hit |= f[k];
    if (__syncthreads_or(hit) && threadIdx.x == 0) atomicOr(out, 1ull);
}

cudaError_t launch_amr_any(const unsigned char* flags, size_t n, unsigned long long* out, cudaStream_t st) {
    size_t b = (n + 255) / 256;
    if (b > device_sm_count() * 4) b = device_sm_count() * 4;
    amr_any_kernel<<<(int)(b ? b : 1), 256, 0, st>>>(flags, n, out);
    count_launch();
    return cudaGetLastError();
}

// ------------------------------------------------------------------ state-level functions
// The reference's per-state functions (state vectors, equations of state, slope limiters, the
// black-hole eigenvalues) for n independent items, one thread per item, with the same arithmetic
// as the sweeps.  Item k reads in_stride doubles at in + k in_stride (and, for the black-hole
// system, its coordinates at xyz + 3k) and writes out_stride doubles at out + k out_stride.
template <class Sys>
CG_D void state_vector_op(const Sys& S, int op, const double* v, Pt q, double* o) {
    if (op == kStateCons) S.cons(v, q, o);
    else if (op == kStatePrim) S.prim(v, q, o);
    else S.flux(v, op == kStateFluxX ? 0 : 1, q, o);
}

// BlackHoleEuler/BlackHoleEulerEigenvalues.cpp:3-96: material, fast and slow acoustic eigenvalues
// along x, y, z (the terms whose largest value is GRExact::sound_speed).
CG_D void gr_eigenvalues(const GRExact& S, const double* p, Pt q, double* o) {
    double al, be[3];
    S.bh.lapse_shift(q.x, q.y, q.z, al, be);
    double gm[9], gs[9];
    S.bh.gamma(q.x, q.y, q.z, gm);
    inverse3(gm, gs);
    const double cs = sr_sound(p[0], p[4], S.g);
    const double v[3] = {p[1], p[2], p[3]};
    double v2 = 0.0;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) v2 = v2 + ((gm[3 * i + j] * v[i]) * v[j]);
    for (int i = 0; i < 3; i++) {
        const double rt = sqrt((1.0 - v2) * ((gs[3 * i + i] * (1.0 - (v2 * (cs * cs)))) - ((v[i] * v[i]) * (1.0 - (cs * cs)))));
        const double pre = al / (1.0 - (v2 * (cs * cs)));
        o[i] = (al * v[i]) - be[i];
        o[3 + i] = (pre * ((v[i] * (1.0 - (cs * cs))) + (cs * rt))) - be[i];
        o[6 + i] = (pre * ((v[i] * (1.0 - (cs * cs))) - (cs * rt))) - be[i];
    }
}

__global__ void state_eval_kernel(StateEvalArgs a, NewtonExact<double> nw, SRExact sr, GRExact gr) {
    for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < a.n; k += (size_t)gridDim.x * blockDim.x) {
        const double* v = a.in + a.in_stride * k;
        double* o = a.out + a.out_stride * k;
        const Pt q = a.xyz ? Pt{a.xyz[3 * k], a.xyz[3 * k + 1], a.xyz[3 * k + 2]} : Pt{0.0, 0.0, 0.0};
        const double g = a.gamma;
        switch (a.op) {
            case kStateCons:
            case kStatePrim:
            case kStateFluxX:
            case kStateFluxY:
                if (a.system == 0) state_vector_op(nw, a.op, v, q, o);
                else if (a.system == 1) state_vector_op(sr, a.op, v, q, o);
                else state_vector_op(gr, a.op, v, q, o);
                break;
            case kStateSound:  // Euler/EulerEquationOfState.cpp:17-22; SR :10-18; black hole :519-549
                if (a.system == 0) o[0] = sqrt((g * v[4]) / v[0]);
                else if (a.system == 1) o[0] = sr_sound(v[0], v[4], g);
                else o[0] = gr.sound_speed(v, q);
                break;
            case kStateInternalEnergy:  // Euler/EulerEquationOfState.cpp:3-8
                o[0] = v[4] / ((g - 1.0) * v[0]);
                break;
            case kStateTotalEnergy: {  // Euler/EulerStateVector.cpp:129-134 (the conserved energy)
                double u[5];
                nw.cons(v, q, u);
                o[0] = u[4];
                break;
            }
            case kStatePressure:  // Euler/EulerEquationOfState.cpp:10-15 from (rho, ., ., ., e)
                o[0] = (v[4] * (g - 1.0)) * v[0];
                break;
            case kStateEnthalpy:  // RelativisticEuler/RelativisticEulerEquationOfState.cpp:3-8
                o[0] = sr_enthalpy(v[0], v[4], g);
                break;
            case kStateSource:  // BlackHoleEuler/BlackHoleEulerStateVector.cpp:359-510
                gr.source(v, q, o);
                break;
            case kStateEigenvalues:
                gr_eigenvalues(gr, v, q, o);
                break;
            case kStateGradientRatio:  // Solvers/SlopeLimiters.cpp:3-6
                o[0] = gradient_ratio(v[0], a.bias);
                break;
            case kStateLimiter:  // Solvers/SlopeLimiters.cpp:8-69
                o[0] = limiter_exact(v[0], a.bias, a.lim);
                break;
            case kStateSlope:  // Solvers/SlopeLimiters.cpp:71-101 on three conserved vectors
                slope_exact(v, v + 5, v + 10, a.bias, a.lim, o);
                break;
            default:
                break;
        }
    }
}

cudaError_t launch_state_eval(const SweepArgs& s, const StateEvalArgs& a) {
    size_t b = (a.n + 127) / 128;
    if (b > device_sm_count() * 8) b = device_sm_count() * 8;
    state_eval_kernel<<<(int)(b ? b : 1), 128, 0, s.stream>>>(a, NewtonExact<double>{s.gamma, nullptr},
                                                                SRExact{s.gamma, nullptr}, make_gr(s));
    count_launch();
    return cudaGetLastError();
}

// ------------------------------------------------------------------ per-interface functions
// The reference's static building blocks, one item per thread, in the reference's operation order
// (this unit is compiled without FMA contraction):
//   0 computeLaxFriedrichsFlux, 1 computeRichtmyerFlux (the intermediate state), 2 computeFORCEFlux,
//   3 computeFORCEUpdate (Solvers/EulerFirstOrderSolver.cpp:3-24, :96-101), 4 computeFractional-
//   EvolutionVector, 5 computeEvolutionVector (Solvers/EulerSolvers.cpp:163-172);
//   6..11 computeX/Y{LaxFriedrichs,Richtmyer,FORCE}Flux of primitive states
//   (Solvers/EulerFirstOrderSolver.cpp:26-94 and the SR and black-hole twins; black hole: states
//   at x -/+ dx/2, the intermediate state's flux at x);
//   12/13 computeX/YSLICFlux (Solvers/EulerSecondOrderSolver.cpp:3-25; black hole
//   Solvers/BlackHoleEulerSecondOrderSolver.cpp:3-39: evolutions at x -/+ dx/2);
//   14/15 evolveStateByHalfX/YTimeStep of states, 16/17 evolveStateByHalfTimeStep of vectors
//   (Solvers/EulerSolvers.cpp:174-223; black hole Solvers/BlackHoleEulerSolvers.cpp:234-307);
//   black hole only: 18/19 evolveStateByFractionalX/YTimeStep, 20 evolveStateByFractionalTimeStep
//   (Solvers/BlackHoleEulerSolvers.cpp:159-232), 21/22 the forcing solver's
//   evolveConservedVariableVector / ...2D (Solvers/BlackHoleEulerForcingSolver.cpp:3-185).
template <class Sys>
CG_D void iface_item(const Sys& S, bool gr, const IfaceArgs& A, const double* a, Pt q, double* o) {
    const double* b = a + 5;
    const double* c = a + 10;
    const double* d = a + 15;
    const int op = A.op;
    const int axis = (op & 1) ? 1 : 0;
    const double dx = A.dx, dt = A.dt;
    switch (op) {
        case 0: { const double r = dx / dt; for (int k = 0; k < 5; k++) o[k] = 0.5 * ((c[k] + d[k]) + (r * (a[k] - b[k]))); break; }
        case 1: { const double r = dt / dx; for (int k = 0; k < 5; k++) o[k] = 0.5 * ((a[k] + b[k]) + (r * (c[k] - d[k]))); break; }
        case 2: for (int k = 0; k < 5; k++) o[k] = 0.5 * (a[k] + b[k]); break;
        case 3: { const double r = dt / dx; for (int k = 0; k < 5; k++) o[k] = a[k] + (r * (b[k] - c[k])); break; }
        case 4: case 5: {
            const double r = (op == 4 ? A.frac : 0.5) * (dt / dx);
            for (int k = 0; k < 5; k++) o[k] = r * (a[k] - b[k]);
            break;
        }
        case 6: case 7: case 8: case 9: {
            double uL[5], uR[5], fL[5], fR[5];
            const Pt pl = shift_pt(q, axis, -(dx * 0.5)), pr = shift_pt(q, axis, dx * 0.5);
            S.cons(a, pl, uL);
            S.cons(b, pr, uR);
            S.flux(uL, axis, pl, fL);
            S.flux(uR, axis, pr, fR);
            if (op <= 7) {
                const double r = dx / dt;
                for (int k = 0; k < 5; k++) o[k] = 0.5 * ((fL[k] + fR[k]) + (r * (uL[k] - uR[k])));
                break;
            }
            const double r = dt / dx;
            double us[5];
            for (int k = 0; k < 5; k++) us[k] = 0.5 * ((uL[k] + uR[k]) + (r * (fL[k] - fR[k])));
            S.flux(us, axis, q, o);
            break;
        }
        case 10: case 11: force_exact(S, a, b, q, axis, dx, dt, o); break;
        case 12: case 13: {
            double eR[5], eL[5];
            evolve_half_exact(S, a, b, c, shift_pt(q, axis, -(dx * 0.5)), axis, dx, dt, A.bias, A.lim, (double*)nullptr, eR);
            evolve_half_exact(S, b, c, d, shift_pt(q, axis, dx * 0.5), axis, dx, dt, A.bias, A.lim, eL, (double*)nullptr);
            force_exact(S, eR, eL, q, axis, dx, dt, o);
            break;
        }
        case 14: case 15:
            evolve_half_exact(S, a, b, c, q, axis, dx, dt, A.bias, A.lim, A.side == 0 ? o : nullptr,
                              A.side == 0 ? nullptr : o);
            break;
        case 16: case 17: {
            double u[5];
            const double* x = A.side == 0 ? a : b;
            for (int k = 0; k < 5; k++) u[k] = x[k] + c[k];
            S.prim(u, gr ? shift_pt(q, axis, A.side == 0 ? -(dx * 0.5) : dx * 0.5) : q, o);
            break;
        }
        default: break;
    }
}

__global__ void iface_kernel(IfaceArgs A, NewtonExact<double> nw, SRExact sr, GRExact gr) {
    const int w = A.width;
    for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < A.n; k += (size_t)gridDim.x * blockDim.x) {
        const double* a = A.in + (size_t)w * k;
        double* o = A.out + 5 * k;
        const Pt q = A.xyz ? Pt{A.xyz[3 * k], A.xyz[3 * k + 1], A.xyz[3 * k + 2]} : Pt{0.0, 0.0, 0.0};
        if (A.system == 0) iface_item(nw, false, A, a, q, o);
        else if (A.system == 1) iface_item(sr, false, A, a, q, o);
        else if (A.op <= 17) iface_item(gr, true, A, a, q, o);
        else if (A.op <= 19) evolve_fraction_exact(gr, A.frac, a, a + 5, a + 10, q, A.op - 18, A.dx, A.dt, A.bias, A.lim, o);
        else if (A.op == 20) {
            double u[5];
            for (int f = 0; f < 5; f++) u[f] = a[f] + a[5 + f];
            gr.prim(u, q, o);
        } else if (A.op == 21) {
            rk_cell_exact(gr, 1, a, a + 5, a + 10, a, a, q, A.dx, A.dt, A.bias, A.lim, o);
        } else {
            rk_cell_exact(gr, 2, a, a + 5, a + 10, a + 15, a + 20, q, A.dx, A.dt, A.bias, A.lim, o);
        }
    }
}

cudaError_t launch_interface_eval(const SweepArgs& s, const IfaceArgs& a) {
    size_t b = (a.n + 127) / 128;
    if (b > (size_t)device_sm_count() * 8) b = (size_t)device_sm_count() * 8;
    SweepArgs g = s;
    g.dx = a.dx;  // the black-hole metric derivatives take the cell spacing (the reference's h)
    iface_kernel<<<(int)(b ? b : 1), 128, 0, s.stream>>>(a, NewtonExact<double>{s.gamma, nullptr}, SRExact{s.gamma, nullptr},
                                                         make_gr(g));
    count_launch();
    return cudaGetLastError();
}

// ------------------------------------------------------------------ spacetime record
// Every public quantity of the reference's BlackHoleSpacetime (BlackHoleEuler/BlackHoleSpacetime.cpp:
// 54-386) at one point, metric derivatives by the reference's centred differences with spacing
// S.h, in the layout of the public COSMOS_ST_* offsets.
__global__ void spacetime_kernel(GRExact S, size_t n, const double* __restrict__ xyz, double* __restrict__ out) {
    for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
        const Pt q{xyz[3 * k], xyz[3 * k + 1], xyz[3 * k + 2]};
        double* o = out + (size_t)kSpacetimeWidth * k;
        const BHExact& b = S.bh;
        o[0] = b.H(q.x, q.y, q.z);                            // computeKerrSchildScalar
        b.l(q.x, q.y, q.z, o + 1);                            // computeKerrSchildVector
        b.L4(q.x, q.y, q.z, o + 4);                           // computeKerrSchildSpacetimeVector
        const double h = S.h, hs = 0.5 * h;
        for (int d = 0; d < 3; d++) {                         // the scalar and vector derivatives
            const Pt p1 = S.off(q, d, hs), p0 = S.off(q, d, -hs);
            double h1, h0, a1[3], a0[3];
            b.Hl(p1.x, p1.y, p1.z, h1, a1);
            b.Hl(p0.x, p0.y, p0.z, h0, a0);
            o[8 + d] = (h1 - h0) / h;
            for (int c = 0; c < 3; c++) o[11 + 3 * d + c] = (1.0 / h) * (a1[c] - a0[c]);
        }
        double m[9], g4m[16];
        b.gamma(q.x, q.y, q.z, m);
        b.g4(q.x, q.y, q.z, g4m);
        for (int i = 0; i < 9; i++) o[20 + i] = m[i];
        for (int i = 0; i < 16; i++) o[29 + i] = g4m[i];
        inverse3(m, o + 45);
        inverse4(g4m, o + 54);
        o[70] = det3(m);
        o[71] = det4(g4m);
        double al, gi[16];
        b.lapse_shift(q.x, q.y, q.z, al, o + 100);
        o[99] = al;
        // lapse, shift and spatial-metric derivatives and K_ij as the source term takes them
        S.source_metric(q, al, gi, o + 103, o + 106, o + 72, o + 115);
        o[124] = b.excised(q.x, q.y, q.z) ? 1.0 : 0.0;
    }
}

cudaError_t launch_spacetime_eval(const SweepArgs& s, size_t n, const double* xyz, double* out) {
    size_t blocks = (n + 127) / 128;
    if (blocks > (size_t)device_sm_count() * 8) blocks = (size_t)device_sm_count() * 8;
    spacetime_kernel<<<(int)(blocks ? blocks : 1), 128, 0, s.stream>>>(make_gr(s), n, xyz, out);
    count_launch();
    return cudaGetLastError();
}

// ------------------------------------------------------------------ conservation sums
// Sum of each stored field over the grid with Kahan-Babuska (Neumaier) compensation per thread,
// then compensated double atomics are avoided: per-block partials go to a small buffer summed by
// the last block in a fixed order, so the result is deterministic.
__global__ void field_sums_kernel(const void* __restrict__ state, Geom G, int precision, double* partial,
                                  unsigned int* counter, double* out5) {
    double s[5] = {0, 0, 0, 0, 0}, comp[5] = {0, 0, 0, 0, 0};
    const size_t n = (size_t)G.nx * G.ny;
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
        const size_t i = c / G.nx, j = c % G.nx, k = i * G.pitch + j;
#pragma unroll
        for (int f = 0; f < 5; f++) {
            const double v = precision == 1 ? (double)((const float*)state)[f * G.fstride + k]
                                            : ((const double*)state)[f * G.fstride + k];
            const double t = s[f] + v;
            comp[f] += (fabs(s[f]) >= fabs(v)) ? ((s[f] - t) + v) : ((v - t) + s[f]);
            s[f] = t;
        }
    }
    __shared__ double red[5][256];
#pragma unroll
    for (int f = 0; f < 5; f++) red[f][threadIdx.x] = s[f] + comp[f];
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int f = 0; f < 5; f++) {
            double a = 0.0, ca = 0.0;
            for (int q = 0; q < blockDim.x; q++) {
                const double v = red[f][q], t = a + v;
                ca += (fabs(a) >= fabs(v)) ? ((a - t) + v) : ((v - t) + a);
                a = t;
            }
            partial[blockIdx.x * 5 + f] = a + ca;
        }
        __threadfence();
        const unsigned int done = atomicAdd(counter, 1u);
        if (done == gridDim.x - 1) {
            __threadfence();
            for (int f = 0; f < 5; f++) {
                double a = 0.0, ca = 0.0;
                for (unsigned q = 0; q < gridDim.x; q++) {
                    const double v = ((volatile double*)partial)[q * 5 + f], t = a + v;
                    ca += (fabs(a) >= fabs(v)) ? ((a - t) + v) : ((v - t) + a);
                    a = t;
                }
                out5[f] = a + ca;
            }
            *counter = 0;
        }
    }
}

cudaError_t launch_field_sums(const void* soa, const Geom& G, int precision, double* out5, cudaStream_t st) {
    // scratch: 152*4 blocks * 5 partials + a counter, carved from out5's companion buffer
    constexpr int kBlocks = 152 * 4;
    double* partial = out5 + 8;
    unsigned int* counter = (unsigned int*)(out5 + 8 + kBlocks * 5);
    field_sums_kernel<<<kBlocks, 256, 0, st>>>(soa, G, precision, partial, counter, out5);
    count_launch();
    return cudaGetLastError();
}

}  // namespace cg
