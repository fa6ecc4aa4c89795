// FP32 bulk kernels of the black-hole system (physics_gr_fast.cuh): FP64 metric tables built once
// per grid, FP32 sweeps on the one-cell tile functions, the RK4 source step, the CFL reduction and
// the primitive conversions.
#include <algorithm>

#include "launch.h"
#include "physics_gr_fast.cuh"
#include "policies.cuh"

namespace cg {

namespace {

GRExact make_gr_exact(const SweepArgs& a) {
    GRExact s;
    s.g = a.gamma;
    s.bh = BHExact{a.bh[0], a.bh[1], a.bh[2], a.bh[3], a.bh[4]};
    s.h = a.dx;
    s.capped = nullptr;
    return s;
}

// ---------------------------------------------------------------- metric tables (FP64 -> FP32)
// Point (i, j) of a table at x = (j + xo) dx, y = (i + yo) dx (y = 0 on 1D grids), with xo, yo
// 0 for centres and -0.5 along the face axis.
__global__ void gr_met_table_kernel(GRExact sys, int dims, double dx, int ni, int nj, int i0, int j0, double yo,
                                    double xo, float* out, size_t stride) {
    const size_t n = (size_t)ni * nj;
    for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(k / nj) + i0, j = (int)(k % nj) + j0;
        const double x = (j + xo) * dx, y = dims == 1 ? 0.0 : (i + yo) * dx;
        double m[9], al, be[3];
        sys.bh.gamma(x, y, 0.0, m);
        sys.bh.lapse_shift(x, y, 0.0, al, be);
        const double sg = sqrt(det3(m));
        const int sym[6] = {0, 1, 2, 4, 5, 8};
#pragma unroll
        for (int q = 0; q < 6; q++) out[q * stride + k] = (float)m[sym[q]];
        out[6 * stride + k] = (float)sg;
        out[7 * stride + k] = (float)al;
#pragma unroll
        for (int q = 0; q < 3; q++) out[(8 + q) * stride + k] = (float)be[q];
    }
}

// Source data at cell centres and the CFL point data and masks per cell.
__global__ void gr_cell_table_kernel(GRExact sys, int dims, int order, double dx, int nx, int ny, float* src,
                                     float* ws, unsigned char* flags) {
    const size_t n = (size_t)nx * ny;
    const BHExact& b = sys.bh;
    for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(k / nx), j = (int)(k % nx);
        const double y = dims == 1 ? 0.0 : i * dx;
        const Pt q{j * dx, y, 0.0};
        double al, be[3];
        b.lapse_shift(q.x, q.y, q.z, al, be);
        double gi[16], da[3], db[9], dgm[27], K[9];
        sys.source_metric(q, al, gi, da, db, dgm, K);
        const int s4[10] = {0, 1, 2, 3, 5, 6, 7, 10, 11, 15};
        const int s3[6] = {0, 1, 2, 4, 5, 8};
        int o = 0;
        for (int t = 0; t < 10; t++) src[(o++) * n + k] = (float)gi[s4[t]];
        for (int t = 0; t < 3; t++) src[(o++) * n + k] = (float)da[t];
        for (int t = 0; t < 9; t++) src[(o++) * n + k] = (float)db[t];
        for (int d = 0; d < 3; d++)
            for (int t = 0; t < 6; t++) src[(o++) * n + k] = (float)dgm[9 * d + s3[t]];
        for (int t = 0; t < 6; t++) src[(o++) * n + k] = (float)K[s3[t]];
        // excision masks (Solvers/BlackHoleEulerSecondOrderSolver.cpp:44-46, :81-85; the source
        // step's five-point test, Solvers/BlackHoleEulerSecondOrderSolver.cpp:195-209)
        auto stencil_clear = [&](int reach) {
            if (dims == 1) {
                for (int d = -reach; d <= reach; d++)
                    if (b.excised((j + d) * dx, 0.0, 0.0)) return false;
                return true;
            }
            if (b.excised(j * dx, i * dx, 0.0)) return false;
            for (int d = 1; d <= reach; d++)
                if (b.excised((j - d) * dx, i * dx, 0.0) || b.excised((j + d) * dx, i * dx, 0.0) ||
                    b.excised(j * dx, (i - d) * dx, 0.0) || b.excised(j * dx, (i + d) * dx, 0.0))
                    return false;
            return true;
        };
        unsigned char f = 0;
        if (stencil_clear(2)) f |= 1;
        if (stencil_clear(1)) f |= 2 | 4;
        // CFL point (Solvers/BlackHoleEulerSolvers.cpp:87-131): spacing 1/N; in 2D the excision test
        // reads (j/nx, i/ny) and the speed is evaluated at (i/ny, j/nx)
        double px, py;
        if (dims == 1) {
            const double cs = 1.0 / nx;
            if (b.excised(j * cs, 0.0, 0.0)) f |= 8;
            px = j * cs;
            py = 0.0;
        } else {
            const double rs = 1.0 / ny, cs = 1.0 / nx;
            if (b.excised(j * cs, i * rs, 0.0)) f |= 8;
            px = i * rs;
            py = j * cs;
        }
        flags[k] = f;
        double wal, wbe[3], gm[9], gs[9];
        b.lapse_shift(px, py, 0.0, wal, wbe);
        b.gamma(px, py, 0.0, gm);
        inverse3(gm, gs);
        o = 0;
        ws[(o++) * n + k] = (float)wal;
        for (int t = 0; t < 3; t++) ws[(o++) * n + k] = (float)wbe[t];
        for (int t = 0; t < 6; t++) ws[(o++) * n + k] = (float)gm[s3[t]];
        for (int t = 0; t < 3; t++) ws[(o++) * n + k] = (float)gs[4 * t];
    }
}

int blocks_for(size_t n) { return (int)std::min<size_t>((n + 255) / 256, device_sm_count() * 16); }

// ---------------------------------------------------------------- sweep policy
// Plugs into the one-cell tile functions (sweep_x_own_kernel, sweep_y_kernel) on primitive cells:
// one evolution per cell for both faces, metric from the tables by (line, position).
template <int AXIS, int LIM, bool MASKED>
struct GRFastPolicy {
    using S = float;
    using X = float;
    using W = float;
    using Cell = V5<float>;
    using Face = V5<float>;
    using Coef = FastCoef;
    static constexpr bool kShared = true;
    static constexpr bool kMasked = true;  // excision: cells with an excised stencil keep their state
    static constexpr bool kHasDx = false;
    NewtonFastParams NP;
    SRFastParams P;
    GRTables T;
    LineMap lm;
    int dims, order;
    float dtdx, half_dtdx, q_dxdt;
    int flags;

    CG_D Coef make_coef(const DtSrc& ds, double) const { return ds.fast_coef(); }
    CG_D void use_coef(const Coef& c) {
        dtdx = c.dtdx;
        half_dtdx = c.half_dtdx;
        q_dxdt = c.q_dxdt;
    }
    CG_D GRMet center(int line, int k) const {
        int i, j;
        lm.ij(line, k, i, j);
        GRMet m;
        load_met(GRTab{T.center, T.center_stride}, (size_t)(i + 2) * (T.nx + 4) + (j + 2), m);
        return m;
    }
    // face f of the line: between positions f - 1 and f along the sweep axis
    CG_D GRMet face(int line, int f) const {
        GRMet m;
        if (AXIS == 0) load_met(GRTab{T.xface, T.xface_stride}, (size_t)(line + 2) * (T.nx + 5) + (f + 2), m);
        else load_met(GRTab{T.yface, T.yface_stride}, (size_t)(f + 2) * (T.nx + 4) + (line + 2), m);
        return m;
    }
    CG_D void recon(const Cell& l, const Cell& m, const Cell& r, int line, int k, Face& L, Face& R) {
        gr_evolve_fast<AXIS, LIM>(P, NP, l.v, m.v, r.v, center(line, k - 1), center(line, k), center(line, k + 1),
                                  face(line, k), face(line, k + 1), half_dtdx, L.v, R.v, &flags);
    }
    CG_D void recon_side(const Cell&, const Cell&, const Cell&, int, int, int, Face&) const {}
    CG_D void face_of(const Cell& c, Face& f) const { f = c; }
    CG_D void flux(const Face& L, const Face& R, int line, int f, V5<float>& F) {
        gr_force_fast<AXIS>(P, L.v, R.v, center(line, f - 1), face(line, f), center(line, f), half_dtdx, q_dxdt, F.v,
                            &flags);
    }
    CG_D Cell update(const Cell& c, const V5<float>& FL, const V5<float>& FR, int line, int k) {
        Cell o;
        gr_update_fast(P, c.v, FL.v, FR.v, center(line, k), dtdx, o.v, &flags);
        return o;
    }
    CG_D bool active(int line, int k, const unsigned char* mask) const {
        if (MASKED && !lm.mask_on(mask, line, k)) return false;
        int i, j;
        lm.ij(line, k, i, j);
        return (T.flags[(size_t)i * T.nx + j] & (order == 2 ? 1 : 2)) != 0;
    }
    CG_D float wavespeed(const Cell& c, int line, int k) {
        int i, j;
        lm.ij(line, k, i, j);
        const size_t q = (size_t)i * T.nx + j;
        if (T.flags[q] & 8) return 0.0f;
        float w[kWsFields];
#pragma unroll
        for (int t = 0; t < kWsFields; t++) w[t] = T.ws[t * T.cell_stride + q];
        return speed_or_inf(c.v[0], c.v[4], gr_speed_fast(P, c.v, w));
    }
    CG_D void flush_status(int* st) const {
        if (st && flags) atomicOr(st, ST_NEWTON_CAP);
    }
};

template <int AXIS, int LIM, bool MASKED>
GRFastPolicy<AXIS, LIM, MASKED> make_pol(const SweepArgs& a, double bias) {
    GRFastPolicy<AXIS, LIM, MASKED> p;
    const SRFastPolicy<AXIS, LIM, MASKED> s = make_sr_fast<AXIS, LIM, MASKED>(a.gamma, bias, a.G.nx, a.G.dims,
                                                                               a.c2p64_above);
    p.NP = s.NP;
    p.P = s.P;
    p.T = *a.grt;
    p.lm.axis = AXIS;
    p.lm.nx = a.G.nx;
    p.dims = a.G.dims;
    p.order = a.order;
    p.dtdx = p.half_dtdx = p.q_dxdt = 0.0f;
    p.flags = 0;
    return p;
}

constexpr int kXThreads = 256;
// One warp of columns per Y block, 8 rows per segment: the cells near the hole (FP64 recovery
// stage) make some column segments several times costlier than the rest, and many small blocks
// spread them over the SMs (at 1024^2, 4096 blocks of 32 x 8 cells against 256 of 128 x 32; the
// 4-row halo of each segment costs less than the imbalance it removes: 2.49 vs 2.65 ms per step
// against 32 x 16).
constexpr int kYThreads = 32;
constexpr int kYSeg = 8;

template <int AXIS, int LIM, bool MASKED>
void run(const SweepArgs& a) {
    const Geom& G = a.G;
    const float* src = (const float*)a.src;
    float* dst = (float*)a.dst;
    auto pol = make_pol<AXIS, LIM, MASKED>(a, a.bias);
    using Pol = decltype(pol);
    if constexpr (AXIS == 0) {
        dim3 grid((G.nx + kXThreads - 3) / (kXThreads - 2), G.ny);
        if (a.order == 2) sweep_x_own_kernel<Pol, 2, kXThreads><<<grid, kXThreads, 0, a.stream>>>(pol, G, src, dst, a.ds, a.out);
        else sweep_x_own_kernel<Pol, 1, kXThreads><<<grid, kXThreads, 0, a.stream>>>(pol, G, src, dst, a.ds, a.out);
    } else {
        dim3 grid((G.nx + kYThreads - 1) / kYThreads, (G.ny + kYSeg - 1) / kYSeg);
        if (a.order == 2) sweep_y_kernel<Pol, 2, kYThreads, kYSeg><<<grid, kYThreads, 0, a.stream>>>(pol, G, src, dst, a.ds, a.out);
        else sweep_y_kernel<Pol, 1, kYThreads, kYSeg><<<grid, kYThreads, 0, a.stream>>>(pol, G, src, dst, a.ds, a.out);
    }
}

template <int AXIS, bool MASKED>
void run_lim(const SweepArgs& a) {
    if (a.lim == 0) run<AXIS, 0, MASKED>(a);
    else if (a.lim == 1) run<AXIS, 1, MASKED>(a);
    else run<AXIS, 2, MASKED>(a);
}

// ---------------------------------------------------------------- source step
// One cell per thread; cells whose five-point stencil touches the excised region keep their state.
// Capped at three blocks of 128 threads per SM (168 registers, a small L1-resident spill): on the
// evolved 1024^2 accretion grid that beat 205 registers at two blocks (2.65 vs 2.81 ms per step).
template <int LIM>
__global__ void __launch_bounds__(128, 3) gr_rk_kernel(SRFastParams P, NewtonFastParams NP, GRTables T, Geom G, double dx,
                                                    const float* __restrict__ src, float* __restrict__ dst, DtSrc ds,
                                                    int* status) {
    // the step's dt (0.5 dt / subcycles from the controller) and dt/dx, once per block
    __shared__ float s_dt, s_dtdx;
    __shared__ int s_on;
    if (threadIdx.x == 0) {
        double d;
        s_on = ds.get(d);
        s_dt = (float)d;
        s_dtdx = (float)(d / dx);
    }
    __syncthreads();
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;
    if (j >= G.nx) return;
    const size_t idx = (size_t)i * G.pitch + j;
    const bool on = s_on && (T.flags[(size_t)i * G.nx + j] & 4);
    if (!on) {
#pragma unroll
        for (int f = 0; f < 5; f++) dst[f * G.fstride + idx] = src[f * G.fstride + idx];
        return;
    }
    const float dtdx = s_dtdx;
    auto ld = [&](int ii, int jj, float* p) {
        const size_t k = (size_t)ghost_index(ii, G.ny, 0) * G.pitch + ghost_index(jj, G.nx, 0);
#pragma unroll
        for (int f = 0; f < 5; f++) p[f] = src[f * G.fstride + k];
    };
    auto met = [&](int ii, int jj) {
        GRMet m;
        load_met(GRTab{T.center, T.center_stride}, (size_t)(ii + 2) * (T.nx + 4) + (jj + 2), m);
        return m;
    };
    // primitives of the cell and its neighbours, made conserved at their own centres
    // (the reference's kernel, Solvers/BlackHoleEulerForcingSolver.cpp:72-99)
    const int ii = G.dims == 1 ? 0 : i;
    const GRMet Ml = met(ii, j - 1), Mc = met(ii, j), Mr = met(ii, j + 1);
    GRMet Mt = Mc, Mb = Mc;
    float p[5], cl[5], cm[5], cr[5], ct[5], cb[5], out[5];
    ld(i, j - 1, p);
    gr_cons_fast(P, p, Ml, cl);
    ld(i, j, p);
    gr_cons_fast(P, p, Mc, cm);
    ld(i, j + 1, p);
    gr_cons_fast(P, p, Mr, cr);
    if (G.dims == 2) {
        Mt = met(i - 1, j);
        Mb = met(i + 1, j);
        ld(i - 1, j, p);
        gr_cons_fast(P, p, Mt, ct);
        ld(i + 1, j, p);
        gr_cons_fast(P, p, Mb, cb);
    }
    GRSrc X;
    load_src(GRTab{T.src, T.cell_stride}, (size_t)i * G.nx + j, X);
    int flags = 0;
    gr_rk_fast<LIM>(P, NP, G.dims, cl, cm, cr, ct, cb, Ml, Mc, Mr, Mt, Mb, X, s_dt, dtdx, out, &flags);
#pragma unroll
    for (int f = 0; f < 5; f++) dst[f * G.fstride + idx] = out[f];
    if (flags && status) atomicOr(status, ST_NEWTON_CAP);
}

// ---------------------------------------------------------------- conversions
// The FP32 black-hole path stores primitives, like the reference's grids: upload and download
// round them to and from FP32.
__global__ void gr_prim_in_kernel(const double* __restrict__ aos, float* __restrict__ soa, Geom G) {
    const size_t n = (size_t)G.nx * G.ny;
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
        const size_t i = c / G.nx, j = c % G.nx;
#pragma unroll
        for (int f = 0; f < 5; f++) soa[f * G.fstride + i * G.pitch + j] = (float)aos[5 * c + f];
    }
}
__global__ void gr_prim_out_kernel(const float* __restrict__ soa, double* __restrict__ aos, Geom G) {
    const size_t n = (size_t)G.nx * G.ny;
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
        const size_t i = c / G.nx, j = c % G.nx;
#pragma unroll
        for (int f = 0; f < 5; f++) aos[5 * c + f] = (double)soa[f * G.fstride + i * G.pitch + j];
    }
}

size_t rup(size_t v) { return (v + 63) / 64 * 64; }

}  // namespace

size_t gr_tables_bytes(int nx, int ny) {
    const size_t c = rup((size_t)(nx + 4) * (ny + 4)), xf = rup((size_t)(nx + 5) * (ny + 4)),
                 yf = rup((size_t)(nx + 4) * (ny + 5)), cell = rup((size_t)nx * ny);
    return sizeof(float) * (kMetFields * (c + xf + yf) + (kSrcFields + kWsFields) * cell) + cell;
}

cudaError_t build_gr_tables(const SweepArgs& a, void* storage, GRTables* out) {
    const int nx = a.G.nx, ny = a.G.ny;
    GRTables t;
    t.nx = nx;
    t.ny = ny;
    t.center_stride = rup((size_t)(nx + 4) * (ny + 4));
    t.xface_stride = rup((size_t)(nx + 5) * (ny + 4));
    t.yface_stride = rup((size_t)(nx + 4) * (ny + 5));
    t.cell_stride = rup((size_t)nx * ny);
    float* p = (float*)storage;
    float* center = p;
    float* xface = center + kMetFields * t.center_stride;
    float* yface = xface + kMetFields * t.xface_stride;
    float* src = yface + kMetFields * t.yface_stride;
    float* ws = src + kSrcFields * t.cell_stride;
    unsigned char* flags = (unsigned char*)(ws + kWsFields * t.cell_stride);
    t.center = center;
    t.xface = xface;
    t.yface = yface;
    t.src = src;
    t.ws = ws;
    t.flags = flags;
    const GRExact sys = make_gr_exact(a);
    const int d = a.G.dims;
    const double dx = a.dx;
    gr_met_table_kernel<<<blocks_for(t.center_stride), 256, 0, a.stream>>>(sys, d, dx, ny + 4, nx + 4, -2, -2, 0.0,
                                                                             0.0, center, t.center_stride);
    gr_met_table_kernel<<<blocks_for(t.xface_stride), 256, 0, a.stream>>>(sys, d, dx, ny + 4, nx + 5, -2, -2, 0.0,
                                                                            -0.5, xface, t.xface_stride);
    gr_met_table_kernel<<<blocks_for(t.yface_stride), 256, 0, a.stream>>>(sys, d, dx, ny + 5, nx + 4, -2, -2, -0.5,
                                                                            0.0, yface, t.yface_stride);
    // the cell tables use a compact stride of nx * ny inside their rounded-up slots
    GRTables u = t;
    u.cell_stride = (size_t)nx * ny;
    gr_cell_table_kernel<<<blocks_for(u.cell_stride), 128, 0, a.stream>>>(sys, d, 2, dx, nx, ny, src, ws, flags);
    count_launch(4);
    *out = u;
    return cudaGetLastError();
}

cudaError_t launch_sweep_gr_fast(const SweepArgs& a) {
    const bool masked = a.out.mask != nullptr;
    if (a.G.axis == 0) masked ? run_lim<0, true>(a) : run_lim<0, false>(a);
    else masked ? run_lim<1, true>(a) : run_lim<1, false>(a);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_rk_source_gr_fast(const SweepArgs& a) {
    const SRFastPolicy<0, 1, false> s = make_sr_fast<0, 1, false>(a.gamma, a.bias, a.G.nx, a.G.dims, a.c2p64_above);
    dim3 grid((a.G.nx + 127) / 128, a.G.ny);
    auto k = a.lim == 0 ? gr_rk_kernel<0> : (a.lim == 1 ? gr_rk_kernel<1> : gr_rk_kernel<2>);
    k<<<grid, 128, 0, a.stream>>>(s.P, s.NP, *a.grt, a.G, a.dx, (const float*)a.src, (float*)a.dst, a.ds, a.out.status);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_wavespeed_gr_fast(const SweepArgs& a, unsigned long long* slot) {
    constexpr int NT = 256;
    SweepArgs b = a;
    b.G.axis = 0;
    SweepOut o = a.out;
    if (slot) { o.smax = slot; o.ws_ctl = nullptr; }
    auto pol = make_pol<0, 2, false>(b, 0.0);
    wavespeed_kernel<decltype(pol), NT><<<blocks_for((size_t)a.G.nx * a.G.ny), NT, 0, a.stream>>>(
        pol, b.G, (const float*)a.src, o);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_prim_in_gr_fast(const SweepArgs& a, const double* aos, void* soa) {
    gr_prim_in_kernel<<<blocks_for((size_t)a.G.nx * a.G.ny), 256, 0, a.stream>>>(aos, (float*)soa, a.G);
    count_launch();
    return cudaGetLastError();
}
cudaError_t launch_prim_out_gr_fast(const SweepArgs& a, const void* soa, double* aos) {
    gr_prim_out_kernel<<<blocks_for((size_t)a.G.nx * a.G.ny), 256, 0, a.stream>>>((const float*)soa, aos, a.G);
    count_launch();
    return cudaGetLastError();
}

}  // namespace cg
