// C-ABI implementation: contexts, grids, solver runs (device-side dt, CUDA-graph replay).
#include <algorithm>
#include <atomic>
#include <climits>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>

#include "../../include/cosmos_gb300.h"
#include "capi_internal.h"
#include "launch.h"

namespace cg {
static std::atomic<unsigned long long> g_launches{0};
static thread_local bool t_capturing = false;  // launches recorded into a graph are not launches
void count_launch(unsigned n) {
    if (!t_capturing) g_launches.fetch_add(n, std::memory_order_relaxed);
}
int device_sm_count() {
    static std::atomic<int> counts[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
    int c = counts[dev].load(std::memory_order_relaxed);
    if (c <= 0) {
        if (cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || c <= 0) c = 152;
        counts[dev].store(c, std::memory_order_relaxed);
    }
    return c;
}
}  // namespace cg

using namespace cg;

namespace {

thread_local std::string t_err;

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    t_err = buf;
    return code;
}

#define CK(call)                                                                                    \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess) return fail(COSMOS_ECUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                                           __FILE__, __LINE__);                                     \
    } while (0)

}  // namespace

namespace cg {
// lets other translation units report an error through cosmos_last_error()
void set_error(const char* msg) { t_err = msg ? msg : ""; }
// lets other translation units keep launches recorded into a graph out of the launch count
void set_capturing(bool on) { t_capturing = on; }
}  // namespace cg

namespace cg {
void ctx_retain(cosmos_ctx* c) { c->refs.fetch_add(1); }
void ctx_release(cosmos_ctx* c) {
    if (c->refs.fetch_sub(1) != 1) return;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    cudaStreamSynchronize(c->copy);
    for (int k = 0; k < 2; k++) cudaEventDestroy(c->ev[k]);
    cudaStreamDestroy(c->copy);
    cudaStreamDestroy(c->stream);
    delete c;
}
}  // namespace cg

namespace cg {
SweepArgs base_args(cosmos_grid* g) {
    SweepArgs a;
    memset(&a, 0, sizeof a);
    a.system = g->p.system;
    a.G = g->G;
    a.order = 2;
    a.dx = g->p.dx;
    a.gamma = g->p.gamma;
    a.bh[0] = g->p.bh_mass; a.bh[1] = g->p.bh_spin; a.bh[2] = g->p.bh_x; a.bh[3] = g->p.bh_y; a.bh[4] = g->p.bh_z;
    a.c2p64_above = g->p.sr_c2p64_above;
    a.grt = &g->grt;
    a.stream = g->ctx->stream;
    return a;
}

cudaError_t sweep_launch(cosmos_grid* g, const SweepArgs& a) {
    return g->p.precision == COSMOS_FP64 ? launch_sweep_exact(a) : launch_sweep_fast(a);
}

}  // namespace cg

namespace {

size_t round_up(size_t v, size_t a) { return (v + a - 1) / a * a; }
constexpr int kChunkSteps = 8;  // steps per replayed chunk graph (even)

bool valid_params(const cosmos_params* p, std::string& why) {
    if (!p) { why = "null params"; return false; }
    if (p->system < 0 || p->system > 2) { why = "system must be 0 (Newtonian), 1 (SR) or 2 (GR)"; return false; }
    if (p->dims != 1 && p->dims != 2) { why = "dims must be 1 or 2"; return false; }
    if (p->nx < 2 || (p->dims == 2 && p->ny < 2)) { why = "need at least 2 cells per dimension (the reference's 2-cell ghost mirror reads c[1] and c[n-2])"; return false; }
    if (p->dims == 1 && p->ny != 1) { why = "1D grids have ny == 1"; return false; }
    if ((long long)p->nx * p->ny > (1ll << 31)) { why = "grid larger than 2^31 cells"; return false; }
    // row-parallel kernels (X sweeps, source step, AMR passes) launch one block row per grid row
    if (p->ny > 65535) { why = "at most 65535 rows (one launch row per grid row)"; return false; }
    if (p->precision != COSMOS_FP64 && p->precision != COSMOS_FP32) { why = "precision must be COSMOS_FP64 or COSMOS_FP32"; return false; }
    if (p->boundary != COSMOS_BC_TRANSMISSIVE && p->boundary != COSMOS_BC_PERIODIC) { why = "unknown boundary"; return false; }
    if (!(p->dx > 0.0)) { why = "dx must be positive"; return false; }
    if (!(p->gamma > 1.0)) { why = "gamma must exceed 1"; return false; }
    if (p->system == COSMOS_GR && p->boundary != COSMOS_BC_TRANSMISSIVE) { why = "the GR system supports transmissive boundaries only"; return false; }
    return true;
}

// Enqueue one full solver step starting from buffer `cur`; *cur_out receives the buffer holding
// the result and *nk the number of kernels enqueued.
// Step structure (Solvers/EulerSecondOrderSolver.cpp:124-147, :102-122; GR
// Solvers/BlackHoleEulerSecondOrderSolver.cpp:144-218): dt from the last CFL reduction, then
// [GR: subcycles RK source half-steps], X(dt/2) Y(dt) X(dt/2) in 2D or one sweep in 1D,
// [GR: subcycles RK source half-steps], and the CFL reduction for the next step.
int enqueue_step(cosmos_grid* g, int cur, int* cur_out, unsigned* nk) {
    const cosmos_solve_opts& o = g->run;
    CK(launch_dt_kernel(g->ctl, g->ctx->stream));
    unsigned k = 1;
    SweepArgs a = base_args(g);
    a.order = o.order;
    a.bias = o.bias;
    a.lim = o.limiter;
    a.out.status = &g->ctl->status;
    a.ds.ctl = g->ctl;
    auto sweep = [&](int axis, double scale, bool ws) -> int {
        a.G.axis = axis;
        a.ds.scale = scale;
        a.ds.nsub = 0;
        a.ds.fsel = scale == 0.5 ? 1 : 0;  // the controller forms FP32 coefficients for dt and dt/2
        a.src = g->buf[cur];
        a.dst = g->buf[cur ^ 1];
        a.out.ws_ctl = ws ? g->ctl : nullptr;
        CK(sweep_launch(g, a));
        cur ^= 1;
        k++;
        return COSMOS_OK;
    };
    auto rk = [&]() -> int {
        SweepArgs r = a;
        r.bias = 0.0;  // the GR solvers call the forcing step with bias 0, limiter 1
        r.lim = 1;     // (Solvers/BlackHoleEulerSecondOrderSolver.cpp:195-209)
        r.ds.nsub = o.subcycles;
        r.src = g->buf[cur];
        r.dst = g->buf[cur ^ 1];
        CK(g->p.precision == COSMOS_FP64 ? launch_rk_source_exact(r) : launch_rk_source_gr_fast(r));
        cur ^= 1;
        k++;
        return COSMOS_OK;
    };
    const bool gr = g->p.system == COSMOS_GR;
    int rc;
    if (gr)
        for (int s = 0; s < o.subcycles; s++)
            if ((rc = rk())) return rc;
    if (g->p.dims == 1) {
        if ((rc = sweep(0, 1.0, !gr))) return rc;
    } else {
        if ((rc = sweep(0, 0.5, false))) return rc;
        if ((rc = sweep(1, 1.0, false))) return rc;
        if ((rc = sweep(0, 0.5, !gr))) return rc;
    }
    if (gr) {
        for (int s = 0; s < o.subcycles; s++)
            if ((rc = rk())) return rc;
        // GR CFL reduction on the final state of the step
        SweepArgs w = base_args(g);
        w.src = g->buf[cur];
        w.out.ws_ctl = g->ctl;
        CK(g->p.precision == COSMOS_FP64 ? launch_wavespeed_exact(w, nullptr) : launch_wavespeed_gr_fast(w, nullptr));
        k++;
    }
    *nk = k;
    *cur_out = cur;
    return COSMOS_OK;
}

}  // namespace

namespace cg {
// One step of a Newtonian or SR run -- the launches enqueue_step records into the step graph, with
// the same device time step -- on explicit buffers: the step reads `src` and its sweep k writes
// dst[k] (three sweeps in 2D, one in 1D).
int enqueue_step_into(cosmos_grid* g, const void* src, void* const* dst) {
    const bool gr = g->p.system == COSMOS_GR;
    const cosmos_solve_opts& o = g->run;
    const int nsub = gr ? o.subcycles : 0;  // RK source half-steps before and after the flux sweeps
    CK(launch_dt_kernel(g->ctl, g->ctx->stream));
    SweepArgs a = base_args(g);
    a.order = o.order;
    a.bias = o.bias;
    a.lim = o.limiter;
    a.out.status = &g->ctl->status;
    a.ds.ctl = g->ctl;
    const int ns = g->p.dims == 2 ? 3 : 1;
    int k = 0;  // operations done; operation k reads dst[k - 1] (src for k = 0) and writes dst[k]
    for (int half = 0; half < 2; half++) {
        for (int s = 0; s < nsub; s++, k++) {  // as enqueue_step's RK half-steps: bias 0, limiter 1
            SweepArgs r = a;
            r.bias = 0.0;
            r.lim = 1;
            r.ds.nsub = nsub;
            r.src = k == 0 ? src : dst[k - 1];
            r.dst = dst[k];
            CK(g->p.precision == COSMOS_FP64 ? launch_rk_source_exact(r) : launch_rk_source_gr_fast(r));
        }
        if (half == 1) break;
        for (int m = 0; m < ns; m++, k++) {
            const double scale = ns == 3 && m != 1 ? 0.5 : 1.0;
            a.G.axis = ns == 3 && m == 1 ? 1 : 0;
            a.ds.scale = scale;
            a.ds.nsub = 0;
            a.ds.fsel = scale == 0.5 ? 1 : 0;
            a.src = k == 0 ? src : dst[k - 1];
            a.dst = dst[k];
            a.out.ws_ctl = m == ns - 1 && !gr ? g->ctl : nullptr;  // the CFL reduction of the step's last sweep
            CK(sweep_launch(g, a));
        }
    }
    if (gr) {  // the black-hole CFL reduction runs on the step's final state, as in enqueue_step
        SweepArgs w = base_args(g);
        w.src = dst[k - 1];
        w.out.ws_ctl = g->ctl;
        CK(g->p.precision == COSMOS_FP64 ? launch_wavespeed_exact(w, nullptr) : launch_wavespeed_gr_fast(w, nullptr));
    }
    return COSMOS_OK;
}
}  // namespace cg

extern "C" {

const char* cosmos_version(void) { return "cosmos_gb300 0.1 (sm_103a)"; }
const char* cosmos_last_error(void) { return t_err.c_str(); }
unsigned long long cosmos_kernel_launches(void) { return g_launches.load(); }

void cosmos_params_default(cosmos_params* p) {
    if (!p) return;
    memset(p, 0, sizeof *p);
    p->system = COSMOS_NEWTONIAN;
    p->dims = 1;
    p->nx = 100;
    p->ny = 1;
    p->precision = COSMOS_FP64;
    p->boundary = COSMOS_BC_TRANSMISSIVE;
    p->gamma = 1.4;
    p->dx = 0.01;
    p->bh_mass = 1.0;   // BlackHoleSpacetime() defaults (BlackHoleEuler/BlackHoleSpacetime.cpp:3-11)
    p->bh_spin = 0.0;
    p->bh_x = 0.5;
    p->bh_y = 0.5;
    p->bh_z = 0.0;
    p->sr_c2p64_above = 2.0;  // SR FP32: primitive recovery finishes in FP64 above Lorentz factor 2
}

void cosmos_solve_opts_default(cosmos_solve_opts* o) {
    if (!o) return;
    o->order = 2;
    o->cfl = 0.9;
    o->t_final = 0.25;
    o->bias = 0.0;
    o->limiter = COSMOS_VANLEER;
    o->subcycles = 1;
    o->max_steps = -1;
}

double cosmos_stable_dt_rule(double dt, double t, double t_final, int iteration) {
    double n = dt;
    if (iteration <= 5) n = n * 0.2;
    if ((t + n) > t_final) n = t_final - t;
    return n;
}

int cosmos_ctx_create(int device, cosmos_ctx** out) {
    if (!out) return fail(COSMOS_EINVAL, "null output pointer");
    int n = 0;
    CK(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n) return fail(COSMOS_EINVAL, "device %d out of range (%d devices)", device, n);
    CK(cudaSetDevice(device));
    cosmos_ctx* c = new cosmos_ctx();
    c->device = device;
    c->refs.store(1);
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->copy, cudaStreamNonBlocking);
    for (int k = 0; k < 2 && e == cudaSuccess; k++) e = cudaEventCreateWithFlags(&c->ev[k], cudaEventDisableTiming);
    if (e != cudaSuccess) {
        delete c;
        return fail(COSMOS_ECUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
    }
    *out = c;
    return COSMOS_OK;
}

int cosmos_ctx_destroy(cosmos_ctx* c) {
    if (c) ctx_release(c);
    return COSMOS_OK;
}

int cosmos_ctx_synchronize(cosmos_ctx* c) {
    if (!c) return fail(COSMOS_EINVAL, "null context");
    CK(cudaStreamSynchronize(c->stream));
    return COSMOS_OK;
}

void* cosmos_ctx_stream(cosmos_ctx* c) { return c ? (void*)c->stream : nullptr; }

int cosmos_grid_create(cosmos_ctx* ctx, const cosmos_params* p, cosmos_grid** out) {
    if (!ctx || !out) return fail(COSMOS_EINVAL, "null context or output pointer");
    std::string why;
    if (!valid_params(p, why)) return fail(COSMOS_EINVAL, "invalid params: %s", why.c_str());
    CK(cudaSetDevice(ctx->device));
    cosmos_grid* g = new cosmos_grid();
    memset((void*)g, 0, sizeof *g);
    g->ctx = ctx;
    ctx_retain(ctx);
    g->p = *p;
    g->elem = p->precision == COSMOS_FP64 ? sizeof(double) : sizeof(float);
    g->G.nx = p->nx;
    g->G.ny = p->dims == 1 ? 1 : p->ny;
    g->G.pitch = (int)round_up((size_t)p->nx, 64);
    g->G.dims = p->dims;
    g->G.axis = 0;
    g->G.bc = p->boundary;
    g->G.fstride = round_up((size_t)g->G.pitch * g->G.ny, 64);
    const size_t bytes = g->G.fstride * 5 * g->elem;
    const size_t ncell = (size_t)g->G.nx * g->G.ny;
    cudaError_t e = cudaSuccess;
    for (int b = 0; b < 2 && e == cudaSuccess; b++) e = cudaMalloc(&g->buf[b], bytes);
    if (e == cudaSuccess) e = cudaMalloc(&g->ctl, sizeof(StepCtl));
    if (e == cudaSuccess) e = cudaMalloc(&g->staging, ncell * 5 * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&g->sums, (8 + 152 * 4 * 5 + 8) * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&g->status, sizeof(int));
    if (e == cudaSuccess && p->system == COSMOS_GR && p->precision == COSMOS_FP32) {
        e = cudaMalloc(&g->gr_mem, gr_tables_bytes(g->G.nx, g->G.ny));
        if (e == cudaSuccess) e = build_gr_tables(base_args(g), g->gr_mem, &g->grt);
    }
    if (e == cudaSuccess) e = cudaMemsetAsync(g->buf[0], 0, bytes, ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(g->buf[1], 0, bytes, ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(g->sums, 0, (8 + 152 * 4 * 5 + 8) * sizeof(double), ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(g->ctl, 0, sizeof(StepCtl), ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(g->status, 0, sizeof(int), ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
        cosmos_grid_destroy(g);
        return fail(COSMOS_ECUDA, "grid allocation (%zu bytes of state): %s", 2 * bytes, cudaGetErrorString(e));
    }
    *out = g;
    return COSMOS_OK;
}

int cosmos_grid_destroy(cosmos_grid* g) {
    if (!g) return COSMOS_OK;
    cudaSetDevice(g->ctx->device);
    cudaStreamSynchronize(g->ctx->stream);
    for (int b = 0; b < 2; b++) {
        if (g->step_graph[b]) cudaGraphExecDestroy(g->step_graph[b]);
        if (g->chunk_graph[b]) cudaGraphExecDestroy(g->chunk_graph[b]);
        if (g->buf[b]) cudaFree(g->buf[b]);
    }
    if (g->ctl) cudaFree(g->ctl);
    if (g->staging) cudaFree(g->staging);
    if (g->sums) cudaFree(g->sums);
    if (g->status) cudaFree(g->status);
    if (g->gr_mem) cudaFree(g->gr_mem);
    cosmos_ctx* ctx = g->ctx;
    delete g;
    ctx_release(ctx);
    return COSMOS_OK;
}

namespace {
// Rows per chunk of a host <-> device transfer: about eight chunks, at least 64 rows each.
int chunk_rows(const Geom& G) { return std::max(64, (G.ny + 7) / 8); }

cudaError_t convert_in(cosmos_grid* g, const double* staging, void* state, const Geom& G) {
    if (g->p.precision == COSMOS_FP64) return launch_prim_in_exact(staging, state, G, g->ctx->stream);
    if (g->p.system == COSMOS_GR) {
        SweepArgs a = base_args(g);
        a.G = G;
        return launch_prim_in_gr_fast(a, staging, state);
    }
    return launch_prim_in_fast(staging, state, G, g->p.system, g->p.gamma, g->ctx->stream);
}
cudaError_t convert_out(cosmos_grid* g, const void* state, double* staging, const Geom& G) {
    if (g->p.precision == COSMOS_FP64) return launch_prim_out_exact(state, staging, G, g->ctx->stream);
    if (g->p.system == COSMOS_GR) {
        SweepArgs a = base_args(g);
        a.G = G;
        return launch_prim_out_gr_fast(a, state, staging);
    }
    return launch_prim_out_fast(state, staging, G, g->p.system, g->p.gamma, g->ctx->stream);
}
}  // namespace

// Uploads and downloads move row chunks on the context's copy stream while the conversion kernels
// of the previous chunk run on its compute stream (two engines busy at once); events order them.
int cosmos_grid_set_prim(cosmos_grid* g, const double* prim, size_t n) {
    if (!g || !prim) return fail(COSMOS_EINVAL, "null grid or buffer");
    const size_t want = (size_t)5 * g->G.nx * g->G.ny;
    if (n != want) return fail(COSMOS_EINVAL, "buffer holds %zu doubles, grid needs %zu", n, want);
    CK(cudaSetDevice(g->ctx->device));
    cosmos_ctx* c = g->ctx;
    // the staging buffer may still be read by earlier work on the compute stream
    CK(cudaEventRecord(c->ev[0], c->stream));
    CK(cudaStreamWaitEvent(c->copy, c->ev[0], 0));
    const int rows = chunk_rows(g->G);
    for (int r0 = 0; r0 < g->G.ny; r0 += rows) {
        Geom G = g->G;
        G.ny = std::min(rows, g->G.ny - r0);
        const size_t off = (size_t)5 * g->G.nx * r0;
        CK(cudaMemcpyAsync(g->staging + off, prim + off, (size_t)5 * g->G.nx * G.ny * sizeof(double),
                           cudaMemcpyHostToDevice, c->copy));
        CK(cudaEventRecord(c->ev[1], c->copy));
        CK(cudaStreamWaitEvent(c->stream, c->ev[1], 0));
        CK(convert_in(g, g->staging + off, (char*)g->buf[g->cur] + (size_t)r0 * g->G.pitch * g->elem, G));
    }
    // the caller's buffer may be reused once this returns
    CK(cudaStreamSynchronize(c->copy));
    return COSMOS_OK;
}

int cosmos_grid_get_prim(cosmos_grid* g, double* prim, size_t n) {
    if (!g || !prim) return fail(COSMOS_EINVAL, "null grid or buffer");
    const size_t want = (size_t)5 * g->G.nx * g->G.ny;
    if (n != want) return fail(COSMOS_EINVAL, "buffer holds %zu doubles, grid needs %zu", n, want);
    CK(cudaSetDevice(g->ctx->device));
    cosmos_ctx* c = g->ctx;
    const int rows = chunk_rows(g->G);
    for (int r0 = 0; r0 < g->G.ny; r0 += rows) {
        Geom G = g->G;
        G.ny = std::min(rows, g->G.ny - r0);
        const size_t off = (size_t)5 * g->G.nx * r0;
        CK(convert_out(g, (const char*)g->buf[g->cur] + (size_t)r0 * g->G.pitch * g->elem, g->staging + off, G));
        CK(cudaEventRecord(c->ev[0], c->stream));
        CK(cudaStreamWaitEvent(c->copy, c->ev[0], 0));
        CK(cudaMemcpyAsync(prim + off, g->staging + off, (size_t)5 * g->G.nx * G.ny * sizeof(double),
                           cudaMemcpyDeviceToHost, c->copy));
    }
    CK(cudaStreamSynchronize(c->copy));
    return COSMOS_OK;
}

int cosmos_grid_sweep(cosmos_grid* g, int axis, int order, double dt, double bias, int limiter) {
    if (!g) return fail(COSMOS_EINVAL, "null grid");
    if (axis != 0 && !(axis == 1 && g->p.dims == 2)) return fail(COSMOS_EINVAL, "axis %d invalid for a %dD grid", axis, g->p.dims);
    if (order != 1 && order != 2) return fail(COSMOS_EINVAL, "order must be 1 (FORCE) or 2 (SLIC)");
    if (!(dt > 0.0)) return fail(COSMOS_EINVAL, "dt must be positive");
    CK(cudaSetDevice(g->ctx->device));
    SweepArgs a = base_args(g);
    a.G.axis = axis;
    a.order = order;
    a.bias = bias;
    a.lim = limiter;
    a.ds.fixed = dt;
    a.ds.ffix = make_fast_coef(dt, g->p.dx);
    a.src = g->buf[g->cur];
    a.dst = g->buf[g->cur ^ 1];
    a.out.status = g->status;
    CK(sweep_launch(g, a));
    g->cur ^= 1;
    return COSMOS_OK;
}

int cosmos_grid_rk_source(cosmos_grid* g, double dt, double bias, int limiter) {
    if (!g) return fail(COSMOS_EINVAL, "null grid");
    if (g->p.system != COSMOS_GR) return fail(COSMOS_EUNSUPPORTED, "the source step exists for the GR system only");
    if (!(dt > 0.0)) return fail(COSMOS_EINVAL, "dt must be positive");
    CK(cudaSetDevice(g->ctx->device));
    SweepArgs a = base_args(g);
    a.bias = bias;
    a.lim = limiter;
    a.ds.fixed = dt;
    a.src = g->buf[g->cur];
    a.dst = g->buf[g->cur ^ 1];
    a.out.status = g->status;
    CK(g->p.precision == COSMOS_FP64 ? launch_rk_source_exact(a) : launch_rk_source_gr_fast(a));
    g->cur ^= 1;
    return COSMOS_OK;
}

int cosmos_grid_max_wavespeed(cosmos_grid* g, double* out) {
    if (!g || !out) return fail(COSMOS_EINVAL, "null grid or output");
    CK(cudaSetDevice(g->ctx->device));
    unsigned long long* slot = (unsigned long long*)(g->sums + 8 + 152 * 4 * 5 + 4);
    CK(cudaMemsetAsync(slot, 0, sizeof *slot, g->ctx->stream));
    SweepArgs a = base_args(g);
    a.src = g->buf[g->cur];
    if (g->p.precision == COSMOS_FP64) CK(launch_wavespeed_exact(a, slot));
    else CK(launch_wavespeed_fast(a, slot));
    unsigned long long bits = 0;
    CK(cudaMemcpyAsync(&bits, slot, sizeof bits, cudaMemcpyDeviceToHost, g->ctx->stream));
    CK(cudaStreamSynchronize(g->ctx->stream));
    double v;
    memcpy(&v, &bits, sizeof v);
    *out = v;
    return COSMOS_OK;
}

int cosmos_grid_stable_dt(cosmos_grid* g, double cfl, double t, double t_final, int iteration, double* dt_out) {
    if (!dt_out) return fail(COSMOS_EINVAL, "null output");
    double s = 0.0;
    int rc = cosmos_grid_max_wavespeed(g, &s);
    if (rc) return rc;
    *dt_out = cosmos_stable_dt_rule(cfl * (g->p.dx / s), t, t_final, iteration);
    return COSMOS_OK;
}

int cosmos_grid_run_begin(cosmos_grid* g, const cosmos_solve_opts* o) {
    if (!g || !o) return fail(COSMOS_EINVAL, "null grid or options");
    if (o->order != 1 && o->order != 2) return fail(COSMOS_EINVAL, "order must be 1 or 2");
    if (!(o->cfl > 0.0)) return fail(COSMOS_EINVAL, "cfl must be positive");
    // 0 subcycles: no source step, the flux sweeps alone (the reference's loops over
    // subcyclingIterations run zero times, Solvers/BlackHoleEulerSecondOrderSolver.cpp:158-170)
    if (g->p.system == COSMOS_GR && o->subcycles < 0) return fail(COSMOS_EINVAL, "GR runs need subcycles >= 0");
    CK(cudaSetDevice(g->ctx->device));
    cudaStream_t st = g->ctx->stream;
    const bool same = g->run_ready && g->run.order == o->order && g->run.bias == o->bias &&
                      g->run.limiter == o->limiter && g->run.subcycles == o->subcycles;
    g->run = *o;
    // controller reset: t = 0, iteration 0 (the reference's solve() locals)
    StepCtl h;
    memset(&h, 0, sizeof h);
    h.t = 0.0;
    h.t_final = o->t_final;
    h.cfl = o->cfl;
    h.dx = g->p.dx;
    h.it = 0;
    h.it_limit = o->max_steps < 0 ? INT_MAX : o->max_steps;
    h.active = 1;
    CK(cudaMemcpyAsync(g->ctl, &h, sizeof h, cudaMemcpyHostToDevice, st));
    // initial CFL reduction into slot 0
    SweepArgs a = base_args(g);
    a.src = g->buf[g->cur];
    if (g->p.precision == COSMOS_FP64) CK(launch_wavespeed_exact(a, &g->ctl->smax[0]));
    else CK(launch_wavespeed_fast(a, &g->ctl->smax[0]));
    if (!same) {
        // one step, and kChunkSteps steps, from each starting buffer; replaying a chunk saves the
        // launch gap between consecutive graphs
        for (int b = 0; b < 2; b++)
            for (int chunk = 0; chunk < 2; chunk++) {
                cudaGraphExec_t& exec = chunk ? g->chunk_graph[b] : g->step_graph[b];
                if (exec) { cudaGraphExecDestroy(exec); exec = nullptr; }
                cudaGraph_t graph;
                CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
                unsigned nk = 0;
                int cur = b, r = 0;
                t_capturing = true;
                for (int s = 0; s < (chunk ? kChunkSteps : 1) && !r; s++) {
                    int end = 0;
                    r = enqueue_step(g, cur, &end, &nk);
                    if (!r && end != (cur ^ 1)) r = fail(COSMOS_ESTATE, "step writes an even number of times");
                    cur ^= 1;
                }
                t_capturing = false;
                cudaError_t ec = cudaStreamEndCapture(st, &graph);
                if (r) { if (ec == cudaSuccess) cudaGraphDestroy(graph); return r; }
                if (ec != cudaSuccess) return fail(COSMOS_ECUDA, "graph capture: %s", cudaGetErrorString(ec));
                cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
                cudaGraphDestroy(graph);
                if (ei != cudaSuccess) return fail(COSMOS_ECUDA, "graph instantiate: %s", cudaGetErrorString(ei));
                if (!chunk) g->step_kernels = nk;
            }
        g->run_ready = true;
    }
    return COSMOS_OK;
}

int cosmos_grid_run_steps(cosmos_grid* g, int n) {
    if (!g) return fail(COSMOS_EINVAL, "null grid");
    if (!g->run_ready) return fail(COSMOS_ESTATE, "cosmos_grid_run_begin has not been called");
    if (n < 0) return fail(COSMOS_EINVAL, "negative step count");
    int s = 0;
    for (; s + kChunkSteps <= n; s += kChunkSteps) {  // an even number of steps: the buffer stays
        CK(cudaGraphLaunch(g->chunk_graph[g->cur], g->ctx->stream));
        count_launch(g->step_kernels * kChunkSteps);
    }
    for (; s < n; s++) {
        CK(cudaGraphLaunch(g->step_graph[g->cur], g->ctx->stream));
        count_launch(g->step_kernels);
        g->cur ^= 1;  // every step has an odd number of state-writing kernels
    }
    return COSMOS_OK;
}

int cosmos_grid_run_end(cosmos_grid* g, cosmos_solve_result* r) {
    if (!g) return fail(COSMOS_EINVAL, "null grid");
    StepCtl h;
    CK(cudaMemcpyAsync(&h, g->ctl, sizeof h, cudaMemcpyDeviceToHost, g->ctx->stream));
    CK(cudaStreamSynchronize(g->ctx->stream));
    if (r) {
        r->steps = h.it;
        r->t = h.t;
        r->status = h.status;
    }
    if (h.status & ST_NONFINITE) return fail(COSMOS_ENONFINITE, "non-finite or non-positive time step at iteration %d (t = %g)", h.it, h.t);
    return COSMOS_OK;
}

int cosmos_grid_solve(cosmos_grid* g, const cosmos_solve_opts* o, cosmos_solve_result* r) {
    int rc = cosmos_grid_run_begin(g, o);
    if (rc) return rc;
    const int chunk = 32;
    for (;;) {
        if ((rc = cosmos_grid_run_steps(g, chunk))) return rc;
        StepCtl h;
        CK(cudaMemcpyAsync(&h, g->ctl, sizeof h, cudaMemcpyDeviceToHost, g->ctx->stream));
        CK(cudaStreamSynchronize(g->ctx->stream));
        if (h.status & ST_NONFINITE) break;
        if (!(h.t < h.t_final) || h.it >= h.it_limit) break;
    }
    return cosmos_grid_run_end(g, r);
}

int cosmos_grid_field_sums(cosmos_grid* g, double out[5]) {
    if (!g || !out) return fail(COSMOS_EINVAL, "null grid or output");
    CK(cudaSetDevice(g->ctx->device));
    CK(launch_field_sums(g->buf[g->cur], g->G, g->p.precision, g->sums, g->ctx->stream));
    CK(cudaMemcpyAsync(out, g->sums, 5 * sizeof(double), cudaMemcpyDeviceToHost, g->ctx->stream));
    CK(cudaStreamSynchronize(g->ctx->stream));
    return COSMOS_OK;
}

int cosmos_grid_amr_flags(cosmos_grid* g, double tol, unsigned char* coarse, unsigned char* fine) {
    if (!g || !coarse || !fine) return fail(COSMOS_EINVAL, "null grid or flag buffer");
    CK(cudaSetDevice(g->ctx->device));
    const size_t nc = (size_t)g->G.nx * g->G.ny, nf = nc * (g->p.dims == 2 ? 4 : 2);
    unsigned char* d = nullptr;
    CK(cudaMallocAsync((void**)&d, nc + nf, g->ctx->stream));
    CK(cudaMemcpyAsync(d, coarse, nc, cudaMemcpyHostToDevice, g->ctx->stream));
    CK(cudaMemcpyAsync(d + nc, fine, nf, cudaMemcpyHostToDevice, g->ctx->stream));
    SweepArgs a = base_args(g);
    a.src = g->buf[g->cur];
    CK(launch_amr_flags(a, g->p.precision, tol, d, d + nc));
    CK(cudaMemcpyAsync(coarse, d, nc, cudaMemcpyDeviceToHost, g->ctx->stream));
    CK(cudaMemcpyAsync(fine, d + nc, nf, cudaMemcpyDeviceToHost, g->ctx->stream));
    CK(cudaFreeAsync(d, g->ctx->stream));
    CK(cudaStreamSynchronize(g->ctx->stream));
    return COSMOS_OK;
}

int cosmos_grid_amr_derefine(cosmos_grid* coarse, cosmos_grid* fine, double tol, unsigned char* cflags,
                             unsigned char* fflags) {
    if (!coarse || !fine || !cflags || !fflags) return fail(COSMOS_EINVAL, "null argument");
    if (coarse->p.system != fine->p.system || coarse->p.precision != fine->p.precision ||
        coarse->p.dims != fine->p.dims || fine->G.nx != 2 * coarse->G.nx ||
        (coarse->p.dims == 2 && fine->G.ny != 2 * coarse->G.ny))
        return fail(COSMOS_EINVAL, "fine grid must be the 2x refinement of the coarse grid");
    if (coarse->p.system == COSMOS_GR && coarse->p.precision == COSMOS_FP32)
        return fail(COSMOS_EUNSUPPORTED, "derefinement of FP32 black-hole grids is not provided");
    CK(cudaSetDevice(coarse->ctx->device));
    cudaStream_t st = coarse->ctx->stream;
    CK(cudaStreamSynchronize(fine->ctx->stream));
    const size_t nc = (size_t)coarse->G.nx * coarse->G.ny, nf = nc * (coarse->p.dims == 2 ? 4 : 2);
    unsigned char* d = nullptr;
    CK(cudaMallocAsync((void**)&d, nc + nf, st));
    CK(cudaMemcpyAsync(d, cflags, nc, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(d + nc, fflags, nf, cudaMemcpyHostToDevice, st));
    SweepArgs a = base_args(coarse);
    CK(launch_amr_derefine(a, coarse->p.precision, fine->buf[fine->cur], fine->G, tol, d, d + nc,
                           coarse->buf[coarse->cur]));
    CK(cudaMemcpyAsync(cflags, d, nc, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(fflags, d + nc, nf, cudaMemcpyDeviceToHost, st));
    CK(cudaFreeAsync(d, st));
    CK(cudaStreamSynchronize(st));
    return COSMOS_OK;
}

int cosmos_solve_prim(const cosmos_params* p, const double* prim_in, double* prim_out, const cosmos_solve_opts* o,
                      cosmos_solve_result* r) {
    if (!p || !prim_in || !prim_out || !o) return fail(COSMOS_EINVAL, "null argument");
    int dev = 0;
    CK(cudaGetDevice(&dev));
    cosmos_ctx* ctx = nullptr;
    int rc = cosmos_ctx_create(dev, &ctx);
    if (rc) return rc;
    cosmos_grid* g = nullptr;
    const size_t n = (size_t)5 * p->nx * (p->dims == 2 ? p->ny : 1);
    if (!(rc = cosmos_grid_create(ctx, p, &g)) && !(rc = cosmos_grid_set_prim(g, prim_in, n)) &&
        !(rc = cosmos_grid_solve(g, o, r)))
        rc = cosmos_grid_get_prim(g, prim_out, n);
    std::string keep = t_err;
    cosmos_grid_destroy(g);
    cosmos_ctx_destroy(ctx);
    t_err = keep;
    return rc;
}

}  // extern "C"
