// C ABI of the Level-1 AMR drivers (EulerAMR::solveLevel1AMR / solve2DLevel1AMR,
// AMR/EulerAMR.cpp:169-592; RelativisticEulerAMR twins, AMR/RelativisticEulerAMR.cpp:181-603).
//
// Both levels are ordinary device grids (the fine one at 2x resolution and dx / 2) plus one flag
// byte per cell.  The host keeps the reference's loop control (times, iteration counters, the
// 1e-4 sub-cycling slack) in FP64 exactly as written; everything that touches cells runs on the
// device: CFL reductions, the flag passes, masked sweeps (cells whose flag is off are copied),
// the level exchange and the derefinement.  Each coarse step makes one host round trip (its CFL
// maximum and the any-fine-flag word in one 16-byte read) plus one per fine step (its CFL
// maximum); the masked sweeps take the host's dt as a launch argument.
#include <cmath>
#include <cstring>
#include <string>

#include "capi_internal.h"

using namespace cg;

struct cosmos_amr {
    cosmos_ctx* ctx;
    cosmos_grid* level[2];       // 0 coarse, 1 fine
    unsigned char* flags;        // device: coarse flags (nc bytes), then fine flags (nf bytes)
    size_t nc, nf;
    unsigned long long* word;    // device: [0] CFL maximum (bits of a non-negative double), [1] any fine flag
    unsigned long long* host;    // page-locked copy of word
};

namespace {

int afail(int code, const std::string& msg) {
    set_error(msg.c_str());
    return code;
}
#define MCK(call)                                                                                    \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess) return afail(COSMOS_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)
#define MRC(call)                      \
    do {                               \
        int r_ = (call);               \
        if (r_ != COSMOS_OK) return r_; \
    } while (0)

// A masked sweep with a host time step: the reference drivers' computeSLICTimeStepAMR /
// computeX/YSLICTimeStep2DAMR (AMR/EulerAMR.cpp:83-167) and FORCE twins (:3-81), bias 0 and
// limiter 1 (:231-239).  Cells whose flag is off keep their state.
int masked_sweep(cosmos_grid* g, int axis, int order, double dt, const unsigned char* mask) {
    SweepArgs a = base_args(g);
    a.G.axis = axis;
    a.order = order;
    a.bias = 0.0;
    a.lim = 1;
    a.ds.fixed = dt;
    a.ds.ffix = make_fast_coef(dt, g->p.dx);
    a.src = g->buf[g->cur];
    a.dst = g->buf[g->cur ^ 1];
    a.out.status = g->status;
    a.out.mask = mask;
    MCK(sweep_launch(g, a));
    g->cur ^= 1;
    return COSMOS_OK;
}

// One masked step of a level: one sweep in 1D, X(dt/2) Y(dt) X(dt/2) in 2D (AMR/EulerAMR.cpp:231-239, :434-444).
int masked_step(cosmos_grid* g, int order, double dt, const unsigned char* mask) {
    if (g->p.dims == 1) return masked_sweep(g, 0, order, dt, mask);
    MRC(masked_sweep(g, 0, order, dt * 0.5, mask));
    MRC(masked_sweep(g, 1, order, dt, mask));
    return masked_sweep(g, 0, order, dt * 0.5, mask);
}

// Enqueues the CFL maximum of a level into word[0] (and, with `any`, whether a fine flag is set into
// word[1]), reads both back and returns them.
int read_word(cosmos_amr* a, cosmos_grid* g, bool any, double* smax, bool* refined) {
    cudaStream_t st = a->ctx->stream;
    MCK(cudaMemsetAsync(a->word, 0, 2 * sizeof(unsigned long long), st));
    SweepArgs w = base_args(g);
    w.src = g->buf[g->cur];
    MCK(g->p.precision == COSMOS_FP64 ? launch_wavespeed_exact(w, a->word) : launch_wavespeed_fast(w, a->word));
    if (any) MCK(launch_amr_any(a->flags + a->nc, a->nf, a->word + 1, st));
    MCK(cudaMemcpyAsync(a->host, a->word, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    MCK(cudaStreamSynchronize(st));
    memcpy(smax, &a->host[0], sizeof(double));
    if (refined) *refined = a->host[1] != 0;
    return COSMOS_OK;
}

int bad_dt(double dt) {
    if (dt > 0.0 && std::isfinite(dt)) return COSMOS_OK;
    return afail(COSMOS_ENONFINITE, "AMR driver: non-finite or non-positive time step " + std::to_string(dt));
}

}  // namespace

extern "C" {

int cosmos_amr_create(cosmos_ctx* ctx, const cosmos_params* p, cosmos_amr** out) {
    if (!ctx || !p || !out) return afail(COSMOS_EINVAL, "null context, params or output pointer");
    if (p->system == COSMOS_GR)
        return afail(COSMOS_EUNSUPPORTED, "the AMR driver covers the Newtonian and SR systems (the reference's "
                                          "black-hole AMR driver does not compile)");
    if (p->boundary != COSMOS_BC_TRANSMISSIVE)
        return afail(COSMOS_EUNSUPPORTED, "the AMR driver uses the reference's transmissive boundaries");
    cosmos_amr* a = new cosmos_amr();
    memset((void*)a, 0, sizeof *a);
    a->ctx = ctx;
    cosmos_params fp = *p;
    fp.nx = 2 * p->nx;
    fp.ny = p->dims == 2 ? 2 * p->ny : 1;
    fp.dx = p->dx * 0.5;
    int rc = cosmos_grid_create(ctx, p, &a->level[0]);
    if (!rc) rc = cosmos_grid_create(ctx, &fp, &a->level[1]);
    if (rc) {
        cosmos_amr_destroy(a);
        return rc;
    }
    a->nc = (size_t)a->level[0]->G.nx * a->level[0]->G.ny;
    a->nf = (size_t)a->level[1]->G.nx * a->level[1]->G.ny;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e == cudaSuccess) e = cudaMalloc((void**)&a->flags, a->nc + a->nf);
    if (e == cudaSuccess) e = cudaMalloc((void**)&a->word, 2 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMallocHost((void**)&a->host, 2 * sizeof(unsigned long long));
    if (e != cudaSuccess) {
        cosmos_amr_destroy(a);
        return afail(COSMOS_ECUDA, std::string("AMR allocation: ") + cudaGetErrorString(e));
    }
    *out = a;
    return COSMOS_OK;
}

int cosmos_amr_destroy(cosmos_amr* a) {
    if (!a) return COSMOS_OK;
    if (a->level[0]) cudaSetDevice(a->level[0]->ctx->device);
    if (a->ctx) cudaStreamSynchronize(a->ctx->stream);
    if (a->flags) cudaFree(a->flags);
    if (a->word) cudaFree(a->word);
    if (a->host) cudaFreeHost(a->host);
    for (int l = 0; l < 2; l++) cosmos_grid_destroy(a->level[l]);
    delete a;
    return COSMOS_OK;
}

int cosmos_amr_set_prim(cosmos_amr* a, const double* prim, size_t n) {
    if (!a) return afail(COSMOS_EINVAL, "null AMR handle");
    return cosmos_grid_set_prim(a->level[0], prim, n);
}

int cosmos_amr_solve(cosmos_amr* a, double cfl, double t_final, double tol, int order, cosmos_amr_result* r) {
    if (!a) return afail(COSMOS_EINVAL, "null AMR handle");
    if (order != 1 && order != 2) return afail(COSMOS_EINVAL, "order must be 1 (FORCE) or 2 (SLIC)");
    if (!(cfl > 0.0)) return afail(COSMOS_EINVAL, "cfl must be positive");
    cosmos_grid* C = a->level[0];
    cosmos_grid* F = a->level[1];
    const int prec = C->p.precision;
    MCK(cudaSetDevice(a->ctx->device));
    cudaStream_t st = a->ctx->stream;
    unsigned char* cflags = a->flags;
    unsigned char* fflags = a->flags + a->nc;
    MCK(cudaMemsetAsync(C->status, 0, sizeof(int), st));
    MCK(cudaMemsetAsync(F->status, 0, sizeof(int), st));
    // initial flags (AMR/EulerAMR.cpp:181-190) and fine cells copied from their parents (:197-202):
    // with every coarse flag on and every fine flag off, the level exchange is exactly that copy
    MCK(cudaMemsetAsync(cflags, 1, a->nc, st));
    MCK(cudaMemsetAsync(fflags, 0, a->nf, st));
    SweepArgs ca = base_args(C);
    MCK(launch_amr_sync(ca, prec, C->buf[C->cur], F->buf[F->cur], F->G, cflags, fflags));
    const double dx = C->p.dx;
    double t = 0.0;
    int it = 0, fit = 0, run = 0;
    int rc = COSMOS_OK;
    while (t < t_final) {
        double smax = 0.0;
        bool refined = false;
        // the coarse time step is taken before the flag pass (AMR/EulerAMR.cpp:197-198); both read
        // the same coarse state, so the flag pass is enqueued first and one read returns both
        SweepArgs fa = base_args(C);
        fa.src = C->buf[C->cur];
        MCK(launch_amr_flags(fa, prec, tol, cflags, fflags));
        if ((rc = read_word(a, C, true, &smax, &refined))) break;
        const double dt = cosmos_stable_dt_rule(cfl * (dx / smax), t, t_final, fit);
        if ((rc = bad_dt(dt))) break;
        if ((rc = masked_step(C, order, dt, cflags))) break;
        if (refined) {
            double ft = t;
            while (ft < (t + dt - 1e-4)) {
                double fs = 0.0;
                if ((rc = read_word(a, F, false, &fs, nullptr))) break;
                const double fdt = cosmos_stable_dt_rule(cfl * ((dx * 0.5) / fs), ft, t + dt, fit);
                if ((rc = bad_dt(fdt))) break;
                if ((rc = masked_step(F, order, fdt, fflags))) break;
                ft += fdt;
                fit += 1;
                run += 1;
            }
            if (rc) break;
        } else {
            fit += 1;
        }
        t += dt;
        it += 1;
        // restriction and injection (AMR/EulerAMR.cpp:287-307), then derefinement (:309-345)
        SweepArgs sa = base_args(C);
        MCK(launch_amr_sync(sa, prec, C->buf[C->cur], F->buf[F->cur], F->G, cflags, fflags));
        MCK(launch_amr_derefine(sa, prec, F->buf[F->cur], F->G, tol, cflags, fflags, C->buf[C->cur]));
    }
    int st2[2] = {0, 0};
    MCK(cudaMemcpyAsync(&st2[0], C->status, sizeof(int), cudaMemcpyDeviceToHost, st));
    MCK(cudaMemcpyAsync(&st2[1], F->status, sizeof(int), cudaMemcpyDeviceToHost, st));
    MCK(cudaStreamSynchronize(st));
    if (r) {
        r->coarse_steps = it;
        r->fine_steps = fit;
        r->t = t;
        r->status = st2[0] | st2[1] | (rc == COSMOS_ENONFINITE ? COSMOS_STATUS_NONFINITE : 0);
        r->fine_run = run;
    }
    return rc;
}

int cosmos_amr_get(cosmos_amr* a, double* coarse_prim, double* fine_prim, unsigned char* coarse_flags,
                   unsigned char* fine_flags) {
    if (!a) return afail(COSMOS_EINVAL, "null AMR handle");
    MCK(cudaSetDevice(a->ctx->device));
    if (coarse_prim) MRC(cosmos_grid_get_prim(a->level[0], coarse_prim, 5 * a->nc));
    if (fine_prim) MRC(cosmos_grid_get_prim(a->level[1], fine_prim, 5 * a->nf));
    cudaStream_t st = a->ctx->stream;
    if (coarse_flags) MCK(cudaMemcpyAsync(coarse_flags, a->flags, a->nc, cudaMemcpyDeviceToHost, st));
    if (fine_flags) MCK(cudaMemcpyAsync(fine_flags, a->flags + a->nc, a->nf, cudaMemcpyDeviceToHost, st));
    MCK(cudaStreamSynchronize(st));
    return COSMOS_OK;
}

}  // extern "C"
