// C ABI of the AMR drivers: Level 1 (EulerAMR::solveLevel1AMR / solve2DLevel1AMR,
// AMR/EulerAMR.cpp:169-592; RelativisticEulerAMR twins, AMR/RelativisticEulerAMR.cpp:181-603) and
// Level 2 (solveLevel2AMR / solve2DLevel2AMR, AMR/EulerAMR.cpp:593-1379,
// AMR/RelativisticEulerAMR.cpp:604-1392).
//
// Every level is an ordinary device grid (each at twice the previous resolution) plus one flag byte
// per cell.  The host keeps the reference's loop control (times, iteration counters, the 1e-4
// sub-cycling slack) in FP64 exactly as written; everything that touches cells runs on the device:
// CFL reductions, the flag passes, masked sweeps (cells whose flag is off are copied), the level
// exchanges and the derefinement passes.  Each level step makes one host round trip (its CFL
// maximum, with the next level's any-flag word where the loop needs it, in one 16-byte read); the
// masked sweeps take the host's dt as a launch argument.
#include <cmath>
#include <cstring>
#include <string>

#include "capi_internal.h"

using namespace cg;

struct cosmos_amr {
    cosmos_ctx* ctx;
    int nlev;                    // 2: the Level-1 driver (coarse, fine); 3: Level 2 (coarse, intermediate, fine)
    cosmos_grid* level[3];
    unsigned char* flags;        // device: every level's flags, level after level
    size_t n[3], off[3];         // cells and flag offset per level
    unsigned long long* word;    // device: [0] CFL maximum (bits of a non-negative double), [1] any flag
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

// Enqueues the CFL maximum of level l into word[0] (and, with any_level >= 0, whether a flag of that
// level is set into word[1]), reads both back and returns them.
int read_word(cosmos_amr* a, int l, int any_level, double* smax, bool* refined) {
    cudaStream_t st = a->ctx->stream;
    cosmos_grid* g = a->level[l];
    MCK(cudaMemsetAsync(a->word, 0, 2 * sizeof(unsigned long long), st));
    SweepArgs w = base_args(g);
    w.src = g->buf[g->cur];
    MCK(g->p.precision == COSMOS_FP64 ? launch_wavespeed_exact(w, a->word) : launch_wavespeed_fast(w, a->word));
    if (any_level >= 0) MCK(launch_amr_any(a->flags + a->off[any_level], a->n[any_level], a->word + 1, st));
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

// A finer level takes about 2 steps per parent step; a run that needs this many has a collapsed
// time step (the reference would keep looping), so the driver stops with an error instead.
constexpr int kMaxSubSteps = 1 << 20;
int too_many(int k) {
    if (k < kMaxSubSteps) return COSMOS_OK;
    return afail(COSMOS_ENONFINITE, "AMR driver: more than 2^20 sub-steps in one parent step (collapsed time step)");
}

// Sweep arguments of level l reading its current state.
SweepArgs level_args(cosmos_amr* a, int l) {
    SweepArgs s = base_args(a->level[l]);
    s.src = a->level[l]->buf[a->level[l]->cur];
    return s;
}
void* state(cosmos_amr* a, int l) { return a->level[l]->buf[a->level[l]->cur]; }
unsigned char* flags(cosmos_amr* a, int l) { return a->flags + a->off[l]; }

int create(cosmos_ctx* ctx, const cosmos_params* p, int nlev, cosmos_amr** out) {
    if (!ctx || !p || !out) return afail(COSMOS_EINVAL, "null context, params or output pointer");
    if (p->system == COSMOS_GR)
        return afail(COSMOS_EUNSUPPORTED, "the AMR drivers cover the Newtonian and SR systems (the reference's "
                                          "black-hole AMR driver does not compile)");
    if (p->boundary != COSMOS_BC_TRANSMISSIVE)
        return afail(COSMOS_EUNSUPPORTED, "the AMR drivers use the reference's transmissive boundaries");
    cosmos_amr* a = new cosmos_amr();
    memset((void*)a, 0, sizeof *a);
    a->ctx = ctx;
    a->nlev = nlev;
    int rc = COSMOS_OK;
    size_t total = 0;
    for (int l = 0; l < nlev && !rc; l++) {
        cosmos_params q = *p;
        const int s = 1 << l;
        q.nx = s * p->nx;
        q.ny = p->dims == 2 ? s * p->ny : 1;
        q.dx = l == 0 ? p->dx : (l == 1 ? p->dx * 0.5 : p->dx * 0.25);  // the reference's cellSpacing * 0.5, * 0.25
        rc = cosmos_grid_create(ctx, &q, &a->level[l]);
        if (!rc) {
            a->n[l] = (size_t)a->level[l]->G.nx * a->level[l]->G.ny;
            a->off[l] = total;
            total += a->n[l];
        }
    }
    if (rc) {
        cosmos_amr_destroy(a);
        return rc;
    }
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e == cudaSuccess) e = cudaMalloc((void**)&a->flags, total);
    if (e == cudaSuccess) e = cudaMalloc((void**)&a->word, 2 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMallocHost((void**)&a->host, 2 * sizeof(unsigned long long));
    if (e != cudaSuccess) {
        cosmos_amr_destroy(a);
        return afail(COSMOS_ECUDA, std::string("AMR allocation: ") + cudaGetErrorString(e));
    }
    *out = a;
    return COSMOS_OK;
}

// Initial state of the drivers (AMR/EulerAMR.cpp:181-202, :606-636): every coarse flag on, every
// other flag off, each finer level a copy of its parent.  The level exchange with the parent on
// and the children off is exactly that copy; the intermediate flags are switched on for the
// copy into the fine level and off again.
int init_levels(cosmos_amr* a) {
    cudaStream_t st = a->ctx->stream;
    const int prec = a->level[0]->p.precision;
    MCK(cudaMemsetAsync(flags(a, 0), 1, a->n[0], st));
    for (int l = 1; l < a->nlev; l++) MCK(cudaMemsetAsync(flags(a, l), 0, a->n[l], st));
    for (int l = 0; l + 1 < a->nlev; l++) {
        if (l > 0) MCK(cudaMemsetAsync(flags(a, l), 1, a->n[l], st));
        MCK(launch_amr_sync(level_args(a, l), prec, state(a, l), state(a, l + 1), a->level[l + 1]->G, flags(a, l),
                            flags(a, l + 1)));
        if (l > 0) MCK(cudaMemsetAsync(flags(a, l), 0, a->n[l], st));
    }
    return COSMOS_OK;
}

struct Counts {
    int it = 0, fit = 0, mid_run = 0, fine_run = 0;
};

// Level-1 driver loop (AMR/EulerAMR.cpp:195-346).
int run_level1(cosmos_amr* a, double cfl, double t_final, double tol, int order, double* t_out, Counts* c) {
    cosmos_grid* C = a->level[0];
    cosmos_grid* F = a->level[1];
    const int prec = C->p.precision;
    const double dx = C->p.dx;
    double t = 0.0;
    int rc = COSMOS_OK;
    while (t < t_final) {
        double smax = 0.0;
        bool refined = false;
        // the coarse time step is taken before the flag pass (AMR/EulerAMR.cpp:197-198); both read
        // the same coarse state, so the flag pass is enqueued first and one read returns both
        MCK(launch_amr_flags(level_args(a, 0), prec, tol, flags(a, 0), flags(a, 1)));
        if ((rc = read_word(a, 0, 1, &smax, &refined))) break;
        const double dt = cosmos_stable_dt_rule(cfl * (dx / smax), t, t_final, c->fit);
        if ((rc = bad_dt(dt))) break;
        if ((rc = masked_step(C, order, dt, flags(a, 0)))) break;
        if (refined) {
            double ft = t;
            for (int sub = 0; ft < (t + dt - 1e-4); sub++) {
                double fs = 0.0;
                if ((rc = too_many(sub)) || (rc = read_word(a, 1, -1, &fs, nullptr))) break;
                const double fdt = cosmos_stable_dt_rule(cfl * ((dx * 0.5) / fs), ft, t + dt, c->fit);
                if ((rc = bad_dt(fdt))) break;
                if ((rc = masked_step(F, order, fdt, flags(a, 1)))) break;
                ft += fdt;
                c->fit += 1;
                c->fine_run += 1;
            }
            if (rc) break;
        } else {
            c->fit += 1;
        }
        t += dt;
        c->it += 1;
        // restriction and injection (AMR/EulerAMR.cpp:287-307), then derefinement (:309-345)
        SweepArgs sa = base_args(C);
        MCK(launch_amr_sync(sa, prec, state(a, 0), state(a, 1), F->G, flags(a, 0), flags(a, 1)));
        MCK(launch_amr_derefine(sa, prec, state(a, 1), F->G, tol, flags(a, 0), flags(a, 1), state(a, 0)));
    }
    *t_out = t;
    return rc;
}

// Level-2 driver loop (AMR/EulerAMR.cpp:638-914; 2D :973-1376): coarse flags with the Newtonian
// neighbours for both systems; intermediate steps while an intermediate flag is on, each with its
// own flag pass (tol * 2 * order, coarse spacing, cells that are on), fine sub-steps while a fine
// flag is on, the total fine count advancing per fine step (or once when none runs) and once more
// per intermediate step, then the strict exchange and derefinement (tol) between intermediate and
// fine; after the coarse step the exchange and derefinement (tol * 0.5 / order) between coarse and
// intermediate.
int run_level2(cosmos_amr* a, double cfl, double t_final, double tol, int order, double* t_out, Counts* c) {
    cosmos_grid* C = a->level[0];
    cosmos_grid* M = a->level[1];
    cosmos_grid* F = a->level[2];
    const int prec = C->p.precision;
    const double dx = C->p.dx;
    double t = 0.0;
    int rc = COSMOS_OK;
    while (t < t_final && !rc) {
        double smax = 0.0;
        bool refined = false;
        MCK(launch_amr_flags_ex(level_args(a, 0), prec, tol, dx, true, false, flags(a, 0), flags(a, 1)));
        if ((rc = read_word(a, 0, 1, &smax, &refined))) break;
        const double dt = cosmos_stable_dt_rule(cfl * (dx / smax), t, t_final, c->fit);
        if ((rc = bad_dt(dt))) break;
        if ((rc = masked_step(C, order, dt, flags(a, 0)))) break;
        if (refined) {
            double mt = t;
            for (int msub = 0; mt < (t + dt - 1e-4); msub++) {
                double ms = 0.0;
                bool refined2 = false;
                // the intermediate time step precedes its flag pass; both read the same state
                if ((rc = too_many(msub)) || (rc = read_word(a, 1, -1, &ms, nullptr))) break;
                const double mdt = cosmos_stable_dt_rule(cfl * ((dx * 0.5) / ms), mt, t + dt, c->fit);
                if ((rc = bad_dt(mdt))) break;
                MCK(launch_amr_flags_ex(level_args(a, 1), prec, tol * 2.0 * order, dx, true, true, flags(a, 1),
                                        flags(a, 2)));
                if ((rc = masked_step(M, order, mdt, flags(a, 1)))) break;
                MCK(cudaMemsetAsync(a->word + 1, 0, sizeof(unsigned long long), a->ctx->stream));
                MCK(launch_amr_any(flags(a, 2), a->n[2], a->word + 1, a->ctx->stream));
                MCK(cudaMemcpyAsync(a->host + 1, a->word + 1, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                    a->ctx->stream));
                MCK(cudaStreamSynchronize(a->ctx->stream));
                refined2 = a->host[1] != 0;
                if (refined2) {
                    double ft = mt;
                    for (int fsub = 0; ft < (mt + mdt - 1e-4); fsub++) {
                        double fs = 0.0;
                        if ((rc = too_many(fsub)) || (rc = read_word(a, 2, -1, &fs, nullptr))) break;
                        const double fdt = cosmos_stable_dt_rule(cfl * ((dx * 0.25) / fs), ft, mt + mdt, c->fit);
                        if ((rc = bad_dt(fdt))) break;
                        if ((rc = masked_step(F, order, fdt, flags(a, 2)))) break;
                        ft += fdt;
                        c->fit += 1;
                        c->fine_run += 1;
                    }
                    if (rc) break;
                } else {
                    c->fit += 1;
                }
                mt += mdt;
                c->fit += 1;
                c->mid_run += 1;
                SweepArgs ma = base_args(M);
                MCK(launch_amr_sync(ma, prec, state(a, 1), state(a, 2), F->G, flags(a, 1), flags(a, 2), true));
                MCK(launch_amr_derefine_ex(ma, prec, state(a, 2), F->G, tol, dx, true, flags(a, 1), flags(a, 2),
                                           state(a, 1)));
            }
            if (rc) break;
        } else {
            c->fit += 1;
        }
        t += dt;
        c->it += 1;
        SweepArgs sa = base_args(C);
        MCK(launch_amr_sync(sa, prec, state(a, 0), state(a, 1), M->G, flags(a, 0), flags(a, 1)));
        MCK(launch_amr_derefine_ex(sa, prec, state(a, 1), M->G, tol * 0.5 * (1.0 / order), dx, true, flags(a, 0),
                                   flags(a, 1), state(a, 0)));
    }
    *t_out = t;
    return rc;
}

}  // namespace

extern "C" {

int cosmos_amr_create(cosmos_ctx* ctx, const cosmos_params* p, cosmos_amr** out) { return create(ctx, p, 2, out); }

int cosmos_amr_create_level2(cosmos_ctx* ctx, const cosmos_params* p, cosmos_amr** out) {
    return create(ctx, p, 3, out);
}

int cosmos_amr_destroy(cosmos_amr* a) {
    if (!a) return COSMOS_OK;
    if (a->ctx) {
        cudaSetDevice(a->ctx->device);
        cudaStreamSynchronize(a->ctx->stream);
    }
    if (a->flags) cudaFree(a->flags);
    if (a->word) cudaFree(a->word);
    if (a->host) cudaFreeHost(a->host);
    for (int l = 0; l < 3; l++) cosmos_grid_destroy(a->level[l]);
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
    MCK(cudaSetDevice(a->ctx->device));
    cudaStream_t st = a->ctx->stream;
    for (int l = 0; l < a->nlev; l++) MCK(cudaMemsetAsync(a->level[l]->status, 0, sizeof(int), st));
    MRC(init_levels(a));
    Counts c;
    double t = 0.0;
    const int rc = a->nlev == 2 ? run_level1(a, cfl, t_final, tol, order, &t, &c)
                                : run_level2(a, cfl, t_final, tol, order, &t, &c);
    if (rc != COSMOS_OK && rc != COSMOS_ENONFINITE) return rc;
    int sts[3] = {0, 0, 0};
    for (int l = 0; l < a->nlev; l++)
        MCK(cudaMemcpyAsync(&sts[l], a->level[l]->status, sizeof(int), cudaMemcpyDeviceToHost, st));
    MCK(cudaStreamSynchronize(st));
    if (r) {
        r->coarse_steps = c.it;
        r->fine_steps = c.fit;
        r->t = t;
        r->status = sts[0] | sts[1] | sts[2] | (rc == COSMOS_ENONFINITE ? COSMOS_STATUS_NONFINITE : 0);
        r->fine_run = c.fine_run;
        r->mid_run = c.mid_run;
    }
    return rc;
}

int cosmos_amr_get_level(cosmos_amr* a, int level, double* prim, unsigned char* level_flags) {
    if (!a) return afail(COSMOS_EINVAL, "null AMR handle");
    if (level < 0 || level >= a->nlev) return afail(COSMOS_EINVAL, "level out of range");
    MCK(cudaSetDevice(a->ctx->device));
    if (prim) MRC(cosmos_grid_get_prim(a->level[level], prim, 5 * a->n[level]));
    if (level_flags) {
        MCK(cudaMemcpyAsync(level_flags, flags(a, level), a->n[level], cudaMemcpyDeviceToHost, a->ctx->stream));
        MCK(cudaStreamSynchronize(a->ctx->stream));
    }
    return COSMOS_OK;
}

int cosmos_amr_get(cosmos_amr* a, double* coarse_prim, double* fine_prim, unsigned char* coarse_flags,
                   unsigned char* fine_flags) {
    if (!a) return afail(COSMOS_EINVAL, "null AMR handle");
    MRC(cosmos_amr_get_level(a, 0, coarse_prim, coarse_flags));
    return cosmos_amr_get_level(a, a->nlev - 1, fine_prim, fine_flags);
}

}  // extern "C"
