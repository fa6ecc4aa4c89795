// C ABI of the hand-written adjoint: reverse-mode gradient of a final-density misfit through
// nsteps SLIC steps of a Newtonian grid (or an FP64 SR grid, or an FP64 black-hole grid with its RK
// source half-steps), with checkpoints every `checkpoint_every` steps.
//
// Forward: the grid's own steps (device dt from the CFL rule, or the caller's dts) with each
// step's dt logged.  The last segments -- as many as fit in the keep budget (cosmos_grid_set_
// adjoint_keep; by default half of the device memory free at the call, at least the last segment)
// -- run with every sweep's input written to a store of its own (same kernels and device time
// steps as the graph-replayed steps); the earlier ones run from the captured step graph with the
// state copied to a checkpoint store before each segment.
// Backward, segment by segment from the last: a kept segment's sweep inputs are in place; an
// earlier segment is recomputed from its checkpoint with the same sweep kernels and dts, keeping
// every sweep's input, on a second stream while the following segment's adjoints run.  The sweep
// adjoints run in reverse order (X(dt/2) Y(dt) X(dt/2) per 2D step, X(dt) per 1D step).  The
// gradient is the same bit for bit whatever the budget and the checkpoint interval.
#include <algorithm>
#include <climits>
#include <cstddef>
#include <cstring>
#include <string>
#include <vector>

#include "adjoint_kernels.cuh"
#include "capi_internal.h"

using namespace cg;

namespace {

int afail(int code, const std::string& msg) {
    set_error(msg.c_str());
    return code;
}
#define ACK(call)                                                                                    \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess) return afail(COSMOS_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// Device scratch of one adjoint call, released on every exit path.
struct Scratch {
    cudaStream_t st = nullptr;
    std::vector<void*> ptrs;
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    cudaEvent_t rec_done[2] = {nullptr, nullptr}, adj_done[2] = {nullptr, nullptr};
    StepCtl* patched = nullptr;  // controller whose dt pointers point into this scratch
    std::vector<cudaGraphExec_t> graphs;  // the kept segments' captured forward steps
    cudaError_t alloc(void** p, size_t bytes) {
        cudaError_t e = cudaMallocAsync(p, bytes, st);
        if (e == cudaSuccess) ptrs.push_back(*p);
        return e;
    }
    void unpatch() {
        if (!patched) return;
        // dt_log and dt_fixed are adjacent; a pageable source is staged before the call returns
        const double* nul[2] = {nullptr, nullptr};
        cudaMemcpyAsync((char*)patched + offsetof(StepCtl, dt_log), nul, sizeof nul, cudaMemcpyHostToDevice, st);
        patched = nullptr;
    }
    ~Scratch() {
        if (!graphs.empty()) {
            cudaStreamSynchronize(st);  // no captured segment is still running when it is destroyed
            for (cudaGraphExec_t x : graphs) cudaGraphExecDestroy(x);
        }
        unpatch();
        for (void* p : ptrs) cudaFreeAsync(p, st);
        for (auto& e : ev)
            if (e) cudaEventDestroy(e);
        for (int k = 0; k < 2; k++) {
            if (rec_done[k]) cudaEventDestroy(rec_done[k]);
            if (adj_done[k]) cudaEventDestroy(adj_done[k]);
        }
    }
};

}  // namespace

extern "C" int cosmos_grid_adjoint(cosmos_grid* g, const cosmos_solve_opts* o, int nsteps, int checkpoint_every,
                                   const double* target, const double* dts_in, double* grad_prim, double* loss,
                                   double* dts_out, double* ms) {
    if (!g || !o || !target || !grad_prim) return afail(COSMOS_EINVAL, "null grid, options, target or gradient");
    // SR and black-hole grids (FP64) run the relativistic adjoints on primitive adjoints; a black-hole
    // step is o->subcycles RK source half-steps, the flux sweeps, o->subcycles more
    const bool rel = g->p.system == COSMOS_SR || g->p.system == COSMOS_GR;
    if (rel && g->p.precision != COSMOS_FP64)
        return afail(COSMOS_EUNSUPPORTED, "the relativistic adjoints cover FP64 grids");
    if (rel && (g->G.nx < 2 || (g->p.dims == 2 && g->G.ny < 2)))
        return afail(COSMOS_EUNSUPPORTED, "the relativistic adjoints need at least two cells per swept line");
    if (o->order != 2) return afail(COSMOS_EUNSUPPORTED, "the adjoint covers SLIC (order 2)");
    if (g->p.system == COSMOS_GR && o->subcycles < 0) return afail(COSMOS_EINVAL, "subcycles must be >= 0");
    if (nsteps < 1 || checkpoint_every < 1) return afail(COSMOS_EINVAL, "nsteps and checkpoint_every must be >= 1");
    if (!dts_in && !(o->cfl > 0.0)) return afail(COSMOS_EINVAL, "cfl must be positive when no dts are given");
    if (dts_in)
        for (int s = 0; s < nsteps; s++)
            if (!(dts_in[s] > 0.0)) return afail(COSMOS_EINVAL, "dts_in[" + std::to_string(s) + "] is not positive");
    ACK(cudaSetDevice(g->ctx->device));
    const bool fp64 = g->p.precision == COSMOS_FP64;
    const Geom G0 = g->G;
    const size_t ncell = (size_t)G0.nx * G0.ny;
    const size_t sbytes = G0.fstride * 5 * g->elem;                         // one state, storage precision
    const size_t abytes = G0.fstride * 5 * (fp64 ? sizeof(double) : sizeof(float));  // one adjoint state
    const int K = std::min(checkpoint_every, nsteps);
    const int nck = (nsteps + K - 1) / K;
    // operations per step: the sweeps, and around them a black-hole grid's RK source half-steps
    const int nsw = g->p.dims == 2 ? 3 : 1;
    const int nsub = g->p.system == COSMOS_GR ? o->subcycles : 0;
    const int spp = nsw + 2 * nsub;
    Scratch sc;
    sc.st = g->ctx->stream;
    cudaStream_t st = sc.st;
    // segments c >= ckeep keep their sweep inputs from the forward pass; the others are recomputed
    const size_t seg_bytes = (size_t)K * spp * sbytes;
    long long budget = g->adj_keep;
    if (budget < 0) {
        size_t fr = 0, tot = 0;
        ACK(cudaMemGetInfo(&fr, &tot));
        budget = (long long)(fr / 2);
    }
    const int nkeep = (int)std::max<long long>(1, std::min<long long>(nck, budget / (long long)seg_bytes));
    const int ckeep = nck - nkeep;
    char *ck, *seg = nullptr, *keep, *adj;
    double *d_target, *d_dts, *d_rows, *d_loss;
    ACK(sc.alloc((void**)&ck, (size_t)std::max(ckeep, 1) * sbytes));  // checkpoints of the recomputed segments (and 0)
    if (ckeep > 0) ACK(sc.alloc((void**)&seg, 2 * seg_bytes));       // two segments: recompute one, reverse the other
    ACK(sc.alloc((void**)&keep, (size_t)nkeep * seg_bytes));
    ACK(sc.alloc((void**)&adj, 2 * abytes));
    ACK(sc.alloc((void**)&d_target, ncell * sizeof(double)));
    ACK(sc.alloc((void**)&d_dts, nsteps * sizeof(double)));
    ACK(sc.alloc((void**)&d_rows, (size_t)G0.ny * sizeof(double)));
    ACK(sc.alloc((void**)&d_loss, sizeof(double)));
    for (auto& e : sc.ev) ACK(cudaEventCreate(&e));
    for (int k = 0; k < 2; k++) {
        ACK(cudaEventCreateWithFlags(&sc.rec_done[k], cudaEventDisableTiming));
        ACK(cudaEventCreateWithFlags(&sc.adj_done[k], cudaEventDisableTiming));
    }
    ACK(cudaMemcpyAsync(d_target, target, ncell * sizeof(double), cudaMemcpyHostToDevice, st));
    if (dts_in) ACK(cudaMemcpyAsync(d_dts, dts_in, nsteps * sizeof(double), cudaMemcpyHostToDevice, st));

    // ---- forward with checkpoints
    ACK(cudaEventRecord(sc.ev[0], st));
    cosmos_solve_opts fo = *o;
    fo.t_final = 1e300;  // exactly nsteps steps
    fo.max_steps = nsteps;
    fo.subcycles = g->p.system == COSMOS_GR ? nsub : 1;
    if (dts_in) fo.cfl = 1.0;
    int rc = cosmos_grid_run_begin(g, &fo);
    if (rc) return rc;
    double* logp = dts_in ? nullptr : d_dts;
    const double* fixp = dts_in ? d_dts : nullptr;
    static_assert(offsetof(StepCtl, dt_fixed) == offsetof(StepCtl, dt_log) + sizeof(double*), "adjacent dt pointers");
    const void* dtp[2] = {logp, fixp};
    sc.patched = g->ctl;
    ACK(cudaMemcpyAsync((char*)g->ctl + offsetof(StepCtl, dt_log), dtp, sizeof dtp, cudaMemcpyHostToDevice, st));
    // input of operation q of segment c: the keep store, or the recomputation store's half c & 1
    auto slot = [&](int c, int q) {
        return c >= ckeep ? keep + (size_t)(c - ckeep) * seg_bytes + (size_t)q * sbytes
                          : seg + (size_t)(c & 1) * seg_bytes + (size_t)q * sbytes;
    };
    for (int c = 0; c < nck; c++) {
        const int ns = std::min(K, nsteps - c * K);
        if (c < ckeep) {
            ACK(cudaMemcpyAsync(ck + (size_t)c * sbytes, g->buf[g->cur], sbytes, cudaMemcpyDeviceToDevice, st));
            if ((rc = cosmos_grid_run_steps(g, ns))) return rc;
            continue;
        }
        // a kept segment: its first input is the grid's state (c == ckeep) or the previous kept
        // segment's last output; its own last output goes to the next segment, or for the last
        // segment to the grid's other buffer
        if (c == ckeep) ACK(cudaMemcpyAsync(slot(c, 0), g->buf[g->cur], sbytes, cudaMemcpyDeviceToDevice, st));
        if (c == 0) ACK(cudaMemcpyAsync(ck, slot(c, 0), sbytes, cudaMemcpyDeviceToDevice, st));  // the gradient's state
        // the segment's steps are captured into one graph and replayed once, so they run with the
        // launch gaps of the graph-replayed steps
        cudaGraph_t graph;
        ACK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        set_capturing(true);
        for (int s = 0; s < ns && !rc; s++) {
            std::vector<void*> outs(spp);
            for (int k = 0; k < spp; k++) {
                const int q = s * spp + k + 1;
                outs[k] = q < ns * spp ? (void*)slot(c, q) : (c + 1 < nck ? (void*)slot(c + 1, 0) : g->buf[g->cur ^ 1]);
            }
            rc = enqueue_step_into(g, slot(c, s * spp), outs.data());
        }
        set_capturing(false);
        const cudaError_t ec = cudaStreamEndCapture(st, &graph);
        if (ec == cudaSuccess && rc) cudaGraphDestroy(graph);
        if (rc) return rc;
        ACK(ec);
        cudaGraphExec_t exec;
        const cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        ACK(ei);
        sc.graphs.push_back(exec);
        ACK(cudaGraphLaunch(exec, st));
        // per step: the dt kernel, the operations, and a black-hole grid's CFL reduction
        count_launch((unsigned)(ns * (1 + spp + (g->p.system == COSMOS_GR ? 1 : 0))));
    }
    g->cur ^= 1;
    ACK(cudaEventRecord(sc.ev[1], st));
    sc.unpatch();  // the controller's dt pointers point into this call's scratch

    // ---- loss and its adjoint seed at the final state
    int cur = 0;
    ACK(fp64 ? launch_adjoint_loss_exact(G0, g->buf[g->cur], d_target, adj, d_rows, d_loss, st)
             : launch_adjoint_loss_fast(G0, g->buf[g->cur], d_target, adj, d_rows, d_loss, st));
    // The dts of the forward pass: a recomputation (and the relativistic adjoints) take them as
    // launch arguments, so the host waits for them here.  A Newtonian run that keeps every
    // segment reads its sweeps' coefficients from device memory instead, so its backward pass is
    // queued behind the forward pass with no wait; the forward's status is checked at the end.
    const bool devdt = !rel && ckeep == 0;
    std::vector<double> dts(nsteps);
    StepCtl h;
    AdjCoefs* d_coefs = nullptr;
    auto check_forward = [&]() -> int {
        ACK(cudaMemcpyAsync(dts.data(), d_dts, nsteps * sizeof(double), cudaMemcpyDeviceToHost, st));
        ACK(cudaMemcpyAsync(&h, g->ctl, sizeof h, cudaMemcpyDeviceToHost, st));
        ACK(cudaStreamSynchronize(st));
        if (h.status & ST_NONFINITE) return afail(COSMOS_ENONFINITE, "non-finite or non-positive time step in the forward run");
        if (h.it != nsteps) return afail(COSMOS_ESTATE, "the forward run stopped after " + std::to_string(h.it) + " steps");
        return COSMOS_OK;
    };
    if (devdt) {
        ACK(sc.alloc((void**)&d_coefs, (size_t)nsteps * nsw * sizeof(AdjCoefs)));
        ACK(launch_adjoint_coefs(d_dts, nsteps, nsw, g->p.dx, g->p.gamma, o->bias, d_coefs, st));
    } else if ((rc = check_forward())) {
        return rc;
    }

    // ---- backward, one checkpoint segment at a time
    SweepArgs fa = base_args(g);
    fa.order = 2;
    fa.bias = o->bias;
    fa.lim = o->limiter;
    fa.out.status = g->status;
    AdjSweepParams ap;
    ap.G = G0;
    ap.dx = g->p.dx;
    ap.bias = o->bias;
    ap.gamma = g->p.gamma;
    ap.coefp = nullptr;
    const double bh[5] = {g->p.bh_mass, g->p.bh_spin, g->p.bh_x, g->p.bh_y, g->p.bh_z};
    // The recomputation of segment c - 1 (forward sweeps, on the context's second stream) runs
    // while the sweep adjoints of segment c run on the compute stream; the two segments use
    // alternate halves of `seg`, and events order each half's writer and reader.
    cudaStream_t rs = g->ctx->copy;
    fa.stream = rs;
    for (int k = 0; k < 2; k++) ACK(cudaEventRecord(sc.adj_done[k], st));  // after the forward pass and the loss
    // operation q of segment c: its axis and dt; true for an RK source half-step (dt / (2 nsub))
    auto op_of = [&](int c, int q, int& axis, double& dt) -> bool {
        const double d = dts[c * K + q / spp];
        int m = q % spp;
        if (m < nsub || m >= nsub + nsw) {
            axis = 0;
            dt = 0.5 * (d / nsub);
            return true;
        }
        m -= nsub;
        axis = nsw == 3 && m == 1 ? 1 : 0;
        dt = nsw == 3 && m != 1 ? 0.5 * d : d;
        return false;
    };
    auto nops_of = [&](int c) { return (std::min(nsteps, c * K + K) - c * K) * spp; };
    auto recompute = [&](int c) -> int {
        ACK(cudaStreamWaitEvent(rs, sc.adj_done[c & 1], 0));  // this half's previous reader is done
        ACK(cudaMemcpyAsync(slot(c, 0), ck + (size_t)c * sbytes, sbytes, cudaMemcpyDeviceToDevice, rs));
        const int nops = nops_of(c);
        for (int q = 0; q + 1 < nops; q++) {  // the last operation's output is not needed
            int axis;
            double dt;
            if (op_of(c, q, axis, dt)) {  // RK source half-step: bias 0, limiter 1, as in the forward
                SweepArgs r = fa;
                r.bias = 0.0;
                r.lim = 1;
                r.ds.fixed = dt;
                r.src = slot(c, q);
                r.dst = slot(c, q + 1);
                ACK(launch_rk_source_exact(r));
                continue;
            }
            fa.G.axis = axis;
            fa.ds.fixed = dt;
            fa.ds.ffix = make_fast_coef(dt, g->p.dx);
            fa.src = slot(c, q);
            fa.dst = slot(c, q + 1);
            ACK(sweep_launch(g, fa));
        }
        ACK(cudaEventRecord(sc.rec_done[c & 1], rs));
        return COSMOS_OK;
    };
    // the sweep adjoints of segment c in reverse order, on `st`
    auto reverse = [&](int c) -> int {
        for (int q = nops_of(c) - 1; q >= 0; q--) {
            int axis;
            double dt = 0.0;
            if (devdt) {  // Newtonian: the sweeps only; coefficients from device memory
                const int m = q % spp;
                axis = nsw == 3 && m == 1 ? 1 : 0;
                ap.G.axis = axis;
                ap.coefp = d_coefs + (size_t)(c * K + q / spp) * nsw + m;
                ap.state = slot(c, q);
                ap.ubar_out = adj + (size_t)cur * abytes;
                ap.ubar_in = adj + (size_t)(cur ^ 1) * abytes;
                ACK(fp64 ? launch_adjoint_sweep_exact(ap, o->limiter, st) : launch_adjoint_sweep_fast(ap, o->limiter, st));
                cur ^= 1;
                continue;
            }
            if (op_of(c, q, axis, dt)) {
                ACK(launch_adjoint_rel_rk(G0, g->p.gamma, bh, g->p.dx, dt, slot(c, q), adj + (size_t)cur * abytes,
                                          adj + (size_t)(cur ^ 1) * abytes, st));
                cur ^= 1;
                continue;
            }
            ap.G.axis = axis;
            ap.dt = dt;
            {
                const AdjCoefs cs = adj_coefs(dt, g->p.dx, g->p.gamma, o->bias);
                ap.cd = cs.d;
                ap.cf = cs.f;
            }
            ap.state = slot(c, q);
            ap.ubar_out = adj + (size_t)cur * abytes;
            ap.ubar_in = adj + (size_t)(cur ^ 1) * abytes;
            if (rel)
                ACK(launch_adjoint_rel_sweep(ap.G, g->p.system, g->p.gamma, bh, g->p.dx, dt, o->bias, o->limiter, ap.state,
                                             ap.ubar_out, ap.ubar_in, st));
            else
                ACK(fp64 ? launch_adjoint_sweep_exact(ap, o->limiter, st) : launch_adjoint_sweep_fast(ap, o->limiter, st));
            cur ^= 1;
        }
        return COSMOS_OK;
    };
    for (int c = nck - 1; c >= 0; c--) {
        if (c > 0 && c - 1 < ckeep && (rc = recompute(c - 1))) return rc;
        if (c < ckeep) ACK(cudaStreamWaitEvent(st, sc.rec_done[c & 1], 0));
        if (c == nck - 1) {  // the first segment reversed launches at once (the device waits for it)
            if ((rc = reverse(c))) return rc;
            ACK(cudaEventRecord(sc.adj_done[c & 1], st));
            continue;
        }
        // later segments are captured into one graph each while the device runs the previous
        // ones, and replayed once: no launch gaps between their kernels beyond the graph's own
        cudaGraph_t graph;
        ACK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        set_capturing(true);
        rc = reverse(c);
        set_capturing(false);
        const cudaError_t ec = cudaStreamEndCapture(st, &graph);
        if (ec == cudaSuccess && rc) cudaGraphDestroy(graph);
        if (rc) return rc;
        ACK(ec);
        cudaGraphExec_t exec;
        const cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        ACK(ei);
        sc.graphs.push_back(exec);
        ACK(cudaGraphLaunch(exec, st));
        count_launch((unsigned)nops_of(c));
        ACK(cudaEventRecord(sc.adj_done[c & 1], st));
    }
    // ---- gradient with respect to the initial primitives
    if (rel)  // the relativistic sweep adjoints carry primitive adjoints already
        ACK(launch_adjoint_rel_grad(G0, adj + (size_t)cur * abytes, g->staging, st));
    else
        ACK(fp64 ? launch_adjoint_grad_exact(G0, g->p.gamma, ck, adj + (size_t)cur * abytes, g->staging, st)
                 : launch_adjoint_grad_fast(G0, g->p.gamma, ck, adj + (size_t)cur * abytes, g->staging, st));
    ACK(cudaEventRecord(sc.ev[2], st));
    if (devdt && (rc = check_forward())) return rc;  // the forward's dts and status, read only now
    ACK(cudaMemcpyAsync(grad_prim, g->staging, ncell * 5 * sizeof(double), cudaMemcpyDeviceToHost, st));
    double lv = 0.0;
    ACK(cudaMemcpyAsync(&lv, d_loss, sizeof lv, cudaMemcpyDeviceToHost, st));
    ACK(cudaStreamSynchronize(st));
    if (loss) *loss = lv;
    if (dts_out) std::copy(dts.begin(), dts.end(), dts_out);
    if (ms) {
        float f = 0.f, b = 0.f;
        ACK(cudaEventElapsedTime(&f, sc.ev[0], sc.ev[1]));
        ACK(cudaEventElapsedTime(&b, sc.ev[1], sc.ev[2]));
        ms[0] = f;
        ms[1] = b;
    }
    return COSMOS_OK;
}

extern "C" int cosmos_grid_set_adjoint_keep(cosmos_grid* g, long long bytes) {
    if (!g) return afail(COSMOS_EINVAL, "null grid");
    if (bytes < -1) return afail(COSMOS_EINVAL, "keep budget must be -1 (automatic) or a byte count");
    g->adj_keep = bytes;
    return COSMOS_OK;
}
