// Batched Newtonian SLIC for many independent grids of uneven sizes in ONE persistent launch.
//
// Every grid keeps its own step controller (t, dt, iteration, CFL maximum), exactly as if each
// were solved alone by the reference's solve / solve2D loop (Solvers/EulerSecondOrderSolver.cpp:
// 102-147); the grids only share the launch.  One launch runs `nsteps` steps; each step is four
// phases:
//   A  dt of every grid from its last CFL reduction (the reference's computeStableTimeStep);
//   B  the X sweep of every grid (full dt for 1D grids, dt/2 for 2D grids);
//   C  the Y sweep of every 2D grid (dt);
//   D  the second X sweep of every 2D grid (dt/2), with each grid's CFL reduction fused in.
// Work is a list of items per phase (X: a few rows of one grid, tiled; Y: a block of columns
// times a run of rows).  FP64: the items are dealt on the host, longest first, to the resident
// blocks so that their loads by cells swept are even, and grid-wide barriers separate the phases.
// FP32: the warps take the items as they become free and each item waits only for its own grid's
// earlier phase (per-grid counters; one barrier per launch).  Both need co-residency, so the launch
// is cooperative; every wait is bounded and reports a timeout instead of hanging.
#pragma once
#include "policies.cuh"
#include "sweep_pairs.cuh"

namespace cg {

struct BatchGrid {
    size_t off;   // element offset of the grid's state inside each pool buffer
    Geom G;       // geometry (axis field unused)
    double dx;
};

// One-cell tiles (FP64): X item rows [a, b) of grid g, each row in tiles of NT - 2 cells; Y item
// columns [a, a + NT) and rows [b, c) of grid g.  Cell pairs (FP32): X item the grid's 60-cell
// segments a .. b - 1, numbered row by row; Y item columns [a, a + 64) and rows [b, c).  Items
// hold several tiles so that the per-item set-up (descriptor loads, time step) and the CFL
// reduction are paid once per few thousand cells.
struct BatchItem { int g, a, b, c; };

// Most 60-cell segments in one FP32 X item (fewer when the batch gives each warp few items).
constexpr int kBatchXSegs = 64;

struct GridBarrier {
    unsigned int count;
    unsigned int gen;
    int err;
    int pad;
    long long limit;  // polls before a waiting block gives up (0: 2^26, about 4 s)
};

struct BatchDev {
    const BatchGrid* grids;
    StepCtl* ctl;
    int ngrids;
    const BatchItem* items[3];  // phases B, C, D: FP64 worker by worker, FP32 longest first
    const int* offs[3];         // FP64: worker w's items are items[offs[w]] .. items[offs[w + 1] - 1]
    int nitems[3];
    unsigned int* flow;         // FP32: the launch's dataflow counters (batch_flow_words)
    const int* gcount;          // FP32: items of grid g in phase ph at gcount[3 g + ph]
    void* buf[2];
    GridBarrier* bar;
    int* gstep;                 // steps completed by the batch (buffer parity)
    const CUtensorMap* maps;    // FP32: tensor map of buffer k's grid g at maps[k * ngrids + g] (null: per-field copies)
};

// dt of one step from the last CFL reduction (Solvers/EulerSolvers.cpp:130-161); the solver loop's
// `while (t < t_final)` becomes `active`.
CG_D void step_ctl_advance(StepCtl* c) {
    if (!(c->t < c->t_final) || c->it >= c->it_limit) {
        c->active = 0;
        c->dt = 0.0;
        return;
    }
    const double smax = __longlong_as_double((long long)c->smax[c->it & 1]);
    double dt = c->cfl * (c->dx / smax);
    if (c->it <= 5) dt = dt * 0.2;
    if ((c->t + dt) > c->t_final) dt = c->t_final - c->t;
    if (!(dt > 0.0) || !isfinite(dt)) c->status |= ST_NONFINITE;
    c->dt = dt;
    c->fc[0] = make_fast_coef(dt, c->dx);
    c->fc[1] = make_fast_coef(dt * 0.5, c->dx);
    c->active = 1;
    c->smax[(c->it + 1) & 1] = 0ull;
    c->t = c->t + dt;
    c->it = c->it + 1;
}

// Grid-wide barrier for a cooperative launch.  Waits are bounded (b->limit polls of about 64 ns,
// by default 2^26, about 4 s); a block that gives up sets err, and every block returns at its next
// barrier (a block that is last to arrive passes, sees err and returns too).
CG_D bool grid_sync(GridBarrier* b) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned int* vgen = &b->gen;
        volatile int* verr = &b->err;
        const unsigned int g = *vgen;
        __threadfence();
        int ok = 1;
        if (atomicAdd(&b->count, 1u) == gridDim.x - 1) {
            atomicExch(&b->count, 0u);
            __threadfence();
            atomicAdd(&b->gen, 1u);
        } else {
            const long long limit = b->limit > 0 ? b->limit : (1ll << 26);
            long long spins = 0;
            while (*vgen == g) {
                if (*verr) { ok = 0; break; }
                __nanosleep(64);
                if (++spins > limit) { atomicOr(&b->err, ST_TIMEOUT); ok = 0; break; }
            }
        }
        __threadfence();
        s_ok = ok && !*verr;
    }
    __syncthreads();
    return s_ok != 0;
}

// Policies specialised per grid (dims, nx, dx) for one work item.
template <class Pol>
CG_D void bind_grid(Pol& p, const BatchGrid& bg) {
    p.lm.nx = bg.G.nx;
    p.dims = bg.G.dims;
    if constexpr (Pol::kHasDx) p.dx = bg.dx;
}

// MINB: minimum resident blocks per SM requested from the compiler (1 = no register cap;
// 768 / NT caps registers near 80 so that more warps hide latency, at the price of a few spills).
template <class PolX, class PolY, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) batch_step_kernel(PolX polx0, PolY poly0, BatchDev B, int nsteps) {
    using X = typename PolX::X;
    using S = typename PolX::S;
    using W = typename PolX::W;
    __shared__ XTileSmem<X, NT> sm;
    __shared__ typename PolX::Coef s_cx;
    __shared__ typename PolY::Coef s_cy;
    __shared__ int s_act;
    const int step0 = *B.gstep;
    for (int s = 0; s < nsteps; s++) {
        const int p = (step0 + s) & 1;
        // ---- A: per-grid time steps
        for (int g = blockIdx.x * NT + threadIdx.x; g < B.ngrids; g += gridDim.x * NT) step_ctl_advance(&B.ctl[g]);
        if (!grid_sync(B.bar)) return;
        // ---- B, C, D
        for (int ph = 0; ph < 3; ph++) {
            // selects rather than indexing, so the descriptor stays in the parameter bank
            void* b0 = p ? B.buf[1] : B.buf[0];
            void* b1 = p ? B.buf[0] : B.buf[1];
            const S* src = (const S*)(ph == 1 ? b1 : b0);
            S* dst = (S*)(ph == 1 ? b0 : b1);
            const BatchItem* items = ph == 0 ? B.items[0] : (ph == 1 ? B.items[1] : B.items[2]);
            const int* offs = ph == 0 ? B.offs[0] : (ph == 1 ? B.offs[1] : B.offs[2]);
            const int k1 = offs[blockIdx.x + 1];
            for (int k = offs[blockIdx.x]; k < k1; k++) {
                const BatchItem it = items[k];
                const BatchGrid bg = B.grids[it.g];
                StepCtl* ctl = &B.ctl[it.g];
                const bool one_d = bg.G.dims == 1;
                DtSrc ds;
                ds.ctl = ctl;
                ds.fixed = 0.0;
                ds.nsub = 0;
                ds.scale = (ph == 1 || one_d) ? 1.0 : 0.5;
                ds.fsel = (ph == 1 || one_d) ? 0 : 1;
                SweepOut out;
                out.smax = nullptr;
                out.ws_ctl = nullptr;
                out.status = &ctl->status;
                out.mask = nullptr;
                // CFL reduction on the last sweep of the grid's step
                const bool ws = (ph == 0 && one_d) || ph == 2;
                __syncthreads();  // the previous item's shared memory (coefficients, reduction) is no longer read
                if (threadIdx.x == 0) {
                    double dt;
                    s_act = ds.get(dt);
                    if (s_act) {
                        if (ph == 1) s_cy = poly0.make_coef(ds, dt);
                        else s_cx = polx0.make_coef(ds, dt);
                    }
                }
                __syncthreads();
                const bool act = s_act != 0;
                W w = W(0);
                Geom G = bg.G;
                if (ph == 1) {
                    G.axis = 1;
                    PolY pol = poly0;
                    bind_grid(pol, bg);
                    if (act) pol.use_coef(s_cy);
                    w = y_march_seg<PolY, 2, NT>(pol, G, src + bg.off, dst + bg.off, it.a, it.b, it.c, act, out, ws);
                } else {
                    G.axis = 0;
                    PolX pol = polx0;
                    bind_grid(pol, bg);
                    if (act) pol.use_coef(s_cx);
                    for (int row = it.a; row < it.b; row++)
                        for (int s0 = 0; s0 < G.nx; s0 += NT - 2) {
                            const W wt = x_own_tile<PolX, 2, NT>(pol, G, src + bg.off, dst + bg.off, row, s0, act, out,
                                                                 ws, sm);
                            w = wt > w ? wt : w;
                        }
                }
                if (ws && act) block_max_to<NT>(&ctl->smax[ctl->it & 1], w);
            }
            if (!grid_sync(B.bar)) return;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *B.gstep = step0 + nsteps;
}

// Rows of each warp's Y ring in the FP32 batched launch, and the launch's dynamic shared memory
// (the rings and their mbarriers) for NT threads.
constexpr int kBatchRingRows = 8;
constexpr size_t batch_pair_smem(int nt) {
    return (size_t)(nt / 32) * kBatchRingRows * (5 * 64 * sizeof(float) + sizeof(unsigned long long));
}

// Counters of the FP32 batched launch's dataflow, cleared before every launch (words of flow[]):
//   [0] items taken; the launch's items are numbered step by step, in each step phase B's list,
//       then C's, then D's (each grid by grid, the grids by descending cost); [1] items finished;
//   [2 + 3 g + ph] items of grid g finished in phase ph, summed over the launch's steps;
//   [2 + 3 n + g] steps after the launch's first whose time step grid g has set (n = number of
//       grids; the first step's are set before the launch's one barrier).
CG_HD size_t batch_flow_words(int ngrids) { return 2 + 4 * (size_t)ngrids; }

// Lane 0 of a warp: wait until *c >= target, then order the warp's later reads after the writes
// that the counter's increments released (the caller follows with __syncwarp).  Polls are bounded
// as the grid barrier's; false when the wait ran out (err gets ST_TIMEOUT) or another warp
// reported an error.
CG_D bool flow_wait(const unsigned int* c, unsigned int target, GridBarrier* b) {
    const volatile unsigned int* vc = c;
    const volatile int* verr = &b->err;
    if (*vc < target) {
        const long long limit = b->limit > 0 ? b->limit : (1ll << 26);
        long long spins = 0;
        do {
            if (*verr) return false;
            if (++spins > limit) {
                atomicOr(&b->err, ST_TIMEOUT);
                return false;
            }
            __nanosleep(32);
        } while (*vc < target);
    }
    __threadfence();
    return true;
}

// FP32 batch on cell pairs (sweep_pairs.cuh), one warp per item, no barrier after the launch's
// first: the warps take the launch's items in order through an atomic counter (the next one is
// taken while an item runs), and an item waits only for the items of its own grid that it reads
// from or overwrites:
//   B (X sweep) of step s: the grid's time step for s is set -- at the launch's start for its
//     first step, else by the warp that finished the grid's last item of step s - 1;
//   C (Y sweep): the grid's B items of step s are finished;
//   D (X sweep with the CFL reduction): the grid's C items of step s are finished.
// Items are numbered step by step and phase by phase, so every item waits only for items taken
// before it by warps that are running: the launch cannot stall (and every wait is bounded).  Within
// a phase the items come grid by grid, so a grid's items of one phase finish early in it and the
// next phase's items of that grid rarely wait.  The last finisher of a grid's step (D; B for a 1D grid) computes the grid's next time
// step.  X items are runs of 60-cell segments of one grid (the next segment loaded while the
// current one is computed); Y items are 64 columns (a pair per lane) x a run of rows, marched
// through the warp's ring of rows staged by one tensor-map copy per row (y_ring_march; the grid's
// map of the source buffer), its barriers initialised again before each item.  Each warp reads its
// item's time step and reduces its own CFL maximum.  A wait that runs out sets ST_TIMEOUT in the
// barrier's error word and the warps leave at their next wait.
template <int LIM, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) batch_pair_kernel(NewtonFastParams P, BatchDev B, int nsteps) {
    constexpr int W = NT / 32;
    constexpr int TSW = 60;
    constexpr int R = kBatchRingRows;
    constexpr unsigned FULL = 0xffffffffu;
    extern __shared__ __align__(128) unsigned char batch_smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float(*ring)[R][5][64] = reinterpret_cast<float(*)[R][5][64]>(batch_smem);
    unsigned long long* rbar = reinterpret_cast<unsigned long long*>(batch_smem + W * sizeof(float[R][5][64]));
    unsigned long long* wbar = rbar + warp * R;
    ring_init<R>(wbar, false);
    bool ring_ok = true;     // warp-uniform
    bool ring_used = false;  // warp-uniform: the ring's barriers have been used since their initialisation
    const int step0 = *B.gstep;
    const int n = B.ngrids;
    unsigned int* done = B.flow + 2;
    unsigned int* ready = B.flow + 2 + 3 * (size_t)n;
    // the time steps of the launch's first step, then the one barrier
    for (int g = blockIdx.x * NT + threadIdx.x; g < n; g += gridDim.x * NT) step_ctl_advance(&B.ctl[g]);
    if (!grid_sync(B.bar)) return;
    const int nb = B.nitems[0], nc = B.nitems[1];
    const int per_step = nb + nc + B.nitems[2];
    const int total = nsteps * per_step;
    int k = __shfl_sync(FULL, lane == 0 ? (int)atomicAdd(&B.flow[0], 1u) : 0, 0);
    while (k < total) {  // warp-uniform
        const int kn_own = lane == 0 ? (int)atomicAdd(&B.flow[0], 1u) : 0;
        const int s = k / per_step;
        int r = k - s * per_step;
        const int ph = r < nb ? 0 : (r < nb + nc ? 1 : 2);
        r -= ph == 0 ? 0 : (ph == 1 ? nb : nb + nc);
        const BatchItem it = (ph == 0 ? B.items[0] : (ph == 1 ? B.items[1] : B.items[2]))[r];
        const BatchGrid bg = B.grids[it.g];
        StepCtl* ctl = &B.ctl[it.g];
        const bool one_d = bg.G.dims == 1;
        // the items this one depends on
        int ok = 1;
        if (lane == 0) {
            if (ph == 0) {
                if (s > 0) ok = flow_wait(&ready[it.g], (unsigned)s, B.bar);
            } else {
                const unsigned need = (unsigned)(s + 1) * (unsigned)B.gcount[3 * it.g + ph - 1];
                ok = flow_wait(&done[3 * it.g + ph - 1], need, B.bar);
            }
        }
        if (!__shfl_sync(FULL, ok, 0)) return;
        __syncwarp();
        const int p = (step0 + s) & 1;
        void* b0 = p ? B.buf[1] : B.buf[0];
        void* b1 = p ? B.buf[0] : B.buf[1];
        const float* src = (const float*)(ph == 1 ? b1 : b0);
        float* dst = (float*)(ph == 1 ? b0 : b1);
        DtSrc ds;
        ds.ctl = ctl;
        ds.fixed = 0.0;
        ds.nsub = 0;
        ds.scale = (ph == 1 || one_d) ? 1.0 : 0.5;
        ds.fsel = (ph == 1 || one_d) ? 0 : 1;
        const bool ws = (ph == 0 && one_d) || ph == 2;
        int act = 0;
        FastCoef cf{0.0f, 0.0f, 0.0f};
        if (lane == 0) {
            double dt;
            act = ds.get(dt);
            if (act) cf = ds.fast_coef();
        }
        act = __shfl_sync(FULL, act, 0);
        cf.dtdx = __shfl_sync(FULL, cf.dtdx, 0);
        cf.half_dtdx = __shfl_sync(FULL, cf.half_dtdx, 0);
        cf.q_dxdt = __shfl_sync(FULL, cf.q_dxdt, 0);
        const Geom& G = bg.G;
        const float* sg = src + bg.off;
        float* dg = dst + bg.off;
        float w = 0.0f;
        if (ph == 1) {
            if (!act) {
                const int j = it.a + 2 * lane;
                if (j < G.nx) y_pair_march<LIM>(P, G.dims, G, sg, dg, j, it.b, it.c, false, cf, false);
            } else if (ring_ok) {
                if (ring_used) ring_init<R>(wbar, true);
                ring_used = true;
                // the Y phase never reduces the CFL maximum (the last X sweep does)
                const CUtensorMap* tm = B.maps ? B.maps + (size_t)(p ? 0 : 1) * n + it.g : nullptr;
                y_ring_march<LIM, R, 2>(P, G.dims, G, sg, dg, it.a, it.b, it.c, cf, false, ring[warp], wbar,
                                        ring_ok, tm);
                if (!ring_ok) {
                    if (lane == 0) {
                        atomicOr(&ctl->status, ST_TIMEOUT);
                        atomicOr(&B.bar->err, ST_TIMEOUT);
                    }
                    return;
                }
            }
        } else {
            const int spr = (G.nx + TSW - 1) / TSW;
            Cell2 ahead;
            x_pair_load(G, sg, it.a / spr, (it.a % spr) * TSW, ahead);
            for (int q = it.a; q < it.b; q++) {
                const Cell2 m = ahead;
                if (q + 1 < it.b) x_pair_load(G, sg, (q + 1) / spr, ((q + 1) % spr) * TSW, ahead);
                w = fmaxf(w, x_pair_update<LIM>(P, G.dims, G, dg, q / spr, (q % spr) * TSW, m, act, cf, ws));
            }
        }
        if (ws && act) {
            w = warp_max(w);
            if (lane == 0) atomic_max_nonneg(&ctl->smax[ctl->it & 1], (double)w);
        }
        // publish the item: every lane's stores (and the CFL maximum) before the counter
        __threadfence();
        __syncwarp();
        if (lane == 0) {
            const unsigned fin = atomicAdd(&done[3 * it.g + ph], 1u) + 1u;
            const bool last_phase = ph == 2 || one_d;
            if (last_phase && s + 1 < nsteps && fin == (unsigned)(s + 1) * (unsigned)B.gcount[3 * it.g + ph]) {
                // every item of the grid's step is finished: its next time step
                __threadfence();
                step_ctl_advance(ctl);
                __threadfence();
                atomicExch(&ready[it.g], (unsigned)(s + 1));
            }
            if (atomicAdd(&B.flow[1], 1u) + 1u == (unsigned)total) *B.gstep = step0 + nsteps;
        }
        k = __shfl_sync(FULL, kn_own, 0);
    }
}

}  // namespace cg
