// C ABI of the batched persistent launch: many independent Newtonian grids of uneven sizes,
// advanced together by one cooperative kernel launch per chunk of steps (replayed from a CUDA
// graph), with the tile shape picked by an autotuner.
#include <algorithm>
#include <climits>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <queue>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/cosmos_gb300.h"
#include "batch_kernels.cuh"
#include "capi_internal.h"

namespace cg {
void* batch_fast_fn(int nt, int cap, int lim);
size_t batch_fast_smem(int nt);
void* batch_exact_fn(int nt, int cap);
}  // namespace cg

using namespace cg;

namespace {

int bfail(int code, const std::string& msg) {
    set_error(msg.c_str());
    return code;
}
#define BCK(call)                                                                                      \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess) return bfail(COSMOS_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

size_t rup(size_t v, size_t a) { return (v + a - 1) / a * a; }

}  // namespace

struct cosmos_batch {
    cosmos_ctx* ctx;
    int device;
    cudaStream_t stream;
    int precision;
    int boundary;
    double gamma;
    std::vector<BatchGrid> grids;  // host copy
    size_t pool_elems;
    size_t elem;
    void* buf[2];
    BatchGrid* d_grids;
    StepCtl* d_ctl;
    GridBarrier* d_bar;
    int* d_gstep;
    unsigned int* d_flow;  // FP32: the launch's dataflow counters, cleared before every launch
    int* d_gcount;         // FP32: items per grid and phase for the current tile shape
    CUtensorMap* d_maps;   // FP32: per buffer and 2D grid, the Y items' tensor maps (null: per-field copies)
    double* d_staging;
    size_t max_cells;
    // work lists for the current tile shape
    int nt, seg, cap, blocks;
    BatchItem* d_items[3];  // per phase, worker by worker
    int* d_offs[3];         // per phase: worker w's items are d_items[off[w] .. off[w + 1] - 1]
    int nitems[3];
    // run state
    cosmos_solve_opts run;
    bool run_ready;
    long long steps_done;  // steps completed since creation (buffer parity)
    int chunk;
    cudaGraphExec_t graph;
    bool graph_ok;
    long long wait_limit;  // grid-barrier polls before a wait gives up (0: the default)
    GridBarrier h_bar;     // staging for the barrier's initial state
};

namespace {

BatchDev dev_desc(cosmos_batch* b) {
    BatchDev B;
    B.grids = b->d_grids;
    B.ctl = b->d_ctl;
    B.ngrids = (int)b->grids.size();
    for (int k = 0; k < 3; k++) {
        B.items[k] = b->d_items[k];
        B.offs[k] = b->d_offs[k];
        B.nitems[k] = b->nitems[k];
    }
    B.buf[0] = b->buf[0];
    B.buf[1] = b->buf[1];
    B.bar = b->d_bar;
    B.gstep = b->d_gstep;
    B.flow = b->d_flow;
    B.gcount = b->d_gcount;
    B.maps = b->d_maps;
    return B;
}

void* kernel_fn(cosmos_batch* b, int nt, int seg, int cap, int lim) {
    if (seg < 1) return nullptr;
    return b->precision == COSMOS_FP32 ? batch_fast_fn(nt, cap, lim) : batch_exact_fn(nt, cap);
}

// Work lists for a tile shape, one per phase.  FP64 (one-cell tiles, one block per item): X items
// are whole rows of one grid, as many as make about 8 tiles of nt - 2 cells; Y items nt columns x
// seg rows.  FP32 (cell pairs, one warp per item): X items are runs of up to kBatchXSegs 60-cell
// segments of one grid, numbered row by row (a = first, b = one past the last); Y items 64 columns
// x seg rows.
// Costs are cells swept (Y counting its four halo rows) plus a per-item overhead.  FP32: the warps
// take the items as they become free (one atomic counter over the launch's steps and phases), grid
// by grid, the grids by descending cost.  FP64: sorted longest item first, each item is dealt onto
// the least-loaded resident block, and block w's items are stored at off[w] .. off[w + 1] - 1.
int build_items(cosmos_batch* b, int nt, int seg, int cap) {
    void* fn = kernel_fn(b, nt, seg, cap, b->run.limiter);
    if (!fn) return bfail(COSMOS_EUNSUPPORTED, "batch tile shape not provided for this precision");
    int per_sm = 0, sms = 0;
    const size_t smem = b->precision == COSMOS_FP32 ? batch_fast_smem(nt) : 0;
    BCK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, nt, smem));
    BCK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device));
    if (per_sm < 1) return bfail(COSMOS_EUNSUPPORTED, "batch kernel does not fit on an SM");
    const bool pairs = b->precision == COSMOS_FP32;
    const int blocks = per_sm * sms;
    const int workers = blocks;  // FP64 deal
    struct Costed { long long cost; BatchItem it; };
    std::vector<Costed> ph[3];
    std::vector<int> gcount(3 * b->grids.size(), 0);  // FP32: items per grid and phase
    const long long overhead = 32;
    // FP32 X items: about four per warp in a phase, 8 to kBatchXSegs segments.  An item waits for
    // its grid's previous phase, so a grid's phase takes at least one item's time: with few
    // items per warp, long items set the step's critical path (16 grids: 0.675 ms per step with
    // 64-segment items, 0.188 with 8; 64 grids: 0.928 and 0.485 ms), with many (256 grids) short
    // items only add set-up (64 segments: 1.575 ms, 16: 1.647).
    int xsegs = kBatchXSegs;
    if (pairs) {
        long long segs = 0;
        for (const BatchGrid& bg : b->grids) segs += (long long)((bg.G.nx + 59) / 60) * bg.G.ny;
        const long long per = 4ll * blocks * (nt / 32);
        xsegs = (int)std::max<long long>(8, std::min<long long>(kBatchXSegs, (segs + per - 1) / per));
    }
    for (int g = 0; g < (int)b->grids.size(); g++) {
        const Geom& G = b->grids[g].G;
        if (pairs) {
            const int spr = (G.nx + 59) / 60, total = spr * G.ny;
            for (int q = 0; q < total; q += xsegs) {
                const BatchItem it{g, q, std::min(q + xsegs, total), 0};
                const long long c = 64ll * (it.b - it.a) + overhead;
                ph[0].push_back({c, it});
                if (G.dims == 2) ph[2].push_back({c, it});
            }
            if (G.dims == 2)
                for (int j0 = 0; j0 < G.nx; j0 += 64)
                    for (int y0 = 0; y0 < G.ny; y0 += seg) {
                        const int y1 = std::min(y0 + seg, G.ny);
                        ph[1].push_back({64ll * (y1 - y0 + 4) + overhead, BatchItem{g, j0, y0, y1}});
                    }
        } else {
            const int tiles = (G.nx + nt - 3) / (nt - 2);
            const int rows = std::max(1, 8 / tiles);
            for (int r = 0; r < G.ny; r += rows) {
                const BatchItem it{g, r, std::min(r + rows, G.ny), 0};
                const long long c = (long long)nt * tiles * (it.b - it.a) + overhead;
                ph[0].push_back({c, it});
                if (G.dims == 2) ph[2].push_back({c, it});
            }
            if (G.dims == 2)
                for (int j0 = 0; j0 < G.nx; j0 += nt)
                    for (int y0 = 0; y0 < G.ny; y0 += seg) {
                        const int y1 = std::min(y0 + seg, G.ny);
                        ph[1].push_back({(long long)nt * (y1 - y0 + 4) + overhead, BatchItem{g, j0, y0, y1}});
                    }
        }
    }
    for (int k = 0; k < 3; k++) {
        if (b->d_items[k]) cudaFree(b->d_items[k]);
        if (b->d_offs[k]) cudaFree(b->d_offs[k]);
        b->d_items[k] = nullptr;
        b->d_offs[k] = nullptr;
        b->nitems[k] = (int)ph[k].size();
        if (pairs) {
            // FP32: grids by descending cost in the phase, each grid's items together in building
            // order.  An item waits for its grid's previous phase, so a grid's items finish early
            // in their phase and the next phase's items of the same grid find them done; sorted
            // item by item instead (longest first), every grid's short last item sat at the
            // phase's end and the next phase waited for it (1.80 against 1.58 ms per step of the
            // 256-grid batch).
            std::vector<long long> gc(b->grids.size(), 0);
            for (const Costed& c : ph[k]) gc[c.it.g] += c.cost;
            std::stable_sort(ph[k].begin(), ph[k].end(), [&](const Costed& x, const Costed& y) {
                return gc[x.it.g] != gc[y.it.g] ? gc[x.it.g] > gc[y.it.g] : x.it.g < y.it.g;
            });
            std::vector<BatchItem> flat;
            flat.reserve(ph[k].size());
            for (const Costed& c : ph[k]) {
                flat.push_back(c.it);
                gcount[3 * (size_t)c.it.g + k]++;
            }
            if (flat.empty()) continue;
            BCK(cudaMalloc(&b->d_items[k], flat.size() * sizeof(BatchItem)));
            BCK(cudaMemcpy(b->d_items[k], flat.data(), flat.size() * sizeof(BatchItem), cudaMemcpyHostToDevice));
            continue;
        }
        // longest processing time first (ties: the building order)
        std::stable_sort(ph[k].begin(), ph[k].end(), [](const Costed& x, const Costed& y) { return x.cost > y.cost; });
        // FP64: each item onto the least-loaded block (ties: the lower index)
        using Load = std::pair<long long, int>;
        std::priority_queue<Load, std::vector<Load>, std::greater<Load>> pq;
        for (int w = 0; w < workers; w++) pq.push({0ll, w});
        std::vector<std::vector<BatchItem>> per(workers);
        for (const Costed& c : ph[k]) {
            Load l = pq.top();
            pq.pop();
            per[l.second].push_back(c.it);
            pq.push({l.first + c.cost, l.second});
        }
        std::vector<BatchItem> flat;
        std::vector<int> off(workers + 1, 0);
        flat.reserve(ph[k].size());
        for (int w = 0; w < workers; w++) {
            flat.insert(flat.end(), per[w].begin(), per[w].end());
            off[w + 1] = (int)flat.size();
        }
        BCK(cudaMalloc(&b->d_offs[k], off.size() * sizeof(int)));
        BCK(cudaMemcpy(b->d_offs[k], off.data(), off.size() * sizeof(int), cudaMemcpyHostToDevice));
        if (flat.empty()) continue;
        BCK(cudaMalloc(&b->d_items[k], flat.size() * sizeof(BatchItem)));
        BCK(cudaMemcpy(b->d_items[k], flat.data(), flat.size() * sizeof(BatchItem), cudaMemcpyHostToDevice));
    }
    if (pairs)
        BCK(cudaMemcpy(b->d_gcount, gcount.data(), gcount.size() * sizeof(int), cudaMemcpyHostToDevice));
    b->nt = nt;
    b->seg = seg;
    b->cap = cap;
    b->blocks = blocks;
    return COSMOS_OK;
}

cudaError_t launch_chunk(cosmos_batch* b, int nsteps) {
    if (b->precision == COSMOS_FP32) {  // the dataflow counters start at zero in every launch
        const cudaError_t e =
            cudaMemsetAsync(b->d_flow, 0, batch_flow_words((int)b->grids.size()) * sizeof(unsigned int), b->stream);
        if (e != cudaSuccess) return e;
    }
    BatchDev B = dev_desc(b);
    BatchLaunch L;
    L.B = &B;
    L.nsteps = nsteps;
    L.nt = b->nt;
    L.seg = b->seg;
    L.cap = b->cap;
    L.lim = b->run.limiter;
    L.gamma = b->gamma;
    L.bias = b->run.bias;
    L.blocks = b->blocks;
    L.stream = b->stream;
    return b->precision == COSMOS_FP32 ? launch_batch_fast(L) : launch_batch_exact(L);
}

// Controllers reset (t = 0, iteration 0) and the initial CFL reduction of every grid.
int reset_controllers(cosmos_batch* b) {
    const int n = (int)b->grids.size();
    std::vector<StepCtl> h(n);
    for (int g = 0; g < n; g++) {
        memset(&h[g], 0, sizeof(StepCtl));
        h[g].t_final = b->run.t_final;
        h[g].cfl = b->run.cfl;
        h[g].dx = b->grids[g].dx;
        h[g].it_limit = b->run.max_steps < 0 ? INT_MAX : b->run.max_steps;
        h[g].active = 1;
    }
    BCK(cudaMemcpyAsync(b->d_ctl, h.data(), n * sizeof(StepCtl), cudaMemcpyHostToDevice, b->stream));
    {
        // the barrier's counters start at zero; its wait limit comes from cosmos_batch_set_wait_limit
        static_assert(sizeof(GridBarrier) == 24, "barrier layout");
        GridBarrier* hb = &b->h_bar;
        memset(hb, 0, sizeof *hb);
        hb->limit = b->wait_limit;
        BCK(cudaMemcpyAsync(b->d_bar, hb, sizeof *hb, cudaMemcpyHostToDevice, b->stream));
        BCK(cudaStreamSynchronize(b->stream));  // hb is host memory read by the copy
    }
    const int cur = (int)(b->steps_done & 1);
    for (int g = 0; g < n; g++) {
        SweepArgs a;
        memset(&a, 0, sizeof a);
        a.system = COSMOS_NEWTONIAN;
        a.G = b->grids[g].G;
        a.dx = b->grids[g].dx;
        a.gamma = b->gamma;
        a.stream = b->stream;
        a.src = (const char*)b->buf[cur] + b->grids[g].off * b->elem;
        unsigned long long* slot = &b->d_ctl[g].smax[0];
        BCK(b->precision == COSMOS_FP32 ? launch_wavespeed_fast(a, slot) : launch_wavespeed_exact(a, slot));
    }
    return COSMOS_OK;
}

int capture_graph(cosmos_batch* b) {
    if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
    b->graph_ok = false;
    cudaGraph_t gr;
    if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return COSMOS_OK;
    set_capturing(true);
    cudaError_t el = launch_chunk(b, b->chunk);
    set_capturing(false);
    cudaError_t ec = cudaStreamEndCapture(b->stream, &gr);
    if (el == cudaSuccess && ec == cudaSuccess) {
        if (cudaGraphInstantiate(&b->graph, gr, 0) == cudaSuccess) b->graph_ok = true;
        cudaGraphDestroy(gr);
    }
    cudaGetLastError();  // a refused capture leaves direct launches as the fallback
    return COSMOS_OK;
}

int set_shape(cosmos_batch* b, int nt, int seg, int cap) {
    int rc = build_items(b, nt, seg, cap);
    if (rc) return rc;
    return capture_graph(b);
}

}  // namespace

extern "C" {

int cosmos_batch_create(cosmos_ctx* ctx, int ngrids, const int* dims, const int* nx, const int* ny, const double* dx,
                        double gamma, int boundary, int precision, cosmos_batch** out) {
    if (!ctx || !dims || !nx || !ny || !dx || !out || ngrids < 1) return bfail(COSMOS_EINVAL, "null argument or no grids");
    if (precision != COSMOS_FP32 && precision != COSMOS_FP64) return bfail(COSMOS_EINVAL, "precision must be FP32 or FP64");
    if (boundary != COSMOS_BC_TRANSMISSIVE && boundary != COSMOS_BC_PERIODIC) return bfail(COSMOS_EINVAL, "unknown boundary");
    if (!(gamma > 1.0)) return bfail(COSMOS_EINVAL, "gamma must exceed 1");
    for (int g = 0; g < ngrids; g++)
        if ((dims[g] != 1 && dims[g] != 2) || nx[g] < 2 || (dims[g] == 2 && ny[g] < 2) || !(dx[g] > 0.0))
            return bfail(COSMOS_EINVAL, "grid " + std::to_string(g) + ": need dims 1 or 2, at least 2 cells per dimension, dx > 0");
    cudaStream_t st = (cudaStream_t)cosmos_ctx_stream(ctx);
    int dev = 0;
    BCK(cudaGetDevice(&dev));
    cosmos_batch* b = new cosmos_batch();
    b->ctx = ctx;
    ctx_retain(ctx);
    b->device = dev;
    b->stream = st;
    b->precision = precision;
    b->boundary = boundary;
    b->gamma = gamma;
    b->elem = precision == COSMOS_FP32 ? sizeof(float) : sizeof(double);
    b->chunk = 10;
    size_t off = 0, maxc = 0;
    for (int g = 0; g < ngrids; g++) {
        BatchGrid bg;
        bg.G.nx = nx[g];
        bg.G.ny = dims[g] == 1 ? 1 : ny[g];
        bg.G.pitch = (int)rup((size_t)nx[g], 32);
        bg.G.dims = dims[g];
        bg.G.axis = 0;
        bg.G.bc = boundary;
        bg.G.fstride = rup((size_t)bg.G.pitch * bg.G.ny, 32);
        bg.off = off;
        bg.dx = dx[g];
        off += rup(bg.G.fstride * 5, 64);
        maxc = std::max(maxc, (size_t)bg.G.nx * bg.G.ny);
        b->grids.push_back(bg);
    }
    b->pool_elems = off;
    b->max_cells = maxc;
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < 2 && e == cudaSuccess; k++) e = cudaMalloc(&b->buf[k], off * b->elem);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_grids, ngrids * sizeof(BatchGrid));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_ctl, ngrids * sizeof(StepCtl));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_bar, sizeof(GridBarrier));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_gstep, sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_flow, batch_flow_words(ngrids) * sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_gcount, 3 * (size_t)ngrids * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_staging, maxc * 5 * sizeof(double));
    if (e == cudaSuccess) e = cudaMemcpy(b->d_grids, b->grids.data(), ngrids * sizeof(BatchGrid), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(b->d_gstep, 0, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(b->d_bar, 0, sizeof(GridBarrier));
    if (e == cudaSuccess) e = cudaMemset(b->d_ctl, 0, ngrids * sizeof(StepCtl));
    for (int k = 0; k < 2 && e == cudaSuccess; k++) e = cudaMemset(b->buf[k], 0, off * b->elem);
    if (e == cudaSuccess && precision == COSMOS_FP32) {  // the Y items' rows: one tensor-map copy each
        std::vector<CUtensorMap> maps(2 * (size_t)ngrids);
        bool ok = true;
        for (int k = 0; k < 2; k++)
            for (int g = 0; g < ngrids; g++)
                if (b->grids[g].G.dims == 2)
                    ok = ok && field_map(&maps[(size_t)k * ngrids + g], (const float*)b->buf[k] + b->grids[g].off,
                                         b->grids[g].G, 64);
        if (ok) {
            e = cudaMalloc(&b->d_maps, maps.size() * sizeof(CUtensorMap));
            if (e == cudaSuccess)
                e = cudaMemcpy(b->d_maps, maps.data(), maps.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice);
        }
    }
    if (e != cudaSuccess) {
        std::string msg = std::string("batch allocation: ") + cudaGetErrorString(e);
        cosmos_batch_destroy(b);
        return bfail(COSMOS_ECUDA, msg);
    }
    b->nt = 128;
    b->seg = 16;
    b->cap = 0;
    b->run.limiter = COSMOS_MINBEE;
    *out = b;
    return COSMOS_OK;
}

int cosmos_batch_destroy(cosmos_batch* b) {
    if (!b) return COSMOS_OK;
    cudaStreamSynchronize(b->stream);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    for (int k = 0; k < 2; k++) if (b->buf[k]) cudaFree(b->buf[k]);
    if (b->d_maps) cudaFree(b->d_maps);
    for (int k = 0; k < 3; k++) {
        if (b->d_items[k]) cudaFree(b->d_items[k]);
        if (b->d_offs[k]) cudaFree(b->d_offs[k]);
    }
    if (b->d_grids) cudaFree(b->d_grids);
    if (b->d_ctl) cudaFree(b->d_ctl);
    if (b->d_bar) cudaFree(b->d_bar);
    if (b->d_gstep) cudaFree(b->d_gstep);
    if (b->d_flow) cudaFree(b->d_flow);
    if (b->d_gcount) cudaFree(b->d_gcount);
    if (b->d_staging) cudaFree(b->d_staging);
    cosmos_ctx* ctx = b->ctx;
    delete b;
    ctx_release(ctx);
    return COSMOS_OK;
}

int cosmos_batch_size(cosmos_batch* b, int* ngrids, long long* cells) {
    if (!b) return bfail(COSMOS_EINVAL, "null batch");
    long long c = 0;
    for (auto& g : b->grids) c += (long long)g.G.nx * g.G.ny;
    if (ngrids) *ngrids = (int)b->grids.size();
    if (cells) *cells = c;
    return COSMOS_OK;
}

static int batch_grid_args(cosmos_batch* b, int grid, size_t n, Geom& G, void** state) {
    if (!b || grid < 0 || grid >= (int)b->grids.size()) return bfail(COSMOS_EINVAL, "bad batch or grid index");
    G = b->grids[grid].G;
    if (n != (size_t)5 * G.nx * G.ny) return bfail(COSMOS_EINVAL, "buffer size does not match the grid");
    *state = (char*)b->buf[b->steps_done & 1] + b->grids[grid].off * b->elem;
    return COSMOS_OK;
}

int cosmos_batch_set_prim(cosmos_batch* b, int grid, const double* prim, size_t n) {
    Geom G;
    void* st;
    int rc = batch_grid_args(b, grid, n, G, &st);
    if (rc) return rc;
    if (!prim) return bfail(COSMOS_EINVAL, "null buffer");
    BCK(cudaMemcpyAsync(b->d_staging, prim, n * sizeof(double), cudaMemcpyHostToDevice, b->stream));
    if (b->precision == COSMOS_FP32) BCK(launch_prim_in_fast(b->d_staging, st, G, COSMOS_NEWTONIAN, b->gamma, b->stream));
    else BCK(launch_prim_in_exact(b->d_staging, st, G, b->stream));
    BCK(cudaStreamSynchronize(b->stream));  // the staging buffer is reused by the next call
    return COSMOS_OK;
}

int cosmos_batch_get_prim(cosmos_batch* b, int grid, double* prim, size_t n) {
    Geom G;
    void* st;
    int rc = batch_grid_args(b, grid, n, G, &st);
    if (rc) return rc;
    if (!prim) return bfail(COSMOS_EINVAL, "null buffer");
    if (b->precision == COSMOS_FP32) BCK(launch_prim_out_fast(st, b->d_staging, G, COSMOS_NEWTONIAN, b->gamma, b->stream));
    else BCK(launch_prim_out_exact(st, b->d_staging, G, b->stream));
    BCK(cudaMemcpyAsync(prim, b->d_staging, n * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    return COSMOS_OK;
}

int cosmos_batch_run_begin(cosmos_batch* b, const cosmos_solve_opts* o) {
    if (!b || !o) return bfail(COSMOS_EINVAL, "null argument");
    if (o->order != 2) return bfail(COSMOS_EUNSUPPORTED, "the batched launch runs SLIC (order 2)");
    if (!(o->cfl > 0.0)) return bfail(COSMOS_EINVAL, "cfl must be positive");
    const bool reshape = !b->run_ready || b->run.limiter != o->limiter || b->run.bias != o->bias;
    b->run = *o;
    int rc = reset_controllers(b);
    if (rc) return rc;
    if (reshape || !b->d_items[0]) {
        if ((rc = set_shape(b, b->nt, b->seg, b->cap))) return rc;
    }
    b->run_ready = true;
    return COSMOS_OK;
}

int cosmos_batch_run_steps(cosmos_batch* b, int n) {
    if (!b) return bfail(COSMOS_EINVAL, "null batch");
    if (!b->run_ready) return bfail(COSMOS_ESTATE, "cosmos_batch_run_begin has not been called");
    if (n < 0) return bfail(COSMOS_EINVAL, "negative step count");
    int left = n;
    while (left >= b->chunk && b->graph_ok) {
        BCK(cudaGraphLaunch(b->graph, b->stream));
        count_launch(1);
        left -= b->chunk;
    }
    while (left > 0) {
        const int k = std::min(left, b->chunk);
        BCK(launch_chunk(b, k));
        left -= k;
    }
    b->steps_done += n;
    return COSMOS_OK;
}

int cosmos_batch_run_end(cosmos_batch* b, cosmos_solve_result* results) {
    if (!b) return bfail(COSMOS_EINVAL, "null batch");
    const int n = (int)b->grids.size();
    std::vector<StepCtl> h(n);
    GridBarrier bar;
    BCK(cudaMemcpyAsync(h.data(), b->d_ctl, n * sizeof(StepCtl), cudaMemcpyDeviceToHost, b->stream));
    BCK(cudaMemcpyAsync(&bar, b->d_bar, sizeof bar, cudaMemcpyDeviceToHost, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    int bad = 0;
    for (int g = 0; g < n; g++) {
        if (results) { results[g].steps = h[g].it; results[g].t = h[g].t; results[g].status = h[g].status; }
        if (h[g].status & ST_NONFINITE) bad = 1;
    }
    if (bar.err) return bfail(COSMOS_ECUDA, "batched launch: a grid barrier wait timed out");
    if (bad) return bfail(COSMOS_ENONFINITE, "a grid produced a non-finite or non-positive time step");
    return COSMOS_OK;
}

int cosmos_batch_time_shape(cosmos_batch* b, int nt, int seg, int cap, int steps, double* ms_per_step) {
    if (!b || !ms_per_step || steps < 1) return bfail(COSMOS_EINVAL, "bad argument");
    if (!b->run_ready) return bfail(COSMOS_ESTATE, "cosmos_batch_run_begin has not been called");
    // the timing run must leave the caller's state untouched: snapshot buffers and controllers
    const size_t bytes = b->pool_elems * b->elem;
    const int n = (int)b->grids.size();
    void* save = nullptr;
    BCK(cudaMallocAsync(&save, 2 * bytes + n * sizeof(StepCtl) + sizeof(int), b->stream));
    BCK(cudaMemcpyAsync(save, b->buf[0], bytes, cudaMemcpyDeviceToDevice, b->stream));
    BCK(cudaMemcpyAsync((char*)save + bytes, b->buf[1], bytes, cudaMemcpyDeviceToDevice, b->stream));
    BCK(cudaMemcpyAsync((char*)save + 2 * bytes, b->d_ctl, n * sizeof(StepCtl), cudaMemcpyDeviceToDevice, b->stream));
    BCK(cudaMemcpyAsync((char*)save + 2 * bytes + n * sizeof(StepCtl), b->d_gstep, sizeof(int), cudaMemcpyDeviceToDevice, b->stream));
    const int nt0 = b->nt, seg0 = b->seg, cap0 = b->cap;
    int rc = build_items(b, nt, seg, cap);
    cudaEvent_t e0, e1;
    float ms = 0.0f;
    if (!rc) {
        BCK(cudaEventCreate(&e0));
        BCK(cudaEventCreate(&e1));
        BCK(launch_chunk(b, 1));  // warm-up
        BCK(cudaEventRecord(e0, b->stream));
        BCK(launch_chunk(b, steps));
        BCK(cudaEventRecord(e1, b->stream));
        BCK(cudaEventSynchronize(e1));
        BCK(cudaEventElapsedTime(&ms, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    }
    BCK(cudaMemcpyAsync(b->buf[0], save, bytes, cudaMemcpyDeviceToDevice, b->stream));
    BCK(cudaMemcpyAsync(b->buf[1], (char*)save + bytes, bytes, cudaMemcpyDeviceToDevice, b->stream));
    BCK(cudaMemcpyAsync(b->d_ctl, (char*)save + 2 * bytes, n * sizeof(StepCtl), cudaMemcpyDeviceToDevice, b->stream));
    BCK(cudaMemcpyAsync(b->d_gstep, (char*)save + 2 * bytes + n * sizeof(StepCtl), sizeof(int), cudaMemcpyDeviceToDevice, b->stream));
    BCK(cudaFreeAsync(save, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    int rc2 = set_shape(b, nt0, seg0, cap0);
    if (rc) return rc;
    if (rc2) return rc2;
    *ms_per_step = ms / steps;
    return COSMOS_OK;
}

int cosmos_batch_autotune(cosmos_batch* b, const char* cache_path, int* nt_out, int* seg_out, int* cap_out,
                          double* ms_out) {
    if (!b) return bfail(COSMOS_EINVAL, "null batch");
    if (!b->run_ready) return bfail(COSMOS_ESTATE, "cosmos_batch_run_begin has not been called");
    cudaDeviceProp prop;
    BCK(cudaGetDeviceProperties(&prop, b->device));
    long long cells = 0, sig = 1469598103934665603ll;
    for (auto& g : b->grids) {
        cells += (long long)g.G.nx * g.G.ny;
        sig = (sig ^ (g.G.nx * 131 + g.G.ny * 7 + g.G.dims)) * 1099511628211ll;
    }
    std::ostringstream key;
    std::string dev_name(prop.name);
    std::replace(dev_name.begin(), dev_name.end(), ' ', '_');  // the cache is whitespace-separated
    key << dev_name << "/" << prop.multiProcessorCount << "/p" << b->precision << "/l" << b->run.limiter << "/n"
        << b->grids.size() << "/c" << cells << "/s" << (unsigned long long)sig;
    int best_nt = 0, best_seg = 0, best_cap = 0;
    double best = 1e300;
    if (cache_path && *cache_path) {
        std::ifstream in(cache_path);
        std::string k;
        int nt, seg, cap;
        double ms;
        while (in >> k >> nt >> seg >> cap >> ms)
            if (k == key.str()) { best_nt = nt; best_seg = seg; best_cap = cap; best = ms; }
    }
    if (!best_nt) {
        for (int s = 0; s < kNumBatchShapes; s++) {
            double ms = 0.0;
            int rc = cosmos_batch_time_shape(b, kBatchShapes[s][0], kBatchShapes[s][1], kBatchShapes[s][2], 3, &ms);
            if (rc == COSMOS_EUNSUPPORTED) continue;
            if (rc) return rc;
            if (ms < best) {
                best = ms;
                best_nt = kBatchShapes[s][0];
                best_seg = kBatchShapes[s][1];
                best_cap = kBatchShapes[s][2];
            }
        }
        if (!best_nt) return bfail(COSMOS_EUNSUPPORTED, "no batch tile shape fits this device");
        if (cache_path && *cache_path) {
            std::ofstream outf(cache_path, std::ios::app);
            outf << std::setprecision(17) << key.str() << " " << best_nt << " " << best_seg << " " << best_cap << " " << best << "\n";
        }
    }
    int rc = set_shape(b, best_nt, best_seg, best_cap);
    if (rc) return rc;
    if (nt_out) *nt_out = best_nt;
    if (seg_out) *seg_out = best_seg;
    if (cap_out) *cap_out = best_cap;
    if (ms_out) *ms_out = best;
    return COSMOS_OK;
}

int cosmos_batch_set_wait_limit(cosmos_batch* b, long long polls) {
    if (!b) return bfail(COSMOS_EINVAL, "null batch");
    if (polls < 0) return bfail(COSMOS_EINVAL, "the wait limit must be >= 0 (0 restores the default)");
    b->wait_limit = polls;
    return COSMOS_OK;
}

int cosmos_batch_set_shape(cosmos_batch* b, int nt, int seg, int cap) {
    if (!b) return bfail(COSMOS_EINVAL, "null batch");
    if (!kernel_fn(b, nt, seg, cap, b->run.limiter)) return bfail(COSMOS_EUNSUPPORTED, "batch tile shape not provided for this precision");
    if (!b->run_ready) { b->nt = nt; b->seg = seg; b->cap = cap; return COSMOS_OK; }
    return set_shape(b, nt, seg, cap);
}

}  // extern "C"
