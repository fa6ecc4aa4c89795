// Internal layout of the C-ABI objects, shared by the translation units that implement them.
#pragma once
#include <atomic>

#include "../../include/cosmos_gb300.h"
#include "launch.h"

// A context lives until cosmos_ctx_destroy has been called AND its last grid or batch is
// destroyed: objects hold a reference, so teardown in any order never touches a freed stream.
struct cosmos_ctx {
    int device;
    cudaStream_t stream;
    std::atomic<int> refs;
    // host <-> device copies of set_prim / get_prim run here, chunk by chunk, overlapping the
    // conversion kernels on `stream`; events order the two streams
    cudaStream_t copy;
    cudaEvent_t ev[2];
};

struct cosmos_grid {
    cosmos_ctx* ctx;
    cosmos_params p;
    cg::Geom G;              // geometry of the stored state (axis set per sweep)
    size_t elem;             // bytes per stored scalar
    void* buf[2];            // ping-pong state buffers (5 fields each)
    int cur;                 // buffer holding the current state
    cg::StepCtl* ctl;        // device step controller
    double* staging;         // device AoS primitives for set/get
    double* sums;            // field-sum output + scratch
    int* status;             // device status word for explicit sweeps
    // run configuration and captured one-step graphs (one per starting buffer)
    cosmos_solve_opts run;
    bool run_ready;
    cudaGraphExec_t step_graph[2];
    cudaGraphExec_t chunk_graph[2];  // kChunkSteps steps from each starting buffer (an even count: back to it)
    unsigned step_kernels;   // kernels per captured step
    // black-hole grids with FP32 storage: metric tables built once at creation
    void* gr_mem;
    cg::GRTables grt;
    // adjoint: device bytes for sweep inputs kept from the forward pass (-1: half the free memory)
    long long adj_keep = -1;
};

namespace cg {
void ctx_retain(cosmos_ctx* c);
void ctx_release(cosmos_ctx* c);
void set_error(const char* msg);
void set_capturing(bool on);
// sweep arguments of a grid (geometry, physics, stream) with everything else zeroed
SweepArgs base_args(cosmos_grid* g);
// the sweep kernel of the grid's precision
cudaError_t sweep_launch(cosmos_grid* g, const SweepArgs& a);
// one step of a running (cosmos_grid_run_begin) grid reading `src`, its k-th operation writing dst[k]:
// the sweeps, and for a black-hole grid `subcycles` RK source half-steps before and after them;
// returns a cosmos status code
int enqueue_step_into(cosmos_grid* g, const void* src, void* const* dst);
}  // namespace cg
