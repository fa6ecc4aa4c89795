// Batched persistent launch, reference-exact FP64 Newtonian policy.  Compiled with --fmad=false:
// every grid of the batch evolves bit-identically to the reference's solver run on it alone.
#include "batch_kernels.cuh"
#include "launch.h"

namespace cg {

namespace {

using PE = ExactPolicy<NewtonExact<double>>;

PE make_exact(const BatchLaunch& L, int axis) {
    PE p;
    p.sys = NewtonExact<double>{L.gamma, nullptr};
    p.lm.axis = axis;
    p.lm.nx = 0;
    p.dims = 2;
    p.order = 2;
    p.ny = 0;
    p.dx = 0.0;
    p.dt = 0.0;
    p.w = L.bias;
    p.lim = L.lim;
    p.capped = 0;
    return p;
}

template <int NT>
cudaError_t launch_shape(const BatchLaunch& L) {
    PE px = make_exact(L, 0), py = make_exact(L, 1);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(L.blocks);
    cfg.blockDim = dim3(NT);
    cfg.stream = L.stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, batch_step_kernel<PE, PE, NT, 1>, px, py, *L.B, L.nsteps);
}

}  // namespace

// The FP64 batch has no register-capped variant (it would spill heavily).
cudaError_t launch_batch_exact(const BatchLaunch& L) {
    cudaError_t e;
    if (L.cap) e = cudaErrorInvalidValue;
    else if (L.nt == 128) e = launch_shape<128>(L);
    else if (L.nt == 256) e = launch_shape<256>(L);
    else e = cudaErrorInvalidValue;
    count_launch();
    return e;
}

void* batch_exact_fn(int nt, int cap) {
    if (cap) return nullptr;
    if (nt == 128) return (void*)batch_step_kernel<PE, PE, 128, 1>;
    if (nt == 256) return (void*)batch_step_kernel<PE, PE, 256, 1>;
    return nullptr;
}

}  // namespace cg
