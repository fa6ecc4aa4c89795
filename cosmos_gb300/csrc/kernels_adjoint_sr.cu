// Special-relativistic sweep adjoint (FP64): one thread per cell over the gather form of
// adjoint_sr.cuh, and the copy of the final adjoint into the caller's layout.  Compiled with
// --fmad=false like the reference-exact forward whose arithmetic it differentiates.
#include <algorithm>

#include "adjoint_sr.cuh"
#include "launch.h"

namespace cg {

__global__ void __launch_bounds__(128) sr_adjoint_sweep_kernel(sra::Params p) {
    const size_t n = (size_t)p.nx * p.ny;
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x)
        sra::cell_adjoint(p, c);
}

// grad[5 c + f] = pbar[f fstride + i pitch + j] for c = i nx + j (the layout of cosmos_grid_set_prim).
__global__ void sr_adjoint_grad_kernel(Geom G, const double* pbar, double* grad) {
    const size_t n = (size_t)G.nx * G.ny;
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
        const size_t q = (c / (size_t)G.nx) * (size_t)G.pitch + c % (size_t)G.nx;
        for (int f = 0; f < 5; f++) grad[5 * c + f] = pbar[f * G.fstride + q];
    }
}

cudaError_t launch_adjoint_sr_sweep(const Geom& G, double gamma, double dx, double dt, double bias, int lim,
                                    const void* state, const void* pbar_out, void* pbar_in, cudaStream_t st) {
    sra::Params p;
    p.nx = G.nx;
    p.ny = G.ny;
    p.pitch = G.pitch;
    p.axis = G.axis;
    p.periodic = G.bc == 1;
    p.fstride = G.fstride;
    p.s = sra::Step{gamma, dx, dt, bias, lim, G.axis};
    p.state = (const double*)state;
    p.pbar_out = (const double*)pbar_out;
    p.pbar_in = (double*)pbar_in;
    const size_t n = (size_t)G.nx * G.ny;
    const int blocks = (int)std::max<size_t>(1, std::min<size_t>((n + 127) / 128, 152 * 16));
    sr_adjoint_sweep_kernel<<<blocks, 128, 0, st>>>(p);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_adjoint_sr_grad(const Geom& G, const void* pbar, double* grad, cudaStream_t st) {
    const size_t n = (size_t)G.nx * G.ny;
    const int blocks = (int)std::max<size_t>(1, std::min<size_t>((n + 255) / 256, 152 * 16));
    sr_adjoint_grad_kernel<<<blocks, 256, 0, st>>>(G, (const double*)pbar, grad);
    count_launch();
    return cudaGetLastError();
}

}  // namespace cg
