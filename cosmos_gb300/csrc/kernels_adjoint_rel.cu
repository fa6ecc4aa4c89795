// Relativistic adjoints (FP64; special-relativistic sweeps, black-hole flux sweeps and RK source
// steps): one thread per cell over the gather forms of adjoint_rel.cuh, and the copy of the final
// adjoint into the caller's layout.  Compiled with --fmad=false like the reference-exact forward whose
// arithmetic it differentiates.
#include <algorithm>

#include "adjoint_rel.cuh"
#include "launch.h"

namespace cg {

__global__ void __launch_bounds__(128) rel_adjoint_sweep_kernel(radj::Params p) {
    const size_t n = (size_t)p.nx * p.ny;
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x)
        radj::cell_adjoint(p, c);
}

__global__ void __launch_bounds__(128) rel_adjoint_rk_kernel(radj::Params p) {
    const size_t n = (size_t)p.nx * p.ny;
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x)
        radj::rk_cell_adjoint(p, c);
}

// grad[5 c + f] = pbar[f fstride + i pitch + j] for c = i nx + j (the layout of cosmos_grid_set_prim).
__global__ void rel_adjoint_grad_kernel(Geom G, const double* pbar, double* grad) {
    const size_t n = (size_t)G.nx * G.ny;
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
        const size_t q = (c / (size_t)G.nx) * (size_t)G.pitch + c % (size_t)G.nx;
        for (int f = 0; f < 5; f++) grad[5 * c + f] = pbar[f * G.fstride + q];
    }
}

cudaError_t launch_adjoint_rel_sweep(const Geom& G, int system, double gamma, const double* bh, double dx, double dt,
                                     double bias, int lim, const void* state, const void* pbar_out, void* pbar_in,
                                     cudaStream_t st) {
    radj::Params p;
    p.system = system;
    p.dims = G.dims;
    p.nx = G.nx;
    p.ny = G.ny;
    p.pitch = G.pitch;
    p.periodic = G.bc == 1;
    p.fstride = G.fstride;
    p.gamma = gamma;
    for (int k = 0; k < 5; k++) p.bh[k] = bh ? bh[k] : 0.0;
    p.s = radj::Step{dx, dt, bias, lim, G.axis};
    p.state = (const double*)state;
    p.pbar_out = (const double*)pbar_out;
    p.pbar_in = (double*)pbar_in;
    const size_t n = (size_t)G.nx * G.ny;
    const int blocks = (int)std::max<size_t>(1, std::min<size_t>((n + 127) / 128, device_sm_count() * 16));
    rel_adjoint_sweep_kernel<<<blocks, 128, 0, st>>>(p);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_adjoint_rel_rk(const Geom& G, double gamma, const double* bh, double dx, double dt, const void* state,
                                  const void* pbar_out, void* pbar_in, cudaStream_t st) {
    radj::Params p;
    p.system = 2;
    p.dims = G.dims;
    p.nx = G.nx;
    p.ny = G.ny;
    p.pitch = G.pitch;
    p.periodic = 0;
    p.fstride = G.fstride;
    p.gamma = gamma;
    for (int k = 0; k < 5; k++) p.bh[k] = bh[k];
    p.s = radj::Step{dx, dt, 0.0, 1, 0};  // the forcing step's slopes: bias 0, van Leer
    p.state = (const double*)state;
    p.pbar_out = (const double*)pbar_out;
    p.pbar_in = (double*)pbar_in;
    const size_t n = (size_t)G.nx * G.ny;
    const int blocks = (int)std::max<size_t>(1, std::min<size_t>((n + 127) / 128, device_sm_count() * 16));
    rel_adjoint_rk_kernel<<<blocks, 128, 0, st>>>(p);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_adjoint_rel_grad(const Geom& G, const void* pbar, double* grad, cudaStream_t st) {
    const size_t n = (size_t)G.nx * G.ny;
    const int blocks = (int)std::max<size_t>(1, std::min<size_t>((n + 255) / 256, device_sm_count() * 16));
    rel_adjoint_grad_kernel<<<blocks, 256, 0, st>>>(G, (const double*)pbar, grad);
    count_launch();
    return cudaGetLastError();
}

}  // namespace cg
