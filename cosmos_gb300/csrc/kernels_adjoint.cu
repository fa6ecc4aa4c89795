// Sweep adjoint, FP64 (primitive storage of the reference-exact path).  Compiled with
// --fmad=false like the forward it differentiates.
#include <algorithm>

#include "adjoint_kernels.cuh"
#include "launch.h"

namespace cg {

cudaError_t launch_adjoint_sweep_exact(const AdjSweepParams& a, int lim, cudaStream_t st) {
    count_launch();
    return launch_adjoint_sweep_any<double, double, true>(a, lim, st);
}
cudaError_t launch_adjoint_loss_exact(const Geom& G, const void* state, const double* target, void* ubar,
                                      double* row_sums, double* loss, cudaStream_t st) {
    count_launch(2);
    return launch_adjoint_loss_t<double, double, true>(G, state, target, ubar, row_sums, loss, st);
}
cudaError_t launch_adjoint_grad_exact(const Geom& G, double gamma, const void* state, const void* ubar, double* grad,
                                      cudaStream_t st) {
    count_launch();
    return launch_adjoint_grad_t<double, double, true>(G, gamma, state, ubar, grad, st);
}

__global__ void adjoint_coef_kernel(const double* dts, int nsteps, int nsw, double dx, double gam, double w,
                                    AdjCoefs* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nsteps * nsw) return;
    const int m = i % nsw;
    const double d = dts[i / nsw];
    out[i] = adj_coefs(nsw == 3 && m != 1 ? 0.5 * d : d, dx, gam, w);
}
cudaError_t launch_adjoint_coefs(const double* dts, int nsteps, int nsw, double dx, double gamma, double bias,
                                 AdjCoefs* out, cudaStream_t st) {
    count_launch();
    const int n = nsteps * nsw;
    adjoint_coef_kernel<<<(n + 127) / 128, 128, 0, st>>>(dts, nsteps, nsw, dx, gamma, bias, out);
    return cudaGetLastError();
}

}  // namespace cg
