// Sweep adjoint, FP32 (conserved storage of the bulk path; FP32 arithmetic throughout).
#include <algorithm>

#include "adjoint_kernels.cuh"
#include "launch.h"

namespace cg {

cudaError_t launch_adjoint_sweep_fast(const AdjSweepParams& a, int lim, cudaStream_t st) {
    count_launch();
    return launch_adjoint_sweep_any<f2, float, false>(a, lim, st);
}
cudaError_t launch_adjoint_loss_fast(const Geom& G, const void* state, const double* target, void* ubar,
                                     double* row_sums, double* loss, cudaStream_t st) {
    count_launch(2);
    return launch_adjoint_loss_t<float, float, false>(G, state, target, ubar, row_sums, loss, st);
}
cudaError_t launch_adjoint_grad_fast(const Geom& G, double gamma, const void* state, const void* ubar, double* grad,
                                     cudaStream_t st) {
    count_launch();
    return launch_adjoint_grad_t<float, float, false>(G, gamma, state, ubar, grad, st);
}

}  // namespace cg
