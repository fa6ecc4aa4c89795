// Internal launch interface between the C-ABI layer (capi.cu) and the kernel translation units.
// kernels_exact.cu is compiled with --fmad=false (reference-exact FP64 arithmetic);
// kernels_fast.cu with contraction on (FP32 bulk path).
#pragma once
#include <cuda_runtime.h>
#include "device_common.cuh"
#include "sweep_kernels.cuh"

namespace cg {

struct SweepArgs {
    int system;  // 0 Newtonian, 1 SR, 2 GR
    Geom G;
    int order;   // 1 FORCE, 2 SLIC
    double dx, bias, gamma;
    int lim;
    double bh[5];  // mass, spin, x, y, z
    double c2p64_above;  // SR FP32: Lorentz factor above which primitive recovery finishes in FP64 (<= 0: always)
    const void* src;
    void* dst;
    DtSrc ds;
    SweepOut out;
    cudaStream_t stream;
};

// FP64 reference-exact path (primitive SoA storage, double)
cudaError_t launch_sweep_exact(const SweepArgs& a);
cudaError_t launch_wavespeed_exact(const SweepArgs& a, unsigned long long* slot);
cudaError_t launch_rk_source_exact(const SweepArgs& a);
cudaError_t launch_prim_in_exact(const double* aos, void* soa, const Geom& G, cudaStream_t st);
cudaError_t launch_prim_out_exact(const void* soa, double* aos, const Geom& G, cudaStream_t st);
cudaError_t launch_dt_kernel(StepCtl* ctl, cudaStream_t st);
// AMR flag pass (refine marks) and derefinement marks; precision 0 = FP64 prim storage,
// 1 = FP32 conserved storage.
cudaError_t launch_amr_flags(const SweepArgs& a, int precision, double tol, unsigned char* coarse,
                             unsigned char* fine);
cudaError_t launch_amr_derefine(const SweepArgs& a, int precision, const void* fine_state, const Geom& FG,
                                double tol, unsigned char* coarse, unsigned char* fine, void* coarse_state);

// FP32 bulk path (conserved SoA storage, float)
cudaError_t launch_sweep_fast(const SweepArgs& a);
cudaError_t launch_wavespeed_fast(const SweepArgs& a, unsigned long long* slot);
cudaError_t launch_prim_in_fast(const double* aos, void* soa, const Geom& G, int system, double gamma,
                                cudaStream_t st);
cudaError_t launch_prim_out_fast(const void* soa, double* aos, const Geom& G, int system, double gamma,
                                 cudaStream_t st);

// FP32 bulk path of the special-relativistic system (kernels_sr_fast.cu); reached through the
// launch_*_fast functions above for system 1
cudaError_t launch_sweep_sr_fast(const SweepArgs& a);
cudaError_t launch_wavespeed_sr_fast(const SweepArgs& a, unsigned long long* slot);
cudaError_t launch_prim_in_sr_fast(const double* aos, void* soa, const Geom& G, double gamma, cudaStream_t st);
cudaError_t launch_prim_out_sr_fast(const void* soa, double* aos, const Geom& G, double gamma, cudaStream_t st);

// device-side sums for conservation checks (compensated, FP64 accumulation)
cudaError_t launch_field_sums(const void* soa, const Geom& G, int precision, double* out5, cudaStream_t st);

// bookkeeping: every kernel launch made by the library bumps this counter
void count_launch(unsigned n = 1);

// ---- batched persistent launch (batch_kernels.cuh); BatchDev is declared there
struct BatchDev;
struct BatchLaunch {
    const BatchDev* B;  // host copy of the device descriptor
    int nsteps;
    int nt, seg, cap, lim;  // tile shape (threads, Y rows, register cap) and limiter
    double gamma, bias;
    int blocks;             // resident blocks (cooperative grid size)
    cudaStream_t stream;
};
// Tile shapes of the batched launch: (threads per block, rows per Y work item, register cap).
constexpr int kBatchShapes[][3] = {{128, 32, 0}, {128, 64, 0}, {256, 32, 0}, {256, 64, 0},
                                   {128, 32, 1}, {128, 64, 1}, {256, 32, 1}, {256, 64, 1}};
constexpr int kNumBatchShapes = 8;
cudaError_t launch_batch_fast(const BatchLaunch& L);
cudaError_t launch_batch_exact(const BatchLaunch& L);

// ---- sweep adjoint (adjoint_kernels.cuh); _exact: FP64 primitive storage, _fast: FP32 conserved
struct AdjSweepParams;
cudaError_t launch_adjoint_sweep_exact(const AdjSweepParams& a, int lim, cudaStream_t st);
cudaError_t launch_adjoint_sweep_fast(const AdjSweepParams& a, int lim, cudaStream_t st);
cudaError_t launch_adjoint_loss_exact(const Geom& G, const void* state, const double* target, void* ubar,
                                      double* row_sums, double* loss, cudaStream_t st);
cudaError_t launch_adjoint_loss_fast(const Geom& G, const void* state, const double* target, void* ubar,
                                     double* row_sums, double* loss, cudaStream_t st);
cudaError_t launch_adjoint_grad_exact(const Geom& G, double gamma, const void* state, const void* ubar, double* grad,
                                      cudaStream_t st);
cudaError_t launch_adjoint_grad_fast(const Geom& G, double gamma, const void* state, const void* ubar, double* grad,
                                     cudaStream_t st);

}  // namespace cg
