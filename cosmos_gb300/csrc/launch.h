// Internal launch interface between the C-ABI layer (capi.cu) and the kernel translation units.
// kernels_exact.cu is compiled with --fmad=false (reference-exact FP64 arithmetic);
// kernels_fast.cu with contraction on (FP32 bulk path).
#pragma once
#include <cuda_runtime.h>
#include "device_common.cuh"
#include "sweep_kernels.cuh"

struct CUtensorMap_st;  // <cuda.h>'s tensor-map descriptor (CUtensorMap)

namespace cg {

// Metric tables of a black-hole grid with FP32 storage (physics_gr_fast.cuh), built once in FP64.
// Centres carry a two-cell border, faces f (between cells f - 1 and f) run over [-2, n + 2].
struct GRTables {
    const float* center;  // kMetFields x (ny + 4) x (nx + 4), index (i + 2) (nx + 4) + (j + 2)
    const float* xface;   // kMetFields x (ny + 4) x (nx + 5), index (i + 2) (nx + 5) + (f + 2)
    const float* yface;   // kMetFields x (ny + 5) x (nx + 4), index (f + 2) (nx + 4) + (j + 2)
    const float* src;     // kSrcFields x ny x nx
    const float* ws;      // kWsFields x ny x nx
    const unsigned char* flags;  // per cell: bit 0 sweep active (reach 2), bit 1 reach 1, bit 2 source
                                 // step active, bit 3 CFL point excised
    int nx, ny;
    size_t center_stride, xface_stride, yface_stride, cell_stride;
};

struct SweepArgs {
    int system;  // 0 Newtonian, 1 SR, 2 GR
    Geom G;
    int order;   // 1 FORCE, 2 SLIC
    double dx, bias, gamma;
    int lim;
    double bh[5];  // mass, spin, x, y, z
    double c2p64_above;  // SR/GR FP32: Lorentz factor above which primitive recovery finishes in FP64 (<= 0: always)
    const GRTables* grt;  // GR FP32: the grid's metric tables
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
// The Level-2 drivers' forms: threshold `thr`, divisor `div` (the coarse spacing on a finer grid),
// `plain` (Newtonian neighbours for every system), `need_on` (test only cells that are on), `strict`
// (derefine only where every child is flagged).
cudaError_t launch_amr_flags_ex(const SweepArgs& a, int precision, double thr, double div, bool plain, bool need_on,
                                unsigned char* coarse, unsigned char* fine);
cudaError_t launch_amr_derefine_ex(const SweepArgs& a, int precision, const void* fine_state, const Geom& FG, double thr,
                                   double div, bool strict, unsigned char* coarse, unsigned char* fine,
                                   void* coarse_state);
// End-of-step level exchange (restriction into unflagged parent cells, injection into unflagged
// children; strict: restriction only where every child is flagged, injection only under a flagged
// parent; Newtonian and SR) and the any-flag test of n bytes (ORs 1 into *out).
cudaError_t launch_amr_sync(const SweepArgs& a, int precision, void* coarse_state, void* fine_state, const Geom& FG,
                            const unsigned char* coarse, const unsigned char* fine, bool strict = false);
cudaError_t launch_amr_any(const unsigned char* flags, size_t n, unsigned long long* out, cudaStream_t st);

// State-level functions (kernels_exact.cu), the operations of cosmos_state_eval: values equal to
// the public COSMOS_STATE_* constants.
enum StateOp : int {
    kStateCons = 0, kStatePrim = 1, kStateFluxX = 2, kStateFluxY = 3, kStateSound = 4, kStateInternalEnergy = 5,
    kStateTotalEnergy = 6, kStatePressure = 7, kStateEnthalpy = 8, kStateSource = 9, kStateEigenvalues = 10,
    kStateGradientRatio = 11, kStateLimiter = 12, kStateSlope = 13
};
struct StateEvalArgs {
    int system, op;
    size_t n;
    const double* in;   // device, in_stride doubles per item
    const double* xyz;  // device, 3 per item (black-hole system) or null
    double* out;        // device, out_stride doubles per item
    size_t in_stride, out_stride;
    double gamma, bias;
    int lim;
};
// s supplies gamma, the hole and dx (the metric derivatives' spacing) and the stream
cudaError_t launch_state_eval(const SweepArgs& s, const StateEvalArgs& a);

// Per-interface solver functions (kernels_exact.cu), the operations of cosmos_interface_eval
// (op numbers: the public COSMOS_IF_* values; input widths kIfaceWidth).
constexpr int kIfaceOps = 23;
constexpr int kIfaceWidth[kIfaceOps] = {20, 20, 10, 15, 10, 10, 10, 10, 10, 10, 10, 10,
                                        20, 20, 15, 15, 15, 15, 15, 15, 10, 15, 25};
struct IfaceArgs {
    int system, op;
    size_t n;
    const double* in;   // device, kIfaceWidth[op] doubles per item
    const double* xyz;  // device, 3 per item (black-hole system) or null
    double* out;        // device, 5 per item
    double dx, dt, bias, frac;
    int lim, side;
    int width;          // kIfaceWidth[op]
};
// s supplies gamma, the hole and the stream
cudaError_t launch_interface_eval(const SweepArgs& s, const IfaceArgs& a);
// BlackHoleSpacetime's public quantities at n points (kSpacetimeWidth doubles each; s supplies the
// hole and, in s.dx, the derivative spacing)
constexpr int kSpacetimeWidth = 125;
cudaError_t launch_spacetime_eval(const SweepArgs& s, size_t n, const double* xyz, double* out);

// FP32 bulk path (conserved SoA storage, float)
cudaError_t launch_sweep_fast(const SweepArgs& a);
// A 3-D tensor map of an FP32 SoA state at `base` (x: nx cells, y: ny rows G.pitch apart, z: the
// five fields G.fstride apart) whose box is `box_x` cells of one row in every field; false when
// the state cannot be described (the sweeps then copy each field by itself).
bool field_map(CUtensorMap_st* m, const float* base, const Geom& G, unsigned box_x);
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

// FP32 bulk path of the black-hole system (kernels_gr_fast.cu)
size_t gr_tables_bytes(int nx, int ny);
cudaError_t build_gr_tables(const SweepArgs& a, void* storage, GRTables* out);
cudaError_t launch_sweep_gr_fast(const SweepArgs& a);
cudaError_t launch_rk_source_gr_fast(const SweepArgs& a);
cudaError_t launch_wavespeed_gr_fast(const SweepArgs& a, unsigned long long* slot);
cudaError_t launch_prim_in_gr_fast(const SweepArgs& a, const double* aos, void* soa);
cudaError_t launch_prim_out_gr_fast(const SweepArgs& a, const void* soa, double* aos);

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
                                   {128, 32, 1}, {128, 64, 1}, {256, 32, 1}, {256, 64, 1},
                                   {128, 128, 1}, {256, 128, 1}};
constexpr int kNumBatchShapes = 10;
cudaError_t launch_batch_fast(const BatchLaunch& L);
cudaError_t launch_batch_exact(const BatchLaunch& L);

// ---- sweep adjoint (adjoint_kernels.cuh); _exact: FP64 primitive storage, _fast: FP32 conserved
struct AdjSweepParams;
struct AdjCoefs;
// the adjoint coefficients of every sweep from the forward pass's dts (kernels_adjoint.cu)
cudaError_t launch_adjoint_coefs(const double* dts, int nsteps, int nsw, double dx, double gamma, double bias,
                                 AdjCoefs* out, cudaStream_t st);
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
// Relativistic FP64 sweep adjoints on primitive adjoints (kernels_adjoint_rel.cu; system 1 SR,
// 2 black hole with bh = M, a, x, y, z), and the copy of the final primitive adjoint into AoS doubles.
cudaError_t launch_adjoint_rel_sweep(const Geom& G, int system, double gamma, const double* bh, double dx, double dt,
                                     double bias, int lim, const void* state, const void* pbar_out, void* pbar_in,
                                     cudaStream_t st);
// One black-hole RK source step's adjoint (dt the step's, bias 0, limiter 1, transmissive).
cudaError_t launch_adjoint_rel_rk(const Geom& G, double gamma, const double* bh, double dx, double dt, const void* state,
                                  const void* pbar_out, void* pbar_in, cudaStream_t st);
cudaError_t launch_adjoint_rel_grad(const Geom& G, const void* pbar, double* grad, cudaStream_t st);

}  // namespace cg
