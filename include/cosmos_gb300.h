/*
 * cosmos_gb300 -- C ABI of the GB300 implementation of the Cosmos finite-volume SLIC/FORCE path
 * (Newtonian, special-relativistic and black-hole (Kerr-Schild 3+1) Euler equations).
 *
 * The reference exposes this path as static C++ methods on value-semantics grids
 * (vector<StateVector> / vector<vector<StateVector>>, primitive variables rho, vx, vy, vz, p).
 * This ABI keeps the same operations and argument meaning with plain pointers:
 *   - grids are device-resident handles (cosmos_grid) created from a cosmos_params;
 *   - host data crosses as arrays of primitive states, 5 doubles per cell, row-major
 *     [ny][nx] (row i = y, column j = x), exactly the reference's grid layout;
 *   - every call returns a status code (COSMOS_OK == 0); cosmos_last_error() describes failures
 *     (the reference itself has no error reporting).
 * Reference paths are relative to the JonathanGorard/Cosmos tree.
 *
 * Precision: COSMOS_FP64 runs the reference's arithmetic in the reference's operation order
 * (results are bit-identical to the reference's CPU solver); COSMOS_FP32 runs the Newtonian
 * system with FP32 conserved storage and arithmetic.
 *
 * Threading: one cosmos_ctx per host thread; calls on a context are serialised on its stream.
 */
#ifndef COSMOS_GB300_H
#define COSMOS_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- return codes */
#define COSMOS_OK 0
#define COSMOS_EINVAL 1       /* bad argument (size, enum, pointer) */
#define COSMOS_ECUDA 2        /* CUDA runtime error */
#define COSMOS_ENONFINITE 3   /* the solver produced a non-finite time step */
#define COSMOS_EUNSUPPORTED 4 /* combination not provided (e.g. FP32 for the GR system) */
#define COSMOS_ESTATE 5       /* call order violated */

/* ---- device status bits reported by cosmos_solve_result.status */
#define COSMOS_STATUS_NONFINITE 1  /* a non-finite or non-positive dt was produced; a cell whose density
                                      or energy (FP64 grids: pressure) is not finite has an infinite CFL
                                      speed and so yields a zero dt (the reference carries NaNs on) */
#define COSMOS_STATUS_NEWTON_CAP 2 /* a con2prim Newton solve stopped at its iteration cap (FP64 path: the
                                      reference's 1000; FP32 path: 40 FP32 + 8 FP64), or (FP32 path) a state
                                      beyond FP32's range was replaced by the floor state */
#define COSMOS_STATUS_TIMEOUT 4    /* a bounded device wait gave up (the Y sweep's bulk-copy waits, about
                                      a second of SM clocks) */

/* ---- enumerations */
enum { COSMOS_NEWTONIAN = 0, COSMOS_SR = 1, COSMOS_GR = 2 };
enum { COSMOS_FP64 = 0, COSMOS_FP32 = 1 };
enum { COSMOS_BC_TRANSMISSIVE = 0, COSMOS_BC_PERIODIC = 1 };
/* Solvers/SlopeLimiters.cpp:55-69: 0 SuperBee, 1 van Leer, anything else MinBee */
enum { COSMOS_SUPERBEE = 0, COSMOS_VANLEER = 1, COSMOS_MINBEE = 2 };

/* Grid description.  Replaces the reference's (initialCells shape, cellSpacing,
 * EulerMaterialParameters, BlackHoleSpacetime) arguments:
 *   gamma  -- EulerMaterialParameters adiabatic index (Euler/EulerMaterialParameters.cpp:3-21)
 *   bh_*   -- BlackHoleSpacetime(mass, spin, x, y, z) (BlackHoleEuler/BlackHoleSpacetime.cpp:3-52)
 * dims 1 uses ny = 1; 2D grids have at most 65535 rows and 2^31 cells.  boundary: the reference
 * only has transmissive ghost cells (Solvers/EulerSolvers.cpp:3-85); periodic is an extension
 * (Newtonian and SR only). */
typedef struct cosmos_params {
    int system;
    int dims;
    int nx;
    int ny;
    int precision;
    int boundary;
    double gamma;
    double dx;
    double bh_mass, bh_spin, bh_x, bh_y, bh_z;
    /* SR system with COSMOS_FP32 storage: each conserved-to-primitive Newton solve iterates in
     * FP32, then finishes in FP64 (to the reference's 1e-8 step tolerance) when the state's
     * Lorentz factor exceeds this value or the FP32 iteration did not converge; <= 0 finishes
     * every solve in FP64.  Default 2. */
    double sr_c2p64_above;
} cosmos_params;

/* Solver options: the reference's solve() arguments (CFLCoefficient, finalTime, bias,
 * slopeLimiter, subcyclingIterations; Solvers/EulerSecondOrderSolver.hpp:24-28,
 * Solvers/BlackHoleEulerSecondOrderSolver.hpp:26-32) plus run control. */
typedef struct cosmos_solve_opts {
    int order;       /* 2 = SLIC (SecondOrderSolver), 1 = FORCE (FirstOrderSolver) */
    double cfl;
    double t_final;
    double bias;
    int limiter;
    int subcycles;   /* GR only: RK source half-steps before and after the flux step (0: none) */
    int max_steps;   /* < 0: run until t >= t_final; otherwise stop after max_steps steps */
} cosmos_solve_opts;

typedef struct cosmos_solve_result {
    int steps;       /* the reference's currentIteration at exit */
    double t;        /* the reference's currentTime at exit */
    int status;      /* COSMOS_STATUS_* bits */
} cosmos_solve_result;

typedef struct cosmos_ctx cosmos_ctx;
typedef struct cosmos_grid cosmos_grid;

/* ---- context */
int cosmos_ctx_create(int device, cosmos_ctx** out);
/* Releases the caller's reference: the stream is destroyed once the last grid or batch created on
 * the context has been destroyed too, so objects may be destroyed in any order. */
int cosmos_ctx_destroy(cosmos_ctx* ctx);
int cosmos_ctx_synchronize(cosmos_ctx* ctx);
void* cosmos_ctx_stream(cosmos_ctx* ctx); /* the cudaStream_t all work of this context runs on */
const char* cosmos_last_error(void);      /* thread-local description of the last failure */
unsigned long long cosmos_kernel_launches(void); /* kernels launched by this library (all threads) */
const char* cosmos_version(void);
/* FP32 sweeps stage their rows through TMA tensor maps (one copy of a row's five fields) when
 * `enable` is nonzero (the default), else by one copy per field; the results are bit-identical.
 * Read when a sweep is launched or captured and when a batch is created.  Library-wide (the
 * reference has no counterpart); returns the previous setting. */
int cosmos_set_tensor_maps(int enable);

void cosmos_params_default(cosmos_params* p);
void cosmos_solve_opts_default(cosmos_solve_opts* o);

/* ---- grids (device state: structure of arrays; FP64 keeps primitives, FP32 conserved) */
int cosmos_grid_create(cosmos_ctx* ctx, const cosmos_params* p, cosmos_grid** out);
int cosmos_grid_destroy(cosmos_grid* g);
/* n_doubles must equal 5 * nx * ny.  Replaces constructing the reference's initialCells. */
int cosmos_grid_set_prim(cosmos_grid* g, const double* prim, size_t n_doubles);
/* Returns the grid as primitive states (the reference's returned grid). */
int cosmos_grid_get_prim(cosmos_grid* g, double* prim, size_t n_doubles);

/* One dimensional sweep with time step dt, in place on the grid.
 * axis 0 / order 2: EulerSecondOrderSolver::computeXSLICTimeStep2D (2D) or computeSLICTimeStep (1D)
 *   (Solvers/EulerSecondOrderSolver.cpp:27-73); axis 1: computeYSLICTimeStep2D (:75-100);
 * order 1: EulerFirstOrderSolver::computeFORCETimeStep / computeX/YFORCETimeStep2D
 *   (Solvers/EulerFirstOrderSolver.cpp:103-155);
 * SR and GR twins: Solvers/RelativisticEulerSecondOrderSolver.cpp:27-130,
 *   Solvers/BlackHoleEulerSecondOrderSolver.cpp:39-179 (with excision),
 *   Solvers/BlackHoleEulerFirstOrderSolver.cpp:89-165. */
int cosmos_grid_sweep(cosmos_grid* g, int axis, int order, double dt, double bias, int limiter);

/* GR source term step: BlackHoleEulerForcingSolver::computeRungeKuttaTimeStep(2D)
 * (Solvers/BlackHoleEulerForcingSolver.cpp:187-250; classical RK4 with interleaved
 * fractional flux sweeps). */
int cosmos_grid_rk_source(cosmos_grid* g, double dt, double bias, int limiter);

/* EulerSolvers::computeMaximumWaveSpeed(2D) (Solvers/EulerSolvers.cpp:87-128) and twins
 * (Solvers/RelativisticEulerSolvers.cpp:87-128, Solvers/BlackHoleEulerSolvers.cpp:87-131). */
int cosmos_grid_max_wavespeed(cosmos_grid* g, double* out);
/* EulerSolvers::computeStableTimeStep(2D) with the grid's state (Solvers/EulerSolvers.cpp:147-161). */
int cosmos_grid_stable_dt(cosmos_grid* g, double cfl, double t, double t_final, int iteration, double* dt_out);
/* EulerSolvers::computeStableTimeStep(dt, t, T, it) (Solvers/EulerSolvers.cpp:130-145). */
double cosmos_stable_dt_rule(double dt, double t, double t_final, int iteration);

/* Full solve on the device: EulerSecondOrderSolver::solve / solve2D
 * (Solvers/EulerSecondOrderSolver.cpp:102-147), EulerFirstOrderSolver::solve / solve2D
 * (Solvers/EulerFirstOrderSolver.cpp:171-216), the SR twins and
 * BlackHoleEulerSecondOrderSolver::solve / solve2D (Solvers/BlackHoleEulerSecondOrderSolver.cpp:
 * 144-218).  The time step is computed on the device every step and the step sequence replays
 * from captured CUDA graphs. */
int cosmos_grid_solve(cosmos_grid* g, const cosmos_solve_opts* o, cosmos_solve_result* r);

/* Split form of cosmos_grid_solve for callers that time or pipeline steps:
 * run_begin resets the step controller (t = 0, iteration 0) and enqueues the initial CFL
 * reduction; run_steps enqueues n steps without synchronising; run_end synchronises and reports. */
int cosmos_grid_run_begin(cosmos_grid* g, const cosmos_solve_opts* o);
int cosmos_grid_run_steps(cosmos_grid* g, int n);
int cosmos_grid_run_end(cosmos_grid* g, cosmos_solve_result* r);

/* Per-field sums of the stored state (FP64 grids: primitives; FP32 grids: conserved),
 * compensated FP64 accumulation, deterministic order.  Used for conservation drift. */
int cosmos_grid_field_sums(cosmos_grid* g, double out[5]);

/* AMR refinement flag pass of the Level-1 drivers (AMR/EulerAMR.cpp:207-229 1D, :400-431 2D;
 * AMR/RelativisticEulerAMR.cpp:404-435; AMR/BlackHoleEulerAMR.cpp:276-300, :484-515):
 * coarse[c] = 0 and its fine children = 1 where any conserved one-sided gradient reaches tol;
 * other flags are left as passed in.  coarse: nx*ny bytes, fine: 2*nx (1D) or 4*nx*ny (2D). */
int cosmos_grid_amr_flags(cosmos_grid* g, double tol, unsigned char* coarse, unsigned char* fine);
/* AMR derefinement pass (AMR/EulerAMR.cpp:310-345, :538-586): on the fine grid with the coarse
 * dx at tol/2; unflags children, flags the parent and restricts the coarse state. */
int cosmos_grid_amr_derefine(cosmos_grid* coarse, cosmos_grid* fine, double tol, unsigned char* coarse_flags,
                             unsigned char* fine_flags);

/* ---- batched grids: many independent Newtonian grids of uneven sizes (1D and 2D) advanced by
 * one persistent cooperative launch per chunk of steps, replayed from a CUDA graph.  Each grid
 * keeps its own time step, iteration count and CFL reduction -- the same results as running the
 * reference's EulerSecondOrderSolver::solve / solve2D (Solvers/EulerSecondOrderSolver.cpp:102-147)
 * on every grid separately (bit-identical with COSMOS_FP64).  dims/nx/ny/dx hold one entry per
 * grid (ny ignored for 1D grids). */
typedef struct cosmos_batch cosmos_batch;
int cosmos_batch_create(cosmos_ctx* ctx, int ngrids, const int* dims, const int* nx, const int* ny, const double* dx,
                        double gamma, int boundary, int precision, cosmos_batch** out);
int cosmos_batch_destroy(cosmos_batch* b);
int cosmos_batch_size(cosmos_batch* b, int* ngrids, long long* cells);
int cosmos_batch_set_prim(cosmos_batch* b, int grid, const double* prim, size_t n_doubles);
int cosmos_batch_get_prim(cosmos_batch* b, int grid, double* prim, size_t n_doubles);
/* Resets every grid's controller (t = 0, iteration 0) and enqueues the initial CFL reductions;
 * o->order must be 2.  results of run_end: one cosmos_solve_result per grid (may be NULL). */
int cosmos_batch_run_begin(cosmos_batch* b, const cosmos_solve_opts* o);
int cosmos_batch_run_steps(cosmos_batch* b, int n);
int cosmos_batch_run_end(cosmos_batch* b, cosmos_solve_result* results);
/* Tile shape of the persistent launch: threads per block (128 or 256), rows per Y-sweep work
 * item (seg >= 1; the autotuner tries 32 and 64), and cap (1 = registers capped so that 768
 * threads fit an SM, FP32 only; COSMOS_EUNSUPPORTED for FP64).  cosmos_batch_time_shape times `steps` steps of a shape and
 * restores the state; cosmos_batch_autotune times every shape, keeps the fastest, and caches the
 * choice in cache_path (one line per device and batch signature; NULL for no cache). */
int cosmos_batch_set_shape(cosmos_batch* b, int nt, int seg, int cap);
/* Bound on each grid-barrier wait of the persistent launch, in polls of about 64 ns (0: the
 * default 2^26, about 4 s), taking effect at the next cosmos_batch_run_begin.  A wait that runs
 * out ends the launch (every block leaves at its next barrier) and cosmos_batch_run_end returns
 * COSMOS_ECUDA ("a grid barrier wait timed out"); the grids' states are then partly advanced.
 * No counterpart in the reference (which has no batched launch): it exists so that the timeout
 * path can be exercised without a hung device. */
int cosmos_batch_set_wait_limit(cosmos_batch* b, long long polls);
int cosmos_batch_time_shape(cosmos_batch* b, int nt, int seg, int cap, int steps, double* ms_per_step);
int cosmos_batch_autotune(cosmos_batch* b, const char* cache_path, int* nt, int* seg, int* cap, double* ms_per_step);

/* ---- adjoint.  Reverse-mode gradient (hand-written sweep adjoints) of the scalar loss
 *     L = 1/2 * sum over cells (rho_T - target)^2,
 * rho_T the density after `nsteps` SLIC steps (o->order must be 2; o->bias, o->limiter used) of a
 * Newtonian grid, or of a special-relativistic or black-hole FP64 grid, from its current state,
 * with respect to that initial state's primitives.  No counterpart in the reference (it has no
 * derivatives); it differentiates the reference's EulerSecondOrderSolver::solve / solve2D step
 * (Solvers/EulerSecondOrderSolver.cpp:102-147; RelativisticEulerSecondOrderSolver for SR grids;
 * BlackHoleEulerSecondOrderSolver's step for black-hole grids, with o->subcycles RK source
 * half-steps before and after each flux step, 0 for the flux step alone; through every primitive
 * recovery's Newton iteration; lines of at least two cells) with
 * each step's dt held fixed: the caller's dts_in[nsteps] if non-NULL, else the CFL rule's dts
 * (o->cfl) of the forward run, which are returned in dts_out[nsteps] if non-NULL.  Checkpoints
 * every `checkpoint_every` steps; each segment whose sweep inputs were not kept from the forward
 * pass (cosmos_grid_set_adjoint_keep) is recomputed once.  target: ny*nx doubles (row
 * major, the grid's rows); grad_prim: 5*nx*ny doubles in the layout of cosmos_grid_set_prim;
 * loss and ms (2 doubles: forward and backward milliseconds on the context's stream) may be NULL.
 * On return the grid holds the final state.  FP64 grids differentiate the reference-exact FP64
 * steps in FP64; FP32 grids the FP32 steps in FP32. */
int cosmos_grid_adjoint(cosmos_grid* g, const cosmos_solve_opts* o, int nsteps, int checkpoint_every,
                        const double* target, const double* dts_in, double* grad_prim, double* loss,
                        double* dts_out, double* ms);
/* Device memory (bytes) cosmos_grid_adjoint may use to keep sweep inputs from its forward pass:
 * the last checkpoint segments whose sweep inputs fit (always at least the last one) are not
 * recomputed in the backward pass, the earlier ones are recomputed once from their checkpoints.
 * -1 (the default): half of the device memory free when the call starts; 0: keep the last
 * segment only.  The gradient is the same bit for bit whatever the budget. */
int cosmos_grid_set_adjoint_keep(cosmos_grid* g, long long bytes);

/* ---- Level-1 adaptive mesh refinement: EulerAMR::solveLevel1AMR / solve2DLevel1AMR
 * (AMR/EulerAMR.cpp:169-592) and RelativisticEulerAMR::solveLevel1AMR / solve2DLevel1AMR
 * (AMR/RelativisticEulerAMR.cpp:181-603), Newtonian and SR systems, transmissive boundaries.
 * A coarse grid (described by the params) and its 2x refinement (2 nx, and 2 ny in 2D, spacing
 * dx / 2) stay on the device with one flag byte per cell.  Each coarse step: the CFL time step of
 * the coarse grid (its iteration count is the total fine step count, as in the reference), the
 * refinement flag pass, a masked coarse step (bias 0, limiter 1, as the reference's drivers
 * hard-code; 2D: X(dt/2) Y(dt) X(dt/2)), masked fine steps until the fine time reaches
 * (t + dt) - 1e-4 when any fine flag is set, restriction and injection between the levels, and the
 * derefinement pass.  FP64 grids give the reference's results bit for bit. */
typedef struct cosmos_amr cosmos_amr;
typedef struct cosmos_amr_result {
    int coarse_steps;  /* the reference's coarseCurrentIteration at exit */
    int fine_steps;    /* the reference's fineTotalIteration at exit */
    double t;          /* coarseCurrentTime at exit */
    int status;        /* COSMOS_STATUS_* bits of both levels' kernels */
    int fine_run;      /* fine steps actually taken (fine_steps also counts coarse steps with no refinement) */
    int mid_run;       /* Level-2 drivers: intermediate steps taken (0 for Level 1) */
} cosmos_amr_result;
int cosmos_amr_create(cosmos_ctx* ctx, const cosmos_params* coarse, cosmos_amr** out);
/* Level-2 drivers: EulerAMR::solveLevel2AMR / solve2DLevel2AMR (AMR/EulerAMR.cpp:593-1379) and the
 * RelativisticEulerAMR twins (AMR/RelativisticEulerAMR.cpp:604-1392): three levels (coarse,
 * intermediate at dx / 2, fine at dx / 4).  The intermediate level sub-cycles inside each coarse
 * step and the fine level inside each intermediate step, with the reference's thresholds
 * (intermediate flags at tol * 2 * order, fine derefinement at tol, intermediate derefinement at
 * tol * 0.5 / order, all with the coarse spacing) and its counters.  Same calls as Level 1. */
int cosmos_amr_create_level2(cosmos_ctx* ctx, const cosmos_params* coarse, cosmos_amr** out);
int cosmos_amr_destroy(cosmos_amr* a);
/* The coarse grid's initial cells (5 * nx * ny doubles, the layout of cosmos_grid_set_prim). */
int cosmos_amr_set_prim(cosmos_amr* a, const double* prim, size_t n_doubles);
/* Runs the driver from t = 0 on the current coarse cells: flags reset (coarse on, fine off), fine
 * cells injected from their parents, then coarse steps until t >= t_final.  order 1: FORCE,
 * 2: SLIC.  tol: the AMRTolerance argument. */
int cosmos_amr_solve(cosmos_amr* a, double cfl, double t_final, double tol, int order, cosmos_amr_result* r);
/* The Level-1 driver's returned tuple: coarse cells (5 nx ny doubles), fine cells (4x or 2x as
 * many), coarse and fine flags (1 byte per cell); for a Level-2 driver the fine level is the finest.
 * Any pointer may be NULL. */
int cosmos_amr_get(cosmos_amr* a, double* coarse_prim, double* fine_prim, unsigned char* coarse_flags,
                   unsigned char* fine_flags);
/* One level's cells and flags: level 0 coarse, 1 the next finer, 2 the finest of a Level-2 driver. */
int cosmos_amr_get_level(cosmos_amr* a, int level, double* prim, unsigned char* flags);

/* ---- state-level functions: the reference's per-state functions for arrays of n states, evaluated
 * on the device with the sweeps' arithmetic (FP64, bit-identical to the reference).  p supplies the
 * system, gamma and, for the black-hole system, the hole and dx (the spacing of the source term's
 * metric derivatives).  in holds in_width doubles per item, out receives out_width doubles per item
 * (cosmos_state_width); black-hole items take their coordinates from xyz (3 doubles per item).
 *   COSMOS_STATE_CONS       prim -> conserved: StateVector::computeConservedVariableVector
 *                           (Euler/EulerStateVector.cpp:55-66; SR and black-hole twins)
 *   COSMOS_STATE_PRIM       conserved -> prim: setConservedVariableVector (:30-40; SR :30-101)
 *   COSMOS_STATE_FLUX_X/_Y  conserved -> flux: static computeX/YFluxVector (:68-117; SR :138-309)
 *   COSMOS_STATE_SOUND      prim -> sound speed (1): computeSoundSpeed / EquationOfState::computeSoundSpeed
 *                           (the black-hole one is the largest signed eigenvalue, BlackHoleEulerStateVector.cpp:519-549)
 *   COSMOS_STATE_INTERNAL_ENERGY, _TOTAL_ENERGY   Newtonian prim -> e, E (Euler/EulerEquationOfState.cpp:3-8,
 *                           Euler/EulerStateVector.cpp:129-134)
 *   COSMOS_STATE_PRESSURE   Newtonian (rho, -, -, -, e) -> p (Euler/EulerEquationOfState.cpp:10-15)
 *   COSMOS_STATE_ENTHALPY   SR/black-hole prim -> h (RelativisticEuler/RelativisticEulerEquationOfState.cpp:3-8)
 *   COSMOS_STATE_SOURCE     black-hole conserved -> source term: computeSourceTermVector (:359-510)
 *   COSMOS_STATE_EIGENVALUES  black-hole prim -> 9 values: material, fast and slow acoustic eigenvalues
 *                           along x, y, z (BlackHoleEuler/BlackHoleEulerEigenvalues.cpp:3-96)
 *   COSMOS_STATE_GRADIENT_RATIO, _LIMITER   r -> SlopeLimiters::computeGradientRatio / computeSlopeLimiter
 *                           (Solvers/SlopeLimiters.cpp:3-69; bias and limiter as given)
 *   COSMOS_STATE_SLOPE      three conserved vectors (left, middle, right: 15 doubles) -> computeSlopeVector (:71-101) */
enum {
    COSMOS_STATE_CONS = 0, COSMOS_STATE_PRIM = 1, COSMOS_STATE_FLUX_X = 2, COSMOS_STATE_FLUX_Y = 3,
    COSMOS_STATE_SOUND = 4, COSMOS_STATE_INTERNAL_ENERGY = 5, COSMOS_STATE_TOTAL_ENERGY = 6, COSMOS_STATE_PRESSURE = 7,
    COSMOS_STATE_ENTHALPY = 8, COSMOS_STATE_SOURCE = 9, COSMOS_STATE_EIGENVALUES = 10, COSMOS_STATE_GRADIENT_RATIO = 11,
    COSMOS_STATE_LIMITER = 12, COSMOS_STATE_SLOPE = 13
};
int cosmos_state_width(int op, size_t* in_width, size_t* out_width);
int cosmos_state_eval(cosmos_ctx* ctx, const cosmos_params* p, int op, size_t n, const double* in, const double* xyz,
                      double bias, int limiter, double* out);

/* ---- per-interface solver functions: the reference's static building blocks of the sweeps for
 * arrays of items, evaluated on the device in the reference's operation order (bit for bit).
 * in: n items of cosmos_interface_width(op) doubles (5-vectors back to back: conserved vectors,
 * flux vectors or primitive states (rho, vx, vy, vz, p), in the reference function's argument
 * order); out: n items of 5 doubles (a vector, or the primitives of the returned state).
 * p supplies the system, gamma (materialParameters), dx (cellSpacing) and, for the black-hole
 * system, the hole; xyz: 3 doubles per item, the (xCoordinate, yCoordinate, zCoordinate)
 * arguments of the black-hole functions (NULL otherwise).  dt is timeStep; bias, limiter, frac
 * (stepFraction) and side are the functions' arguments of those names where they have them. */
enum {
    COSMOS_IF_LAX_FRIEDRICHS = 0,   /* EulerFirstOrderSolver::computeLaxFriedrichsFlux (UL, UR, FL, FR)
                                       Solvers/EulerFirstOrderSolver.hpp:11 */
    COSMOS_IF_RICHTMYER = 1,        /* ::computeRichtmyerFlux (UL, UR, FL, FR) -> intermediate state, :13 */
    COSMOS_IF_FORCE = 2,            /* ::computeFORCEFlux (LF flux, Richtmyer flux), :15 */
    COSMOS_IF_FORCE_UPDATE = 3,     /* ::computeFORCEUpdate (U, FL, FR), :31 */
    COSMOS_IF_FRACTIONAL_EVOLUTION = 4, /* EulerSolvers::computeFractionalEvolutionVector (FL, FR; frac),
                                           Solvers/EulerSolvers.hpp:25 */
    COSMOS_IF_EVOLUTION = 5,        /* EulerSolvers::computeEvolutionVector (FL, FR), :27 */
    COSMOS_IF_X_LAX_FRIEDRICHS_FLUX = 6, /* *FirstOrderSolver::computeXLaxFriedrichsFlux (L, R states),
                                            Solvers/EulerFirstOrderSolver.hpp:18, SR and black-hole twins */
    COSMOS_IF_Y_LAX_FRIEDRICHS_FLUX = 7,
    COSMOS_IF_X_RICHTMYER_FLUX = 8,
    COSMOS_IF_Y_RICHTMYER_FLUX = 9,
    COSMOS_IF_X_FORCE_FLUX = 10,
    COSMOS_IF_Y_FORCE_FLUX = 11,
    COSMOS_IF_X_SLIC_FLUX = 12,     /* *SecondOrderSolver::computeXSLICFlux (LL, L, R, RR states; bias, limiter),
                                       Solvers/EulerSecondOrderSolver.hpp:9-14, SR and black-hole twins */
    COSMOS_IF_Y_SLIC_FLUX = 13,
    COSMOS_IF_EVOLVE_HALF_X = 14,   /* *Solvers::evolveStateByHalfXTimeStep (l, m, r states; bias, limiter, side),
                                       Solvers/EulerSolvers.hpp:30-34, SR and black-hole twins */
    COSMOS_IF_EVOLVE_HALF_Y = 15,
    COSMOS_IF_EVOLVE_HALF_VECTOR_X = 16, /* *Solvers::evolveStateByHalfTimeStep (UL, UR, evolution; side),
                                            Solvers/EulerSolvers.hpp:29; black hole: the vector form of
                                            evolveStateByHalfXTimeStep, Solvers/BlackHoleEulerSolvers.hpp:37 */
    COSMOS_IF_EVOLVE_HALF_VECTOR_Y = 17, /* the same (Newtonian, SR); black hole: evolveStateByHalfYTimeStep's :45 */
    COSMOS_IF_EVOLVE_FRACTION_X = 18, /* black hole: evolveStateByFractionalXTimeStep (l, m, r; frac, bias, limiter),
                                         Solvers/BlackHoleEulerSolvers.hpp:26 */
    COSMOS_IF_EVOLVE_FRACTION_Y = 19,
    COSMOS_IF_EVOLVE_FRACTION_VECTOR = 20, /* black hole: evolveStateByFractionalTimeStep (U, evolution), :22 */
    COSMOS_IF_RK_CELL_1D = 21,      /* BlackHoleEulerForcingSolver::evolveConservedVariableVector (conserved l, m, r),
                                       Solvers/BlackHoleEulerForcingSolver.hpp:9 */
    COSMOS_IF_RK_CELL_2D = 22       /* ::evolveConservedVariableVector2D (conserved l, m, r, t, b), :13 */
};
int cosmos_interface_width(int op, size_t* in_width, size_t* out_width);
int cosmos_interface_eval(cosmos_ctx* ctx, const cosmos_params* p, int op, size_t n, const double* in, const double* xyz,
                          double dt, double bias, int limiter, double frac, int side, double* out);

/* ---- the black-hole spacetime (BlackHoleEuler/BlackHoleSpacetime.hpp:16-42): every public quantity
 * of the reference's BlackHoleSpacetime at n points xyz (3 doubles each), COSMOS_SPACETIME_WIDTH
 * doubles per point at the offsets below (matrices row-major; derivatives [direction][...]), bit for
 * bit with the reference.  p supplies the hole (bh_*) and, in dx, the cellSpacing of the derivative
 * methods (centred differences at -/+ dx/2). */
#define COSMOS_ST_KS_SCALAR 0                /* computeKerrSchildScalar */
#define COSMOS_ST_KS_VECTOR 1                /* computeKerrSchildVector (3) */
#define COSMOS_ST_KS_SPACETIME_VECTOR 4      /* computeKerrSchildSpacetimeVector (4) */
#define COSMOS_ST_KS_SCALAR_DERIVATIVE 8     /* computeKerrSchildScalarDerivative (3) */
#define COSMOS_ST_KS_VECTOR_DERIVATIVE 11    /* computeKerrSchildVectorDerivative (3 x 3) */
#define COSMOS_ST_SPATIAL_METRIC 20          /* computeSpatialMetricTensor (3 x 3) */
#define COSMOS_ST_SPACETIME_METRIC 29        /* computeSpacetimeMetricTensor (4 x 4) */
#define COSMOS_ST_INVERSE_SPATIAL_METRIC 45  /* computeInverseSpatialMetricTensor (3 x 3) */
#define COSMOS_ST_INVERSE_SPACETIME_METRIC 54 /* computeInverseSpacetimeMetricTensor (4 x 4) */
#define COSMOS_ST_SPATIAL_DETERMINANT 70     /* computeSpatialMetricDeterminant */
#define COSMOS_ST_SPACETIME_DETERMINANT 71   /* computeSpacetimeMetricDeterminant */
#define COSMOS_ST_SPATIAL_METRIC_DERIVATIVE 72 /* computeSpatialMetricTensorDerivative (3 x 3 x 3) */
#define COSMOS_ST_LAPSE 99                   /* computeLapseFunction */
#define COSMOS_ST_SHIFT 100                  /* computeShiftVector (3) */
#define COSMOS_ST_LAPSE_DERIVATIVE 103       /* computeLapseFunctionDerivative (3) */
#define COSMOS_ST_SHIFT_DERIVATIVE 106       /* computeShiftVectorDerivative (3 x 3) */
#define COSMOS_ST_EXTRINSIC_CURVATURE 115    /* computeExtrinsicCurvatureTensor (3 x 3) */
#define COSMOS_ST_EXCISED 124                /* inExcisionRegion (1.0 or 0.0) */
#define COSMOS_SPACETIME_WIDTH 125
int cosmos_spacetime_eval(cosmos_ctx* ctx, const cosmos_params* p, size_t n, const double* xyz, double* out);

/* Allocation-free conservation sums.  No counterpart in the reference: it exists for callers that
 * cannot allocate device memory where they need the sums -- runtimes that own the device
 * allocator and its pool, embedded callers with a fixed memory budget, pipelines that must not
 * stall on cudaMalloc's device synchronisation.  Same sums as cosmos_grid_field_sums, on a
 * caller-owned structure-of-arrays state: field f of cell (i, j) at
 * state[f * field_stride + i * pitch + j], doubles (COSMOS_FP64) or floats (COSMOS_FP32).
 * out5 is caller-owned device memory for 5 doubles; the work is enqueued on `stream` (a
 * cudaStream_t, 0 for the legacy stream) and not synchronised.  It allocates nothing: its
 * reduction scratch is a fixed device array of COSMOS_NOALLOC_MAX_ROWS rows (640 KB, held on
 * every device that loads the library), so grids with more rows are rejected (COSMOS_EINVAL).
 * The first call on a device looks up that array's device address (make it before any stream
 * capture); the address is kept, so do not call it again after a cudaDeviceReset.  All calls
 * share the array: calls whose kernels overlap on the GPU race.  A CUDA error already pending
 * when it is called is returned (COSMOS_ECUDA) before anything is enqueued. */
#define COSMOS_NOALLOC_MAX_ROWS 16384
int cosmos_field_sums_noalloc(const void* state, int precision, int nx, int ny, int pitch, size_t field_stride,
                              double* out5, void* stream);

/* One-shot drop-in for the reference's static solve entry points with host buffers:
 * prim_in/prim_out are 5*nx*ny doubles (may alias). */
int cosmos_solve_prim(const cosmos_params* p, const double* prim_in, double* prim_out, const cosmos_solve_opts* o,
                      cosmos_solve_result* r);

#ifdef __cplusplus
}
#endif

#endif /* COSMOS_GB300_H */
