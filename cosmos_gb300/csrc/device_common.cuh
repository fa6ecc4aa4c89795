// Shared device-side definitions for the cosmos_gb300 kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace cg {

#define CG_HD __host__ __device__ __forceinline__
#define CG_D __device__ __forceinline__

struct Pt { double x, y, z; };

// Streaming multiprocessors of the current device (host code; cached per device): grid-stride
// launches size their grids as a multiple of it.
int device_sm_count();

CG_HD Pt shift_pt(Pt p, int axis, double d) {
    if (axis == 0) p.x = p.x + d; else p.y = p.y + d;
    return p;
}

template <class T> struct V5 { T v[5]; };

// Ghost-cell index along a line of n cells.  Transmissive mirrors the reference's
// insertBoundaryCells (Solvers/EulerSolvers.cpp:13-19, :52-73): g[-1]=c[0], g[-2]=c[1],
// g[n]=c[n-1], g[n+1]=c[n-2].  Periodic wraps (an extension; the reference has no periodic BC).
// k is at most two cells outside [0, n) and n >= 2, so no modulo is needed.
CG_HD int ghost_index(int k, int n, int bc) {
    if (k < 0) return bc == 1 ? k + n : -1 - k;
    if (k >= n) return bc == 1 ? k - n : 2 * n - 1 - k;
    return k;
}

// A cell whose density or energy (FP64 grids: pressure) is not finite gets an infinite CFL speed:
// the step's time step becomes zero and the run reports a non-finite time step
// (COSMOS_STATUS_NONFINITE / COSMOS_ENONFINITE), where the reference carries the NaN on (its
// `if (w > max)` drops a NaN speed).  Finite states keep the reference's speed bit for bit.
CG_HD double speed_or_inf(double a, double b, double ws) { return isfinite(a + b) ? ws : (double)INFINITY; }
CG_HD float speed_or_inf(float a, float b, float ws) { return fabsf(a + b) < INFINITY ? ws : INFINITY; }

// std::min / std::max semantics as used by the reference.
template <class T> CG_HD T mn(T a, T b) { return (b < a) ? b : a; }
template <class T> CG_HD T mx(T a, T b) { return (a < b) ? b : a; }

// FP32 sweep coefficients for one time step: dt/dx, dt/(2 dx), dx/(4 dt).
struct FastCoef { float dtdx, half_dtdx, q_dxdt; };

CG_HD FastCoef make_fast_coef(double dt, double dx) {
    return FastCoef{(float)(dt / dx), (float)(0.5 * (dt / dx)), (float)(0.25 * (dx / dt))};
}

// Device-resident step controller.  The time step is computed on the device from the last
// wavespeed reduction so that whole runs replay from a captured CUDA graph with no host sync.
struct StepCtl {
    double t;          // simulation time at the start of the current step
    double t_final;
    double cfl;
    double dx;
    double dt;         // the current step's dt (0 when inactive)
    int it;            // completed steps (the reference's currentIteration)
    int it_limit;      // stop after this many steps (INT_MAX for none)
    int active;        // 1 while the current step runs, 0 once t >= t_final or it >= it_limit
    int status;        // sticky error bits, see COSMOS_STATUS_* in the public header
    unsigned long long smax[2];  // wavespeed maxima (bit patterns of non-negative doubles), ping-pong by it parity
    FastCoef fc[2];    // FP32 coefficients of dt (fc[0]) and dt/2 (fc[1]), formed by the dt kernel
    double* dt_log;           // non-null: the dt kernel records each step's dt at dt_log[it]
    const double* dt_fixed;   // non-null: step `it` takes dt_fixed[it] instead of the CFL rule
};

// Status bits written by kernels (mirrored in include/cosmos_gb300.h)
enum : int {
    ST_NONFINITE = 1,       // a non-finite state was produced
    ST_NEWTON_CAP = 2,      // a con2prim Newton solve stopped at its iteration cap
    ST_TIMEOUT = 4,         // a bounded device wait gave up
    ST_NEGATIVE = 8,        // non-positive density or pressure produced by the FP32 path
};

// Max of non-negative doubles (ordering of their bit patterns equals numeric ordering).
// The slot only grows while a kernel reduces into it, so a block whose value does not exceed what
// an L2 read already finds there skips the atomic: with one block per 120 cells of a 4096^2 sweep,
// unconditional atomics on one address serialise into about 0.1 ms per launch.
CG_D void atomic_max_nonneg(unsigned long long* slot, double v) {
    if (!(v > 0.0)) return;  // also drops NaN, like the reference's `if (w > max)` test
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    if (__ldcg(slot) >= b) return;
    atomicMax(slot, b);
}

template <class W>
CG_D W warp_max(W v) {
    for (int o = 16; o > 0; o >>= 1) {
        W w = __shfl_xor_sync(0xffffffffu, v, o);
        v = (w > v) ? w : v;
    }
    return v;
}

// Block-wide max reduction into *slot; every thread passes its value (0 if none).  W is the
// policy's arithmetic type (float for the FP32 path, so no FP64 instruction runs per cell).
template <int NT, class W>
CG_D void block_max_to(unsigned long long* slot, W v) {
    __shared__ W red[NT / 32];
    v = warp_max(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) red[wid] = v;
    __syncthreads();
    if (wid == 0) {
        W w = lane < NT / 32 ? red[lane] : W(0);
        w = warp_max(w);
        if (lane == 0) atomic_max_nonneg(slot, (double)w);
    }
}

}  // namespace cg
