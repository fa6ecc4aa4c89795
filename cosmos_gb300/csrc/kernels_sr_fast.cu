// FP32 bulk kernels of the special-relativistic system: conserved SoA float storage, FMA
// contraction on, primitive recovery finishing in FP64 (physics_sr_fast.cuh).
#include "launch.h"
#include "policies.cuh"

namespace cg {

namespace {

constexpr int kXThreads = 256;
constexpr int kYThreads = 128;
constexpr int kYSeg = 32;

template <int AXIS, int LIM, bool MASKED>
SRFastPolicy<AXIS, LIM, MASKED> make_pol(const SweepArgs& a) {
    return make_sr_fast<AXIS, LIM, MASKED>(a.gamma, a.bias, a.G.nx, a.G.dims, a.c2p64_above);
}

template <int AXIS, int LIM, bool MASKED>
void run(const SweepArgs& a) {
    const Geom& G = a.G;
    const float* src = (const float*)a.src;
    float* dst = (float*)a.dst;
    auto pol = make_pol<AXIS, LIM, MASKED>(a);
    using Pol = decltype(pol);
    if constexpr (AXIS == 0) {
        dim3 grid((G.nx + kXThreads - 3) / (kXThreads - 2), G.ny);
        if (a.order == 2) sweep_x_own_kernel<Pol, 2, kXThreads><<<grid, kXThreads, 0, a.stream>>>(pol, G, src, dst, a.ds, a.out);
        else sweep_x_own_kernel<Pol, 1, kXThreads><<<grid, kXThreads, 0, a.stream>>>(pol, G, src, dst, a.ds, a.out);
    } else {
        dim3 grid((G.nx + kYThreads - 1) / kYThreads, (G.ny + kYSeg - 1) / kYSeg);
        if (a.order == 2) sweep_y_kernel<Pol, 2, kYThreads, kYSeg><<<grid, kYThreads, 0, a.stream>>>(pol, G, src, dst, a.ds, a.out);
        else sweep_y_kernel<Pol, 1, kYThreads, kYSeg><<<grid, kYThreads, 0, a.stream>>>(pol, G, src, dst, a.ds, a.out);
    }
}

template <int AXIS, bool MASKED>
void run_lim(const SweepArgs& a) {
    if (a.lim == 0) run<AXIS, 0, MASKED>(a);
    else if (a.lim == 1) run<AXIS, 1, MASKED>(a);
    else run<AXIS, 2, MASKED>(a);
}

// Primitive (double, AoS) -> conserved FP32 SoA with the reference's FP64 formula
// (RelativisticEuler/RelativisticEulerStateVector.cpp:116-136), rounded once.
__global__ void sr_prim_in_kernel(const double* __restrict__ aos, float* __restrict__ soa, Geom G, double gamma) {
    const size_t n = (size_t)G.nx * G.ny;
    SRExact S{gamma, nullptr};
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
        const size_t i = c / G.nx, j = c % G.nx;
        double u[5];
        S.cons(aos + 5 * c, Pt{0, 0, 0}, u);
#pragma unroll
        for (int f = 0; f < 5; f++) soa[f * G.fstride + i * G.pitch + j] = (float)u[f];
    }
}
// Conserved FP32 -> primitives with the reference's full FP64 recovery.
__global__ void sr_prim_out_kernel(const float* __restrict__ soa, double* __restrict__ aos, Geom G, double gamma) {
    const size_t n = (size_t)G.nx * G.ny;
    SRExact S{gamma, nullptr};
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
        const size_t i = c / G.nx, j = c % G.nx;
        double u[5];
#pragma unroll
        for (int f = 0; f < 5; f++) u[f] = (double)soa[f * G.fstride + i * G.pitch + j];
        S.prim(u, Pt{0, 0, 0}, aos + 5 * c);
    }
}
int grid_for(size_t n) {
    size_t b = (n + 255) / 256;
    return (int)(b > device_sm_count() * 32 ? device_sm_count() * 32 : (b ? b : 1));
}

}  // namespace

cudaError_t launch_sweep_sr_fast(const SweepArgs& a) {
    const bool masked = a.out.mask != nullptr;
    if (a.G.axis == 0) masked ? run_lim<0, true>(a) : run_lim<0, false>(a);
    else masked ? run_lim<1, true>(a) : run_lim<1, false>(a);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_wavespeed_sr_fast(const SweepArgs& a, unsigned long long* slot) {
    constexpr int NT = 256;
    SweepArgs b = a;
    b.G.axis = 0;
    SweepOut o = a.out;
    if (slot) { o.smax = slot; o.ws_ctl = nullptr; }
    const size_t n = (size_t)a.G.nx * a.G.ny;
    int blocks = (int)((n + NT - 1) / NT);
    if (blocks > device_sm_count() * 16) blocks = device_sm_count() * 16;
    auto pol = make_pol<0, 2, false>(b);
    wavespeed_kernel<decltype(pol), NT><<<blocks, NT, 0, a.stream>>>(pol, b.G, (const float*)a.src, o);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_prim_in_sr_fast(const double* aos, void* soa, const Geom& G, double gamma, cudaStream_t st) {
    sr_prim_in_kernel<<<grid_for((size_t)G.nx * G.ny), 256, 0, st>>>(aos, (float*)soa, G, gamma);
    count_launch();
    return cudaGetLastError();
}
cudaError_t launch_prim_out_sr_fast(const void* soa, double* aos, const Geom& G, double gamma, cudaStream_t st) {
    sr_prim_out_kernel<<<grid_for((size_t)G.nx * G.ny), 256, 0, st>>>((const float*)soa, aos, G, gamma);
    count_launch();
    return cudaGetLastError();
}

}  // namespace cg
