// FP32 bulk kernels (Newtonian system; the SR system's live in kernels_sr_fast.cu): conserved SoA float storage, FMA contraction on.
#include <cudaTypedefs.h>  // PFN_cuTensorMapEncodeTiled

#include <atomic>

#include "launch.h"
#include "policies.cuh"
#include "sweep_pairs.cuh"

namespace cg {

namespace {

constexpr int kXThreads = 256;  // X sweep tile: 256 evolutions, 255 fluxes, 254 updates
constexpr int kYThreads = 128;
constexpr int kYSeg = 32;
constexpr int kXPairSegs = 3;      // 60-cell segments per one-warp block (4096^2: 0.145 ms against 0.149 with 2)
constexpr int kXRingMinBlocks = 32;  // at most 64 registers: 32 one-warp blocks per SM
constexpr int kYPairThreads = 32;  // one warp (64 columns, two per thread) per block: 0.154 ms at 4096^2
                                   // against 0.168 with two warps per block at the same registers
constexpr int kYRingRows = 8;      // Y rows staged in shared memory per warp (up to 8 in flight)
constexpr int kYRingMinBlocks = 16;  // at most 128 registers: 16 one-warp blocks per SM

// Rows per Y-sweep block: about 32 (each block re-reads four halo rows), adjusted so that the
// blocks fill whole waves of the resident slots.  At 4096^2, 32-row segments make 8192 one-warp
// blocks for 152 x 16 slots (3.37 waves, the last a third full); 36-row segments make 7296, three
// full waves.
int y_ring_seg(const void* kernel, int nx, int ny) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kYPairThreads, 0) != cudaSuccess || per_sm < 1)
        per_sm = kYRingMinBlocks;
    const long long slots = (long long)per_sm * device_sm_count();
    const long long cols = (nx + 2 * kYPairThreads - 1) / (2 * kYPairThreads);
    const long long blocks32 = cols * ((ny + 31) / 32);
    const long long waves = blocks32 / slots > 1 ? blocks32 / slots : 1;
    long long rows = waves * slots / cols;  // block rows that fill `waves` whole waves
    if (rows < 1) rows = 1;
    int seg = (int)((ny + rows - 1) / rows);
    return seg < 8 ? 8 : (seg > 64 ? 64 : seg);
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (nullptr when the driver does
// not provide it).
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    return fn;
}

}  // namespace

std::atomic<int> g_tensor_maps{1};

bool field_map(CUtensorMap* m, const float* base, const Geom& G, unsigned box_x) {
    if (!g_tensor_maps.load(std::memory_order_relaxed)) return false;
    const auto encode = tensor_map_encoder();
    if (!encode || ((uintptr_t)base & 15) || box_x > 256 || (box_x * 4) % 16) return false;
    const cuuint64_t dim[3] = {(cuuint64_t)G.nx, (cuuint64_t)G.ny, 5};
    const cuuint64_t stride[2] = {(cuuint64_t)G.pitch * 4, (cuuint64_t)G.fstride * 4};
    const cuuint32_t box[3] = {box_x, 1, 5}, estride[3] = {1, 1, 1};
    return encode(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dim, stride, box, estride,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

namespace {

template <int AXIS, int LIM, bool MASKED>
NewtonFastPolicy<AXIS, LIM, MASKED> make_fast(const SweepArgs& a) {
    return make_newton_fast<AXIS, LIM, MASKED>(a.gamma, a.bias, a.G.nx, a.G.dims);
}

template <int AXIS, int LIM, bool MASKED>
cudaError_t run_fast(const SweepArgs& a) {
    const Geom& G = a.G;
    const float* src = (const float*)a.src;
    float* dst = (float*)a.dst;
    auto pol = make_fast<AXIS, LIM, MASKED>(a);
    using Pol = decltype(pol);
    if constexpr (AXIS == 0) {
        if (a.order == 2 && !MASKED) {
            const int segs = (G.nx + 59) / 60;
            dim3 grid((segs + kXPairSegs - 1) / kXPairSegs, G.ny);
            CUtensorMap tm{};
            const bool ws = a.out.slot_set();
            // One tensor-map copy per segment only in the sweep that reduces the CFL maximum: there
            // it measured 3 % faster than five per-field copies, in the other sweep (at the
            // 64-register cap) 3 % slower.
            const bool use_tm = ws && field_map(&tm, src, G, 68);
            auto kernel = ws ? (use_tm ? sweep_x_ring_kernel<LIM, kXPairSegs, kXRingMinBlocks, true, true>
                                       : sweep_x_ring_kernel<LIM, kXPairSegs, kXRingMinBlocks, true, false>)
                             : sweep_x_ring_kernel<LIM, kXPairSegs, kXRingMinBlocks, false, false>;
            kernel<<<grid, 32, 0, a.stream>>>(pol.P, G.dims, G, src, dst, a.ds, a.out, tm);
            return cudaSuccess;
        }
        dim3 grid((G.nx + kXThreads - 3) / (kXThreads - 2), G.ny);
        if (a.order == 2) sweep_x_own_kernel<Pol, 2, kXThreads><<<grid, kXThreads, 0, a.stream>>>(pol, G, src, dst, a.ds, a.out);
        else sweep_x_own_kernel<Pol, 1, kXThreads><<<grid, kXThreads, 0, a.stream>>>(pol, G, src, dst, a.ds, a.out);
    } else if (a.order == 2 && !MASKED) {
        CUtensorMap tm{};
        const bool use_tm = field_map(&tm, src, G, 64);  // 4096^2: 0.136 ms against 0.150 with per-field copies
        auto kernel = use_tm ? sweep_y_ring_kernel<LIM, kYPairThreads, kYRingRows, kYRingMinBlocks, true>
                             : sweep_y_ring_kernel<LIM, kYPairThreads, kYRingRows, kYRingMinBlocks, false>;
        const int seg = y_ring_seg((const void*)kernel, G.nx, G.ny);
        dim3 grid((G.nx + 2 * kYPairThreads - 1) / (2 * kYPairThreads), (G.ny + seg - 1) / seg);
        kernel<<<grid, kYPairThreads, 0, a.stream>>>(pol.P, G.dims, G, src, dst, a.ds, a.out, seg, tm);
        return cudaSuccess;
    } else {
        dim3 grid((G.nx + kYThreads - 1) / kYThreads, (G.ny + kYSeg - 1) / kYSeg);
        if (a.order == 2) sweep_y_kernel<Pol, 2, kYThreads, kYSeg><<<grid, kYThreads, 0, a.stream>>>(pol, G, src, dst, a.ds, a.out);
        else sweep_y_kernel<Pol, 1, kYThreads, kYSeg><<<grid, kYThreads, 0, a.stream>>>(pol, G, src, dst, a.ds, a.out);
    }
    return cudaSuccess;
}

template <int AXIS, bool MASKED>
cudaError_t run_fast_lim(const SweepArgs& a) {
    if (a.lim == 0) return run_fast<AXIS, 0, MASKED>(a);
    if (a.lim == 1) return run_fast<AXIS, 1, MASKED>(a);
    return run_fast<AXIS, 2, MASKED>(a);  // Solvers/SlopeLimiters.cpp:66: any other id is MinBee
}

}  // namespace

cudaError_t launch_sweep_fast(const SweepArgs& a) {
    if (a.system == 1) return launch_sweep_sr_fast(a);
    if (a.system == 2) return launch_sweep_gr_fast(a);
    if (a.system != 0) return cudaErrorNotSupported;
    const bool masked = a.out.mask != nullptr;
    cudaError_t e;
    if (a.G.axis == 0) e = masked ? run_fast_lim<0, true>(a) : run_fast_lim<0, false>(a);
    else e = masked ? run_fast_lim<1, true>(a) : run_fast_lim<1, false>(a);
    count_launch();
    return e != cudaSuccess ? e : cudaGetLastError();
}

cudaError_t launch_wavespeed_fast(const SweepArgs& a, unsigned long long* slot) {
    if (a.system == 1) return launch_wavespeed_sr_fast(a, slot);
    if (a.system == 2) return launch_wavespeed_gr_fast(a, slot);
    if (a.system != 0) return cudaErrorNotSupported;
    constexpr int NT = 256;
    SweepArgs b = a;
    b.G.axis = 0;
    SweepOut o = a.out;
    if (slot) { o.smax = slot; o.ws_ctl = nullptr; }
    const size_t n = (size_t)a.G.nx * a.G.ny;
    int blocks = (int)((n + NT - 1) / NT);
    if (blocks > device_sm_count() * 16) blocks = device_sm_count() * 16;
    auto pol = make_fast<0, 2, false>(b);
    wavespeed_kernel<decltype(pol), NT><<<blocks, NT, 0, a.stream>>>(pol, b.G, (const float*)a.src, o);
    count_launch();
    return cudaGetLastError();
}

// Primitive (double, AoS) -> conserved FP32 SoA (Euler/EulerStateVector.cpp:55-66), formed in
// FP64 and rounded once; E = rho v^2 / 2 + p / (gamma - 1) with the reciprocal hoisted (no
// per-cell FP64 division: GB300's FP64 divide costs as much as the whole conversion).
__global__ void prim_in_fast_kernel(const double* __restrict__ aos, float* __restrict__ soa, Geom G, double gamma) {
    const size_t n = (size_t)G.nx * G.ny;
    const double igm1 = 1.0 / (gamma - 1.0);
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
        const size_t i = c / G.nx, j = c % G.nx, k = i * G.pitch + j;
        const double* p = aos + 5 * c;
        const double rho = p[0], vx = p[1], vy = p[2], vz = p[3];
        soa[k] = (float)rho;
        soa[G.fstride + k] = (float)(rho * vx);
        soa[2 * G.fstride + k] = (float)(rho * vy);
        soa[3 * G.fstride + k] = (float)(rho * vz);
        soa[4 * G.fstride + k] = (float)(0.5 * rho * (vx * vx + vy * vy + vz * vz) + p[4] * igm1);
    }
}
// Conserved FP32 -> primitives (double, AoS) (Euler/EulerStateVector.cpp:30-40): 1 / rho from an
// FP32 reciprocal refined by one FP64 Newton step (relative error ~1e-14, no FP64 division).
__global__ void prim_out_fast_kernel(const float* __restrict__ soa, double* __restrict__ aos, Geom G, double gamma) {
    const size_t n = (size_t)G.nx * G.ny;
    const double gm1 = gamma - 1.0;
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
        const size_t i = c / G.nx, j = c % G.nx, k = i * G.pitch + j;
        const double rho = soa[k], m1 = soa[G.fstride + k], m2 = soa[2 * G.fstride + k], m3 = soa[3 * G.fstride + k];
        const double E = soa[4 * G.fstride + k];
        double ir = (double)__frcp_rn((float)rho);
        ir = ir * (2.0 - rho * ir);
        ir = ir * (2.0 - rho * ir);
        const double vx = m1 * ir, vy = m2 * ir, vz = m3 * ir;
        double* p = aos + 5 * c;
        p[0] = rho;
        p[1] = vx;
        p[2] = vy;
        p[3] = vz;
        p[4] = gm1 * (E - 0.5 * (m1 * vx + m2 * vy + m3 * vz));
    }
}
static int grid_for(size_t n) {
    size_t b = (n + 255) / 256;
    return (int)(b > device_sm_count() * 32 ? device_sm_count() * 32 : (b ? b : 1));
}
cudaError_t launch_prim_in_fast(const double* aos, void* soa, const Geom& G, int system, double gamma, cudaStream_t st) {
    if (system == 1) return launch_prim_in_sr_fast(aos, soa, G, gamma, st);
    if (system != 0) return cudaErrorNotSupported;
    prim_in_fast_kernel<<<grid_for((size_t)G.nx * G.ny), 256, 0, st>>>(aos, (float*)soa, G, gamma);
    count_launch();
    return cudaGetLastError();
}
cudaError_t launch_prim_out_fast(const void* soa, double* aos, const Geom& G, int system, double gamma, cudaStream_t st) {
    if (system == 1) return launch_prim_out_sr_fast(soa, aos, G, gamma, st);
    if (system != 0) return cudaErrorNotSupported;
    prim_out_fast_kernel<<<grid_for((size_t)G.nx * G.ny), 256, 0, st>>>((const float*)soa, aos, G, gamma);
    count_launch();
    return cudaGetLastError();
}

}  // namespace cg

extern "C" int cosmos_set_tensor_maps(int enable) { return cg::g_tensor_maps.exchange(enable ? 1 : 0); }
