// Batched persistent launch, FP32 Newtonian system on cell pairs (sweep_pairs.cuh).
#include "batch_kernels.cuh"
#include "launch.h"

namespace cg {

namespace {

template <int LIM, int NT, int CAP>
struct FastBatch {
    static constexpr int MINB = CAP ? 512 / NT : 1;  // cap: at most 128 registers
    // the rings' dynamic shared memory (above the 48 KB default for 256 threads)
    static void* fn() {
        auto k = batch_pair_kernel<LIM, NT, MINB>;
        if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)batch_pair_smem(NT)) != cudaSuccess)
            return nullptr;
        return (void*)k;
    }
    static cudaError_t launch(const BatchLaunch& L) {
        if (!fn()) return cudaErrorInvalidValue;
        const NewtonFastParams P = make_newton_fast<0, LIM, false>(L.gamma, L.bias, 0, 2).P;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(L.blocks);
        cfg.blockDim = dim3(NT);
        cfg.dynamicSmemBytes = batch_pair_smem(NT);
        cfg.stream = L.stream;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        return cudaLaunchKernelEx(&cfg, batch_pair_kernel<LIM, NT, MINB>, P, *L.B, L.nsteps);
    }
};

// Dispatch over the kernel variants: threads per block and register cap.
template <int LIM, class F>
auto by_shape(int nt, int cap, F&& f) -> decltype(f(FastBatch<LIM, 128, 0>())) {
    if (nt == 128) return cap ? f(FastBatch<LIM, 128, 1>()) : f(FastBatch<LIM, 128, 0>());
    return cap ? f(FastBatch<LIM, 256, 1>()) : f(FastBatch<LIM, 256, 0>());
}

template <class F>
auto by_lim(int lim, int nt, int cap, F&& f) -> decltype(f(FastBatch<0, 128, 0>())) {
    if (lim == 0) return by_shape<0>(nt, cap, f);
    if (lim == 1) return by_shape<1>(nt, cap, f);
    return by_shape<2>(nt, cap, f);
}

}  // namespace

cudaError_t launch_batch_fast(const BatchLaunch& L) {
    if (L.nt != 128 && L.nt != 256) return cudaErrorInvalidValue;
    cudaError_t e = by_lim(L.lim, L.nt, L.cap, [&](auto k) { return decltype(k)::launch(L); });
    count_launch();
    return e;
}

size_t batch_fast_smem(int nt) { return batch_pair_smem(nt); }

void* batch_fast_fn(int nt, int cap, int lim) {
    if (nt != 128 && nt != 256) return nullptr;
    return by_lim(lim, nt, cap, [](auto k) { return decltype(k)::fn(); });
}

}  // namespace cg
