// Bulk asynchronous copies (TMA: cp.async.bulk, and cp.async.bulk.tensor on a tensor map) from
// global to shared memory completing on shared-memory mbarriers, and bounded waits on them.  All
// inline PTX written here; sm_90+ forms.
#pragma once
#include <cuda.h>  // CUtensorMap (the descriptor type only; no driver call is linked)

#include <cstdint>

#include "device_common.cuh"

namespace cg {

CG_D uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// One-shot barrier for `count` arrivals (plus the transaction bytes announced by expect_tx).
CG_D void mbar_init(unsigned long long* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
// Invalidates a barrier that has no phase pending, before it is initialised again.
CG_D void mbar_inval(unsigned long long* bar) {
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_addr(bar)) : "memory");
}
// Makes the initialised barriers visible to the copy engine; the caller follows with __syncthreads.
CG_D void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// Arrive once and announce `bytes` of copies that complete this phase.
CG_D void mbar_expect_tx(unsigned long long* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

// Copy `bytes` (a multiple of 16; both addresses 16-byte aligned) from global to shared memory,
// counted against `bar`.
CG_D void bulk_load(void* dst, const void* src, uint32_t bytes, unsigned long long* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

// Copy one box of a 3-D tensor map (x, row, field) to shared memory (128-byte aligned), counted
// against `bar`.  The box's bytes complete the phase in full, parts outside the tensor as zeros.
// x times the element size must be a multiple of 16 bytes.  `map` is the address of a
// __grid_constant__ kernel parameter.
CG_D void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
        : "memory");
}

// Wait until phase `parity` of `bar` has completed.  Gives up after about `cycles` SM clocks and
// returns false (the copies it waited for are then still counted as in flight by the caller).
CG_D bool mbar_wait(unsigned long long* bar, uint32_t parity, long long cycles = 2000000000LL) {
    const uint32_t a = smem_addr(bar);
    long long t0 = -1;
    for (;;) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
        const long long t = clock64();  // the clock is read only once the phase is late
        if (t0 < 0) t0 = t;
        else if (t - t0 > cycles) return false;
    }
}

}  // namespace cg
