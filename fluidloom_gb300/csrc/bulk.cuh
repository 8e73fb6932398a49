// bulk.cuh — the TMA engine's linear (non-tensor) bulk copies from global to
// shared memory, completed on a shared-memory mbarrier (PTX ISA:
// cp.async.bulk, mbarrier.arrive.expect_tx, mbarrier.try_wait.parity).
//
// Rules the callers keep: source and destination 16-byte aligned, sizes a
// multiple of 16 bytes; one thread arms the barrier with the phase's total
// byte count before issuing that phase's copies; every issued phase is waited
// for before the block exits.  Waits are bounded: a wait that runs out
// reports false and the caller records FL_DEVSTAT_TIMEOUT instead of hanging.
#pragma once
#include <cstdint>

namespace flbulk {

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t arrivals) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(arrivals) : "memory");
    // make the initialised barrier visible to the async (copy) proxy
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// One arrival that also adds `bytes` to the transactions the phase waits for.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

// Global -> this CTA's shared memory, `bytes` (multiple of 16) counted on bar.
__device__ __forceinline__ void copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// Wait for the phase with this parity to complete, at most `limit` polls
// (each try_wait may itself suspend the thread for a short time).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t limit) {
    for (uint32_t i = 0; i < limit; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

}  // namespace flbulk
