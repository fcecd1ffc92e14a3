// Bulk asynchronous copies (TMA, cp.async.bulk) into shared memory with
// mbarrier completion, and bounded waits on those barriers.
#pragma once

#include <stdint.h>

#include "tg_common.cuh"

namespace tg {

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;"
                 :: "r"(smem_u32(bar)), "r"(count) : "memory");
}

// Makes barrier initialisation visible to the async (TMA) proxy.
__device__ __forceinline__ void mbar_init_fence()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar,
                                                      uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                 :: "r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// Global -> shared bulk copy.  Both addresses 16-byte aligned, `bytes` a
// multiple of 16; completion is signalled as transaction bytes on `bar`.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src,
                                         uint32_t bytes, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
        "[%0], [%1], %2, [%3];"
        :: "r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok) : "r"(smem_u32(bar)), "r"(parity) : "memory");
    return ok != 0;
}

// Each try_wait suspends the thread for a bounded, implementation-defined
// time; this many failed tries (well above any healthy copy latency) mean
// the copy will not complete.
constexpr uint32_t MBAR_SPIN_LIMIT = 1u << 20;

// Returns false (and records DERR_PIPE_TIMEOUT) if the phase did not
// complete within `limit` tries (MBAR_SPIN_LIMIT by default).  The sweeps'
// main-loop waits take the limit from their launch descriptor
// (pipe_spin_limit(), settable from the host) so that the timeout path can
// be exercised; the waits that drain copies still in flight before a CTA
// returns always use the full bound.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar,
                                                  uint32_t parity,
                                                  unsigned *err,
                                                  uint32_t limit = MBAR_SPIN_LIMIT)
{
    for (uint32_t k = 0; k < limit; ++k)
        if (mbar_try_wait(bar, parity)) return true;
    atomicOr(err, (unsigned)DERR_PIPE_TIMEOUT);
    return false;
}

}  // namespace tg
