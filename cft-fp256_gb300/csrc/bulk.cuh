// bulk.cuh - shared-memory staging by the Tensor Memory Accelerator's bulk
// copies (cp.async.bulk, global -> shared) completed on an mbarrier, with
// every wait bounded in time.
//
// Rules the callers keep: a copy's global source, its shared destination and
// its size are multiples of 16 bytes; one mbarrier tracks one stage, is
// initialised with an arrival count of 1 and is armed by one
// arrive.expect_tx for the stage's total bytes before the copies are issued.
#pragma once
#include <cstdint>

#ifndef SFD
#define SFD __device__ __forceinline__
#endif

namespace cftg {
namespace bulk {

SFD uint32_t saddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

SFD void bar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(bar)), "r"(count) : "memory");
}

// Makes barrier initialisation and earlier generic-proxy accesses to shared
// memory visible to the async proxy (the bulk copies) before they are used.
SFD void fence_async_shared()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

SFD void bar_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(bar)),
                 "r"(bytes)
                 : "memory");
}

// bytes from global src to shared dst; completion is counted on *bar.
SFD void copy_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            saddr(dst)),
        "l"(src), "r"(bytes), "r"(saddr(bar))
        : "memory");
}

SFD bool bar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(saddr(bar)), "r"(parity)
        : "memory");
    return ok != 0u;
}

SFD uint64_t now_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Waits for the phase of parity `parity` to complete, for at most limit_ns
// nanoseconds of the global timer; false when the limit ran out.
SFD bool bar_wait(uint64_t *bar, uint32_t parity, uint64_t limit_ns)
{
    if (bar_try_wait(bar, parity)) return true;
    const uint64_t t0 = now_ns();
    for (;;) {
        if (bar_try_wait(bar, parity)) return true;
        if (now_ns() - t0 > limit_ns) return false;
    }
}

}  // namespace bulk
}  // namespace cftg
