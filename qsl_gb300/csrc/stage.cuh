// stage.cuh -- bulk asynchronous copies into shared memory, completed on
// an mbarrier: the staging of the warp-tiled sweeps (gates.cu).
//
// A warp owns a few buffers of shared memory, each with its own mbarrier.
// Lane 0 arms a buffer's barrier with the bytes it expects and issues the
// bulk copies (cp.async.bulk, global -> shared) that complete on it; the
// warp then waits on the barrier's phase before reading the buffer.  While
// the warp computes on one buffer, the copies of the next ones are in
// flight, so the arithmetic does not wait on global-memory latency and no
// registers are spent on prefetching.
//
// Every wait is bounded (STAGE_WAIT_LIMIT polls of try_wait, which itself
// suspends for a while before it gives up); a wait that runs out reports
// failure to the caller, which records an error word and stops.
#pragma once

#include <cstdint>

namespace qslc {

constexpr long long STAGE_WAIT_LIMIT = 1ll << 20;

__device__ __forceinline__ uint32_t smem_addr(const void *p)
{
    return uint32_t(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
}

// Make the initialised barriers visible to the async proxy (the bulk copies).
__device__ __forceinline__ void mbar_init_fence()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Order this warp's earlier shared-memory reads (generic proxy) before the
// async proxy's later writes into the same buffer.
__device__ __forceinline__ void fence_proxy_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect(uint32_t mbar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
}

// Global -> shared bulk copy of `bytes` (a multiple of 16; both addresses
// 16-byte aligned), completing `bytes` of the barrier's transaction count.
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes, uint32_t mbar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
        "l"(src), "r"(bytes), "r"(mbar)
        : "memory");
}

// Bounded wait for the barrier's phase `parity` to complete.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t mbar, uint32_t parity)
{
    uint32_t done = 0;
    for (long long it = 0; it < STAGE_WAIT_LIMIT && !done; it++) {
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            "selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
    }
    return done != 0;
}

}  // namespace qslc
