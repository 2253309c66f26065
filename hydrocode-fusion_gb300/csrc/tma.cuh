// tma.cuh -- tensor-memory-accelerator tile copies and mbarriers (inline PTX,
// sm_90 and later; used here on sm_103a).
//
// A copy is issued by one thread: mbarrier.arrive.expect_tx announces the
// bytes of the stage, cp.async.bulk.tensor writes the box into shared memory
// and completes those bytes on the mbarrier, and the consumers wait on the
// barrier's phase.  Every wait is bounded (global timer plus a poll cap):
// a wait that gives up returns false and the caller reports an error instead
// of spinning for ever.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace hydro {

__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ unsigned long long timer_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// Makes initialised mbarriers visible to the async proxy (the TMA unit).
__device__ __forceinline__ void fence_mbar_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Orders this CTA's earlier generic-proxy shared-memory accesses before
// later async-proxy (TMA) writes to the same memory.
__device__ __forceinline__ void fence_proxy_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t done;
    asm volatile(
        "{\n"
        " .reg .pred p;\n"
        " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// Waits for the phase with the given parity to complete; false after about
// limit_ns nanoseconds (or 2^26 polls) without completion.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, unsigned long long limit_ns)
{
    if (mbar_try_wait(bar, parity))
        return true;
    const unsigned long long t0 = timer_ns();
    for (uint32_t polls = 1; polls < (1u << 26); ++polls) {
        if (mbar_try_wait(bar, parity))
            return true;
        if ((polls & 255u) == 0u && timer_ns() - t0 > limit_ns)
            return false;
    }
    return false;
}

// 3D tiled copy global -> shared of the box at (x, y, z) (x innermost); x
// times the element size must be a multiple of 16 bytes.
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ void tma_prefetch_desc(const CUtensorMap* map)
{
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

// TMA descriptors of the state a step reads: its 5 value planes and its 8
// previous-slope planes.
struct StepMaps {
    CUtensorMap vals;
    CUtensorMap slopes;
};

}  // namespace hydro
