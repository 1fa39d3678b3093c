/*
 * tma.cuh — tensor-memory-access (TMA) tile loads for sm_103a in inline PTX: a CTA-scope
 * mbarrier per stage, cp.async.bulk.tensor loads that complete on it, and a bounded wait.
 *
 * Every wait has an iteration limit: a wait that runs out returns false, the kernel records
 * ERR_WAIT and stops using the stage, so no launch can spin without end.
 */
#pragma once

#include <cuda.h> /* CUtensorMap */
#include <cuda_runtime.h>

namespace slvof {
namespace tma {

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void bar_init(unsigned long long* bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

/* make the initialised barriers visible to the async proxy (the TMA unit) */
__device__ __forceinline__ void fence_bar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

/* order this thread's earlier shared-memory accesses (generic proxy) before later bulk copies
 * into the same bytes (async proxy) */
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

/* one arrival that also announces `bytes` of bulk-copy transactions for the current phase */
__device__ __forceinline__ void bar_arrive_expect(unsigned long long* bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool bar_test(unsigned long long* bar, unsigned parity)
{
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

/* wait for the phase of the given parity to complete; false after `limit` polls */
__device__ __forceinline__ bool bar_wait(unsigned long long* bar, unsigned parity, int limit = 1 << 22)
{
    for (int it = 0; it < limit; ++it) {
        if (bar_test(bar, parity)) return true;
        if (it > 64) __nanosleep(64);
    }
    return false;
}

/* 3D tile load of the tensor map's box at element coordinates (x, y, z) into shared memory;
 * x times the element size must be a multiple of 16 bytes, dst 128-byte aligned */
__device__ __forceinline__ void load_3d(void* dst, const CUtensorMap* map, int x, int y, int z,
                                        unsigned long long* bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_addr(dst)),
        "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
        : "memory");
}

} // namespace tma
} // namespace slvof
