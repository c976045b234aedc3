// Inline-PTX helpers shared by the kernels that stage operands with the bulk
// copy engine (cp.async.bulk) and wait on shared-memory mbarriers.
//
// Every wait is bounded: a caller that sees `false` records an error, lets the
// copies it issued finish (again with a bounded wait) and returns, so a kernel
// never spins forever on a transfer that does not arrive.
#pragma once

#include <cstdint>

namespace sc {

static constexpr long long kMbarWaitLimit = 1LL << 24;   // polls before a wait gives up

__device__ __forceinline__ uint32_t smem_addr(const void *p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *mbar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_addr(mbar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_init_fence()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ bool mbar_try(uint64_t *mbar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.b32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok) : "r"(smem_addr(mbar)), "r"(parity) : "memory");
    return ok != 0;
}

__device__ __forceinline__ bool mbar_wait(uint64_t *mbar, uint32_t parity, long long limit = kMbarWaitLimit)
{
    for (long long i = 0; i < limit; ++i)
        if (mbar_try(mbar, parity)) return true;
    return false;
}

// One arrival that also announces `bytes` of transaction count.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *mbar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                 :: "r"(smem_addr(mbar)), "r"(bytes) : "memory");
}

// Order earlier generic-proxy accesses of shared memory before later
// async-proxy (bulk copy) writes to it.
__device__ __forceinline__ void fence_proxy_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Bulk copy global -> shared of `bytes` (a multiple of 16; both addresses
// 16-byte aligned), completing as transaction bytes on `mbar`.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *mbar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        :: "r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(mbar)) : "memory");
}

}  // namespace sc
