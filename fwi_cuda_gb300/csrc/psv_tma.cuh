// psv_tma.cuh -- device helpers of the kernels that stage tiles in shared
// memory with TMA tensor copies (psv_tiled.cu, psv_march.cu): shared-memory
// addresses, mbarrier set-up, transaction-count arrival, bounded waits and
// the 3-D tensor load.
#pragma once

#include <cuda.h>
#include <stdint.h>

namespace psv {
namespace {

constexpr unsigned WAIT_LIMIT = 1u << 20;  // try_wait rounds before giving up

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ float *align128(unsigned char *raw)
{
    const uint32_t a = smem_u32(raw);
    return reinterpret_cast<float *>(raw + ((128u - (a & 127u)) & 127u));
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Orders this thread's earlier generic-proxy shared-memory accesses (after
// the block barrier that ended the reads of a stage) before the async-proxy
// copies that refill it.
__device__ __forceinline__ void fence_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity)
{
    for (unsigned n = 0; n < WAIT_LIMIT; n++) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred P;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 P, [%1], %2;\n\t"
            "selp.b32 %0, 1, 0, P;\n\t}"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// One box of a 3-D tensor (x = column, y = row, z = plane) into shared
// memory; completion is signalled on `bar` as transaction bytes.
__device__ __forceinline__ void tma_load(uint32_t dst, const CUtensorMap *map, int x, int y, int z,
                                         uint32_t bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(bar)
        : "memory");
}

}  // namespace
}  // namespace psv
