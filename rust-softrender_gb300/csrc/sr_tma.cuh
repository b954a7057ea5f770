// sr_tma.cuh — 2D tensor copies between a framebuffer plane and shared
// memory (cp.async.bulk.tensor, completion through an mbarrier), for the
// kernels that own one screen tile per CTA.
//
// Rules kept here: a tile's x coordinate times the element size is a
// multiple of 16 bytes (tiles start at multiples of 16 pixels, and the
// planes' row strides are checked on the host), stores start at
// non-negative coordinates, and every wait on the mbarrier gives up after a
// bounded number of polls (then the kernel reports it and skips its tile).
#pragma once
#include <cuda.h>   // CUtensorMap (the type only; maps are encoded on the host)
#include "sr_internal.cuh"

namespace sr {

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// One-shot barrier: `count` arrivals plus the expected transaction bytes.
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    // the initialised barrier must be visible to the copy engine (async proxy)
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok = 0;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Tile load: box of the tensor map at element coordinates (x, y) into `dst`,
// completing `bar`'s transaction count.
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* tm, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(smem_addr(bar))
        : "memory");
}

// Tile store from `src` (elements outside the tensor are not written).
__device__ __forceinline__ void tma_store_2d(const CUtensorMap* tm, int x, int y, const void* src) {
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];" ::"l"(
                     reinterpret_cast<uint64_t>(tm)),
                 "r"(x), "r"(y), "r"(smem_addr(src))
                 : "memory");
}

// Shared-memory writes made by threads, ordered before a tile store.
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// Waits until the committed stores are complete.
__device__ __forceinline__ void bulk_wait() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// Polls before a tile wait gives up (a few milliseconds; a tile load takes
// microseconds).
constexpr uint32_t TMA_WAIT_POLLS = 1u << 22;

}  // namespace sr
