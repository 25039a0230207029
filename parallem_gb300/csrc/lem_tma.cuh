// lem_tma.cuh -- Tensor Memory Accelerator copies and mbarrier waits (inline PTX).
//
// A tile is copied from global to shared memory by cp.async.bulk.tensor with a
// tensor map (made on the host with cuTensorMapEncodeTiled and passed as a
// __grid_constant__ kernel parameter); the copy completes on an mbarrier
// armed with the bytes to expect.  Waits poll mbarrier.try_wait a bounded
// number of times, so a copy that never arrives ends in an error status
// instead of a hang.  The inner coordinate of every copy must be a multiple of
// 16 bytes; copies start at negative coordinates only to read the zero fill.
#pragma once

#include <cstdint>
#include <cuda.h>

namespace lem {

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// makes the initialised barriers visible to the copy engine
__device__ __forceinline__ void fence_mbarrier_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// orders this thread's earlier shared-memory accesses before later bulk copies into it
__device__ __forceinline__ void fence_proxy_async_shared() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// one arrival that also announces `bytes` of copies completing on the barrier
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
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

// waits for the barrier's phase with the given parity; false after `spins` polls
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t spins) {
    for (uint32_t i = 0; i < spins; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// a 2-D box of the tensor at (x, y) (elements; x innermost) into shared memory
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_addr(bar))
        : "memory");
}

}  // namespace lem
