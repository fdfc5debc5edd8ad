// tma.cuh -- tensor-memory-accelerator tile loads with an mbarrier (sm_90 and
// later PTX: cp.async.bulk.tensor, mbarrier.*), used to stage multigrid tiles
// in shared memory.  The wait is bounded: a copy that never completes sets an
// error flag instead of hanging the GPU.
#pragma once
#include <cuda.h>
#include <cstdint>

namespace ifx {

constexpr int TMA_WAIT_LIMIT = 1 << 20;  // try_wait rounds before giving up

__device__ __forceinline__ unsigned smem_u32(const void* p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    // make the initialisation visible to the asynchronous (TMA) proxy
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait for phase `parity`; false when the limit was reached.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity) {
    for (int it = 0; it < TMA_WAIT_LIMIT; it++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// 2-D tiled load of the box at (x, y) of tensor map *map into dst (shared),
// completing on bar.  x * element size must be a multiple of 16 bytes.
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y,
                                            unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

}  // namespace ifx
