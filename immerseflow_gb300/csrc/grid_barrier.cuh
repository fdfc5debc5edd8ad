// grid_barrier.cuh -- software grid barrier of the cooperative launches
// (the per-step kernel of METHOD mode, the REFERENCE-mode step kernel).
#pragma once
#include <cuda_runtime.h>

#include "ifx_persist.h"

namespace ifx {

__device__ __forceinline__ unsigned int vload(const unsigned int* p) { return *(const volatile unsigned int*)p; }

// Flat barrier on a monotonically increasing 64-bit arrival counter: the
// k-th barrier of the launch is passed once the counter reaches
// gridDim.x * k.  Arrival is a release add, the wait an acquire poll, so the
// critical path is one atomic and one poll; the counter never needs a reset
// inside the launch (the host zeroes it before each launch).
// The wait gives up after spin_limit polls: it sets the error flag and every
// block returns, so a lost block ends the launch with an error the host reads
// instead of a hang.
__device__ __forceinline__ bool grid_barrier(GridBar* b, unsigned long long& epoch, long long* trace = nullptr,
                                             int cap = 0, long long spin_limit = kSpinLimit) {
    __syncthreads();
    epoch += 1;
    if (threadIdx.x == 0) {
        const unsigned long long target = epoch * (unsigned long long)gridDim.x;
        unsigned long long v;
        asm volatile("atom.add.release.gpu.u64 %0, [%1], 1;" : "=l"(v) : "l"(&b->count) : "memory");
        long long spins = 0;
        while (true) {
            asm volatile("ld.acquire.gpu.u64 %0, [%1];" : "=l"(v) : "l"(&b->count) : "memory");
            if (v >= target) break;
            if (++spins > spin_limit) {
                atomicExch(&b->err, 1u);
                break;
            }
            __nanosleep(32);
        }
        if (trace && blockIdx.x == 0 && epoch < (unsigned long long)cap) trace[epoch] = clock64();
    }
    __syncthreads();
    return vload(&b->err) == 0u;
}


}  // namespace ifx
