// kernels_persist.cu -- one cooperative launch per time step.
//
// At the benchmark sizes a phase of the step (a smoothing sweep, a
// reduction) touches ~100k cells held in L2 and takes about a microsecond of
// work, so one launch per phase (~1000 per step) is bound by launch and drain
// latency.  This kernel keeps a grid of co-resident blocks (cooperative
// launch, numSMs x occupancy) for the whole step and separates dependent
// phases by a software grid barrier instead of kernel boundaries.  Every
// phase calls the same device bodies as the per-phase kernels
// (method_body.cuh), with the same work decomposition, so both paths give
// bit-identical results; the convergence loops are plain loops whose exit
// test every block evaluates from the per-instance states after a barrier.
//
// The barrier spins on a generation counter with a bounded number of
// iterations: on timeout it raises an error flag, every block leaves at its
// next barrier, and the host reports the failure (the GPU is left usable).
#include <cuda_runtime.h>

#include <mutex>

#include "grid_barrier.cuh"
#include "ifx_persist.h"
#include "method_body.cuh"

namespace ifx {

namespace {

// Loop-exit tests: every block must take the same decision, so the states
// written by other blocks before the last barrier are read with volatile loads.
__device__ __forceinline__ bool any_pred_active(const InstState* S, int n) {
    int a = 0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) a |= (*(const volatile int*)&S[k].pred_state == ST_ACTIVE);
    return __syncthreads_or(a) != 0;
}
__device__ __forceinline__ bool any_restart_due(const InstState* S, int n) {
    int a = 0;
    for (int k = threadIdx.x; k < n; k += blockDim.x)
        a |= *(const volatile int*)&S[k].ppe_state == ST_ACTIVE && *(const volatile int*)&S[k].restart != 0;
    return __syncthreads_or(a) != 0;
}
__device__ __forceinline__ bool any_ppe_active(const InstState* S, int n) {
    int a = 0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) a |= (*(const volatile int*)&S[k].ppe_state == ST_ACTIVE);
    return __syncthreads_or(a) != 0;
}

#define BAR()                                          \
    do {                                               \
        if (!grid_barrier(P.bar, ep, P.trace, P.trace_cap, P.spin_limit)) return false; \
    } while (0)
#define FOR_VB(n) for (int vb = blockIdx.x; vb < (n); vb += gridDim.x)

__device__ __forceinline__ int nchunks(int n) { return (n + TILE_THREADS - 1) / TILE_THREADS; }

__device__ bool ghost_fill(const PersistPlan& P, int comps, unsigned long long& ep) {
    FOR_VB(nchunks(P.ng)) b_ghost_gather(P.G, P.ng, P.I, comps, P.gval, vb);
    BAR();
    FOR_VB(nchunks(P.ng)) b_ghost_scatter(P.G, P.ng, P.I, comps, P.gval, vb);
    BAR();
    return true;
}

// One V-cycle; *res receives the buffer (0: e, 1: e2) of the finest-level
// result.  Levels with at most SUB_MAX_CELLS cells run inside b_subcycle.
template <typename T>
__device__ bool vcycle(const PersistPlan& P, int* res, unsigned long long& ep) {
    FOR_VB(P.nt0) b_smooth<T>(P.t0, P.LV, P.I, P.S, P.G, 1, 0, vb);
    BAR();
    int cur0 = 1;
    for (int k = 1; k < P.mg_pre; k++) {
        FOR_VB(P.nt0) b_smooth<T>(P.t0, P.LV, P.I, P.S, P.G, 0, cur0, vb);
        BAR();
        cur0 ^= 1;
    }
    for (int l = 1; l < P.lmax; l++) {
        if (P.ntre[l] == 0) break;
        FOR_VB(P.ntre[l]) b_restrict<T>(P.tre[l], P.LV, P.I, P.S, P.G, parity_after_pre(l - 1, P.mg_pre), vb);
        BAR();
        if (P.ntsm[l] == 0) continue;  // only first small levels (sub-cycle) at this depth
        int cur = 0;
        for (int k = 1; k < P.mg_pre; k++) {
            FOR_VB(P.ntsm[l]) b_smooth<T>(P.tsm[l], P.LV, P.I, P.S, P.G, 0, cur, vb);
            BAR();
            cur ^= 1;
        }
    }
    {
        extern __shared__ __align__(16) unsigned char sub_smem[];
        const bool resident = P.ninst <= (int)gridDim.x;  // geometry staged at kernel start
        FOR_VB(P.ninst) b_subcycle<T>(P.sub, P.LV, P.I, P.S, P.mg_pre, P.mg_post, sub_smem, resident, vb);
    }
    BAR();
    for (int l = P.lmax - 2; l >= 0; l--) {
        const Tile* tl = l == 0 ? P.t0 : P.tsm[l];
        const int nt = l == 0 ? P.nt0 : P.ntsm[l];
        if (nt == 0) continue;
        int cur = parity_after_pre(l, P.mg_pre);
        FOR_VB(nt) b_prolong<T>(tl, P.LV, P.S, cur, parity_after_post(l + 1, P.mg_pre, P.mg_post), vb);
        BAR();
        for (int k = 0; k < P.mg_post; k++) {
            FOR_VB(nt) b_smooth<T>(tl, P.LV, P.I, P.S, P.G, 0, cur, vb);
            BAR();
            cur ^= 1;
        }
        if (l == 0) cur0 = cur;
    }
    *res = cur0;
    return true;
}

template <typename T>
__device__ bool one_step(const PersistPlan& P, unsigned long long& ep) {
    const int n = P.ninst;
    FOR_VB(nchunks(n)) b_step_begin(P.I, P.S, n, nullptr, vb);
    FOR_VB(nchunks(P.ng)) b_outflow(P.G, P.ng, P.I, vb);
    BAR();
    if (!ghost_fill(P, 3, ep)) return false;
    FOR_VB(P.nt0) b_conv_rhs(P.t0, P.I, P.S, vb);
    BAR();
    FOR_VB(P.nt0) b_pred_guess(P.t0, P.I, vb);
    BAR();
    // predictor: pairs of Jacobi sweeps until every instance converged
    const int npred = P.nt0 + nchunks(P.ng);
    constexpr bool mixed32 = sizeof(T) == 4;
    for (int pair = 0; pair < P.pred_pairs; pair++) {
        if (mixed32) {
            // the FP64 refresh of each inner cycle runs inside the sweeps that start and end it
            for (int par = 0; par < 2; par++) {
                FOR_VB(npred) b_pred_sweep32(P.t0, P.nt0, P.G, P.ng, P.LV, P.I, P.S, P.part, par, vb);
                BAR();
                FOR_VB(n) b_pred_reduce(P.I, P.S, P.part, par, nullptr, 0ull, vb);
                BAR();
            }
        } else {
            FOR_VB(npred) b_pred_sweep(P.t0, P.nt0, P.G, P.ng, P.I, P.S, P.part, 0, vb);
            BAR();
            FOR_VB(n) b_pred_reduce(P.I, P.S, P.part, 0, nullptr, 0ull, vb);
            BAR();
            FOR_VB(npred) b_pred_sweep(P.t0, P.nt0, P.G, P.ng, P.I, P.S, P.part, 1, vb);
            BAR();
            FOR_VB(n) b_pred_reduce(P.I, P.S, P.part, 1, nullptr, 0ull, vb);
            BAR();
        }
        if (!any_pred_active(P.S, n)) break;
    }
    if (mixed32) {
        FOR_VB(npred) b_pred_refresh(P.t0, P.nt0, P.G, P.ng, P.I, P.S, 0, 1, vb);
        BAR();
    }
    if (!ghost_fill(P, 3, ep)) return false;
    FOR_VB(P.nt0) b_face_rhs(P.t0, P.I, P.S, P.part, 0, vb);
    BAR();
    FOR_VB(n) b_rhs_reduce(P.I, P.S, P.part, vb);
    BAR();
    constexpr int mixed = sizeof(T) == 4 ? 1 : 0;
    FOR_VB(P.nt0) b_bicg_start<T>(P.t0, P.LV, P.I, P.S, P.G, P.part, 0, vb);
    BAR();
    FOR_VB(n) b_bicg_reduce_r(P.I, P.S, P.part, 1, mixed, nullptr, 0ull, vb);
    BAR();
    // pressure: BiCGSTAB iterations until every instance converged
    for (int it = 0; it < P.ppe_bodies; it++) {
        if (!any_ppe_active(P.S, n)) break;
        if (mixed && any_restart_due(P.S, n)) {  // FP64 true residual and restart where the FP32 recursion ran its course
            FOR_VB(P.nt0) b_bicg_start<T>(P.t0, P.LV, P.I, P.S, P.G, P.part, 1, vb);
            BAR();
            FOR_VB(n) b_bicg_reduce_r(P.I, P.S, P.part, 2, 1, nullptr, 0ull, vb);
            BAR();
        }
        FOR_VB(P.nt0) b_bicg_p<T>(P.t0, P.LV, P.I, P.S, vb);
        BAR();
        int e1 = 0, e2 = 0;
        if (!vcycle<T>(P, &e1, ep)) return false;
        FOR_VB(P.nt0) b_bicg_apply<T>(P.t0, P.LV, P.I, P.S, P.G, P.part, e1, 0, vb);
        BAR();
        FOR_VB(n) b_bicg_scalar(P.I, P.S, P.part, 0, vb);
        BAR();
        FOR_VB(P.nt0) b_bicg_s<T>(P.t0, P.LV, P.I, P.S, vb);
        BAR();
        if (!vcycle<T>(P, &e2, ep)) return false;
        FOR_VB(P.nt0) b_bicg_apply<T>(P.t0, P.LV, P.I, P.S, P.G, P.part, e2, 1, vb);
        BAR();
        FOR_VB(n) b_bicg_scalar(P.I, P.S, P.part, 1, vb);
        BAR();
        FOR_VB(P.nt0) b_bicg_x<T>(P.t0, P.LV, P.I, P.S, P.part, vb);
        BAR();
        FOR_VB(n) b_bicg_reduce_r(P.I, P.S, P.part, 0, mixed, nullptr, 0ull, vb);
        BAR();
    }
    FOR_VB(P.nt0) b_p_finalize(P.t0, P.I, P.S, vb);
    BAR();
    if (!ghost_fill(P, 4, ep)) return false;
    FOR_VB(P.nt0) b_correct(P.t0, P.I, P.part, vb);
    BAR();
    FOR_VB(n) b_correct_reduce(P.I, P.S, P.part, vb);
    BAR();
    if (!ghost_fill(P, 3, ep)) return false;
    FOR_VB(n * FORCE_BLOCKS) b_forces(P.I, P.S, P.fpart, P.ftick, vb);
    BAR();
    return true;
}

template <typename T>
__global__ void __launch_bounds__(TILE_THREADS) k_persist_step(PersistPlan P) {
    unsigned long long ep = 0;
    if ((int)blockIdx.x < P.ninst && P.ninst <= (int)gridDim.x) {
        // block k runs instance k's small levels all launch long: stage their geometry once
        extern __shared__ __align__(16) unsigned char sub_smem[];
        sub_stage_geometry<T>(P.sub, P.LV, P.I, blockIdx.x, sub_smem);
    }
    if (P.trace && blockIdx.x == 0 && threadIdx.x == 0 && P.trace_cap > 0) P.trace[0] = clock64();
    for (int s = 0; s < P.nsteps; s++)
        if (!one_step<T>(P, ep)) return;
}

// Measurement: `reps` grid barriers back to back (no work between them).
__global__ void __launch_bounds__(TILE_THREADS) k_barrier_bench(GridBar* bar, int reps) {
    unsigned long long ep = 0;
    for (int r = 0; r < reps; r++)
        if (!grid_barrier(bar, ep)) return;
}

}  // namespace

cudaError_t launch_barrier_bench(GridBar* bar, int grid, int reps, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(&bar->count, 0, sizeof(bar->count), s);
    if (e != cudaSuccess) return e;
    void* args[] = {(void*)&bar, (void*)&reps};
    return cudaLaunchCooperativeKernel((const void*)k_barrier_bench, dim3(grid), dim3(TILE_THREADS), args, 0, s);
}

template <typename T>
cudaError_t launch_persist_step(const PersistPlan& P, int grid, cudaStream_t s) {
    // all bits set: 2^64 - 1, one arrival short of zero (the counter wraps)
    cudaError_t e = cudaMemsetAsync(&P.bar->count, P.withhold_arrival ? 0xFF : 0, sizeof(P.bar->count), s);
    if (e != cudaSuccess) return e;
    void* args[] = {(void*)&P};
    return cudaLaunchCooperativeKernel((const void*)k_persist_step<T>, dim3(grid), dim3(TILE_THREADS), args,
                                       (size_t)P.sub_bytes, s);
}

template <typename T>
cudaError_t persist_occupancy(int* blocks_per_sm, int smem_bytes) {
    {
        // the attribute belongs to the kernel, shared by every solver on the device: only raise it
        static std::mutex mu;
        static int cur[64] = {0};
        int dev = 0;
        cudaGetDevice(&dev);
        dev = dev >= 0 && dev < 64 ? dev : 0;
        std::lock_guard<std::mutex> g(mu);
        if (smem_bytes > cur[dev]) {
            cudaError_t e = cudaFuncSetAttribute(k_persist_step<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 smem_bytes);
            if (e != cudaSuccess) return e;
            cur[dev] = smem_bytes;
        }
    }
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_persist_step<T>, TILE_THREADS,
                                                         (size_t)smem_bytes);
}

template cudaError_t launch_persist_step<double>(const PersistPlan&, int, cudaStream_t);
template cudaError_t launch_persist_step<float>(const PersistPlan&, int, cudaStream_t);
template cudaError_t persist_occupancy<double>(int*, int);
template cudaError_t persist_occupancy<float>(int*, int);

}  // namespace ifx
