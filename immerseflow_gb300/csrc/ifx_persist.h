// ifx_persist.h -- plan of the persistent per-step kernel (kernels_persist.cu).
#pragma once
#include <cuda_runtime.h>

#include "ifx_dev.h"

namespace ifx {

constexpr int kMaxLevels = 16;
// polls of a grid barrier before it gives up (x ~50-100 ns per poll: well
// under a second per barrier)
constexpr long long kSpinLimit = 1ll << 23;

// Grid barrier state (zeroed once at allocation; counters return to zero
// after every barrier, the generation only grows).
struct GridBar {
    unsigned long long count;   // arrivals since the launch (reset before each launch)
    unsigned long long pad0[15];
    unsigned int err;
    unsigned int pad1[31];
};

struct PersistPlan {
    const InstDev* I;
    InstState* S;
    const LevelDev* LV;
    const GhostDev* G;
    double* gval;
    double* part;
    double* fpart;      // force partials, 2 * FORCE_BLOCKS per instance
    unsigned* ftick;    // force tickets, one per instance
    const Tile* t0;
    const Tile* tsm[kMaxLevels];
    const Tile* tre[kMaxLevels];
    const Tile* tall;   // tiles of every level, per-level ranges in LevelDev
    const int* sub;     // per instance: LevelDev index of its first small level
    GridBar* bar;
    int nt0, ng, ninst, lmax, mg_pre, mg_post;
    int ntsm[kMaxLevels];
    int ntre[kMaxLevels];
    int pred_pairs, ppe_bodies, nsteps;
    long long* trace;   // optional: SM clock of block 0 after every barrier
    int trace_cap;
    int sub_bytes;      // dynamic shared memory of the sub-cycle (largest instance)
    long long spin_limit;     // polls before a grid barrier gives up (kSpinLimit)
    int withhold_arrival;     // failure-detection hook: the arrival counter starts
                              // one short, so the first barrier never completes
};

template <typename T>
cudaError_t launch_persist_step(const PersistPlan& P, int grid, cudaStream_t s);
template <typename T>
cudaError_t persist_occupancy(int* blocks_per_sm, int smem_bytes);
cudaError_t launch_barrier_bench(GridBar* bar, int grid, int reps, cudaStream_t s);

}  // namespace ifx
