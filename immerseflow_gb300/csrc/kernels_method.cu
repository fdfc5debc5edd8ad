// kernels_method.cu -- one kernel per phase of the fractional step with
// ghost-cell IBM, batched over instances (bodies in method_body.cuh).
//
// The method (written because the reference leaves it unimplemented:
// src/include/AD_PPE_Correction.cu:1-12, src/include/PPESolver.cu:73-135):
//   predictor  (I - dt/Re L) q* = q^n - dt (3/2 N^n - 1/2 N^{n-1})     Jacobi,
//              convection N in the reference's face-flux form
//              (src/include/ADSolver.cu:46-79) with face velocities U, V;
//   pressure   L p = div(U*)/dt, BiCGSTAB in FP64 preconditioned by a
//              multigrid V-cycle in T (weighted Jacobi smoothing,
//              area-weighted restriction, bilinear prolongation, RB-SOR on
//              the coarsest level);
//   projection u = u* - dt grad p (cells), U = U* - dt dp/dn (faces).
// Coefficients follow the reference's 2/(dx_i (dx_i + dx_nb)) form
// (src/include/ADSolver.cu:34-39).  Every phase has a CPU twin in the
// oracle (oracle/oracle.cpp, method_step).
//
// Precision: state in FP64; multigrid corrections in T (double for the plain
// path, float for the mixed path).
#include <cuda_runtime.h>

#include <atomic>
#include <mutex>

#include "method_body.cuh"

namespace ifx {

// Resident blocks per SM the tile kernels are compiled for.  The wide tiles
// (four rows per thread, the batched workloads, many blocks in flight) are
// latency-bound and run fastest at eight blocks of 256 threads per SM, within
// 32 registers a thread (a few spilled to L1); so do the FP64 one-row tiles of
// the plain path's batches.  FP32 one-row tiles keep the 64-register budget.
template <typename T>
constexpr int mg_blocks(int rows) { return rows == 1 ? (sizeof(T) == 8 ? 8 : 4) : 8; }

// Streaming multiprocessors of the current device (read once per device).
static int device_sm_count() {
    static std::atomic<int> cnt[64];
    int dev = 0;
    cudaGetDevice(&dev);
    dev = dev >= 0 && dev < 64 ? dev : 0;
    int n = cnt[dev].load(std::memory_order_relaxed);
    if (n <= 0) {
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 1;
        cnt[dev].store(n, std::memory_order_relaxed);
    }
    return n;
}
// The tile kernels that spill within 32 registers (eight resident blocks per
// SM: the four-row multigrid tiles, the FP64 one-row tiles, the FP64 true
// residual, the prolongation with its first sweep, the convection) come in
// two variants: MINB = 8 for grids of many tiles and MINB = 4 (64 registers,
// no spills), taken for grids of at most four blocks per SM, where the fifth
// to eighth slots would stay empty.
static bool few_tiles(int grid) { return grid <= 4 * device_sm_count(); }

__global__ void k_step_begin(const InstDev* __restrict__ I, InstState* S, int n, LoopCtl* ctl) { b_step_begin(I, S, n, ctl, blockIdx.x); }
__global__ void k_outflow(const GhostDev* __restrict__ G, int ng, const InstDev* __restrict__ I) { b_outflow(G, ng, I, blockIdx.x); }
__global__ void k_ghost_gather(const GhostDev* __restrict__ G, int ng, const InstDev* __restrict__ I,
                               int comps, double* __restrict__ gval) { b_ghost_gather(G, ng, I, comps, gval, blockIdx.x); }
__global__ void k_ghost_scatter(const GhostDev* __restrict__ G, int ng, const InstDev* __restrict__ I,
                                int comps, const double* __restrict__ gval) { b_ghost_scatter(G, ng, I, comps, gval, blockIdx.x); }
template <int MINB>
__global__ void __launch_bounds__(TILE_THREADS, MINB) k_conv_rhs(const Tile* __restrict__ tiles, const InstDev* __restrict__ I,
                           const InstState* __restrict__ S) { b_conv_rhs(tiles, I, S, blockIdx.x); }
__global__ void __launch_bounds__(TILE_THREADS, 8) k_pred_guess(const Tile* __restrict__ tiles,
                                                                const InstDev* __restrict__ I) {
    b_pred_guess(tiles, I, blockIdx.x);
}
__global__ void __launch_bounds__(TILE_THREADS, mg_blocks<double>(1)) k_pred_sweep(const Tile* __restrict__ tiles, int ntiles, const GhostDev* __restrict__ G,
                             int ng, const InstDev* __restrict__ I, const InstState* __restrict__ S,
                             double* __restrict__ part, int parity) {
    pdl_trigger();
    b_pred_sweep(tiles, ntiles, G, ng, I, S, part, parity, blockIdx.x);
}
// one-row variant: five blocks per SM (48 registers), as before the inner
// cycle's FP64 defect moved into the sweep (its branch runs one sweep in
// mixed_inner and may spill)
template <int R>
__global__ void __launch_bounds__(TILE_THREADS, R == 1 ? 5 : mg_blocks<float>(R)) k_pred_sweep32(const Tile* __restrict__ tiles, int ntiles, const GhostDev* __restrict__ G, int ng,
                               const LevelDev* __restrict__ LV, const InstDev* __restrict__ I,
                               const InstState* __restrict__ S, double* __restrict__ part, int parity) {
    pdl_trigger();
    b_pred_sweep32<R>(tiles, ntiles, G, ng, LV, I, S, part, parity, blockIdx.x);
}
// Launch with programmatic stream serialisation (the kernel may start before
// the phase before it has finished and waits for it itself: pdl_wait), for
// the one-block-per-instance phases of small batches only: with many
// instances the early blocks hold SM slots that the phase before still needs
// (256 instances: +0.35% a step; one instance: -0.9%).
constexpr int PDL_MAX_INSTANCES = 8;
template <typename... P, typename... A>
cudaError_t launch_pdl(void (*k)(P...), int grid, int block, size_t smem, cudaStream_t s, A... args) {
    if (grid > PDL_MAX_INSTANCES) {
        k<<<grid, block, smem, s>>>(args...);
        return cudaGetLastError();
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k, args...);
}
// Optional phases (mixed path) run as grid-stride loops on a fixed grid that
// returns at once when the last vote found nothing due.
constexpr int OPT_GRID = 1024;
template <int R>
__global__ void __launch_bounds__(TILE_THREADS, mg_blocks<float>(R)) k_pred_refresh(const Tile* __restrict__ tiles, int ntiles, const GhostDev* __restrict__ G, int ng,
                               const InstDev* __restrict__ I, const InstState* __restrict__ S, int stage,
                               int finalize, const LoopCtl* ctl) {
    if (!finalize && none_due(ctl)) return;
    const int nvb = ntiles + (ng + TILE_THREADS - 1) / TILE_THREADS;
    for (int vb = blockIdx.x; vb < nvb; vb += gridDim.x) b_pred_refresh<R>(tiles, ntiles, G, ng, I, S, stage, finalize, vb);
}
template <bool W>
__global__ void k_pred_reduce(const InstDev* __restrict__ I, InstState* __restrict__ S,
                              const double* __restrict__ part, int parity, LoopCtl* ctl,
                              unsigned long long handle) { b_pred_reduce<W>(I, S, part, parity, ctl, handle, blockIdx.x); }
__global__ void __launch_bounds__(TILE_THREADS, 8) k_face_rhs(const Tile* __restrict__ tiles, const InstDev* __restrict__ I,
                           const InstState* __restrict__ S, double* __restrict__ part, int to_final) {
    b_face_rhs(tiles, I, S, part, to_final, blockIdx.x);
}
template <bool W>
__global__ void k_rhs_reduce(const InstDev* __restrict__ I, InstState* __restrict__ S,
                             const double* __restrict__ part) { b_rhs_reduce<W>(I, S, part, blockIdx.x); }
// restart_only: for a chunk of blockDim instances at a time, every block forms
// the exclusive prefix sum of the finest-level tile counts of the instances
// whose restart is due (others count 0; each instance's tiles are contiguous
// in the list), and the grid strides over the concatenated due tiles: the pass
// costs in proportion to the tiles restarting, spread over the whole grid.
template <typename T, int MINB>
__global__ void __launch_bounds__(TILE_THREADS, MINB) k_bicg_start(const Tile* __restrict__ tiles, const LevelDev* __restrict__ LV,
                             const InstDev* __restrict__ I, const InstState* __restrict__ S,
                             const GhostDev* __restrict__ G, double* __restrict__ part, int restart_only,
                             const LoopCtl* ctl, int nt, int ninst) {
    pdl_trigger();
    if (!restart_only) {
        for (int vb = blockIdx.x; vb < nt; vb += gridDim.x) b_bicg_start<T>(tiles, LV, I, S, G, part, 0, vb);
        return;
    }
    if (none_due(ctl)) return;
    __shared__ int dbeg[TILE_THREADS], doff[TILE_THREADS + 1], wtot[TILE_THREADS / 32];
    const int lane = (int)(threadIdx.x & 31), w = (int)(threadIdx.x >> 5);
    for (int k0 = 0; k0 < ninst; k0 += blockDim.x) {
        const int k = k0 + (int)threadIdx.x;
        const bool d = k < ninst && S[k].ppe_state == ST_ACTIVE && S[k].restart;
        const int cnt = d ? I[k].tile_cnt : 0;
        int inc = cnt;  // inclusive scan within the warp
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += y;
        }
        if (lane == 31) wtot[w] = inc;
        __syncthreads();
        int base = 0;
        for (int q = 0; q < w; q++) base += wtot[q];
        dbeg[threadIdx.x] = d ? I[k].tile_beg : 0;
        doff[threadIdx.x] = base + inc - cnt;
        if ((int)threadIdx.x == (int)blockDim.x - 1) doff[blockDim.x] = base + inc;
        __syncthreads();
        const int total = doff[blockDim.x];
        for (int v = blockIdx.x; v < total; v += gridDim.x) {
            int lo = 0, hi = (int)blockDim.x;  // last entry with doff <= v
            while (hi - lo > 1) {
                const int mid = (lo + hi) >> 1;
                if (doff[mid] <= v) lo = mid;
                else hi = mid;
            }
            b_bicg_start<T>(tiles, LV, I, S, G, part, 1, dbeg[lo] + (v - doff[lo]));
        }
        __syncthreads();
    }
}
template <bool W>
__global__ void k_bicg_reduce_r(const InstDev* __restrict__ I, InstState* __restrict__ S,
                                const double* __restrict__ part, int start, int mixed, LoopCtl* ctl,
                                unsigned long long handle) { b_bicg_reduce_r<W>(I, S, part, start, mixed, ctl, handle, blockIdx.x); }
template <typename T, int R>
__global__ void __launch_bounds__(TILE_THREADS, mg_blocks<T>(R)) k_bicg_p(const Tile* __restrict__ tiles, const LevelDev* __restrict__ LV,
                         const InstDev* __restrict__ I, const InstState* __restrict__ S) { b_bicg_p<T, R>(tiles, LV, I, S, blockIdx.x); }
template <typename T, int R, int MINB = mg_blocks<T>(R)>
__global__ void __launch_bounds__(TILE_THREADS, MINB) k_bicg_dir_smooth(const Tile* __restrict__ tiles, const LevelDev* __restrict__ LV,
                                  const InstDev* __restrict__ I, const InstState* __restrict__ S,
                                  const GhostDev* __restrict__ G, int which) {
    b_bicg_dir_smooth<T, R>(tiles, LV, I, S, G, which, blockIdx.x);
}
template <typename T, int R, int MINB = mg_blocks<T>(R)>
__global__ void __launch_bounds__(TILE_THREADS, MINB) k_bicg_apply(const Tile* __restrict__ tiles, const LevelDev* __restrict__ LV,
                             const InstDev* __restrict__ I, const InstState* __restrict__ S,
                             const GhostDev* __restrict__ G, double* __restrict__ part, int e_alt, int which) {
    pdl_trigger();
    b_bicg_apply<T, R>(tiles, LV, I, S, G, part, e_alt, which, blockIdx.x);
}
template <bool W>
__global__ void k_bicg_scalar(const InstDev* __restrict__ I, InstState* __restrict__ S,
                              const double* __restrict__ part, int which) { b_bicg_scalar<W>(I, S, part, which, blockIdx.x); }
template <typename T, int R>
__global__ void __launch_bounds__(TILE_THREADS, mg_blocks<T>(R)) k_bicg_s(const Tile* __restrict__ tiles, const LevelDev* __restrict__ LV,
                         const InstDev* __restrict__ I, const InstState* __restrict__ S) { b_bicg_s<T, R>(tiles, LV, I, S, blockIdx.x); }
template <typename T, int R>
__global__ void __launch_bounds__(TILE_THREADS, mg_blocks<T>(R)) k_bicg_x(const Tile* __restrict__ tiles, const LevelDev* __restrict__ LV,
                         const InstDev* __restrict__ I, const InstState* __restrict__ S,
                         double* __restrict__ part) {
    pdl_trigger();
    b_bicg_x<T, R>(tiles, LV, I, S, part, blockIdx.x);
}
template <typename T, int R, int MINB = mg_blocks<T>(R)>
__global__ void __launch_bounds__(TILE_THREADS, MINB) k_smooth(const Tile* __restrict__ tiles, const LevelDev* __restrict__ LV,
                         const InstDev* __restrict__ I, const InstState* __restrict__ S,
                         const GhostDev* __restrict__ G, int flags, int src_alt) { b_smooth<T, R>(tiles, LV, I, S, G, flags, src_alt, blockIdx.x); }
template <typename T, int R, int MINB = mg_blocks<T>(R)>
__global__ void __launch_bounds__(TILE_THREADS, MINB) k_smooth_tma(const Tile* __restrict__ tiles, const LevelDev* __restrict__ LV,
                         const InstDev* __restrict__ I, const InstState* __restrict__ S,
                         const GhostDev* __restrict__ G, const CUtensorMap* __restrict__ tm, int flags, int src_alt,
                         unsigned* err) { b_smooth_tma<T, R>(tiles, LV, I, S, G, tm, flags, src_alt, err, blockIdx.x); }
template <typename T, int R>
__global__ void __launch_bounds__(TILE_THREADS, 4) k_smooth_grid_tma(const GridTiles g, const InstState* __restrict__ S,
                                                                    const GhostDev* __restrict__ G,
                                                                    const CUtensorMap* __restrict__ tm, int flags,
                                                                    int src_alt, unsigned* err) {
    b_smooth_grid_tma<T, R>(g, S, G, tm, flags, src_alt, err, blockIdx.x);
}
template <typename T, int R>
__global__ void __launch_bounds__(TILE_THREADS, 4) k_smooth_grid(const GridTiles g, const InstState* __restrict__ S,
                                                                const GhostDev* __restrict__ G, int flags,
                                                                int src_alt) {
    b_smooth_grid<T, R>(g, S, G, flags, src_alt, blockIdx.x);
}
template <typename T, int R, int MINB = mg_blocks<T>(R)>
__global__ void __launch_bounds__(TILE_THREADS, MINB) k_restrict(const Tile* __restrict__ tiles, const LevelDev* __restrict__ LV,
                           const InstDev* __restrict__ I, const InstState* __restrict__ S,
                           const GhostDev* __restrict__ G, int fine_alt) {
    pdl_trigger();  // a programmatically launched sub-cycle may start staging its geometry
    b_restrict<T, R>(tiles, LV, I, S, G, fine_alt, blockIdx.x);
}
template <typename T, int R, int MINB = mg_blocks<T>(R)>
__global__ void __launch_bounds__(TILE_THREADS, MINB) k_prolong(const Tile* __restrict__ tiles, const LevelDev* __restrict__ LV,
                          const InstState* __restrict__ S, int fine_alt, int coarse_alt) { b_prolong<T, R>(tiles, LV, S, fine_alt, coarse_alt, blockIdx.x); }
template <typename T, int MINB>
__global__ void __launch_bounds__(TILE_THREADS, MINB) k_prolong_sweep(const Tile* __restrict__ tiles, const LevelDev* __restrict__ LV,
                                const InstDev* __restrict__ I, const InstState* __restrict__ S, int cur,
                                int coarse_alt) {
    b_prolong_sweep<T>(tiles, LV, I, S, cur, coarse_alt, blockIdx.x);
}
// MINB = 1 lets the compiler keep the two staged levels' views of a
// restriction or prolongation in registers (no spills; one block per SM);
// MINB = 2 fits two blocks per SM for batches of more instances than SMs.
template <typename T, int MINB>
__global__ void __launch_bounds__(SUB_THREADS, MINB) k_subcycle(const int* __restrict__ sub, const LevelDev* __restrict__ LV,
                           const InstDev* __restrict__ I, const InstState* __restrict__ S,
                           int pre, int post) {
    extern __shared__ __align__(16) unsigned char sub_smem[];
    b_subcycle<T>(sub, LV, I, S, pre, post, sub_smem, false, blockIdx.x);
}
__global__ void k_p_finalize(const Tile* __restrict__ tiles, const InstDev* __restrict__ I,
                             const InstState* __restrict__ S) { b_p_finalize(tiles, I, S, blockIdx.x); }
__global__ void __launch_bounds__(TILE_THREADS, 8) k_correct(const Tile* __restrict__ tiles, const InstDev* __restrict__ I,
                          double* __restrict__ part) { b_correct(tiles, I, part, blockIdx.x); }
__global__ void k_correct_reduce(const InstDev* __restrict__ I, InstState* __restrict__ S,
                                 const double* __restrict__ part) { b_correct_reduce(I, S, part, blockIdx.x); }
__global__ void k_forces(const InstDev* __restrict__ I, InstState* __restrict__ S, double* __restrict__ fpart,
                         unsigned* __restrict__ ftick) {
    b_forces(I, S, fpart, ftick, blockIdx.x);
}

// ------------------------------------------------------------ launchers

#define CK(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) return e_; } while (0)

static inline int nblk(int n, int b) { return (n + b - 1) / b; }

cudaError_t launch_step_begin(const InstDev* I, InstState* S, int n, LoopCtl* ctl, cudaStream_t s) {
    k_step_begin<<<nblk(n, 128), 128, 0, s>>>(I, S, n, ctl);
    return cudaGetLastError();
}
cudaError_t launch_outflow(const GhostDev* G, int ng, const InstDev* I, cudaStream_t s) {
    if (ng == 0) return cudaSuccess;
    k_outflow<<<nblk(ng, 256), 256, 0, s>>>(G, ng, I);
    return cudaGetLastError();
}
cudaError_t launch_ghost_fill(const GhostDev* G, int ng, const InstDev* I, int comps, double* gval,
                              cudaStream_t s) {
    if (ng == 0) return cudaSuccess;
    k_ghost_gather<<<nblk(ng, 256), 256, 0, s>>>(G, ng, I, comps, gval);
    CK(cudaGetLastError());
    k_ghost_scatter<<<nblk(ng, 256), 256, 0, s>>>(G, ng, I, comps, gval);
    return cudaGetLastError();
}
// Dense host rows <-> pitched device fields, three fields at a time through a
// dense staging buffer (one contiguous copy each way instead of row copies).
__global__ void k_state_unpack(const double* __restrict__ stage, double* u, double* v, double* p, int nx, int ny,
                               int pitch) {
    const int n = nx * ny;
    double* dst[3] = {u, v, p};
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < 3 * n; q += gridDim.x * blockDim.x) {
        const int f = q / n, r = q - f * n, j = r / nx, i = r - j * nx;
        if (dst[f]) dst[f][i + j * pitch] = stage[q];
    }
}
__global__ void k_state_pack(const double* u, const double* v, const double* p, double* __restrict__ stage, int nx,
                             int ny, int pitch) {
    const int n = nx * ny;
    const double* src[3] = {u, v, p};
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < 3 * n; q += gridDim.x * blockDim.x) {
        const int f = q / n, r = q - f * n, j = r / nx, i = r - j * nx;
        if (src[f]) stage[q] = src[f][i + j * pitch];
    }
}
cudaError_t launch_state_unpack(const double* stage, double* u, double* v, double* p, int nx, int ny, int pitch,
                                cudaStream_t s) {
    const int n = 3 * nx * ny, g = (n + 255) / 256;
    k_state_unpack<<<g < 1216 ? g : 1216, 256, 0, s>>>(stage, u, v, p, nx, ny, pitch);
    return cudaGetLastError();
}
cudaError_t launch_state_pack(const double* u, const double* v, const double* p, double* stage, int nx, int ny,
                              int pitch, cudaStream_t s) {
    const int n = 3 * nx * ny, g = (n + 255) / 256;
    k_state_pack<<<g < 1216 ? g : 1216, 256, 0, s>>>(u, v, p, stage, nx, ny, pitch);
    return cudaGetLastError();
}
cudaError_t launch_pred_guess(const Tile* t, int nt, const InstDev* I, cudaStream_t s) {
    k_pred_guess<<<nt, TILE_THREADS, 0, s>>>(t, I);
    return cudaGetLastError();
}
cudaError_t launch_conv_rhs(const Tile* t, int nt, const InstDev* I, const InstState* S, cudaStream_t s) {
    if (few_tiles(nt)) k_conv_rhs<4><<<nt, TILE_THREADS, 0, s>>>(t, I, S);
    else k_conv_rhs<8><<<nt, TILE_THREADS, 0, s>>>(t, I, S);
    return cudaGetLastError();
}
cudaError_t launch_pred_sweep(const Tile* t, int nt, const GhostDev* G, int ng, const InstDev* I,
                              const InstState* S, double* part, int parity, cudaStream_t s) {
    k_pred_sweep<<<nt + nblk(ng, TILE_THREADS), TILE_THREADS, 0, s>>>(t, nt, G, ng, I, S, part, parity);
    return cudaGetLastError();
}
cudaError_t launch_pred_sweep32(const Tile* t, int nt, const GhostDev* G, int ng, const LevelDev* LV, const InstDev* I,
                                const InstState* S, double* part, int parity, int rows, cudaStream_t s) {
    const int g = nt + nblk(ng, TILE_THREADS);
    if (rows == MG_ROWS_WIDE) k_pred_sweep32<MG_ROWS_WIDE><<<g, TILE_THREADS, 0, s>>>(t, nt, G, ng, LV, I, S, part, parity);
    else k_pred_sweep32<1><<<g, TILE_THREADS, 0, s>>>(t, nt, G, ng, LV, I, S, part, parity);
    return cudaGetLastError();
}
cudaError_t launch_pred_refresh(const Tile* t, int nt, const GhostDev* G, int ng, const InstDev* I, const InstState* S,
                                int stage, int finalize, const LoopCtl* ctl, int rows, cudaStream_t s) {
    const int nvb = nt + nblk(ng, TILE_THREADS), g = nvb < OPT_GRID ? nvb : OPT_GRID;
    if (rows == MG_ROWS_WIDE) k_pred_refresh<MG_ROWS_WIDE><<<g, TILE_THREADS, 0, s>>>(t, nt, G, ng, I, S, stage, finalize, ctl);
    else k_pred_refresh<1><<<g, TILE_THREADS, 0, s>>>(t, nt, G, ng, I, S, stage, finalize, ctl);
    return cudaGetLastError();
}
cudaError_t launch_pred_reduce(const InstDev* I, InstState* S, const double* part, int ninst, int parity,
                               LoopCtl* ctl, unsigned long long handle, cudaStream_t s, int wide) {
    if (wide) return launch_pdl(k_pred_reduce<true>, ninst, 256, 0, s, I, S, part, parity, ctl, handle);
    return launch_pdl(k_pred_reduce<false>, ninst, 256, 0, s, I, S, part, parity, ctl, handle);
}
cudaError_t launch_face_rhs(const Tile* t, int nt, const InstDev* I, const InstState* S, double* part, int to_final,
                            cudaStream_t s) {
    k_face_rhs<<<nt, TILE_THREADS, 0, s>>>(t, I, S, part, to_final);
    return cudaGetLastError();
}
cudaError_t launch_rhs_reduce(const InstDev* I, InstState* S, const double* part, int ninst, cudaStream_t s,
                              int wide) {
    if (wide) k_rhs_reduce<true><<<ninst, 256, 0, s>>>(I, S, part);
    else k_rhs_reduce<false><<<ninst, 256, 0, s>>>(I, S, part);
    return cudaGetLastError();
}
template <typename T>
cudaError_t launch_bicg_start(const Tile* t, int nt, const LevelDev* LV, const InstDev* I, const InstState* S,
                              const GhostDev* G, double* part, int restart_only, const LoopCtl* ctl, int ninst,
                              cudaStream_t s) {
    const int grid = restart_only && nt > OPT_GRID ? OPT_GRID : nt;
    if (few_tiles(grid)) k_bicg_start<T, 4><<<grid, TILE_THREADS, 0, s>>>(t, LV, I, S, G, part, restart_only, ctl, nt, ninst);
    else k_bicg_start<T, 8><<<grid, TILE_THREADS, 0, s>>>(t, LV, I, S, G, part, restart_only, ctl, nt, ninst);
    return cudaGetLastError();
}
cudaError_t launch_bicg_reduce_r(const InstDev* I, InstState* S, const double* part, int ninst, int start,
                                 int mixed, LoopCtl* ctl, unsigned long long handle, cudaStream_t s, int wide) {
    if (wide) return launch_pdl(k_bicg_reduce_r<true>, ninst, 256, 0, s, I, S, part, start, mixed, ctl, handle);
    return launch_pdl(k_bicg_reduce_r<false>, ninst, 256, 0, s, I, S, part, start, mixed, ctl, handle);
}
// Finest-level Krylov phases: rows = 1 on 32x8 tiles, MG_ROWS_WIDE on 32x32 tiles.
template <typename T>
cudaError_t launch_bicg_p(const Tile* t, int nt, const LevelDev* LV, const InstDev* I, const InstState* S,
                          int rows, cudaStream_t s) {
    if (rows == MG_ROWS_WIDE) k_bicg_p<T, MG_ROWS_WIDE><<<nt, TILE_THREADS, 0, s>>>(t, LV, I, S);
    else k_bicg_p<T, 1><<<nt, TILE_THREADS, 0, s>>>(t, LV, I, S);
    return cudaGetLastError();
}
template <typename T>
cudaError_t launch_bicg_dir_smooth(const Tile* t, int nt, const LevelDev* LV, const InstDev* I, const InstState* S,
                                   const GhostDev* G, int which, int rows, cudaStream_t s) {
    if (rows == MG_ROWS_WIDE) k_bicg_dir_smooth<T, MG_ROWS_WIDE><<<nt, TILE_THREADS, 0, s>>>(t, LV, I, S, G, which);
    else if (sizeof(T) == 8 && few_tiles(nt)) k_bicg_dir_smooth<T, 1, 4><<<nt, TILE_THREADS, 0, s>>>(t, LV, I, S, G, which);
    else k_bicg_dir_smooth<T, 1><<<nt, TILE_THREADS, 0, s>>>(t, LV, I, S, G, which);
    return cudaGetLastError();
}
template cudaError_t launch_bicg_dir_smooth<double>(const Tile*, int, const LevelDev*, const InstDev*, const InstState*,
                                                    const GhostDev*, int, int, cudaStream_t);
template cudaError_t launch_bicg_dir_smooth<float>(const Tile*, int, const LevelDev*, const InstDev*, const InstState*,
                                                   const GhostDev*, int, int, cudaStream_t);
template <typename T>
cudaError_t launch_bicg_apply(const Tile* t, int nt, const LevelDev* LV, const InstDev* I, const InstState* S,
                              const GhostDev* G, double* part, int e_alt, int which, int rows, cudaStream_t s) {
    if (rows == MG_ROWS_WIDE) k_bicg_apply<T, MG_ROWS_WIDE><<<nt, TILE_THREADS, 0, s>>>(t, LV, I, S, G, part, e_alt, which);
    else if (sizeof(T) == 8 && few_tiles(nt)) k_bicg_apply<T, 1, 4><<<nt, TILE_THREADS, 0, s>>>(t, LV, I, S, G, part, e_alt, which);
    else k_bicg_apply<T, 1><<<nt, TILE_THREADS, 0, s>>>(t, LV, I, S, G, part, e_alt, which);
    return cudaGetLastError();
}
cudaError_t launch_bicg_scalar(const InstDev* I, InstState* S, const double* part, int ninst, int which,
                               cudaStream_t s, int wide) {
    if (wide) return launch_pdl(k_bicg_scalar<true>, ninst, 256, 0, s, I, S, part, which);
    return launch_pdl(k_bicg_scalar<false>, ninst, 256, 0, s, I, S, part, which);
}
template <typename T>
cudaError_t launch_bicg_s(const Tile* t, int nt, const LevelDev* LV, const InstDev* I, const InstState* S,
                          int rows, cudaStream_t s) {
    if (rows == MG_ROWS_WIDE) k_bicg_s<T, MG_ROWS_WIDE><<<nt, TILE_THREADS, 0, s>>>(t, LV, I, S);
    else k_bicg_s<T, 1><<<nt, TILE_THREADS, 0, s>>>(t, LV, I, S);
    return cudaGetLastError();
}
template <typename T>
cudaError_t launch_bicg_x(const Tile* t, int nt, const LevelDev* LV, const InstDev* I, const InstState* S,
                          double* part, int rows, cudaStream_t s) {
    if (rows == MG_ROWS_WIDE) k_bicg_x<T, MG_ROWS_WIDE><<<nt, TILE_THREADS, 0, s>>>(t, LV, I, S, part);
    else k_bicg_x<T, 1><<<nt, TILE_THREADS, 0, s>>>(t, LV, I, S, part);
    return cudaGetLastError();
}
template <typename T>
cudaError_t launch_smooth(const Tile* t, int nt, const LevelDev* LV, const InstDev* I, const InstState* S,
                          const GhostDev* G, int flags, int src_alt, int rows, cudaStream_t s) {
    if (nt == 0) return cudaSuccess;
    if (rows == MG_ROWS_WIDE && few_tiles(nt))
        k_smooth<T, MG_ROWS_WIDE, 4><<<nt, TILE_THREADS, 0, s>>>(t, LV, I, S, G, flags, src_alt);
    else if (rows == MG_ROWS_WIDE) k_smooth<T, MG_ROWS_WIDE><<<nt, TILE_THREADS, 0, s>>>(t, LV, I, S, G, flags, src_alt);
    else if (sizeof(T) == 8 && few_tiles(nt)) k_smooth<T, 1, 4><<<nt, TILE_THREADS, 0, s>>>(t, LV, I, S, G, flags, src_alt);
    else k_smooth<T, 1><<<nt, TILE_THREADS, 0, s>>>(t, LV, I, S, G, flags, src_alt);
    return cudaGetLastError();
}
template <typename T>
cudaError_t launch_smooth_tma(const Tile* t, int nt, const LevelDev* LV, const InstDev* I, const InstState* S,
                              const GhostDev* G, const CUtensorMap* tm, int flags, int src_alt, int rows, unsigned* err,
                              cudaStream_t s) {
    if (nt == 0) return cudaSuccess;
    if (rows == MG_ROWS_WIDE && few_tiles(nt))
        k_smooth_tma<T, MG_ROWS_WIDE, 4><<<nt, TILE_THREADS, 0, s>>>(t, LV, I, S, G, tm, flags, src_alt, err);
    else if (rows == MG_ROWS_WIDE)
        k_smooth_tma<T, MG_ROWS_WIDE><<<nt, TILE_THREADS, 0, s>>>(t, LV, I, S, G, tm, flags, src_alt, err);
    else if (sizeof(T) == 8 && few_tiles(nt))
        k_smooth_tma<T, 1, 4><<<nt, TILE_THREADS, 0, s>>>(t, LV, I, S, G, tm, flags, src_alt, err);
    else k_smooth_tma<T, 1><<<nt, TILE_THREADS, 0, s>>>(t, LV, I, S, G, tm, flags, src_alt, err);
    return cudaGetLastError();
}
template cudaError_t launch_smooth_tma<double>(const Tile*, int, const LevelDev*, const InstDev*, const InstState*,
                                               const GhostDev*, const CUtensorMap*, int, int, int, unsigned*, cudaStream_t);
template cudaError_t launch_smooth_tma<float>(const Tile*, int, const LevelDev*, const InstDev*, const InstState*,
                                              const GhostDev*, const CUtensorMap*, int, int, int, unsigned*, cudaStream_t);
template <typename T>
cudaError_t launch_smooth_grid_tma(const GridTiles& g, int nt, const InstState* S, const GhostDev* G,
                                   const CUtensorMap* tm, int flags, int src_alt, int rows, unsigned* err,
                                   cudaStream_t s) {
    if (nt == 0) return cudaSuccess;
    if (rows == MG_ROWS_WIDE) k_smooth_grid_tma<T, MG_ROWS_WIDE><<<nt, TILE_THREADS, 0, s>>>(g, S, G, tm, flags, src_alt, err);
    else k_smooth_grid_tma<T, 1><<<nt, TILE_THREADS, 0, s>>>(g, S, G, tm, flags, src_alt, err);
    return cudaGetLastError();
}
template cudaError_t launch_smooth_grid_tma<double>(const GridTiles&, int, const InstState*, const GhostDev*,
                                                    const CUtensorMap*, int, int, int, unsigned*, cudaStream_t);
template cudaError_t launch_smooth_grid_tma<float>(const GridTiles&, int, const InstState*, const GhostDev*,
                                                   const CUtensorMap*, int, int, int, unsigned*, cudaStream_t);
template <typename T>
cudaError_t launch_smooth_grid(const GridTiles& g, int nt, const InstState* S, const GhostDev* G, int flags,
                               int src_alt, int rows, cudaStream_t s) {
    if (nt == 0) return cudaSuccess;
    if (rows == MG_ROWS_WIDE) k_smooth_grid<T, MG_ROWS_WIDE><<<nt, TILE_THREADS, 0, s>>>(g, S, G, flags, src_alt);
    else k_smooth_grid<T, 1><<<nt, TILE_THREADS, 0, s>>>(g, S, G, flags, src_alt);
    return cudaGetLastError();
}
template cudaError_t launch_smooth_grid<double>(const GridTiles&, int, const InstState*, const GhostDev*, int, int,
                                                int, cudaStream_t);
template cudaError_t launch_smooth_grid<float>(const GridTiles&, int, const InstState*, const GhostDev*, int, int,
                                               int, cudaStream_t);
template <typename T>
cudaError_t launch_restrict(const Tile* t, int nt, const LevelDev* LV, const InstDev* I, const InstState* S,
                            const GhostDev* G, int fine_alt, int rows, cudaStream_t s) {
    if (nt == 0) return cudaSuccess;
    if (rows == MG_ROWS_WIDE && few_tiles(nt))
        k_restrict<T, MG_ROWS_WIDE, 4><<<nt, TILE_THREADS, 0, s>>>(t, LV, I, S, G, fine_alt);
    else if (rows == MG_ROWS_WIDE) k_restrict<T, MG_ROWS_WIDE><<<nt, TILE_THREADS, 0, s>>>(t, LV, I, S, G, fine_alt);
    else if (sizeof(T) == 8 && few_tiles(nt)) k_restrict<T, 1, 4><<<nt, TILE_THREADS, 0, s>>>(t, LV, I, S, G, fine_alt);
    else k_restrict<T, 1><<<nt, TILE_THREADS, 0, s>>>(t, LV, I, S, G, fine_alt);
    return cudaGetLastError();
}
template <typename T>
cudaError_t launch_prolong(const Tile* t, int nt, const LevelDev* LV, const InstState* S, int fine_alt,
                           int coarse_alt, int rows, cudaStream_t s) {
    if (nt == 0) return cudaSuccess;
    if (rows == MG_ROWS_WIDE && few_tiles(nt))
        k_prolong<T, MG_ROWS_WIDE, 4><<<nt, TILE_THREADS, 0, s>>>(t, LV, S, fine_alt, coarse_alt);
    else if (rows == MG_ROWS_WIDE) k_prolong<T, MG_ROWS_WIDE><<<nt, TILE_THREADS, 0, s>>>(t, LV, S, fine_alt, coarse_alt);
    else k_prolong<T, 1><<<nt, TILE_THREADS, 0, s>>>(t, LV, S, fine_alt, coarse_alt);
    return cudaGetLastError();
}
template <typename T>
cudaError_t launch_prolong_sweep(const Tile* t, int nt, const LevelDev* LV, const InstDev* I, const InstState* S,
                                 int cur, int coarse_alt, cudaStream_t s) {
    if (nt == 0) return cudaSuccess;
    if (few_tiles(nt)) k_prolong_sweep<T, 4><<<nt, TILE_THREADS, 0, s>>>(t, LV, I, S, cur, coarse_alt);
    else k_prolong_sweep<T, 8><<<nt, TILE_THREADS, 0, s>>>(t, LV, I, S, cur, coarse_alt);
    return cudaGetLastError();
}
template cudaError_t launch_prolong_sweep<double>(const Tile*, int, const LevelDev*, const InstDev*, const InstState*,
                                                  int, int, cudaStream_t);
template cudaError_t launch_prolong_sweep<float>(const Tile*, int, const LevelDev*, const InstDev*, const InstState*,
                                                 int, int, cudaStream_t);
template <typename T>
cudaError_t subcycle_smem_limit(int bytes) {
    // the attribute belongs to the kernel, shared by every solver on the device: only raise it
    static std::mutex mu;
    static int cur[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    dev = dev >= 0 && dev < 64 ? dev : 0;
    std::lock_guard<std::mutex> g(mu);
    if (bytes <= cur[dev]) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(k_subcycle<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_subcycle<T, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess) cur[dev] = bytes;
    return e;
}

template <typename T>
cudaError_t launch_subcycle(const int* sub, int ninst, const LevelDev* LV, const InstDev* I, const InstState* S,
                            int pre, int post, int smem_bytes, cudaStream_t s) {
    if (ninst == 0) return cudaSuccess;
    // programmatic dependent launch: the blocks may start (and stage the
    // geometry image) while the restriction before them runs
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(ninst);
    cfg.blockDim = dim3(SUB_THREADS);
    cfg.dynamicSmemBytes = (size_t)smem_bytes;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    // one block per instance: as many instances as SMs run in one wave of the
    // one-block-per-SM variant
    if (ninst <= device_sm_count()) return cudaLaunchKernelEx(&cfg, k_subcycle<T, 1>, sub, LV, I, S, pre, post);
    return cudaLaunchKernelEx(&cfg, k_subcycle<T, 2>, sub, LV, I, S, pre, post);
}
cudaError_t launch_p_finalize(const Tile* t, int nt, const InstDev* I, const InstState* S, cudaStream_t s) {
    k_p_finalize<<<nt, TILE_THREADS, 0, s>>>(t, I, S);
    return cudaGetLastError();
}
cudaError_t launch_correct(const Tile* t, int nt, const InstDev* I, double* part, cudaStream_t s) {
    k_correct<<<nt, TILE_THREADS, 0, s>>>(t, I, part);
    return cudaGetLastError();
}
cudaError_t launch_correct_reduce(const InstDev* I, InstState* S, const double* part, int ninst,
                                  cudaStream_t s) {
    k_correct_reduce<<<ninst, 256, 0, s>>>(I, S, part);
    return cudaGetLastError();
}
cudaError_t launch_forces(const InstDev* I, InstState* S, double* fpart, unsigned* ftick, int ninst, cudaStream_t s) {
    k_forces<<<ninst * FORCE_BLOCKS, 256, 0, s>>>(I, S, fpart, ftick);
    return cudaGetLastError();
}

template cudaError_t launch_bicg_p<double>(const Tile*, int, const LevelDev*, const InstDev*, const InstState*, int, cudaStream_t);
template cudaError_t launch_bicg_s<double>(const Tile*, int, const LevelDev*, const InstDev*, const InstState*, int, cudaStream_t);
template cudaError_t launch_bicg_apply<double>(const Tile*, int, const LevelDev*, const InstDev*, const InstState*, const GhostDev*, double*, int, int, int, cudaStream_t);
template cudaError_t launch_smooth<double>(const Tile*, int, const LevelDev*, const InstDev*, const InstState*, const GhostDev*, int, int, int, cudaStream_t);
template cudaError_t launch_restrict<double>(const Tile*, int, const LevelDev*, const InstDev*, const InstState*, const GhostDev*, int, int, cudaStream_t);
template cudaError_t launch_bicg_p<float>(const Tile*, int, const LevelDev*, const InstDev*, const InstState*, int, cudaStream_t);
template cudaError_t launch_bicg_s<float>(const Tile*, int, const LevelDev*, const InstDev*, const InstState*, int, cudaStream_t);
template cudaError_t launch_bicg_apply<float>(const Tile*, int, const LevelDev*, const InstDev*, const InstState*, const GhostDev*, double*, int, int, int, cudaStream_t);
template cudaError_t launch_smooth<float>(const Tile*, int, const LevelDev*, const InstDev*, const InstState*, const GhostDev*, int, int, int, cudaStream_t);
template cudaError_t launch_restrict<float>(const Tile*, int, const LevelDev*, const InstDev*, const InstState*, const GhostDev*, int, int, cudaStream_t);
template cudaError_t launch_prolong<double>(const Tile*, int, const LevelDev*, const InstState*, int, int, int,
                                            cudaStream_t);
template cudaError_t launch_prolong<float>(const Tile*, int, const LevelDev*, const InstState*, int, int, int,
                                            cudaStream_t);
template cudaError_t launch_subcycle<double>(const int*, int, const LevelDev*, const InstDev*, const InstState*,
                                             int, int, int, cudaStream_t);
template cudaError_t launch_subcycle<float>(const int*, int, const LevelDev*, const InstDev*, const InstState*,
                                            int, int, int, cudaStream_t);
template cudaError_t subcycle_smem_limit<double>(int);
template cudaError_t subcycle_smem_limit<float>(int);

template cudaError_t launch_bicg_start<double>(const Tile*, int, const LevelDev*, const InstDev*, const InstState*,
                                               const GhostDev*, double*, int, const LoopCtl*, int, cudaStream_t);
template cudaError_t launch_bicg_start<float>(const Tile*, int, const LevelDev*, const InstDev*, const InstState*,
                                              const GhostDev*, double*, int, const LoopCtl*, int, cudaStream_t);
template cudaError_t launch_bicg_x<double>(const Tile*, int, const LevelDev*, const InstDev*, const InstState*, double*,
                                           int, cudaStream_t);
template cudaError_t launch_bicg_x<float>(const Tile*, int, const LevelDev*, const InstDev*, const InstState*, double*,
                                          int, cudaStream_t);

}  // namespace ifx
