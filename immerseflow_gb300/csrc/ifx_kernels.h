// ifx_kernels.h -- host-callable launchers of the CUDA kernels.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include "ifx_dev.h"

namespace ifx {

// ---- method path (kernels_method.cu)
cudaError_t launch_step_begin(const InstDev* I, InstState* S, int n, LoopCtl* ctl, cudaStream_t s);
cudaError_t launch_outflow(const GhostDev* G, int ng, const InstDev* I, cudaStream_t s);
cudaError_t launch_ghost_fill(const GhostDev* G, int ng, const InstDev* I, int comps, double* gval,
                              cudaStream_t s);
cudaError_t launch_conv_rhs(const Tile* t, int nt, const InstDev* I, const InstState* S, cudaStream_t s);
cudaError_t launch_pred_guess(const Tile* t, int nt, const InstDev* I, cudaStream_t s);
// u, v, p (pitched; a null field is skipped) <-> stage (dense rows of nx, the
// three fields one after another)
cudaError_t launch_state_unpack(const double* stage, double* u, double* v, double* p, int nx, int ny, int pitch,
                                cudaStream_t s);
cudaError_t launch_state_pack(const double* u, const double* v, const double* p, double* stage, int nx, int ny,
                              int pitch, cudaStream_t s);
cudaError_t launch_pred_sweep(const Tile* t, int nt, const GhostDev* G, int ng, const InstDev* I,
                              const InstState* S, double* part, int parity, cudaStream_t s);
// Mixed path: FP32 sweep on the correction, and the FP64 refresh (stage 0:
// absorb the correction, stage 1: defect; finalize: absorb after the loop).
// rows: 1 on 32x8 tiles, MG_ROWS_WIDE on 32x32 tiles.
cudaError_t launch_pred_sweep32(const Tile* t, int nt, const GhostDev* G, int ng, const LevelDev* LV, const InstDev* I,
                                const InstState* S, double* part, int parity, int rows, cudaStream_t s);
cudaError_t launch_pred_refresh(const Tile* t, int nt, const GhostDev* G, int ng, const InstDev* I, const InstState* S,
                                int stage, int finalize, const LoopCtl* ctl, int rows, cudaStream_t s);
// One-block-per-instance reductions of the level-0 tile partials; wide: an
// instance has thousands of tiles (loads batched four rows at a time).
cudaError_t launch_pred_reduce(const InstDev* I, InstState* S, const double* part, int ninst, int parity,
                               LoopCtl* ctl, unsigned long long handle, cudaStream_t s, int wide = 0);
cudaError_t launch_face_rhs(const Tile* t, int nt, const InstDev* I, const InstState* S, double* part, int to_final,
                            cudaStream_t s);
cudaError_t launch_rhs_reduce(const InstDev* I, InstState* S, const double* part, int ninst, cudaStream_t s,
                              int wide = 0);
template <typename T>
cudaError_t launch_bicg_start(const Tile* t, int nt, const LevelDev* LV, const InstDev* I, const InstState* S,
                              const GhostDev* G, double* part, int restart_only, const LoopCtl* ctl, int ninst,
                              cudaStream_t s);
cudaError_t launch_bicg_reduce_r(const InstDev* I, InstState* S, const double* part, int ninst, int start,
                                 int mixed, LoopCtl* ctl, unsigned long long handle, cudaStream_t s, int wide = 0);
// Finest-level Krylov phases take rows = 1 (32x8 tiles) or MG_ROWS_WIDE (32x32 tiles).
template <typename T>
cudaError_t launch_bicg_p(const Tile* t, int nt, const LevelDev* LV, const InstDev* I, const InstState* S,
                          int rows, cudaStream_t s);
template <typename T>
cudaError_t launch_bicg_apply(const Tile* t, int nt, const LevelDev* LV, const InstDev* I, const InstState* S,
                              const GhostDev* G, double* part, int e_alt, int which, int rows, cudaStream_t s);
// Direction update (which 0: p_dir, 1: s) fused with the first V-cycle sweep.
template <typename T>
cudaError_t launch_bicg_dir_smooth(const Tile* t, int nt, const LevelDev* LV, const InstDev* I, const InstState* S,
                                   const GhostDev* G, int which, int rows, cudaStream_t s);
cudaError_t launch_bicg_scalar(const InstDev* I, InstState* S, const double* part, int ninst, int which,
                               cudaStream_t s, int wide = 0);
template <typename T>
cudaError_t launch_bicg_s(const Tile* t, int nt, const LevelDev* LV, const InstDev* I, const InstState* S,
                          int rows, cudaStream_t s);
template <typename T>
cudaError_t launch_bicg_x(const Tile* t, int nt, const LevelDev* LV, const InstDev* I, const InstState* S,
                          double* part, int rows, cudaStream_t s);
template <typename T>
cudaError_t launch_smooth(const Tile* t, int nt, const LevelDev* LV, const InstDev* I, const InstState* S,
                          const GhostDev* G, int flags, int src_alt, int rows, cudaStream_t s);
// The same sweep with each tile staged in shared memory by TMA loads (tm:
// TMA_MAPS_PER_LEVEL tensor maps per LevelDev entry); *err is set when a copy
// does not complete.
template <typename T>
cudaError_t launch_smooth_tma(const Tile* t, int nt, const LevelDev* LV, const InstDev* I, const InstState* S,
                              const GhostDev* G, const CUtensorMap* tm, int flags, int src_alt, int rows, unsigned* err,
                              cudaStream_t s);
// The same with each tile staged by TMA (see launch_smooth_tma).
template <typename T>
cudaError_t launch_smooth_grid_tma(const GridTiles& g, int nt, const InstState* S, const GhostDev* G,
                                   const CUtensorMap* tm, int flags, int src_alt, int rows, unsigned* err,
                                   cudaStream_t s);
// Smoothing sweep of one level of a one-instance solver (tiles from the grid).
template <typename T>
cudaError_t launch_smooth_grid(const GridTiles& g, int nt, const InstState* S, const GhostDev* G, int flags,
                               int src_alt, int rows, cudaStream_t s);
template <typename T>
cudaError_t launch_restrict(const Tile* t, int nt, const LevelDev* LV, const InstDev* I, const InstState* S,
                            const GhostDev* G, int fine_alt, int rows, cudaStream_t s);
template <typename T>
cudaError_t launch_prolong(const Tile* t, int nt, const LevelDev* LV, const InstState* S, int fine_alt,
                           int coarse_alt, int rows, cudaStream_t s);
// Prolongation plus the first post-smoothing sweep of a coarse level (32x8
// tiles): reads buffer cur, writes buffer cur ^ 1.
template <typename T>
cudaError_t launch_prolong_sweep(const Tile* t, int nt, const LevelDev* LV, const InstDev* I, const InstState* S,
                                 int cur, int coarse_alt, cudaStream_t s);
template <typename T>
cudaError_t launch_subcycle(const int* sub, int ninst, const LevelDev* LV, const InstDev* I, const InstState* S,
                            int pre, int post, int smem_bytes, cudaStream_t s);
// Cluster V-cycle (kernels_cluster.cu): shared-memory bytes for one instance,
// set-up (attributes; *ok = 1 when ninst clusters fit on the device at once),
// launch (one cluster per instance; writes the finest level's correction).
size_t cluster_vcycle_bytes(int nd, const int* nx, const int* ny, int tsize, size_t sub_bytes);
template <typename T>
cudaError_t cluster_vcycle_setup(int smem_bytes, int ninst, int* ok);
template <typename T>
cudaError_t launch_vcycle_cluster(const int* sub, int ninst, const LevelDev* LV, const InstDev* I, const InstState* S,
                                  const GhostDev* G, int pre, int post, int smem_bytes, cudaStream_t s);
// Allows both k_subcycle<T, MINB> variants `bytes` of dynamic shared memory (above the 48 KB default).
template <typename T>
cudaError_t subcycle_smem_limit(int bytes);
cudaError_t launch_p_finalize(const Tile* t, int nt, const InstDev* I, const InstState* S, cudaStream_t s);
cudaError_t launch_correct(const Tile* t, int nt, const InstDev* I, double* part, cudaStream_t s);
cudaError_t launch_correct_reduce(const InstDev* I, InstState* S, const double* part, int ninst,
                                  cudaStream_t s);
// fpart: 2 * FORCE_BLOCKS doubles per instance; ftick: one zeroed counter per instance
cudaError_t launch_forces(const InstDev* I, InstState* S, double* fpart, unsigned* ftick, int ninst, cudaStream_t s);

// ---- immersed-boundary set-up (kernels_ibm.cu, built without FMA contraction)
cudaError_t launch_tag(const InstDev* I, int inst, int n_cells, uint8_t* type, cudaStream_t s);
cudaError_t launch_mark_ghosts(const InstDev* I, int inst, int n_interior, uint8_t* type, cudaStream_t s);
// threads: block size; small blocks spread the FP64 latency chains of the
// ghosts over more SMs (the per-step refresh of moving bodies uses 32)
cudaError_t launch_ghost_weights(GhostDev* G, const int* ibm, int nibm, const InstDev* I, double* bi_ip,
                                 cudaStream_t s, int threads = 128);
// ---- moving bodies (kernels_move.cu)
cudaError_t launch_move_geometry(InstDev* I, InstState* S, const LevelDev* LV, GhostDev* G, const int* mv, int nmv,
                                 cudaStream_t s);
cudaError_t launch_move_init(InstDev* I, InstState* S, const int* mv, int nmv, const int* n_ibm, cudaStream_t s);
cudaError_t launch_move_forces(const InstDev* I, const InstState* S, const int* mv, int nmv, cudaStream_t s);

// ---- reference path (kernels_ref.cu), one instance, dense rows (pitch = nx)
struct RefDev {
    int nx, ny;
    double dt, re;
    double w_ad;  // relaxation of the velocity Jacobi update (1: none)
    const double *dx, *dy, *iblank;
    double *aP, *aE, *aW, *aN, *aS, *sx, *sy, *uf, *vf, *res;
};
cudaError_t launch_ref_coeffs(const RefDev& R, cudaStream_t s);
cudaError_t launch_ref_velf(const RefDev& R, const double* u, const double* v, cudaStream_t s);
cudaError_t launch_ref_bc(const RefDev& R, double* u, double* v, cudaStream_t s);
cudaError_t launch_ref_source(const RefDev& R, const double* u, const double* v, cudaStream_t s);
cudaError_t launch_ref_jacobi(const RefDev& R, const double* u, const double* v, double* un, double* vn,
                              cudaStream_t s);
// |u_old - u_new| + |v_old - v_new| summed over fluid interior cells -> out[0] (u), out[1] (v)
cudaError_t launch_ref_resid(const RefDev& R, const double* uo, const double* un, const double* vo,
                             const double* vn, double* out, cudaStream_t s);
cudaError_t launch_ref_init(int nx, int ny, const double* xc, const double* yc, double* u, double* v,
                            double* p, cudaStream_t s);
// nsteps ADsolver steps in one cooperative launch of `grid` blocks (grid
// barriers between the phases, stop rule evaluated on the device);
// ref_steps_grid gives the grid (co-resident blocks, at most one per 256-cell
// chunk), 0 when cooperative launch is unavailable.
struct GridBar;
int ref_steps_grid(int nx, int ny);
cudaError_t launch_ref_steps(const RefDev& R, double* u, double* v, double* ut, double* vt, GridBar* bar,
                             int itermax, int nsteps, int* iters, int grid, cudaStream_t s);
// Jacobi Laplace (PPESolver intent): coefficients, BC, sweep, signed residual sum -> out[0]
cudaError_t launch_ref_ppe_coeffs(const RefDev& R, cudaStream_t s);
cudaError_t launch_ref_ppe_bc(const RefDev& R, double* p, cudaStream_t s);
cudaError_t launch_ref_ppe_sweep(const RefDev& R, const double* p, double* pn, double* out, cudaStream_t s);
// One red-black point Gauss-Seidel / SOR iteration in place (red (i+j even)
// cells, then black), then the signed residual sum -> out[0].
cudaError_t launch_ref_ppe_rbgs(const RefDev& R, double* p, double w, double* out, cudaStream_t s);
// One zebra x-line SOR iteration in place (odd rows, then even rows; each row
// solved exactly along x with the Thomas algorithm, scratch cp/dp of nx*ny),
// then the signed residual sum -> out[0].
cudaError_t launch_ref_ppe_lines(const RefDev& R, double* p, double* cp, double* dp, double w, double* out,
                                 cudaStream_t s);

}  // namespace ifx
