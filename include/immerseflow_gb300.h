/*
 * immerseflow_gb300.h -- C ABI of the GB300-native fractional-step / ghost-cell
 * immersed-boundary solver.
 *
 * The reference (ImmerseFlow++) exposes no library API: its boundary is the
 * executable `main` (src/main.cu:75-102) plus the file surface (inputs.txt,
 * xgrid/ygrid files, Tecplot outputs).  Each entry point below names the
 * reference routine it replaces.  All functions return an ifx_status code
 * instead of calling exit(1) (the reference's CHECK_CUDA_ERROR,
 * src/header/globalVariables.cuh:91-107).  Host buffers are owned by the
 * caller, device state by the solver handle.  A handle is used by one host
 * thread at a time.
 *
 * Index convention (same as the reference, src/include/ADSolver.cu:10):
 *   cells (i,j), i = 0..nx-1 fastest, nx = NX+2 (one ghost layer each side),
 *   host arrays are dense: q[i + j*nx].
 *   u faces: uf[i + (j-1)*(nx-1)], i = 0..nx-2, j = 1..ny-2  (east face of cell i)
 *   v faces: vf[(i-1) + j*(nx-2)], i = 1..nx-2, j = 0..ny-2  (north face of cell j)
 */
#ifndef IMMERSEFLOW_GB300_H
#define IMMERSEFLOW_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
typedef int ifx_status;
#define IFX_OK                 0
#define IFX_ERR_ARG            1  /* bad argument / size                       */
#define IFX_ERR_IO             2  /* file cannot be opened or written          */
#define IFX_ERR_PARSE          3  /* malformed inputs.txt or grid file         */
#define IFX_ERR_CUDA           4  /* CUDA runtime error (message in last_error) */
#define IFX_ERR_NOMEM          5  /* device or host allocation failed          */
#define IFX_ERR_NOT_CONVERGED  6  /* an iteration cap was hit                  */
#define IFX_ERR_DIVERGED       7  /* NaN/Inf detected in the state             */
#define IFX_ERR_BUDGET         8  /* request does not fit the HBM budget       */
#define IFX_ERR_STATE          9  /* call not valid in the current state       */
#define IFX_ERR_NODEVICE      10  /* no CUDA device                            */
#define IFX_ERR_GEOMETRY      11  /* a moving body left the domain, or its IBM
                                     ghosts outgrew their slots (the instance is
                                     retired, like IFX_ERR_DIVERGED)            */

/* ---------------------------------------------------------------- enums */
#define IFX_MODE_REFERENCE 0  /* ADsolver-only semantics of the reference      */
#define IFX_MODE_METHOD    1  /* full fractional step: predictor/PPE/projection */

#define IFX_PREC_FP64  0      /* every kernel in FP64                          */
#define IFX_PREC_MIXED 1      /* FP32 sweeps, FP64 residuals / defect correction */

#define IFX_INIT_VORTEX  0    /* vortex in uniform flow, src/include/preSim.cu:70-73 */
#define IFX_INIT_UNIFORM 1    /* u = bc_u[W], v = 0 in the fluid               */
#define IFX_INIT_REST    2    /* u = v = 0                                     */

#define IFX_SIDE_W 0
#define IFX_SIDE_E 1
#define IFX_SIDE_S 2
#define IFX_SIDE_N 3

#define IFX_BC_WALL    0      /* Dirichlet velocity (bc_u, bc_v), Neumann p     */
#define IFX_BC_INFLOW  1      /* Dirichlet velocity (bc_u, bc_v), Neumann p     */
#define IFX_BC_OUTFLOW 2      /* convective outflow, Dirichlet p = 0           */
#define IFX_BC_SLIP    3      /* zero normal velocity, zero shear, Neumann p   */

#define IFX_BODY_NONE    0
#define IFX_BODY_ELLIPSE 1    /* ellipse / circle: centre, semi-axes a >= b, angle */

#define IFX_FIELD_U        0  /* cell u, nx*ny                                 */
#define IFX_FIELD_V        1  /* cell v, nx*ny                                 */
#define IFX_FIELD_P        2  /* cell p, nx*ny                                 */
#define IFX_FIELD_IBLANK   3  /* 1 fluid / 0 solid as double, nx*ny            */
#define IFX_FIELD_UF       4  /* u faces, (nx-1)*(ny-2)                         */
#define IFX_FIELD_VF       5  /* v faces, (nx-2)*(ny-1)                         */
#define IFX_FIELD_CELLTYPE 6  /* 0 solid, 1 fluid, 2 IBM ghost, 3 domain ghost (as double) */
#define IFX_FIELD_DIV      7  /* face divergence per fluid cell, nx*ny           */
#define IFX_FIELD_XC       8  /* cell centres x, nx                             */
#define IFX_FIELD_YC       9  /* cell centres y, ny                             */

/* Pressure-solve method of ifx_ppe_reference (extension keyword PPE-Method).
 * The reference parses PPE_Solver (inputs/inputs.txt:14: 1 point GS, 2 line
 * SOR) but always runs Jacobi (src/include/PPESolver.cu:13-31), also for its
 * own PPE_Solver = 1 inputs; PPE_Solver is therefore kept as read and this
 * field selects, with the same numbering.  METHOD mode accepts only 0. */
#define IFX_PPE_JACOBI   0    /* the reference's Jacobi sweep                   */
#define IFX_PPE_POINT_GS 1    /* red-black point Gauss-Seidel / SOR (w-PPE)     */
#define IFX_PPE_LINE_SOR 2    /* zebra x-line SOR, tridiagonal row solves (w-PPE) */

/* Body motion (METHOD mode, ellipse body).  IFX_MOTION_PRESCRIBED moves the
 * body rigidly: at time t = n dt (step n) the centre and the angle are
 *   x(t) = body_cx + motion_u t + motion_amp_x (sin(w t + phx) - sin(phx))
 *   y(t) = body_cy + motion_v t + motion_amp_y (sin(w t + phy) - sin(phy))
 *   a(t) = body_angle_deg + motion_amp_deg (sin(w t + pha) - sin(pha))
 * with w = 2 pi motion_freq and the phases in degrees, so that t = 0 is the
 * configured pose.  The reference claims moving boundaries (README.md:7,11)
 * but has no code for them. */
#define IFX_MOTION_NONE       0
#define IFX_MOTION_PRESCRIBED 1

#define IFX_PATH_MAX 512

/* --------------------------------------------------------------- config */
/*
 * Fields up to write_interval are the reference's CFDInput
 * (src/header/globalVariables.cuh:15-33) read by the same keyword grammar
 * (src/main.cu:10-59).  The rest are extension keywords that the reference
 * grammar ignores.
 */
typedef struct ifx_config {
    int    restart, restart_time;
    int    nx, ny;                 /* interior cells, as written in inputs.txt */
    double lx, ly;
    int    w_ad, w_ppe, ad_itermax, ppe_itermax, ad_solver, ppe_solver;
    double error_max, tmax, dt, re, mu;
    int    write_interval;

    int    mode;                   /* IFX_MODE_*                                */
    int    precision;              /* IFX_PREC_*                                */
    int    init;                   /* IFX_INIT_*                                */
    int    bc_type[4];             /* per side W,E,S,N: IFX_BC_*                */
    double bc_u[4], bc_v[4];       /* Dirichlet values per side                 */
    double outflow_uc;             /* convective outflow speed                  */
    int    body;                   /* IFX_BODY_*                                */
    double body_cx, body_cy, body_a, body_b, body_angle_deg;
    double ppe_tol;                /* method mode: ||r||_2 <= ppe_tol*||b||_2    */
    double ad_tol;                 /* method mode: mean |Jacobi update| bound   */
    int    mg_pre, mg_post;        /* multigrid smoothing sweeps                */
    double mg_omega;               /* weighted-Jacobi factor                    */
    int    mixed_inner;            /* FP32 predictor sweeps per FP64 residual
                                      (at least 2)                              */
    double force_ref_u, force_ref_len;   /* drag/lift normalisation          */
    int    ppe_method;             /* IFX_PPE_*: REFERENCE-mode pressure solve  */
    double relax_ad, relax_ppe;    /* w-AD, w-PPE as read (0 or 1: none)        */
    int    motion;                 /* IFX_MOTION_*                              */
    double motion_u, motion_v;     /* constant velocity of the centre           */
    double motion_amp_x, motion_amp_y, motion_amp_deg;  /* harmonic amplitudes  */
    double motion_freq;            /* harmonic frequency (1/time)               */
    double motion_phase_x, motion_phase_y, motion_phase_deg;  /* degrees        */
    int    coarse_sweeps;          /* red-black SOR sweeps on the coarsest
                                      multigrid level                           */
    double restart_drop;           /* mixed path: the FP32 Krylov recursion is
                                      restarted from the FP64 true residual once
                                      its residual fell by this factor ...      */
    int    restart_every;          /* ... or after this many iterations         */
    char   xgrid[IFX_PATH_MAX];    /* face-coordinate files (<idx> <coord>)     */
    char   ygrid[IFX_PATH_MAX];
} ifx_config;

/* Per-instance statistics of the last ifx_step call. */
typedef struct ifx_stats {
    long long steps;               /* time steps done since creation            */
    int    last_ad_iters;          /* predictor sweeps in the last step         */
    int    last_ppe_iters;         /* PPE iterations (outer) in the last step   */
    double last_ad_metric;         /* final predictor metric                    */
    double last_ppe_residual;      /* final relative PPE residual               */
    double max_div;                /* max |div U| over fluid cells after projection */
    double cd, cl;                 /* drag and lift coefficients                */
    double mass_flux_in, mass_flux_out;
    long long ad_iters_total, ppe_iters_total;
    long long kernel_launches;     /* kernels of this library launched so far   */
    int    n_fluid, n_ibm_ghost, mg_levels;
    int    status;                 /* sticky per-instance status: IFX_OK,
                                      IFX_ERR_DIVERGED (non-finite state; the
                                      instance is retired, the others go on),
                                      IFX_ERR_NOT_CONVERGED (a pressure solve
                                      stopped at ppe_itermax; steps go on)     */
} ifx_stats;

/* ------------------------------------------------------ library / errors */
const char* ifx_status_string(ifx_status s);
/* Message of the last failing call on this host thread. */
const char* ifx_last_error(void);
/* Library version string. */
const char* ifx_version(void);

/* ---------------------------------------------------------- file surface */
/* Defaults = the reference's inputs/inputs.txt values, mode REFERENCE. */
void       ifx_config_default(ifx_config* cfg);
/* readInputFile (src/main.cu:10-59): keyword line, values on the next line.
 * Grid paths default to xgrid.dat2 / ygrid.dat2 beside the inputs file
 * (src/include/preSim.cu:268,281). */
ifx_status ifx_config_read(const char* inputs_path, ifx_config* cfg);
/* Grid-file loop of readGridData (src/include/preSim.cu:267-291):
 * reads n lines "<index> <coordinate>". */
ifx_status ifx_grid_read(const char* path, int n, double* coords);
/* write_results_to_file (src/include/postSim.cu:41-66): Tecplot ASCII POINT. */
ifx_status ifx_write_tecplot(const char* path, int nx, int ny, const double* x,
                             const double* y, const double* q);

/* ----------------------------------------------------------------- solver */
typedef struct ifx_solver ifx_solver;

/* Largest instance: the kernels index an instance's cells with 32-bit
 * integers over rows padded to a multiple of 32 cells, so the bound applies to
 * IFX_PADDED_CELLS(nx, ny) = roundup(nx+2, 32) * (ny+2), which is at least
 * the cell count with the ghost ring, (nx+2)*(ny+2).  ifx_config_read refuses
 * larger grids with IFX_ERR_PARSE, the create calls with IFX_ERR_ARG. */
#define IFX_MAX_CELLS (1 << 28)
#define IFX_PADDED_CELLS(nx, ny) ((((long long)(nx) + 2 + 31) / 32 * 32) * ((long long)(ny) + 2))

/* allocation + readGridData + initializeData (src/main.cu:86-90,
 * src/include/preSim.cu:147-240).  xf has cfg->nx+1 entries, yf cfg->ny+1. */
ifx_status ifx_create(const ifx_config* cfg, const double* xf, const double* yf,
                      ifx_solver** out);
/* Same, reading inputs.txt and the grid files it names. */
ifx_status ifx_create_from_file(const char* inputs_path, ifx_solver** out);
/* Batched solver: n independent instances of uneven size, advanced together
 * (no reference counterpart; the reference runs one instance per process). */
ifx_status ifx_create_batch(int n, const ifx_config* cfgs, const double* const* xfs,
                            const double* const* yfs, ifx_solver** out);
int        ifx_num_instances(const ifx_solver* s);
/* Grid size of instance inst including the ghost ring (nx = NX+2, ny = NY+2). */
ifx_status ifx_get_dims(const ifx_solver* s, int inst, int* nx, int* ny);

/* One reference time step is ImmerseFlow::ADsolver (src/include/ADSolver.cu:268-395)
 * in REFERENCE mode; in METHOD mode it is predictor -> PPE -> projection.
 * METHOD mode returns IFX_ERR_DIVERGED in the call in which an instance's state
 * becomes non-finite; that instance is retired (its stats.status says so) and
 * the other instances of a batch are unaffected. */
ifx_status ifx_step(ifx_solver* s, int nsteps);

/* Asynchronous form (no reference counterpart): ifx_step_async issues nsteps
 * steps on the solver's own stream and returns; ifx_step_wait waits for them
 * and checks the state (every other call on the handle waits first).  Handles
 * on different streams overlap on the device.  The host-loop execution mode
 * completes the steps inside ifx_step_async. */
ifx_status ifx_step_async(ifx_solver* s, int nsteps);
ifx_status ifx_step_wait(ifx_solver* s);

/* Execution of a METHOD-mode step; all modes give bit-identical results. */
#define IFX_EXEC_DEFAULT    (-1) /* IFX_EXEC environment variable, else persistent */
#define IFX_EXEC_PERSISTENT 0    /* one cooperative launch per ifx_step call        */
#define IFX_EXEC_GRAPH      1    /* one CUDA-graph launch per step (device loops)   */
#define IFX_EXEC_HOST       2    /* one launch per phase, loops driven by the host  */
ifx_status ifx_set_exec_mode(ifx_solver* s, int mode);
ifx_status ifx_get_exec_mode(ifx_solver* s, int* mode);
/* Blocks of the persistent mode's cooperative launch (no reference
 * counterpart): 0 = every block that can be co-resident (the default), else at
 * most that many.  The phases stride over their tiles, so results do not
 * depend on it; fewer blocks make each grid barrier cheaper.  ifx_autotune
 * also tries one block per SM for handles of up to eight instances. */
ifx_status ifx_set_persistent_grid(ifx_solver* s, int blocks);
ifx_status ifx_get_persistent_grid(ifx_solver* s, int* blocks);

/* Autotuner (no reference counterpart): times `steps` steps in each available
 * execution mode, multigrid tile shape and persistent grid (after one warm-up
 * step each),
 * restores the solver state afterwards, and keeps the fastest.  All of them
 * give bit-identical results, so tuning never changes an answer.  A handle with
 * a moving body is refused (IFX_ERR_STATE): trial steps would move its
 * geometry, which the restored state does not hold. */
ifx_status ifx_autotune(ifx_solver* s, int steps, int* chosen_mode, double* ms_per_step);
/* Sweep schedule of a METHOD-mode step (no reference counterpart: the
 * reference reads solver settings in inputs.txt that it never uses,
 * inputs/inputs.txt:14, src/main.cu:39-42).  The pressure solve stops on the
 * same rule whatever the schedule (FP64 true residual <= ppe_tol ||b||), so a
 * schedule changes the fields only within that tolerance; it changes how many
 * iterations, and how much time, the solve takes. */
typedef struct ifx_schedule {
    int    mg_pre, mg_post;        /* weighted-Jacobi sweeps before / after the
                                      coarse-grid correction of the V-cycle     */
    double mg_omega;               /* weighted-Jacobi factor                    */
    int    coarse_sweeps;          /* red-black SOR sweeps on the coarsest level */
    int    mixed_inner;            /* mixed path: FP32 predictor sweeps per FP64
                                      defect (at least 2)                       */
    double restart_drop;           /* mixed path: FP32 Krylov recursion restarted
                                      from the FP64 true residual after this drop */
    int    restart_every;          /* ... or after this many iterations         */
} ifx_schedule;
/* Every instance of the handle takes the schedule (the configuration fields of
 * the same names). */
ifx_status ifx_set_schedule(ifx_solver* s, const ifx_schedule* sched);
ifx_status ifx_get_schedule(const ifx_solver* s, int inst, ifx_schedule* out);
/* Autotuner of the sweep schedule (no reference counterpart): a one-pass
 * coordinate search over the pre/post sweep pair, omega, the coarsest-level
 * sweeps and, in mixed precision, mixed_inner and the restart drop.  Each
 * candidate runs a warm-up step and `steps` timed steps from the same saved
 * state; a candidate counts only if every pressure solve met its stop rule and
 * no instance diverged, and it replaces the current best only when it is more
 * than 1% faster.  The state is restored afterwards and the fastest valid
 * schedule is kept (*chosen, device ms per step).  Run it after
 * ifx_autotune, in the execution mode that will be used.  A handle with a
 * moving body is refused (IFX_ERR_STATE), as by ifx_autotune. */
ifx_status ifx_autotune_schedule(ifx_solver* s, int steps, ifx_schedule* chosen, double* ms_per_step);
/* Multigrid tile shape of the graph and host-loop modes: 1 = 32x8 cells (one
 * row per thread), 4 = 32x32 cells (four rows per thread, more loads in flight;
 * suits large batches).  Results do not depend on it.  The autotuner sets it. */
ifx_status ifx_set_mg_tile_rows(ifx_solver* s, int rows);
ifx_status ifx_get_mg_tile_rows(const ifx_solver* s, int* rows);
/* Cluster V-cycle of the graph and host-loop modes: the multigrid levels above
 * the small ones held in the distributed shared memory of one 16-CTA
 * thread-block cluster per instance, phases separated by cluster barriers.
 * Available when every instance fits (about 100k cells per instance in the
 * mixed path) and the device runs that many clusters at once.  Results do not
 * depend on it.  The autotuner considers it. */
ifx_status ifx_set_cluster_vcycle(ifx_solver* s, int on);
ifx_status ifx_get_cluster_vcycle(const ifx_solver* s, int* available, int* on);

/* Batch membership (no reference counterpart): an inactive instance is left
 * unchanged by later steps while the others advance. */
ifx_status ifx_set_instance_active(ifx_solver* s, int inst, int active);
/* Device memory held by the handle, bytes. */
ifx_status ifx_device_bytes(const ifx_solver* s, size_t* bytes);

/* ImmerseFlow::PPESolver (src/include/PPESolver.cu:137-205): Jacobi Laplace with
 * p = 100 on the i=0 and j=0 ghosts, stopped on the signed residual sum. */
ifx_status ifx_ppe_reference(ifx_solver* s, int* iters);

/* Largest grid (cells including the ghost ring, nx*ny) that
 * ifx_ppe_reference_noalloc accepts: 132 x 132 including the ghost ring, a
 * 130 x 130 interior (the 128 x 128 cavity, 130 x 130 with its ring, fits).
 * Its scratch is ~0.84 MB of device memory per GPU. */
#define IFX_NOALLOC_MAX_CELLS (132 * 132)
/* Pressure solve for callers that cannot allocate device memory (a plug-in
 * whose host application owns every device allocation, a service that budgets
 * device memory up front, a latency-bound loop that cannot afford the device
 * synchronisation cudaFree implies).  No counterpart in the reference: it is the solve of ifx_ppe_reference
 * (PPESolver's Jacobi Laplace with p = 100 on the i=0 / j=0 ghosts, stopped when
 * the signed residual sum drops to tol or after itermax sweeps) run on buffers
 * the caller owns: d_dx, d_dy (nx*ny each, the full width arrays of readGridData,
 * src/include/preSim.cu:328-355) and d_p (nx*ny, initial pressure in, solution
 * out), all device pointers; stream is a cudaStream_t (NULL: default stream).
 * It calls no cudaMalloc/cudaFree: its scratch is one fixed device array inside
 * this library, present on every GPU that loads the library until exit, so
 * nx*ny above IFX_NOALLOC_MAX_CELLS returns IFX_ERR_ARG.  The first call on a
 * device looks up that array's device address (cudaGetSymbolAddress) and keeps
 * it for the life of the process; make that first call before any stream
 * capture, and do not cudaDeviceReset a device between calls (the kept
 * address would no longer be valid).  All calls share the array, so
 * calls that overlap on the GPU (other streams, other threads) race: serialise
 * them. */
ifx_status ifx_ppe_reference_noalloc(const double* d_dx, const double* d_dy, int nx, int ny, double* d_p,
                                     int itermax, double tol, int* iters, void* stream);

/* Host <-> device field copies (saveDataToFile's D2H, src/include/postSim.cu:10-39). */
ifx_status ifx_get_field(ifx_solver* s, int field, double* host, size_t n);
ifx_status ifx_set_field(ifx_solver* s, int field, const double* host, size_t n);
ifx_status ifx_get_field_i(ifx_solver* s, int inst, int field, double* host, size_t n);
ifx_status ifx_set_field_i(ifx_solver* s, int inst, int field, const double* host, size_t n);
/* The state of one instance in one call: u, v and p, each nx*ny doubles in
 * dense rows (a null pointer skips that field), staged through one dense
 * device buffer: one contiguous copy per field, one kernel between the dense
 * and the pitched layout, one synchronisation (the per-field calls above
 * synchronise once per field and copy row by row).  For a caller that passes
 * the whole state in and out every step. */
ifx_status ifx_set_state(ifx_solver* s, int inst, const double* u, const double* v, const double* p, size_t n);
ifx_status ifx_get_state(ifx_solver* s, int inst, double* u, double* v, double* p, size_t n);
/* ifx_set_state, ifx_step(nsteps) and ifx_get_state in one call (no reference
 * counterpart): the state copies, the steps and the result copies are issued
 * back to back on the solver's stream and the call waits once, at the end, so
 * a caller that exchanges the state every step pays one host round trip instead
 * of three.  NULL inputs keep the device values; NULL outputs are not copied;
 * inputs and outputs may be the same buffers.  The outputs are written also
 * when the steps report an error (a diverged instance is flagged, as by
 * ifx_step); the return value is the steps' status. */
ifx_status ifx_step_state(ifx_solver* s, int inst, const double* u_in, const double* v_in, const double* p_in,
                          int nsteps, double* u_out, double* v_out, double* p_out, size_t n);
/* Writes p.dat, uc.dat, vc.dat, final_results.dat into dir (src/include/postSim.cu:10-66). */
ifx_status ifx_write_results(ifx_solver* s, const char* dir);
ifx_status ifx_forces(ifx_solver* s, double* cd, double* cl);
/* Immersed-boundary ghost table of instance inst (no reference counterpart:
 * the reference has no ghost-cell code, src/include/preSim.cu:110-136).
 * Writes up to cap entries in row-major cell order: dense cell index
 * (i + j*nx), the 4 image-point stencil cells, Dirichlet (velocity) and
 * Neumann (pressure) weights, and body-intercept / image-point coordinates
 * (bi_ip[4k..4k+3] = BIx, BIy, IPx, IPy).  Any output may be NULL.
 * *count receives the number of ghost cells. */
ifx_status ifx_get_ibm_ghosts(ifx_solver* s, int inst, int cap, int* cells, int* nb, double* wu,
                              double* wp, double* bi_ip, int* count);
ifx_status ifx_get_stats(ifx_solver* s, int inst, ifx_stats* out);
/* Device milliseconds of the last ifx_step call, timed with CUDA events on
 * the solver's own stream. */
ifx_status ifx_last_step_ms(ifx_solver* s, double* ms);
ifx_status ifx_synchronize(ifx_solver* s);

/* ------------------------------------------------------- restart / checkpoint */
/* The reference parses `Restart Restart_Time` and `Write Interval`
 * (src/main.cu:27-30,50-53) without using them; its Fortran predecessor
 * restarts from an ASCII snapshot (test/UTIL_PRE_SIM.f90:120-149).
 * Binary checkpoint of one instance: every array a step carries into the next
 * (METHOD: cell and face velocities, convection history, pressure and the
 * pressures of the two steps before, the predictor increment of the step
 * before, outflow boundary values, iteration state; REFERENCE: u, v, p), so
 * that a run
 * restarted from it continues bit for bit.  A checkpoint loads into an
 * instance of the same mode, grid, body and boundary types (any precision,
 * any batch position); a header and a checksum are checked.  Loading into a
 * one-instance handle also sets its step count. */
ifx_status ifx_checkpoint_bytes(const ifx_solver* s, int inst, size_t* bytes);
ifx_status ifx_checkpoint_save(ifx_solver* s, int inst, void* buf, size_t n);
ifx_status ifx_checkpoint_load(ifx_solver* s, int inst, const void* buf, size_t n);
/* Every instance of the handle to / from one file (written atomically). */
ifx_status ifx_checkpoint_write(ifx_solver* s, const char* path);
ifx_status ifx_checkpoint_read(ifx_solver* s, const char* path);
/* ASCII snapshot in the predecessor's layout: three header lines (the third
 * names the step), then one row per cell including ghosts, j outer, i inner:
 * x y u v p uf vf iblank (uf / vf: east / north face velocity of the cell).
 * It holds no convection history: the first step after reading it starts the
 * Adams-Bashforth history again (forward-Euler convection, as at t = 0). */
ifx_status ifx_write_snapshot_ascii(ifx_solver* s, int inst, const char* path);
ifx_status ifx_read_snapshot_ascii(ifx_solver* s, int inst, const char* path);

/* ------------------------------------------------------------ time history */
/* probe_init (test/UTIL_PRE_SIM.f90:172-202): probe.dat holds the probe count,
 * a skipped line, then one "x y" line per probe.  *n receives the count; up to
 * cap probes are stored in xy (x0, y0, x1, y1, ...). */
ifx_status ifx_probes_read(const char* path, int cap, double* xy, int* n);
/* METHOD mode: record, at the end of every step, the step count, cd, cl and
 * u, v, p at each probe into a device ring buffer of `capacity` records (0
 * switches recording off).  A probe samples the cell whose centre is nearest
 * in x and in y (first minimum over the cell centres, ghosts included, as
 * probe_init's minloc).  Resets the record count. */
ifx_status ifx_set_history(ifx_solver* s, int inst, int capacity, int nprobes, const double* xy);
/* Cell indices (0-based, ghost cell 0) of the probes; *n = probe count. */
ifx_status ifx_get_probe_cells(ifx_solver* s, int inst, int cap, int* i, int* j, int* n);
/* The newest min(records, capacity, cap) records, oldest first; each row has
 * *width = 3 + 3*nprobes doubles: step, cd, cl, then u, v, p per probe. */
ifx_status ifx_get_history(ifx_solver* s, int inst, int cap, double* rows, int* n, int* width);
/* probe_output.dat: a header line (count, probe cell centres x then y, cell
 * indices i then j), a blank line, " Time  U   V  P", then one row per
 * recorded step: time, and u v p of each probe. */
ifx_status ifx_write_probe_file(ifx_solver* s, int inst, const char* path);
/* Force history: " Time  Cd  Cl", then one row per recorded step. */
ifx_status ifx_write_force_file(ifx_solver* s, int inst, const char* path);

/* ------------------------------------------------------------------ server */
/* Continuous-batching solve server (no reference counterpart; the reference
 * runs one case per process, src/main.cu:75-102).  Submitted METHOD-mode cases
 * wait in FIFO order; each ifx_server_tick admits the waiting requests that
 * fit in the device-memory budget as one batched cohort with its own stream
 * and state kept on the device, then advances every live cohort by up to
 * steps_per_tick time steps (all cohorts issued before any is waited for, so
 * they overlap on the GPU).  A mixed-precision cohort of at least 2^18 cells
 * runs its tile phases on 32x32 tiles (ifx_set_mg_tile_rows), a smaller one on
 * 32x8 tiles.  A request that completed its steps is copied out (u, v, p, stats)
 * and stops computing; a cohort whose requests all finished frees its memory.
 * Results do not depend on the cohort a request ran in.  One host thread per
 * server. */
typedef struct ifx_server ifx_server;
#define IFX_REQ_WAITING  0
#define IFX_REQ_RUNNING  1
#define IFX_REQ_FINISHED 2
#define IFX_REQ_FAILED   3
/* Device bytes one METHOD-mode instance of this configuration needs (estimate). */
ifx_status ifx_estimate_bytes(const ifx_config* cfg, size_t* bytes);
ifx_status ifx_server_create(size_t hbm_budget_bytes, int max_cohort, ifx_server** out);
/* Execution mode of the cohorts (IFX_EXEC_*, default IFX_EXEC_GRAPH). */
ifx_status ifx_server_set_exec_mode(ifx_server* v, int mode);
/* Steps a cohort advances per tick at most (default 1; a cohort never runs past
 * the step count of one of its requests, so results do not depend on it). */
ifx_status ifx_server_set_steps_per_tick(ifx_server* v, int steps);
ifx_status ifx_server_submit(ifx_server* v, const ifx_config* cfg, const double* xf, const double* yf,
                             int nsteps, long long* id);
ifx_status ifx_server_tick(ifx_server* v, int* n_finished);
/* Pre-emption between ticks: a running request's state is saved as a binary
 * checkpoint in host memory, its instance stops, and it waits again (at the
 * front of the queue if front != 0, else at the back).  When admitted again
 * it continues from the checkpoint; its result is the same as if it had not
 * been interrupted. */
ifx_status ifx_server_preempt(ifx_server* v, long long id, int front);
/* Finished (or failed) request ids, oldest first; each is returned once. */
ifx_status ifx_server_poll(ifx_server* v, long long* ids, int cap, int* n);
ifx_status ifx_server_request_state(ifx_server* v, long long id, int* state, int* steps_done, int* nx, int* ny);
/* Field IFX_FIELD_U, _V or _P of a finished request (nx*ny values). */
ifx_status ifx_server_result(ifx_server* v, long long id, int field, double* host, size_t n);
ifx_status ifx_server_request_stats(ifx_server* v, long long id, ifx_stats* out);
/* Forgets a finished request and its results. */
ifx_status ifx_server_release(ifx_server* v, long long id);
ifx_status ifx_server_info(ifx_server* v, int* waiting, int* running, int* cohorts, size_t* used_bytes);
void       ifx_server_destroy(ifx_server* v);
/* Measurement hook (no reference counterpart): launches one kernel of the
 * time step `reps` times back to back on the solver's stream and returns the
 * mean device time per launch (CUDA events).  kernel: 0 finest-level
 * multigrid smoothing sweep (the variant the step launches: from the block
 * index for one instance, TMA-staged on the mixed path), 1 FP64 pressure
 * operator apply (BiCGSTAB),
 * 2 predictor Jacobi sweep, 3 convection / predictor right-hand side,
 * 4 one grid barrier of the persistent per-step kernel (time per barrier),
 * 5 the small-level multigrid sub-cycle (one block per instance).
 * *cells receives the interior cells one launch covers.  Scratch buffers and
 * the per-step iteration state are overwritten; the flow state is not. */
ifx_status ifx_profile_kernel(ifx_solver* s, int kernel, int reps, double* ms_per_launch, long long* cells);
/* Measurement hook (no reference counterpart): runs one time step with the
 * persistent per-step kernel and records the SM clock of block 0 after every
 * grid barrier; us[k] receives the time between barrier k and k+1 in
 * microseconds (SM clock rate), *n the number of intervals (<= cap). */
ifx_status ifx_trace_step(ifx_solver* s, int cap, double* us, int* n);
/* Failure-detection hook (no reference counterpart): the next persistent
 * launch of this handle (IFX_EXEC_PERSISTENT) polls each grid barrier at most
 * spin_limit times (<= 0: the default, about 2^23 polls, well under a second)
 * and, if withhold_arrival is non-zero, starts its arrival counter one short,
 * as if one block of the launch had been lost.  The first barrier then never
 * completes: every block gives up after spin_limit polls, sets the error flag
 * and returns, the step reports IFX_ERR_CUDA and the handle refuses further
 * steps (IFX_ERR_STATE); the device stays usable.  Applies to one launch. */
ifx_status ifx_set_barrier_fault(ifx_solver* s, long long spin_limit, int withhold_arrival);
void       ifx_destroy(ifx_solver* s);

#ifdef __cplusplus
}
#endif
#endif /* IMMERSEFLOW_GB300_H */
