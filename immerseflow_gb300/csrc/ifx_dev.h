// ifx_dev.h -- device-side layout shared by the host orchestration and the
// CUDA kernels.
//
// Every kernel works on a batch of independent instances (a single solve is a
// batch of one).  Work is described by tile lists: a tile is a 32x8 block of
// cells of one grid level of one instance; a launch covers all tiles of all
// instances that take part in a phase.  Per-instance reductions are written
// as one partial per tile and summed per instance in a fixed order, so an
// instance gives bit-identical results alone or inside any batch.
//
// Field layout in HBM: row-major, i fastest, with the reference's one-cell
// ghost ring (src/include/ADSolver.cu:10), rows padded to a pitch that is a
// multiple of 32 elements.  Face velocities live on cell-shaped arrays:
// U[c] is the east face of cell c, V[c] its north face.
#pragma once
#include <cstdint>

#include <vector_types.h>

namespace ifx {

constexpr int TILE_X = 32;
constexpr int TILE_Y = 8;
constexpr int TILE_THREADS = TILE_X * TILE_Y;
constexpr int MG_ROWS_WIDE = 4;  // rows per thread of the wide multigrid tiles (32 x 32 cells)
constexpr int GHOST_BLOCK = 256;
constexpr int NPART = 6;            // partial sums per tile
constexpr int FORCE_SAMPLES = 2048;  // body-surface samples for drag/lift
// blocks per instance that evaluate them (an SM issues 2 FP64 FMA per clock:
// one block took ~30 us for the 2048 samples)
constexpr int FORCE_BLOCKS = 8;
constexpr int TMA_MAPS_PER_LEVEL = 8;  // tensor maps per level: e, e2, r, bits for 32x8 tiles, then for wide tiles
constexpr double COARSE_OMEGA = 1.5;  // RB-SOR factor on the coarsest level
// Threads of the block that runs an instance's small levels in the graph and
// host-loop modes (the persistent kernel runs them with its own blocks).
constexpr int SUB_THREADS = 512;
constexpr int SUB_MAX_CELLS = 2048;  // coarse levels up to this size run in one block per instance
// ... in the plain FP64 path: one SM issues 2 FP64 FMA per clock, so a sweep of
// a 1536-cell level in one block takes ~12 us against ~5 us as a tile phase
constexpr int SUB_MAX_CELLS_FP64 = 512;
constexpr int SUB_SMEM_MAX = 96 * 1024;  // shared memory for those levels (fields, metrics, tables)
constexpr int kSubLevels = 16;           // at most this many levels per instance
constexpr int SUB_COARSE_PER_THREAD = 4;  // coarsest-level cells per thread in the RB-SOR solve

enum CellType : uint8_t { T_SOLID = 0, T_FLUID = 1, T_GHOST = 2, T_DOMAIN = 3 };
// per-cell stencil bits: open faces, and (finest level) faces to an IBM ghost
enum : uint8_t { B_E = 1, B_W = 2, B_N = 4, B_S = 8, G_E = 16, G_W = 32, G_N = 64, G_S = 128 };
// per-instance iteration state
enum : int { ST_ACTIVE = 0, ST_FINAL_IN_ALT = 1, ST_DONE = 2 };

#if defined(__CUDACC__)
#define IFX_HD __host__ __device__
#else
#define IFX_HD
#endif

// Buffer (0: e, 1: e2) that holds a level's multigrid correction after its
// pre- and after its post-smoothing (the finest level starts from a
// zero-start sweep into e2; coarser levels from the fused restriction into e).
IFX_HD inline int parity_after_pre(int depth, int pre) { return depth == 0 ? (pre & 1) : ((pre - 1) & 1); }
IFX_HD inline int parity_after_post(int depth, int pre, int post) { return (parity_after_pre(depth, pre) + post) & 1; }

// Shared-memory layout (byte offsets) of one small multigrid level staged for
// the sub-cycle: fields e, e2, r (n = nx*ny cells of tsize bytes), the face
// coefficient pairs cew = (kx[i] ix[i], kx[i-1] ix[i]) and the widths dw (nx),
// cns and dh (ny), the prolongation tables from the next coarser level (pwx
// pI pIn psx: nx; pwy pJ pJn psy: ny) and the stencil bytes; every array
// starts on a 16-byte boundary.
struct SubLayout {
    size_t e, e2, r, cew, dw, pwx, cns, dh, pwy, pI, pIn, pJ, pJn, b, psx, psy, bytes;
};
IFX_HD inline size_t sub_al16(size_t x) { return (x + 15) & ~(size_t)15; }
IFX_HD inline SubLayout sub_layout(int nx, int ny, int tsize) {
    SubLayout L;
    const size_t n = (size_t)nx * ny, ts = (size_t)tsize, X = (size_t)nx, Y = (size_t)ny;
    size_t o = 0;
    L.e = o;   o += sub_al16(n * ts);
    L.e2 = o;  o += sub_al16(n * ts);
    L.r = o;   o += sub_al16(n * ts);
    L.cew = o; o += sub_al16(X * 2 * ts);
    L.dw = o;  o += sub_al16(X * ts);
    L.pwx = o; o += sub_al16(X * ts);
    L.cns = o; o += sub_al16(Y * 2 * ts);
    L.dh = o;  o += sub_al16(Y * ts);
    L.pwy = o; o += sub_al16(Y * ts);
    L.pI = o;  o += sub_al16(X * 4);
    L.pIn = o; o += sub_al16(X * 4);
    L.pJ = o;  o += sub_al16(Y * 4);
    L.pJn = o; o += sub_al16(Y * 4);
    L.b = o;   o += sub_al16(n);
    L.psx = o; o += sub_al16(X);
    L.psy = o; o += sub_al16(Y);
    L.bytes = o;
    return L;
}
IFX_HD inline size_t sub_level_bytes(int nx, int ny, int tsize) { return sub_layout(nx, ny, tsize).bytes; }
// Header of a staged level at the start of the sub-cycle's shared memory.
struct SubHdr {
    SubLayout o;
    unsigned base;  // byte offset of the level's arrays
    int NX, NY, nx, ny, dirmask, child, depth, ns, cx, cy;
};
constexpr size_t SUB_HDR_BYTES = (kSubLevels * sizeof(SubHdr) + 15) & ~(size_t)15;

// Cluster V-cycle (graph and host-loop modes, instances that fit): the
// multigrid levels above the sub-cycle are row-partitioned across the shared
// memory of one thread-block cluster per instance.
constexpr int CMG_CTAS = 16;        // CTAs per cluster
constexpr int CMG_THREADS = 1024;   // threads per CTA
constexpr int CMG_MAX_LEVELS = 8;   // distributed levels at most
constexpr size_t CMG_SMEM_MAX = 200 * 1024;

// Per-CTA shared-memory layout (byte offsets): for each distributed level the
// CTA's m rows of e, e2, r (T) and stencil bytes, and the cluster-wide row
// pointer tables (one generic pointer per row of the level, for e, e2, r and
// the stencil bytes); a zero row for the ghost ring; the sub-cycle area.
struct CmgLevel {
    unsigned e, e2, r, b, pe, pe2, pr, pb;
    int m;  // rows per CTA
};
struct CmgLayout {
    CmgLevel lv[CMG_MAX_LEVELS];
    unsigned zero, zerob, sub, bytes;
    int nd;
};
IFX_HD inline CmgLayout cmg_layout(int nd, const int* nx, const int* ny, int tsize, size_t sub_bytes) {
    CmgLayout L;
    size_t o = 0, nxmax = 0;
    const size_t ts = (size_t)tsize;
    L.nd = nd;
    for (int l = 0; l < nd && l < CMG_MAX_LEVELS; l++) {
        const int m = (ny[l] - 2 + CMG_CTAS - 1) / CMG_CTAS;
        const size_t n = (size_t)m * nx[l], rows = (size_t)ny[l];
        CmgLevel& c = L.lv[l];
        c.m = m;
        c.e = (unsigned)o;   o += sub_al16(n * ts);
        c.e2 = (unsigned)o;  o += sub_al16(n * ts);
        c.r = (unsigned)o;   o += sub_al16(n * ts);
        c.b = (unsigned)o;   o += sub_al16(n);
        c.pe = (unsigned)o;  o += sub_al16(rows * 8);
        c.pe2 = (unsigned)o; o += sub_al16(rows * 8);
        c.pr = (unsigned)o;  o += sub_al16(rows * 8);
        c.pb = (unsigned)o;  o += sub_al16(rows * 8);
        if ((size_t)nx[l] > nxmax) nxmax = (size_t)nx[l];
    }
    L.zero = (unsigned)o;  o += sub_al16(nxmax * ts);
    L.zerob = (unsigned)o; o += sub_al16(nxmax);
    L.sub = (unsigned)o;   o += sub_al16(sub_bytes);
    L.bytes = (unsigned)o;
    return L;
}

struct alignas(16) Tile {
    int inst;  // instance index
    int lev;   // index into the LevelDev array
    int i0, j0;
};

// One boundary relation q[cell] = c + sum_k w[k] * q[nb[k]].  Domain ghosts
// (one neighbour) carry the wall/inflow/slip/outflow rule; IBM ghosts carry
// image-point weights (Dirichlet for u,v; Neumann for p).
struct alignas(16) GhostDev {
    int cell, inst, side, adj;  // side: -1 IBM ghost, 0..3 domain side, 4 corner
    int nb[4];
    double wu[4], wv[4], wp[4];
    double cu, cv;               // static constants
    int qi[2];                   // outflow face values feeding the constant (-1: none)
    double qf[2];                // ... with these factors
    int qown;                    // outflow face value owned (updated) by this entry, -1 none
    double qh;                   // normal spacing for the convective outflow update
};

struct alignas(16) LevelDev {
    int NX, NY, nx, ny, pitch;
    int inst, depth, dirmask;    // dirmask bit s: side s Dirichlet for pressure
    const double *kx, *ky, *ix, *iy, *dw, *dh;
    const float *kxf, *kyf, *ixf, *iyf, *dwf, *dhf;
    // face coefficients of the pressure operator: (c_E, c_W) of column i =
    // (kx[i] ix[i], kx[i-1] ix[i]) and (c_N, c_S) of row j = (ky[j] iy[j],
    // ky[j-1] iy[j]), the products formed once in the level's precision
    const double2 *cew, *cns;
    const float2 *cewf, *cnsf;
    const uint8_t* bits;
    uint8_t* act;  // coarse level of a moving body's instance: cells taking part (else null)
    void* e;   // correction, T*
    void* e2;  // Jacobi partner, T*
    void* r;   // right-hand side, T*
    // prolongation tables from the next coarser level into this one; at a
    // domain boundary the neighbour is the cell itself mirrored with sign
    // psx/psy (+1 Neumann, -1 Dirichlet)
    const int *pI, *pIn, *pJ, *pJn;
    const double *pwx, *pwy;
    const float *pwxf, *pwyf;
    const signed char *psx, *psy;
    int child;   // LevelDev index of the next coarser level, -1 at the coarsest
    int parent;  // LevelDev index of the next finer level, -1 at the finest
    int tbeg, tcnt;  // this level's tiles in the all-levels tile table
    int cx, cy;      // cells of the parent level per cell of this one, in x and y (1 or 2)
};

// Tiles of one level of one instance, in row-major order from (x0, y0), each
// TILE_X x th cells, with the level's descriptor and the instance's constants
// by value (kernel parameters of the single-instance phases): a block finds
// its tile and level without memory loads, and reads the instance's state
// together with the fields, testing it before the stores (a single instance
// that has converged ends the loop after the phase anyway).
struct GridTiles {
    LevelDev L;
    const int* gidx;
    double omega;
    int inst, lev, x0, y0, ntx, th;
    IFX_HD Tile tile(int vb) const {
        Tile t;
        t.inst = inst;
        t.lev = lev;
        t.i0 = x0 + (vb % ntx) * TILE_X;
        t.j0 = y0 + (vb / ntx) * th;
        return t;
    }
};

// One body-surface sample for drag/lift (stationary body: built once).
// Pressure is sampled bilinearly at the surface point (base cell c0,
// weights xi0/et0), velocity at a probe del along the normal (c1, xi1/et1).
struct alignas(16) ForceSample {
    int c0, c1;
    double xi0, et0, xi1, et1, nx, ny, ds, del;
};

// The geometry arrays below that are declared const (cell types, ghost map,
// force samples, sub-cycle image; and the stencil bytes of LevelDev) are read
// only by every kernel except the per-step geometry of a moving body
// (k_move_geometry, k_move_forces), which rewrites them between the steps'
// phases.
struct alignas(16) InstDev {
    int NX, NY, nx, ny, pitch;
    int singular, dirmask, body, lev0, nlev;
    int tile_beg, tile_cnt;      // level-0 tiles (for per-instance partial sums)
    int ghost_beg, ghost_cnt;
    int retired;                 // set between steps: a step leaves the instance unchanged
    double dt, re, dtre, idt, omega;
    double ad_lim, ppe_tol;
    int ad_itermax, ppe_itermax, n_fluid, mixed_inner;
    // sweep schedule: coarsest-level RB-SOR sweeps; mixed path: the FP32
    // BiCGSTAB restarts from the FP64 true residual once its recursive
    // residual fell by restart_drop since the last restart, or after
    // restart_every iterations
    int coarse_sweeps, restart_every;
    double restart_drop;
    double uc;                   // convective outflow speed
    double area;                 // sum of fluid-cell areas
    double *u, *v, *u2, *v2, *Us, *Vs, *U, *V, *Nu, *Nv, *ru, *rv, *p, *b, *div, *iblank;
    double *pold, *pold2;        // pressures of the two steps before (initial-guess extrapolation)
    double *dup, *dvp;           // predictor increment q* - q^n of the step before (initial guess)
    const double *dx, *dy, *fx, *gx, *fy, *gy, *xc, *yc, *xf, *yf;
    const double *kx, *ky, *ix, *iy;   // finest-level face coefficients and 1/width
    // implicit predictor coefficients: column i (a_E, a_W) = dt/Re (kx[i] ix[i],
    // kx[i-1] ix[i]) with pcs[i] = (1 + a_E) + a_W, row j (a_N, a_S) likewise
    const double2 *pax, *pay;
    const double* pcs;
    const uint8_t* type;
    const int* gidx;             // cell -> global ghost index (IBM ghosts), -1 otherwise
    double *qbu, *qbv;
    // BiCGSTAB vectors of the pressure solve, in T (FP64 plain path, FP32 mixed path)
    void *kr, *krh, *kp, *kv, *ks, *kt, *kph, *ksh;
    // mixed-precision predictor corrections
    float *du, *dv, *du2, *dv2, *rfu, *rfv;
    // body (ellipse), bit-exact predicate constants
    double bcx, bcy, ba, bb, bcs, bsn, bia2, bib2, fref;
    const ForceSample* fs;       // FORCE_SAMPLES entries when body != 0
    // time history: a ring of hist_cap records of hist_w doubles (step, cd, cl,
    // then u, v, p at each probe cell), written at the end of every step
    double* hist;
    const int* probe_cell;       // pitched cell index of each probe
    // the sub-cycle's shared-memory image of this instance's small levels
    // (headers, metric arrays, prolongation tables, stencil bytes; zero fields),
    // staged by one contiguous copy; sub_img_bytes is a multiple of 16
    const unsigned char* sub_img;
    int sub_img_bytes;
    // the first small level: its global correction buffers and right-hand
    // side (read by the sub-cycle, the correction written back), their row
    // pitch, the byte offsets of its e and r in the image, its size (ghost
    // ring included) and whether it has a coarser level
    void *sub_ge, *sub_ge2;
    const void* sub_gr;
    int sub_gpitch, sub_oe, sub_or, sub_nx, sub_ny, sub_child;
    int hist_cap, hist_w, nprobe;
    // prescribed body motion: the pose at t = nstep dt follows from these
    // (centre x0 + u t + ax (sin(2 pi (f t + phx)) - sin(2 pi phx)), likewise y
    // and the angle; angles and phases in turns, w = 2 pi f); bcx, bcy, bcs,
    // bsn above hold the current pose and bu, bv, bw the current velocity of
    // the centre and the rotation rate
    int moving;
    int ibm_beg, ibm_cap;        // this instance's IBM ghost slots in the ghost table
    int sub_lb;                  // LevelDev offset (from lev0) of the first sub-cycle level, 0: none
    double mo_x0, mo_y0, mo_th0, mo_u, mo_v, mo_ax, mo_ay, mo_ath, mo_f, mo_w, mo_phx, mo_phy, mo_pha;
    double bu, bv, bw;
    int* fresh;                  // step in which the cell last turned fluid (0: never)
    const double* fsb;           // body-frame force samples: lx, ly, nlx, nly, ds each
};

// Device-resident per-instance iteration state and diagnostics.
struct InstState {
    int pred_state, pred_iters, ppe_state, ppe_iters;
    int status, have_nold;
    int pold_n, pad_pold;                     // steps that stored their pressure for the extrapolation (saturates at 4)
    int restart, restart_it;                  // mixed path: FP64 residual due next body; iteration of the last one
    double pred_metric, ppe_rel, bmean, bnorm, pmean;
    double rho, alpha, omega, beta;           // BiCGSTAB scalars
    double max_div, cd, cl, flux_in, flux_out;
    double rel_restart;                       // mixed path: true relative residual at the last restart
    long long nstep;                          // time steps this instance has done
    long long hist_n;                         // time-history records written
    // moving body: cell box (i0, i1, j0, j1) of the body at the current pose,
    // IBM ghosts in use, and a geometry error (1 left the domain, 2 ghost slots full)
    int bb[4];
    int n_ibm, geo_err;
};

// Loop control for device-side convergence: reduce kernels vote, the last
// block publishes the result (and sets the CUDA-graph conditional).
struct LoopCtl {
    int active;
    unsigned int ticket;
    int result;
    int due;         // instances that need the optional phases of the next loop body
    int due_result;  // published with result: predictor refresh or Krylov restart due
    int pad[3];
};

}  // namespace ifx
