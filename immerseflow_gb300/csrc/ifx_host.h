// ifx_host.h -- host-side solver object behind the C ABI.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/immerseflow_gb300.h"
#include "ifx_dev.h"
#include "ifx_persist.h"

namespace ifx {

extern thread_local std::string g_last_error;
ifx_status set_error(ifx_status st, const std::string& msg);

// One multigrid level of one instance, host copy.
struct HostLevel {
    int NX = 0, NY = 0, nx = 0, ny = 0, pitch = 0;
    int cx = 1, cy = 1;  // cells of the next finer level per cell of this one, in x and y
    std::vector<double> dw, dh, xc, yc, kx, ky, ix, iy;
    std::vector<uint8_t> act, bits;  // pitched
    std::vector<int> pI, pIn, pJ, pJn;
    std::vector<double> pwx, pwy;
    std::vector<signed char> psx, psy;
    // device
    double *d_kx = nullptr, *d_ky = nullptr, *d_ix = nullptr, *d_iy = nullptr, *d_dw = nullptr, *d_dh = nullptr;
    float *d_kxf = nullptr, *d_kyf = nullptr, *d_ixf = nullptr, *d_iyf = nullptr, *d_dwf = nullptr, *d_dhf = nullptr;
    double2 *d_cew = nullptr, *d_cns = nullptr;
    float2 *d_cewf = nullptr, *d_cnsf = nullptr;
    uint8_t* d_bits = nullptr;
    uint8_t* d_act = nullptr;        // coarse levels of a moving body's instance
    void *d_e = nullptr, *d_e2 = nullptr, *d_r = nullptr;
    int *d_pI = nullptr, *d_pIn = nullptr, *d_pJ = nullptr, *d_pJn = nullptr;
    double *d_pwx = nullptr, *d_pwy = nullptr;
    float *d_pwxf = nullptr, *d_pwyf = nullptr;
    signed char *d_psx = nullptr, *d_psy = nullptr;
};

struct Instance {
    ifx_config cfg;
    int NX = 0, NY = 0, nx = 0, ny = 0, pitch = 0;
    size_t ncell = 0;  // pitch * ny
    std::vector<double> xf, yf, xc, yc, dx, dy, fx, gx, fy, gy;
    std::vector<uint8_t> type;       // pitched, after tagging
    std::vector<HostLevel> lev;
    int n_fluid = 0, n_ibm = 0, lev_base = 0, tile_beg = 0, tile_cnt = 0, ghost_beg = 0, ghost_cnt = 0;
    double area = 0.0;
    bool singular = true;
    int dirmask = 0;
    double cs = 1.0, sn = 0.0, ia2 = 1.0, ib2 = 1.0;
    int qstride = 0;
    bool moving = false;             // prescribed body motion: geometry redone every step
    int ibm_beg = 0, ibm_cap = 0;    // its IBM ghost slots in the ghost table
    InstDev dev{};                   // device pointers (host copy of the InstDev entry)
};

// Waits for steps issued by ifx_step_async and checks their state.
ifx_status finish_pending(ifx_solver* S);
// The checks a METHOD-mode configuration must pass at creation.
ifx_status validate_method_config(const ifx_config* c);

}  // namespace ifx

// The opaque handle of the C ABI.
struct ifx_solver {
    int mode = IFX_MODE_METHOD;
    int prec = IFX_PREC_FP64;
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // after ev1: the step's error flag and instance states copied to pinned
    // host memory, then ev2, so that completing a step takes one wait
    cudaEvent_t ev2 = nullptr;
    unsigned int* h_flag = nullptr;  // pinned
    bool states_enqueued = false;
    double last_ms = 0.0;
    long long launches = 0;
    std::vector<void*> allocs;       // every device allocation, freed at destroy
    size_t device_bytes = 0;         // their total size
    int exec_override = -1;          // IFX_EXEC_*; -1: environment / default
    int pending_mode = 0, pending_steps = 0;  // steps issued and not yet waited for
    std::vector<ifx::Instance> inst;
    std::vector<int> inst_status;    // sticky per-instance status (IFX_*), METHOD mode

    // batched device tables
    ifx::InstDev* dI = nullptr;
    ifx::InstState* dS = nullptr;
    ifx::InstState* hS = nullptr;    // pinned mirror
    ifx::LevelDev* dLV = nullptr;
    std::vector<ifx::LevelDev> hLV;  // host copy of dLV
    ifx::GhostDev* dG = nullptr;
    int ng = 0, nibm = 0;
    int* dIbm = nullptr;             // global indices of IBM ghost entries
    CUtensorMap* dTmap = nullptr;    // TMA tensor maps of the multigrid levels (null: plain tile loads)
    unsigned* dErr = nullptr;        // set by a kernel whose TMA copy did not complete
    int* dMv = nullptr;              // instances with a moving body
    int nmv = 0;
    int* dMvSlots = nullptr;         // their IBM ghost slots (global indices)
    int nmvslots = 0;
    double* dGval = nullptr;         // ghost gather scratch, 3 per entry
    double* dBiIp = nullptr;         // BI/IP per IBM ghost (diagnostics, tests)
    ifx::Tile* dT0 = nullptr;        // finest-level tiles of every instance
    int nt0 = 0;
    std::vector<ifx::Tile*> dTsm;    // per level >= 1: tiles of instances for which it is a middle level
    std::vector<int> ntsm;
    std::vector<ifx::Tile*> dTre;    // per level >= 1: tiles of the next finer level (from (1,1)) of instances that have the level
    std::vector<int> ntre;
    // the same lists with wide tiles (32 x 8*MG_ROWS_WIDE cells) for the multigrid phases
    ifx::Tile* dT0W = nullptr;
    int nt0W = 0;
    std::vector<ifx::Tile*> dTsmW, dTreW;
    std::vector<int> ntsmW, ntreW;
    int mg_rows = 1;                 // rows per thread of the multigrid tile phases: 1 or MG_ROWS_WIDE
    size_t cmg_bytes = 0;            // cluster V-cycle: shared memory per CTA (largest instance)
    int cmg_ok = 0, cmg_use = 0;     // it fits / graph and host-loop modes use it
    // host copies of the full tile lists (every instance, instance order); the
    // device lists hold the tiles of the instances in in_lists only
    std::vector<ifx::Tile> hT0full, hT0Wfull;
    std::vector<std::vector<ifx::Tile>> hTsmFull, hTreFull, hTsmWFull, hTreWFull;
    std::vector<char> in_lists;
    int listed = 0;
    ifx::Tile* dTall = nullptr;      // tiles of every level of every instance
    int* dSub = nullptr;             // LevelDev index of each instance's first small level
    int lmax = 0;
    int sub_bytes = 0;  // dynamic shared memory of the small-level sub-cycle
    int mg_pre = 2, mg_post = 2;
    double* dPart = nullptr;         // NPART partials per finest-level tile
    double* dStage = nullptr;        // state transfers: three dense fields of the largest instance
    double* dFpart = nullptr;        // force partials, 2 * FORCE_BLOCKS per instance
    unsigned* dFtick = nullptr;      // force tickets, one per instance (zero between steps)
    ifx::LoopCtl* dCtl = nullptr;
    ifx::LoopCtl* hCtl = nullptr;    // pinned

    // persistent execution: one cooperative launch per ifx_step call
    ifx::GridBar* dBar = nullptr;
    ifx::PersistPlan plan{};
    int persist_grid = 0;            // 0: cooperative launch unavailable
    int persist_full = 0;            // co-resident grid (SMs x blocks per SM, capped): the default
    int wide_sums = 0;               // some instance has >= 1024 level-0 tile partials (batched reduction loads)
    int persist_sms = 0;             // SMs of the device
    bool poisoned = false;           // a grid barrier timed out: the handle refuses further steps

    // graph execution of one time step (conditional WHILE nodes for the loops)
    bool use_graph = true;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    long long graph_nodes_pre = 0, graph_nodes_pred = 0, graph_nodes_mid = 0, graph_nodes_ppe = 0,
              graph_nodes_post = 0;

    // REFERENCE mode state (one instance, dense rows)
    double *r_u = nullptr, *r_v = nullptr, *r_ut = nullptr, *r_vt = nullptr, *r_p = nullptr, *r_pt = nullptr;
    double *r_dx = nullptr, *r_dy = nullptr, *r_xc = nullptr, *r_yc = nullptr, *r_ib = nullptr;
    double *r_coef = nullptr, *r_sx = nullptr, *r_sy = nullptr, *r_uf = nullptr, *r_vf = nullptr, *r_res = nullptr;
    double* r_out = nullptr;         // device reduction results (+ ticket)
    double* r_line = nullptr;        // line-SOR elimination scratch
    ifx::GridBar* r_bar = nullptr;   // grid barrier of the one-launch step
    int* r_iters_d = nullptr;        // Jacobi iterations per step of one launch (kRefStepsPerLaunch)
    int* r_iters_h = nullptr;        // pinned mirror
    int r_grid = 0;                  // blocks of the one-launch step, 0: host loop
    double* h_out = nullptr;         // pinned
    int r_cur = 0;                   // 0: state in r_u/r_v, 1: in r_ut/r_vt
    std::vector<int> r_iters;
    long long steps_done = 0;
};
