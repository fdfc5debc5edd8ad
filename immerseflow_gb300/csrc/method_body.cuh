// method_body.cuh -- device bodies of the fractional-step kernels with
// ghost-cell IBM, batched over instances.
//
// Each phase of the time step is a __device__ function b_*(..., vb) that
// processes one "virtual block" vb: a tile (32x8 cells of one level of one
// instance), a chunk of ghost relations, or one instance.  The same bodies
// run as ordinary kernels (one launch per phase, kernels_method.cu; used by
// the CUDA-graph and host-loop paths) and inside the persistent per-step
// kernel (kernels_persist.cu), so all paths compute bit-identical results.
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
// oracle (oracle/oracle.cpp, method_step).  State in FP64; multigrid
// corrections in T (double for the plain path, float for the mixed path).
#pragma once
#include <cuda_runtime.h>

#include "ifx_dev.h"
#include "ifx_kernels.h"
#include "tma.cuh"


namespace ifx {

// Read-only data (tile lists, level / instance / ghost tables, stencil bytes,
// metric arrays) does not change during a time step: small structs that are
// used whole (tiles, force samples) and the metric / stencil arrays are
// loaded through the read-only data path.
template <typename S>
__device__ __forceinline__ S ldg_struct(const S* p) {
    static_assert(sizeof(S) % 16 == 0, "16-byte multiple");
    S out;
    const int4* src = reinterpret_cast<const int4*>(p);
    int4* dst = reinterpret_cast<int4*>(&out);
#pragma unroll
    for (int k = 0; k < (int)(sizeof(S) / 16); k++) dst[k] = __ldg(src + k);
    return out;
}

// ---------------------------------------------------------------- helpers

// Programmatic dependent launch: a phase lets its dependents launch early
// (trigger), and a dependent launched that way does its independent work
// (its instance state, its geometry) before waiting for the phase's output
// (wait).  Both are no-ops in launches without a programmatic dependency.
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

__device__ __forceinline__ double rcpa(double d) { return (double)__frcp_rn((float)d); }
__device__ __forceinline__ float rcpa(float d) { return __frcp_rn(d); }

template <typename T> struct LvA;
template <> struct LvA<double> {
    static __device__ __forceinline__ const double* kx(const LevelDev& L) { return L.kx; }
    static __device__ __forceinline__ const double* ky(const LevelDev& L) { return L.ky; }
    static __device__ __forceinline__ const double* ix(const LevelDev& L) { return L.ix; }
    static __device__ __forceinline__ const double* iy(const LevelDev& L) { return L.iy; }
    static __device__ __forceinline__ const double* dw(const LevelDev& L) { return L.dw; }
    static __device__ __forceinline__ const double* dh(const LevelDev& L) { return L.dh; }
    static __device__ __forceinline__ const double* pwx(const LevelDev& L) { return L.pwx; }
    static __device__ __forceinline__ const double* pwy(const LevelDev& L) { return L.pwy; }
    static __device__ __forceinline__ const double2* cew(const LevelDev& L) { return L.cew; }
    static __device__ __forceinline__ const double2* cns(const LevelDev& L) { return L.cns; }
};
template <> struct LvA<float> {
    static __device__ __forceinline__ const float* kx(const LevelDev& L) { return L.kxf; }
    static __device__ __forceinline__ const float* ky(const LevelDev& L) { return L.kyf; }
    static __device__ __forceinline__ const float* ix(const LevelDev& L) { return L.ixf; }
    static __device__ __forceinline__ const float* iy(const LevelDev& L) { return L.iyf; }
    static __device__ __forceinline__ const float* dw(const LevelDev& L) { return L.dwf; }
    static __device__ __forceinline__ const float* dh(const LevelDev& L) { return L.dhf; }
    static __device__ __forceinline__ const float* pwx(const LevelDev& L) { return L.pwxf; }
    static __device__ __forceinline__ const float* pwy(const LevelDev& L) { return L.pwyf; }
    static __device__ __forceinline__ const float2* cew(const LevelDev& L) { return L.cewf; }
    static __device__ __forceinline__ const float2* cns(const LevelDev& L) { return L.cnsf; }
};

__device__ __forceinline__ void tile_ij(const Tile& t, int& i, int& j) {
    i = t.i0 + (int)(threadIdx.x & 31);
    j = t.j0 + (int)(threadIdx.x >> 5);
}

// Deterministic block sum of NV values; result valid in thread 0..NV-1 as out[k].
// RT: arithmetic of the in-warp stage (float on the mixed path, whose Krylov
// vectors are FP32: FP64 butterfly adds on every lane are slow on GB300); the
// warp results are summed in FP64.  The values may be given as float: a
// product or sum of two floats formed in FP64 and rounded to float equals
// the FP32 operation (53 >= 2*24 + 2 bits, so the double rounding is
// innocuous), and GB300 issues FP64 operations and conversions at 1/61 of
// the FP32 rate (2 FP64 FMA per SM and clock), so the mixed path forms its
// FP32 partials in FP32.
template <int NV, typename RT = double, typename VT>
__device__ __forceinline__ void block_sum(VT (&v)[NV], double* out) {
    __shared__ RT sh[NV][32];
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++) {
        RT x = (RT)v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (l == 0) sh[k][w] = x;
    }
    __syncthreads();
    if constexpr (sizeof(RT) == sizeof(double)) {
        if (threadIdx.x < NV) {
            double s = 0.0;
            for (int q = 0; q < nw; q++) s += sh[threadIdx.x][q];
            out[threadIdx.x] = s;
        }
    } else {
        // FP32 warp sums: warp 0 widens all of them at once (one conversion
        // per lane instead of one per warp and value), then sums them in FP64
        // in the same order
        __shared__ double shd[NV][32];
        if (w == 0) {
            for (int q = l; q < NV * nw; q += 32) shd[q / nw][q % nw] = (double)sh[q / nw][q % nw];
            __syncwarp();
            if (l < NV) {
                double s = 0.0;
                for (int q = 0; q < nw; q++) s += shd[l][q];
                out[l] = s;
            }
        }
    }
    __syncthreads();
}

__device__ __forceinline__ double block_max(double v) {
    __shared__ double sh[32];
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (l == 0) sh[w] = v;
    __syncthreads();
    double m = 0.0;
    if (threadIdx.x == 0)
        for (int q = 0; q < nw; q++) m = fmax(m, sh[q]);
    __syncthreads();
    return m;
}

// Per-instance sum of the level-0 tile partials, fixed order; valid in all threads.
// A thread adds rows t, t + B, t + 2B, ... (B threads).  WIDE (instances of
// thousands of tiles): the loads of four rows are issued before their sums, so
// the block waits for a quarter of the round trips (same additions in the same
// order); the plain loop keeps the code of the common case short (a one-block
// kernel fetches its code cold at every launch).
template <int NV, bool WIDE = false>
__device__ __forceinline__ void inst_sum(const double* part, int beg, int cnt, double (&res)[NV]) {
    double acc[NV];
#pragma unroll
    for (int k = 0; k < NV; k++) acc[k] = 0.0;
    if constexpr (WIDE) {
        const int B = (int)blockDim.x;
        int t = (int)threadIdx.x;
        for (; t + 3 * B < cnt; t += 4 * B) {
            double v[4][NV];
#pragma unroll
            for (int u = 0; u < 4; u++)
#pragma unroll
                for (int k = 0; k < NV; k++) v[u][k] = part[(size_t)(beg + t + u * B) * NPART + k];
#pragma unroll
            for (int u = 0; u < 4; u++)
#pragma unroll
                for (int k = 0; k < NV; k++) acc[k] += v[u][k];
        }
        for (; t < cnt; t += B)
#pragma unroll
            for (int k = 0; k < NV; k++) acc[k] += part[(size_t)(beg + t) * NPART + k];
    } else {
        for (int t = threadIdx.x; t < cnt; t += blockDim.x)
#pragma unroll
            for (int k = 0; k < NV; k++) acc[k] += part[(size_t)(beg + t) * NPART + k];
    }
    __shared__ double out[NV];
    block_sum<NV>(acc, out);
#pragma unroll
    for (int k = 0; k < NV; k++) res[k] = out[k];
}

// due: the instance needs the optional phases of the next loop body (mixed
// path: predictor refresh, Krylov restart); their kernels return at once
// when no instance does.
__device__ __forceinline__ void loop_vote(LoopCtl* ctl, bool active, unsigned long long handle, bool due = false) {
    // thread 0 of each voting block; no-op inside the persistent kernel (ctl == nullptr)
    if (!ctl) return;
    if (gridDim.x == 1) {
        // the only voting block (a one-instance solver): the vote is its own,
        // with no other block to count or to order against; the counters stay
        // at zero and the next kernel sees the result at the kernel boundary
        ctl->result = active ? 1 : 0;
        ctl->due_result = due ? 1 : 0;
        if (handle) cudaGraphSetConditional((cudaGraphConditionalHandle)handle, active ? 1u : 0u);
        return;
    }
    if (active) atomicAdd(&ctl->active, 1);
    if (due) atomicAdd(&ctl->due, 1);
    __threadfence();
    unsigned int t = atomicAdd(&ctl->ticket, 1u);
    if (t == gridDim.x - 1) {
        __threadfence();
        int a = atomicAdd(&ctl->active, 0);
        int d = atomicAdd(&ctl->due, 0);
        ctl->result = a;
        ctl->due_result = d;
        ctl->active = 0;
        ctl->due = 0;
        ctl->ticket = 0u;
        __threadfence();
        if (handle) cudaGraphSetConditional((cudaGraphConditionalHandle)handle, a > 0 ? 1u : 0u);
    }
}

// Optional phases: nothing to do when the last vote found no instance due.
__device__ __forceinline__ bool none_due(const LoopCtl* ctl) {
    return ctl != nullptr && *(const volatile int*)&ctl->due_result == 0;
}

__device__ __forceinline__ double ghost_const(const GhostDev& g, const double* qb, double c0) {
    if (g.qi[0] >= 0) c0 += g.qf[0] * qb[g.qi[0]];
    if (g.qi[1] >= 0) c0 += g.qf[1] * qb[g.qi[1]];
    return c0;
}

// Image-point value of the IBM ghost at global entry gid, from field e;
// ws receives the weight on cell `self`.  Pressure stencils reference fluid
// cells only, so this is an exact linear function of the fluid values.
template <typename TC, typename Fetch>
__device__ __forceinline__ TC ghost_eval_f(const GhostDev* G, int gid, Fetch fetch, int self, TC& ws) {
    TC acc = (TC)0;
    ws = (TC)0;
    if (gid < 0) return acc;  // a moving body's ghost beyond its slots (instance retired after the step)
    const GhostDev& g = G[gid];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const TC w = (TC)g.wp[k];
        acc += w * fetch(g.nb[k]);
        if (g.nb[k] == self) ws += w;
    }
    return acc;
}
template <typename TC, typename TE>
__device__ __forceinline__ TC ghost_eval(const GhostDev* G, int gid, const TE* e, int self, TC& ws) {
    return ghost_eval_f<TC>(G, gid, [e](int q) { return (TC)e[q]; }, self, ws);
}

// Face coefficients of cell (i,j) with closed faces dropped, and the
// diagonal with Dirichlet sides adding 2c.
template <typename TC>
struct LapCoef {
    TC ce, cw, cn, cs, dd;
};
template <typename TC>
__device__ __forceinline__ LapCoef<TC> lap_coef(const LevelDev& L, int i, int j, uint8_t bt) {
    const auto ew = __ldg(&LvA<TC>::cew(L)[i]);
    const auto ns = __ldg(&LvA<TC>::cns(L)[j]);
    const TC cE = ew.x, cW = ew.y, cN = ns.x, cS = ns.y;
    LapCoef<TC> c;
    c.ce = (bt & B_E) ? cE : (TC)0;
    c.cw = (bt & B_W) ? cW : (TC)0;
    c.cn = (bt & B_N) ? cN : (TC)0;
    c.cs = (bt & B_S) ? cS : (TC)0;
    TC dd = c.ce + c.cw + c.cn + c.cs;
    if (L.dirmask) {
        if (i == L.NX && (L.dirmask & (1 << 1))) dd += (TC)2 * cE;
        if (i == 1 && (L.dirmask & (1 << 0))) dd += (TC)2 * cW;
        if (j == L.NY && (L.dirmask & (1 << 3))) dd += (TC)2 * cN;
        if (j == 1 && (L.dirmask & (1 << 2))) dd += (TC)2 * cS;
    }
    c.dd = dd;
    return c;
}

// Pressure-type Laplacian at live cell (i,j): Le = sum c (e_nb - e) with
// closed faces dropped, Dirichlet sides adding 2c to the diagonal, and (finest
// level) faces to IBM ghosts using the ghost's image-point value (ghost
// unknowns eliminated).  D is the diagonal of that operator.  Coefficients
// and arithmetic in TC, field values of type TE; P is the row pitch of e
// (L.pitch in global memory, L.nx for a level staged in shared memory).
// Same, from the values of the cell (eP) and its four neighbours; fetch(q)
// returns the value at dense index q for the IBM ghosts' image-point stencils.
template <typename TC, bool LVL0, typename Fetch>
__device__ __forceinline__ void lap_vals(const LevelDev& L, int i, int j, int id, int P, uint8_t bt, const GhostDev* G,
                                         const int* gidx, TC eE, TC eW, TC eN, TC eS, TC eP, Fetch fetch, TC& Le,
                                         TC& D) {
    const LapCoef<TC> c = lap_coef<TC>(L, i, j, bt);
    TC dm = c.dd;
    if (LVL0 && (bt & 0xF0)) {
        TC ws;
        if (bt & G_E) { eE = ghost_eval_f<TC>(G, gidx[id + 1], fetch, id, ws); dm -= c.ce * ws; }
        if (bt & G_W) { eW = ghost_eval_f<TC>(G, gidx[id - 1], fetch, id, ws); dm -= c.cw * ws; }
        if (bt & G_N) { eN = ghost_eval_f<TC>(G, gidx[id + P], fetch, id, ws); dm -= c.cn * ws; }
        if (bt & G_S) { eS = ghost_eval_f<TC>(G, gidx[id - P], fetch, id, ws); dm -= c.cs * ws; }
    }
    Le = c.ce * eE + c.cw * eW + c.cn * eN + c.cs * eS - c.dd * eP;
    D = dm;
}

template <typename TC, typename TE, bool LVL0>
__device__ __forceinline__ void lap_p(const LevelDev& L, const TE* __restrict__ e, int i, int j, int id, int P,
                                      uint8_t bt, const GhostDev* G, const int* gidx, TC& Le, TC& D) {
    lap_vals<TC, LVL0>(L, i, j, id, P, bt, G, gidx, (TC)e[id + 1], (TC)e[id - 1], (TC)e[id + P], (TC)e[id - P],
                       (TC)e[id], [e](int q) { return (TC)e[q]; }, Le, D);
}

// Weighted-Jacobi update of a cell, and the first sweep from zero.
template <typename T>
__device__ __forceinline__ T jacobi_update(T e, T r, T Le, T D, T om) { return e + om * (Le - r) * rcpa(D); }
template <typename T>
__device__ __forceinline__ T jacobi_from_zero(T r, T D, T om) { return -om * r * rcpa(D); }

template <typename TC, typename TE, bool LVL0>
__device__ __forceinline__ void lap(const LevelDev& L, const TE* __restrict__ e, int i, int j, int id,
                                    uint8_t bt, const GhostDev* G, const int* gidx, TC& Le, TC& D) {
    lap_p<TC, TE, LVL0>(L, e, i, j, id, L.pitch, bt, G, gidx, Le, D);
}

// Diagonal of a coarse-level operator (no IBM ghosts below the finest level).
template <typename TC>
__device__ __forceinline__ TC lap_diag(const LevelDev& L, int i, int j, uint8_t bt) {
    return lap_coef<TC>(L, i, j, bt).dd;
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// Finest-level Krylov tiles: 32 columns by 8R rows; thread (w, lane) handles
// column i0+lane of rows j0+w+8r.  Loads use indices clamped into the level's
// interior so that they issue together; stores are for live cells only.  A
// tile of R > 1 rows writes the partial sums of each of its 32x8 sub-tiles,
// formed by the same block reduction over the same threads as a 32x8 tile,
// into that sub-tile's slot: results do not depend on R.
template <int R>
struct Rows0 {
    int ic, id[R], jc[R];
    uint8_t bt[R];
    bool in_i;
};
template <int R>
__device__ __forceinline__ void rows0(const LevelDev& L, const Tile& t, Rows0<R>& q) {
    const int i = t.i0 + (int)(threadIdx.x & 31), jb = t.j0 + (int)(threadIdx.x >> 5);
    q.ic = clampi(i, 1, L.NX);
#pragma unroll
    for (int r = 0; r < R; r++) {
        const int j = jb + 8 * r;
        q.jc[r] = clampi(j, 1, L.NY);
        q.id[r] = q.ic + q.jc[r] * L.pitch;
        q.bt[r] = (i == q.ic && j == q.jc[r]) ? __ldg(&L.bits[q.id[r]]) : (uint8_t)0;
    }
}
// Slot of the partial sums of 32x8 sub-tile r of finest-level tile t: its
// index in the instance's list of 32x8 tiles (rows of tiles outer); ok is
// false below the level's last row of tiles.
__device__ __forceinline__ size_t sub_slot(const InstDev& in, const LevelDev& L, const Tile& t, int r, bool& ok) {
    const int ntx = (L.nx + TILE_X - 1) / TILE_X, nty = (L.ny + TILE_Y - 1) / TILE_Y, row = t.j0 / TILE_Y + r;
    ok = row < nty;
    return (size_t)in.tile_beg + (size_t)row * ntx + t.i0 / TILE_X;
}
template <int NV, typename RT, int R, typename VT>
__device__ __forceinline__ void write_sub_partials(const InstDev& in, const LevelDev& L, const Tile& t,
                                                   VT (&acc)[R][NV], double* __restrict__ part) {
#pragma unroll
    for (int r = 0; r < R; r++) {
        __shared__ double out[NV];
        block_sum<NV, RT>(acc[r], out);
        bool ok;
        const size_t q = sub_slot(in, L, t, r, ok);
        if (ok && threadIdx.x < NV) part[q * NPART + threadIdx.x] = out[threadIdx.x];
    }
}

// ------------------------------------------------------ step bookkeeping

__device__ __forceinline__ void b_step_begin(const InstDev* __restrict__ I, InstState* S, int n, LoopCtl* ctl,
                                             int vb) {
    if (ctl && vb == 0 && threadIdx.x == 0) ctl->due_result = 1;  // the first predictor body refreshes
    int k = vb * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int st = I[k].retired ? ST_DONE : ST_ACTIVE;
    if (st == ST_ACTIVE) {
        S[k].nstep++;
        if (S[k].pold_n < 4) S[k].pold_n++;
    }
    S[k].pred_state = st;
    S[k].pred_iters = 0;
    S[k].ppe_state = st;
    S[k].ppe_iters = 0;
}

// Convective outflow: advance the boundary face value of every outflow
// edge ghost (dq/dt + Uc dq/dn = 0, explicit).
__device__ __forceinline__ void b_outflow(const GhostDev* __restrict__ G, int ng, const InstDev* __restrict__ I, int vb) {
    int g = vb * blockDim.x + threadIdx.x;
    if (g >= ng) return;
    const GhostDev& gh = G[g];
    if (gh.qown < 0) return;
    const InstDev& in = I[gh.inst];
    if (in.retired) return;
    double fac = in.dt * in.uc * 2.0 / gh.qh;
    in.qbu[gh.qown] = in.qbu[gh.qown] - fac * (in.qbu[gh.qown] - in.u[gh.adj]);
    in.qbv[gh.qown] = in.qbv[gh.qown] - fac * (in.qbv[gh.qown] - in.v[gh.adj]);
}

// Ghost refresh in two passes (gather, then scatter) so that ghost-to-ghost
// references read the old values, exactly like one Jacobi pass.
// comps: bit0 u, bit1 v, bit2 p.
__device__ __forceinline__ void b_ghost_gather(const GhostDev* __restrict__ G, int ng, const InstDev* __restrict__ I,
                               int comps, double* __restrict__ gval, int vb) {
    int g = vb * blockDim.x + threadIdx.x;
    if (g >= ng) return;
    const GhostDev& gh = G[g];
    if (gh.cell < 0) return;  // unused slot of a moving body
    const InstDev& in = I[gh.inst];
    if (in.retired) return;
    if (comps & 1) {
        double a = ghost_const(gh, in.qbu, gh.cu);
#pragma unroll
        for (int k = 0; k < 4; k++) a += gh.wu[k] * in.u[gh.nb[k]];
        gval[3 * (size_t)g] = a;
    }
    if (comps & 2) {
        double a = ghost_const(gh, in.qbv, gh.cv);
#pragma unroll
        for (int k = 0; k < 4; k++) a += gh.wv[k] * in.v[gh.nb[k]];
        gval[3 * (size_t)g + 1] = a;
    }
    if (comps & 4) {
        double a = 0.0;
#pragma unroll
        for (int k = 0; k < 4; k++) a += gh.wp[k] * in.p[gh.nb[k]];
        gval[3 * (size_t)g + 2] = a;
    }
}

__device__ __forceinline__ void b_ghost_scatter(const GhostDev* __restrict__ G, int ng, const InstDev* __restrict__ I,
                                int comps, const double* __restrict__ gval, int vb) {
    int g = vb * blockDim.x + threadIdx.x;
    if (g >= ng) return;
    const GhostDev& gh = G[g];
    if (gh.cell < 0) return;
    const InstDev& in = I[gh.inst];
    if (in.retired) return;
    if (comps & 1) in.u[gh.cell] = gval[3 * (size_t)g];
    if (comps & 2) in.v[gh.cell] = gval[3 * (size_t)g + 1];
    if (comps & 4) in.p[gh.cell] = gval[3 * (size_t)g + 2];
}

// ------------------------------------------------------------- predictor

// Convective term in face-flux form and the AB2 right-hand side.
__device__ __forceinline__ void b_conv_rhs(const Tile* __restrict__ tiles, const InstDev* __restrict__ I,
                           const InstState* __restrict__ S, int vb) {
    const Tile t = ldg_struct(&tiles[vb]);
    const InstDev& in = I[t.inst];
    if (in.retired) return;
    int i, j;
    tile_ij(t, i, j);
    if (i < 1 || i > in.NX || j < 1 || j > in.NY) return;
    const int P = in.pitch, id = i + j * P;
    if (__ldg(&in.type[id]) != T_FLUID) {
        in.ru[id] = 0.0;
        in.rv[id] = 0.0;
        return;
    }
    const double* u = in.u;
    const double* v = in.v;
    const double gxi = __ldg(&in.gx[i]), fxi = __ldg(&in.fx[i]), gxw = __ldg(&in.gx[i - 1]), fxw = __ldg(&in.fx[i - 1]);
    const double gyj = __ldg(&in.gy[j]), fyj = __ldg(&in.fy[j]), gys = __ldg(&in.gy[j - 1]), fys = __ldg(&in.fy[j - 1]);
    const double ixi = __ldg(&in.ix[i]), iyj = __ldg(&in.iy[j]);
    const double Ue = in.U[id], Uw = in.U[id - 1], Vn = in.V[id], Vs = in.V[id - P];
    const double ue = u[id] * gxi + u[id + 1] * fxi, uw = u[id - 1] * gxw + u[id] * fxw;
    const double un = u[id] * gyj + u[id + P] * fyj, us = u[id - P] * gys + u[id] * fys;
    const double ve = v[id] * gxi + v[id + 1] * fxi, vw = v[id - 1] * gxw + v[id] * fxw;
    const double vn = v[id] * gyj + v[id + P] * fyj, vs = v[id - P] * gys + v[id] * fys;
    const double Nu = (ue * Ue - uw * Uw) * ixi + (un * Vn - us * Vs) * iyj;
    const double Nv = (ve * Ue - vw * Uw) * ixi + (vn * Vn - vs * Vs) * iyj;
    // AB2, Euler on the first step and in cells that turned fluid in this step
    const bool ab2 = S[t.inst].have_nold != 0 && !(in.fresh && in.fresh[id] == (int)S[t.inst].nstep);
    const double cu = ab2 ? 1.5 * Nu - 0.5 * in.Nu[id] : Nu;
    const double cv = ab2 ? 1.5 * Nv - 0.5 * in.Nv[id] : Nv;
    in.ru[id] = u[id] - in.dt * cu;
    in.rv[id] = v[id] - in.dt * cv;
    in.Nu[id] = Nu;
    in.Nv[id] = Nv;
}

// Initial guess of the predictor: q^n plus the step before's predictor
// increment q* - q^n in the fluid cells (zero on an instance's first step and
// in cells that were not fluid then); the increment buffers keep q^n until
// b_face_rhs forms the new increment.  The predictor's first update then
// starts O(dt^2) instead of O(dt) away: about 12 -> 9 Jacobi sweeps a step on
// the cylinder.
__device__ __forceinline__ void b_pred_guess(const Tile* __restrict__ tiles, const InstDev* __restrict__ I, int vb) {
    const Tile t = ldg_struct(&tiles[vb]);
    const InstDev& in = I[t.inst];
    if (in.retired) return;
    int i, j;
    tile_ij(t, i, j);
    if (i < 1 || i > in.NX || j < 1 || j > in.NY) return;
    const int id = i + j * in.pitch;
    if (__ldg(&in.type[id]) != T_FLUID) return;
    const double un = in.u[id], vn = in.v[id];
    in.u[id] = un + in.dup[id];
    in.v[id] = vn + in.dvp[id];
    in.dup[id] = un;
    in.dvp[id] = vn;
}

// One Jacobi sweep of the predictor for u and v, fluid cells and every
// ghost relation; parity 0 reads (u,v) and writes (u2,v2), parity 1 the
// reverse.  An instance that converged on the parity-0 sweep copies its
// result back on the parity-1 sweep.
__device__ __forceinline__ void b_pred_sweep(const Tile* __restrict__ tiles, int ntiles, const GhostDev* __restrict__ G,
                             int ng, const InstDev* __restrict__ I, const InstState* __restrict__ S,
                             double* __restrict__ part, int parity, int vb) {
    if ((int)vb < ntiles) {
        const Tile t = ldg_struct(&tiles[vb]);
        const InstDev& in = I[t.inst];
        const int st = S[t.inst].pred_state, nxi = in.NX;  // loads in flight together
        if ((st == ST_DONE) | (nxi < 0)) return;
        const double* su = parity ? in.u2 : in.u;
        const double* sv = parity ? in.v2 : in.v;
        double* du = parity ? in.u : in.u2;
        double* dv = parity ? in.v : in.v2;
        int i, j;
        tile_ij(t, i, j);
        const bool ok = i >= 1 && i <= in.NX && j >= 1 && j <= in.NY;
        const int P = in.pitch, id = i + j * P;
        const bool fl = ok && __ldg(&in.type[id]) == T_FLUID;
        if (st == ST_FINAL_IN_ALT) {
            if (fl) {
                du[id] = su[id];
                dv[id] = sv[id];
            }
            return;
        }
        double m[1] = {0.0};
        if (fl) {
            const double2 ax = __ldg(&in.pax[i]), ay = __ldg(&in.pay[j]);
            const double aE = ax.x, aW = ax.y, aN = ay.x, aS = ay.y;
            const double aP = (__ldg(&in.pcs[i]) + aN) + aS;  // 1 + aE + aW + aN + aS, in that order
            const double di = rcpa(aP);
            const double dU = (in.ru[id] + aE * su[id + 1] + aW * su[id - 1] + aN * su[id + P] + aS * su[id - P] -
                               aP * su[id]) * di;
            const double dV = (in.rv[id] + aE * sv[id + 1] + aW * sv[id - 1] + aN * sv[id + P] + aS * sv[id - P] -
                               aP * sv[id]) * di;
            du[id] = su[id] + dU;
            dv[id] = sv[id] + dV;
            m[0] = fabs(dU) + fabs(dV);
        }
        __shared__ double out[1];
        block_sum<1>(m, out);
        if (threadIdx.x == 0) part[(size_t)vb * NPART] = out[0];
    } else {
        const int g = ((int)vb - ntiles) * blockDim.x + threadIdx.x;
        if (g >= ng) return;
        const GhostDev& gh = G[g];
        if (gh.cell < 0) return;
        const InstDev& in = I[gh.inst];
        const int st = S[gh.inst].pred_state;
        if (st == ST_DONE) return;
        const double* su = parity ? in.u2 : in.u;
        const double* sv = parity ? in.v2 : in.v;
        double* du = parity ? in.u : in.u2;
        double* dv = parity ? in.v : in.v2;
        if (st == ST_FINAL_IN_ALT) {
            du[gh.cell] = su[gh.cell];
            dv[gh.cell] = sv[gh.cell];
            return;
        }
        double au = ghost_const(gh, in.qbu, gh.cu), av = ghost_const(gh, in.qbv, gh.cv);
#pragma unroll
        for (int k = 0; k < 4; k++) {
            au += gh.wu[k] * su[gh.nb[k]];
            av += gh.wv[k] * sv[gh.nb[k]];
        }
        du[gh.cell] = au;
        dv[gh.cell] = av;
    }
}

template <bool WIDE = false>
__device__ __forceinline__ void b_pred_reduce(const InstDev* __restrict__ I, InstState* __restrict__ S,
                              const double* __restrict__ part, int parity, LoopCtl* ctl,
                              unsigned long long handle, int vb) {
    const int k = vb;
    const InstDev& in = I[k];
    const int st = S[k].pred_state, beg = in.tile_beg, cnt = in.tile_cnt;
    pdl_wait();  // the sweep's partials; every write below
    bool active = false, due = false;
    if (st == ST_ACTIVE) {
        double r[1];
        inst_sum<1, WIDE>(part, beg, cnt, r);
        if (threadIdx.x == 0) {
            const int it = S[k].pred_iters + 1;
            S[k].pred_iters = it;
            S[k].pred_metric = r[0] / (double)(in.n_fluid > 0 ? in.n_fluid : 1);
            const bool done = r[0] <= in.ad_lim || it >= in.ad_itermax;
            if (done) S[k].pred_state = parity == 0 ? ST_FINAL_IN_ALT : ST_DONE;
            active = !done;
            due = active && it % (in.mixed_inner > 0 ? in.mixed_inner : 8) == 0;
        }
    } else if (st == ST_FINAL_IN_ALT) {
        if (threadIdx.x == 0) S[k].pred_state = ST_DONE;
    }
    if (threadIdx.x == 0) loop_vote(ctl, active, handle, due);
}

// ------------------------------------------- mixed-path predictor (FP32)
//
// FP32 Jacobi sweeps on the correction d = q - q0, q0 = (u, v) in FP64:
//   d <- d + D~^-1 (r0 - M d),   r0 = rhs - M q0 (FP64 defect, stored FP32);
// the ghost relations likewise (d_g <- r0_g + sum w d_nb).  M is linear, so this
// is the FP64 Jacobi iteration up to FP32 rounding of d, and every
// mixed_inner sweeps q0 absorbs d and r0 is recomputed in FP64 (defect
// correction): rounding never accumulates into the state.  The sweep metric
// (sum |update|) and the stop rule are those of the FP64 path.
// The refresh is folded into the sweeps (mixed_inner >= 2): the sweep that
// ends an inner cycle stores q0 + d instead of d (and d = 0), the sweep that
// starts the next one forms r0 from q0 first (its own cell; q0 is not written
// in that launch).  The first sweep of a step starts a cycle with d = 0 (the
// step before ended with q = q0 + d, d = 0).

__device__ __forceinline__ bool pred_refresh_due(const InstDev& in, const InstState& s) {
    return s.pred_state == ST_ACTIVE && s.pred_iters % (in.mixed_inner > 0 ? in.mixed_inner : 8) == 0;
}

// stage 0: q0 += d, d = 0 ; stage 1: r0 = rhs - M q0 (cells), r0_g (ghosts).
// finalize: q = q0 + d, d = 0 after the loop (every instance not retired).
__device__ __forceinline__ void pred_refresh_cell(const InstDev& in, int cell, const GhostDev* gh, int stage,
                                                  int finalize) {
    if (finalize || stage == 0) {
        in.u[cell] += (double)in.du[cell];
        in.v[cell] += (double)in.dv[cell];
        in.du[cell] = 0.0f;
        in.dv[cell] = 0.0f;
        return;
    }
    const double* u = in.u;
    const double* v = in.v;
    if (!gh) {
        const int P = in.pitch, id = cell, j = cell / P, i = cell - j * P;
        const double2 ax = __ldg(&in.pax[i]), ay = __ldg(&in.pay[j]);
        const double aE = ax.x, aW = ax.y, aN = ay.x, aS = ay.y;
        const double aP = (__ldg(&in.pcs[i]) + aN) + aS;  // 1 + aE + aW + aN + aS, in that order
        in.rfu[id] = (float)(in.ru[id] + aE * u[id + 1] + aW * u[id - 1] + aN * u[id + P] + aS * u[id - P] - aP * u[id]);
        in.rfv[id] = (float)(in.rv[id] + aE * v[id + 1] + aW * v[id - 1] + aN * v[id + P] + aS * v[id - P] - aP * v[id]);
    } else {
        double au = ghost_const(*gh, in.qbu, gh->cu), av = ghost_const(*gh, in.qbv, gh->cv);
#pragma unroll
        for (int k = 0; k < 4; k++) {
            au += gh->wu[k] * u[gh->nb[k]];
            av += gh->wv[k] * v[gh->nb[k]];
        }
        in.rfu[cell] = (float)(au - u[cell]);
        in.rfv[cell] = (float)(av - v[cell]);
    }
}

// vb: level-0 tiles of 32 x 8R cells, then ghost chunks (as b_pred_sweep).
template <int R = 1>
__device__ __forceinline__ void b_pred_refresh(const Tile* __restrict__ tiles, int ntiles,
                                               const GhostDev* __restrict__ G, int ng,
                                               const InstDev* __restrict__ I, const InstState* __restrict__ S,
                                               int stage, int finalize, int vb) {
    if ((int)vb < ntiles) {
        const Tile t = ldg_struct(&tiles[vb]);
        const InstDev& in = I[t.inst];
        if (in.retired) return;
        if (!finalize && !pred_refresh_due(in, S[t.inst])) return;
        const int i = t.i0 + (int)(threadIdx.x & 31), jb = t.j0 + (int)(threadIdx.x >> 5);
        if (i < 1 || i > in.NX) return;
#pragma unroll
        for (int r = 0; r < R; r++) {
            const int j = jb + 8 * r;
            if (j < 1 || j > in.NY) continue;
            const int cell = i + j * in.pitch;
            if (__ldg(&in.type[cell]) != T_FLUID) continue;
            pred_refresh_cell(in, cell, nullptr, stage, finalize);
        }
    } else {
        const int g = ((int)vb - ntiles) * blockDim.x + threadIdx.x;
        if (g >= ng) return;
        const GhostDev* gh = &G[g];
        if (gh->cell < 0) return;
        const InstDev& in = I[gh->inst];
        if (in.retired) return;
        if (!finalize && !pred_refresh_due(in, S[gh->inst])) return;
        pred_refresh_cell(in, gh->cell, gh, stage, finalize);
    }
}

// One FP32 sweep on the correction; parity 0 reads (du, dv), writes (du2,
// dv2), parity 1 the reverse.  Tiles of 32 x 8R cells with loads at indices
// clamped into the interior; partials as b_pred_sweep, one per 32x8 sub-tile
// (the same reduction as a 32x8 tile: results do not depend on R).
template <int R = 1>
__device__ __forceinline__ void b_pred_sweep32(const Tile* __restrict__ tiles, int ntiles,
                                               const GhostDev* __restrict__ G, int ng,
                                               const LevelDev* __restrict__ LV, const InstDev* __restrict__ I,
                                               const InstState* __restrict__ S, double* __restrict__ part,
                                               int parity, int vb) {
    if ((int)vb < ntiles) {
        const Tile t = ldg_struct(&tiles[vb]);
        const InstDev& in = I[t.inst];
        const LevelDev& L = LV[t.lev];  // finest-level tiles
        const int st = S[t.inst].pred_state, nxi = in.NX, nxl = L.NX;  // loads in flight together
        if ((st == ST_DONE) | (nxi < 0) | (nxl < 0)) return;
        const float* su = parity ? in.du2 : in.du;
        const float* sv = parity ? in.dv2 : in.dv;
        float* du = parity ? in.du : in.du2;
        float* dv = parity ? in.dv : in.dv2;
        const int i = t.i0 + (int)(threadIdx.x & 31), jb = t.j0 + (int)(threadIdx.x >> 5);
        const int ic = clampi(i, 1, in.NX), P = in.pitch;
        int id[R], jc[R];
        bool fl[R];
#pragma unroll
        for (int r = 0; r < R; r++) {
            const int j = jb + 8 * r;
            jc[r] = clampi(j, 1, in.NY);
            id[r] = ic + jc[r] * P;
            fl[r] = i == ic && j == jc[r] && __ldg(&in.type[id[r]]) == T_FLUID;
        }
        if (st == ST_FINAL_IN_ALT) {
#pragma unroll
            for (int r = 0; r < R; r++)
                if (fl[r]) {
                    du[id[r]] = su[id[r]];
                    dv[id[r]] = sv[id[r]];
                }
            return;
        }
        // inner cycle of mixed_inner sweeps: this sweep starts one (FP64 defect
        // of q0 first) and / or ends one (q0 absorbs the new correction)
        const int mi = in.mixed_inner > 0 ? in.mixed_inner : 8, it = S[t.inst].pred_iters;
        const bool cyc_start = it % mi == 0, cyc_end = (it + 1) % mi == 0;
        if (cyc_start) {
#pragma unroll
            for (int r = 0; r < R; r++)
                if (fl[r]) pred_refresh_cell(in, id[r], nullptr, 1, 0);
        }
        const float dtre = (float)in.dtre;
        const float ixi = __ldg(&L.ixf[ic]);
        const float aE = dtre * (__ldg(&L.kxf[ic]) * ixi), aW = dtre * (__ldg(&L.kxf[ic - 1]) * ixi);
        float m[R][1];
#pragma unroll
        for (int r = 0; r < R; r++) {
            const int q = id[r];
            const float iyj = __ldg(&L.iyf[jc[r]]);
            const float aN = dtre * (__ldg(&L.kyf[jc[r]]) * iyj), aS = dtre * (__ldg(&L.kyf[jc[r] - 1]) * iyj);
            const float aP = 1.0f + aE + aW + aN + aS;
            const float di = rcpa(aP);
            const float dU = (in.rfu[q] + aE * su[q + 1] + aW * su[q - 1] + aN * su[q + P] + aS * su[q - P] -
                              aP * su[q]) * di;
            const float dV = (in.rfv[q] + aE * sv[q + 1] + aW * sv[q - 1] + aN * sv[q + P] + aS * sv[q - P] -
                              aP * sv[q]) * di;
            m[r][0] = 0.0f;
            if (fl[r]) {
                const float nu = su[q] + dU, nv = sv[q] + dV;
                if (cyc_end) {
                    in.u[q] += (double)nu;
                    in.v[q] += (double)nv;
                    du[q] = 0.0f;
                    dv[q] = 0.0f;
                } else {
                    du[q] = nu;
                    dv[q] = nv;
                }
                m[r][0] = fabsf(dU) + fabsf(dV);
            }
        }
        write_sub_partials<1, float, R>(in, L, t, m, part);
    } else {
        const int g = ((int)vb - ntiles) * blockDim.x + threadIdx.x;
        if (g >= ng) return;
        const GhostDev& gh = G[g];
        if (gh.cell < 0) return;
        const InstDev& in = I[gh.inst];
        const int st = S[gh.inst].pred_state;
        if (st == ST_DONE) return;
        const float* su = parity ? in.du2 : in.du;
        const float* sv = parity ? in.dv2 : in.dv;
        float* du = parity ? in.du : in.du2;
        float* dv = parity ? in.dv : in.dv2;
        if (st == ST_FINAL_IN_ALT) {
            du[gh.cell] = su[gh.cell];
            dv[gh.cell] = sv[gh.cell];
            return;
        }
        const int mi = in.mixed_inner > 0 ? in.mixed_inner : 8, it = S[gh.inst].pred_iters;
        if (it % mi == 0) pred_refresh_cell(in, gh.cell, &gh, 1, 0);
        float au = in.rfu[gh.cell], av = in.rfv[gh.cell];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            au += (float)gh.wu[k] * su[gh.nb[k]];
            av += (float)gh.wv[k] * sv[gh.nb[k]];
        }
        if ((it + 1) % mi == 0) {
            in.u[gh.cell] += (double)au;
            in.v[gh.cell] += (double)av;
            du[gh.cell] = 0.0f;
            dv[gh.cell] = 0.0f;
        } else {
            du[gh.cell] = au;
            dv[gh.cell] = av;
        }
    }
}

// -------------------------------------------------- faces and PPE source

// Face values of a 32x8 tile (b_face_rhs, b_correct): x faces i0-1 .. i0+31
// of its rows and y faces j0-1 .. j0+7 of its columns, two fields each.  One
// shared allocation serves both phases (a function-scope __shared__ object).
struct TileFaces {
    double x[2][TILE_Y][TILE_X + 1];
    double y[2][TILE_Y + 1][TILE_X];
};
__device__ __forceinline__ TileFaces& tile_faces() {
    __shared__ TileFaces f;
    return f;
}

__device__ __forceinline__ double face_u(const InstDev& in, const double* u, int i, int id) {
    if (__ldg(&in.type[id]) == T_FLUID || __ldg(&in.type[id + 1]) == T_FLUID) return u[id] * __ldg(&in.gx[i]) + u[id + 1] * __ldg(&in.fx[i]);
    return 0.0;
}
__device__ __forceinline__ double face_v(const InstDev& in, const double* v, int j, int id) {
    const int P = in.pitch;
    if (__ldg(&in.type[id]) == T_FLUID || __ldg(&in.type[id + P]) == T_FLUID) return v[id] * __ldg(&in.gy[j]) + v[id + P] * __ldg(&in.fy[j]);
    return 0.0;
}

// Face velocities of the predicted field (into Us,Vs, or into U,V when
// to_final), the pressure source div(U*)/dt and its area-weighted sum.
// Also sets the pressure solve's initial guess: the extrapolation of the
// instance's last pressures, 3 p^(n-1) - 3 p^(n-2) + p^(n-3) from its fourth
// step on, 2 p^(n-1) - p^(n-2) on its third (the solve from the last pressure
// alone starts O(dt) away, the quadratic extrapolation O(dt^3): fewer Krylov
// iterations under the same stop rule).  Each operation is rounded on its
// own, as in the oracle.  Every face value is formed once, as in b_correct:
// thread (w, lane) forms the east and north faces of its cell, warps 0 and 1
// the south faces of the first row and the west faces of the first column.
__device__ __forceinline__ void b_face_rhs(const Tile* __restrict__ tiles, const InstDev* __restrict__ I,
                           const InstState* __restrict__ S, double* __restrict__ part, int to_final, int vb) {
    const Tile t = ldg_struct(&tiles[vb]);
    const InstDev& in = I[t.inst];
    if (in.retired) return;
    TileFaces& F = tile_faces();
    auto& sU = F.x[0];
    auto& sV = F.y[0];
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    int i, j;
    tile_ij(t, i, j);
    const int P = in.pitch, id = i + j * P, NX = in.NX, NY = in.NY;
    const bool row = j >= 1 && j <= NY, col = i >= 1 && i <= NX;
    double* Uo = to_final ? in.U : in.Us;
    double* Vo = to_final ? in.V : in.Vs;
    {
        double Ue = 0.0, Vn = 0.0;
        if (row && i <= NX) Uo[id] = Ue = face_u(in, in.u, i, id);
        if (col && j <= NY) Vo[id] = Vn = face_v(in, in.v, j, id);
        sU[w][l + 1] = Ue;
        sV[w + 1][l] = Vn;
    }
    if (w == 0) {
        const int js = t.j0 - 1;
        sV[0][l] = (js >= 0 && col) ? face_v(in, in.v, js, i + js * P) : 0.0;
    } else if (w == 1 && l < TILE_Y) {
        const int iw = t.i0 - 1, jw = t.j0 + l;
        sU[l][0] = (iw >= 0 && jw >= 1 && jw <= NY) ? face_u(in, in.u, iw, iw + jw * P) : 0.0;
    }
    __syncthreads();
    double acc[1] = {0.0};
    if (row && col) {
        if (__ldg(&in.type[id]) == T_FLUID) {
            const double Ue = sU[w][l + 1], Uw = sU[w][l];
            const double Vn = sV[w + 1][l], Vs = sV[w][l];
            const double d = (Ue - Uw) * __ldg(&in.ix[i]) + (Vn - Vs) * __ldg(&in.iy[j]);
            const double b = d / in.dt;
            in.b[id] = b;
            if (in.singular) acc[0] = b * (__ldg(&in.dx[i]) * __ldg(&in.dy[j]));
            if (!to_final) {
                const double po = in.p[id], p2 = in.pold[id];
                const int m = S[t.inst].pold_n;
                if (m >= 4) in.p[id] = __dadd_rn(__dsub_rn(__dmul_rn(3.0, po), __dmul_rn(3.0, p2)), in.pold2[id]);
                else if (m >= 3) in.p[id] = __dsub_rn(__dmul_rn(2.0, po), p2);
                in.pold2[id] = p2;
                in.pold[id] = po;
                // the predictor increment for the next step's initial guess
                in.dup[id] = in.u[id] - in.dup[id];
                in.dvp[id] = in.v[id] - in.dvp[id];
            }
        } else {
            in.b[id] = 0.0;
            if (!to_final) in.dup[id] = in.dvp[id] = 0.0;
        }
    }
    // the area-weighted source serves the mean removal of a singular operator only
    __shared__ double out[1];
    if (in.singular) block_sum<1>(acc, out);
    else __syncthreads();  // the block's next tile rewrites the face arrays
    if (threadIdx.x == 0) part[(size_t)vb * NPART] = in.singular ? out[0] : 0.0;
}

template <bool WIDE = false>
__device__ __forceinline__ void b_rhs_reduce(const InstDev* __restrict__ I, InstState* __restrict__ S,
                             const double* __restrict__ part, int vb) {
    const int k = vb;
    const InstDev& in = I[k];
    if (in.retired) return;
    double r[1];
    inst_sum<1, WIDE>(part, in.tile_beg, in.tile_cnt, r);
    if (threadIdx.x == 0) S[k].bmean = in.singular ? r[0] / in.area : 0.0;
}

// ------------------------------------------------------------------ PPE
//
// BiCGSTAB in FP64 on L p = b (ghost-eliminated finest-level operator),
// preconditioned by one multigrid V-cycle in T.  Per-instance scalars live
// in InstState; every reduction is per instance over its tiles, fixed order.

__device__ __forceinline__ bool live0(const LevelDev& L, int i, int j, int& id, uint8_t& bt) {
    if (i < 1 || i > L.NX || j < 1 || j > L.NY) return false;
    id = i + j * L.pitch;
    bt = __ldg(&L.bits[id]);
    return (bt & 0x0F) != 0;
}

// BiCGSTAB of the pressure solve.  The Krylov vectors (r, rh, p_dir, v, s,
// t and the preconditioned p_dir, s) are of type T: FP64 in the plain path,
// FP32 in the mixed path, where the iterate p stays FP64 and the FP32
// iteration restarts from the FP64 true residual b - L p ("defect
// correction": convergence is only accepted on the true residual).  Dot
// products are accumulated in FP64 in both paths.

// True when the tile's instance is still solving.  The state is indexed by
// the tile's own instance (not the level's), and the test also reads the
// level's first field (NX, never negative), so the two loads are in flight
// together instead of one after the other.
__device__ __forceinline__ bool tile_live(const Tile& t, const LevelDev& L, const InstState* __restrict__ S) {
    const int state = S[t.inst].ppe_state, nx = L.NX;
    return (state == ST_ACTIVE) & (nx >= 0);
}
// The same for a finest-level tile, also touching the instance's fields.
__device__ __forceinline__ bool tile_live0(const Tile& t, const LevelDev& L, const InstDev& in,
                                           const InstState* __restrict__ S) {
    const int state = S[t.inst].ppe_state, nx = L.NX, nxi = in.NX;
    return (state == ST_ACTIVE) & (nx >= 0) & (nxi >= 0);
}

// r = (b - mean b) - L p in FP64, rh = r, p_dir = v = 0.  restart_only: only
// the instances whose mixed-path restart is due.
// partials: 0 (r,r)  1 (b,b)  2 (rh,r)  3 (p,area)
template <typename T>
__device__ __forceinline__ void b_bicg_start(const Tile* __restrict__ tiles, const LevelDev* __restrict__ LV,
                                             const InstDev* __restrict__ I, const InstState* __restrict__ S,
                                             const GhostDev* __restrict__ G, double* __restrict__ part,
                                             int restart_only, int vb) {
    const Tile t = ldg_struct(&tiles[vb]);
    const InstDev& in = I[t.inst];
    const InstState& st = S[t.inst];
    const LevelDev& L = LV[t.lev];  // finest-level tiles
    if (!tile_live0(t, L, in, S)) return;
    if (restart_only && !st.restart) return;
    int i, j, id;
    uint8_t bt;
    tile_ij(t, i, j);
    T acc[4] = {(T)0, (T)0, (T)0, (T)0};
    if (live0(L, i, j, id, bt)) {
        double Lp, D;
        lap<double, double, true>(L, in.p, i, j, id, bt, G, in.gidx, Lp, D);
        const double bb = in.b[id] - st.bmean;
        const double r = bb - Lp;
        const T rt = (T)r;
        ((T*)in.kr)[id] = rt;
        ((T*)in.krh)[id] = rt;
        ((T*)in.kp)[id] = (T)0;
        ((T*)in.kv)[id] = (T)0;
        acc[0] = (T)(r * r);
        if (!restart_only) acc[1] = (T)(bb * bb);  // ||b||: the initial residual only
        acc[2] = rt * rt;
        if (in.singular) acc[3] = (T)(in.p[id] * (__ldg(&in.dx[i]) * __ldg(&in.dy[j])));
    }
    __shared__ double out[4];
    block_sum<4, T>(acc, out);
    if (threadIdx.x < 4) part[(size_t)vb * NPART + threadIdx.x] = out[threadIdx.x];
}

// Convergence test on ||r||, then rho, beta for the next direction.  Votes
// (start == 0 only).  start: 1 after the initial residual, 2 after a mixed-path
// restart (instances without one are skipped), 0 after an iteration.  mixed:
// the recursive FP32 residual is never accepted; a restart is scheduled when
// it fell by in.restart_drop (or below the tolerance) since the last one, or
// after in.restart_every iterations.
template <bool WIDE = false>
__device__ __forceinline__ void b_bicg_reduce_r(const InstDev* __restrict__ I, InstState* __restrict__ S,
                                                const double* __restrict__ part, int start, int mixed,
                                                LoopCtl* ctl, unsigned long long handle, int vb) {
    const int k = vb;
    const InstDev& in = I[k];
    bool active = false, due = false;
    if (start == 2 && none_due(ctl)) return;
    const bool run = S[k].ppe_state == ST_ACTIVE && (start != 2 || S[k].restart);
    const int beg = in.tile_beg, cnt = in.tile_cnt;
    pdl_wait();  // the partials of the phase before; every write below
    if (run) {
        double r[4];
        inst_sum<4, WIDE>(part, beg, cnt, r);
        if (threadIdx.x == 0) {
            InstState& st = S[k];
            if (start == 1) {
                st.bnorm = sqrt(r[1]);
                st.rho = st.alpha = st.omega = 1.0;
                st.ppe_iters = 0;
                st.restart = 0;
                st.restart_it = 0;
            } else if (start == 2) {
                st.rho = st.alpha = st.omega = 1.0;
                st.restart = 0;
                st.restart_it = st.ppe_iters;
            } else {
                st.ppe_iters += 1;
            }
            const double rel = sqrt(r[0]) / (st.bnorm > 1e-300 ? st.bnorm : 1e-300);
            st.ppe_rel = rel;
            st.pmean = r[3] / in.area;
            if (start != 0) st.rel_restart = rel;
            const bool true_res = start != 0 || !mixed;
            if ((true_res && rel <= in.ppe_tol) || st.ppe_iters >= in.ppe_itermax) {
                st.ppe_state = ST_DONE;
            } else if (!true_res && (rel <= in.ppe_tol || rel <= in.restart_drop * st.rel_restart ||
                                     st.ppe_iters - st.restart_it >= in.restart_every)) {
                st.restart = 1;
                active = true;
                due = true;
            } else {
                const double rho1 = r[2];
                st.beta = (rho1 / st.rho) * (st.alpha / st.omega);
                st.rho = rho1;
                active = true;
            }
        }
    }
    if (threadIdx.x == 0 && start != 2) loop_vote(ctl, active, handle, due);
}

// p_dir = r + beta (p_dir - omega v); preconditioner input.
template <typename T, int R = 1>
__device__ __forceinline__ void b_bicg_p(const Tile* __restrict__ tiles, const LevelDev* __restrict__ LV,
                                         const InstDev* __restrict__ I, const InstState* __restrict__ S, int vb) {
    const Tile t = ldg_struct(&tiles[vb]);
    const InstDev& in = I[t.inst];
    const InstState& st = S[t.inst];
    const LevelDev& L = LV[t.lev];  // finest-level tiles
    if (!tile_live0(t, L, in, S)) return;
    Rows0<R> q;
    rows0<R>(L, t, q);
    T* kp = (T*)in.kp;
    const T beta = (T)st.beta, om = (T)st.omega;
    T pd[R];
#pragma unroll
    for (int r = 0; r < R; r++) pd[r] = ((const T*)in.kr)[q.id[r]] + beta * (kp[q.id[r]] - om * ((const T*)in.kv)[q.id[r]]);
#pragma unroll
    for (int r = 0; r < R; r++)
        if (q.bt[r] & 0x0F) {
            kp[q.id[r]] = pd[r];
            ((T*)L.r)[q.id[r]] = pd[r];
        }
}

// The direction update (which = 0: p_dir as b_bicg_p; 1: s as b_bicg_s)
// fused with the V-cycle's first, zero-start smoothing sweep of the finest
// level that follows it (as b_smooth with flags = 1, src_alt = 0): the new
// vector is the sweep's right-hand side, so it is used from registers instead
// of being read back.  Same arithmetic as the two phases.
template <typename T, int R = 1>
__device__ __forceinline__ void b_bicg_dir_smooth(const Tile* __restrict__ tiles, const LevelDev* __restrict__ LV,
                                                  const InstDev* __restrict__ I, const InstState* __restrict__ S,
                                                  const GhostDev* __restrict__ G, int which, int vb) {
    const Tile t = ldg_struct(&tiles[vb]);
    const InstDev& in = I[t.inst];
    const InstState& st = S[t.inst];
    const LevelDev& L = LV[t.lev];  // finest-level tiles
    if (!tile_live0(t, L, in, S)) return;
    Rows0<R> q;
    rows0<R>(L, t, q);
    const T* kr = (const T*)in.kr;
    const T* kv = (const T*)in.kv;
    T* out = (T*)(which == 0 ? in.kp : in.ks);
    const T* src = (const T*)L.e;
    T* dst = (T*)L.e2;
    const T om = (T)in.omega;
    // the instance's scalars, converted once per thread
    const T c1 = which == 0 ? (T)st.beta : (T)st.alpha, omg = which == 0 ? (T)st.omega : (T)0;
    T val[R], e1[R];
#pragma unroll
    for (int r = 0; r < R; r++) {
        const int id = q.id[r];
        if (which == 0) val[r] = kr[id] + c1 * (((const T*)in.kp)[id] - omg * kv[id]);
        else val[r] = kr[id] - c1 * kv[id];
        T Le, D;
        lap_p<T, T, true>(L, src, q.ic, q.jc[r], id, L.pitch, q.bt[r], G, in.gidx, Le, D);
        e1[r] = jacobi_from_zero<T>(val[r], D, om);
    }
#pragma unroll
    for (int r = 0; r < R; r++)
        if (q.bt[r] & 0x0F) {
            out[q.id[r]] = val[r];
            ((T*)L.r)[q.id[r]] = val[r];
            dst[q.id[r]] = e1[r];
        }
}

// y = L z with z the preconditioned vector (V-cycle result), operator and z
// in T; z is kept as zo.  partials: which=0 -> (rh, y) ; which=1 -> (y, s), (y, y)
template <typename T, int R = 1>
__device__ __forceinline__ void b_bicg_apply(const Tile* __restrict__ tiles, const LevelDev* __restrict__ LV,
                                             const InstDev* __restrict__ I, const InstState* __restrict__ S,
                                             const GhostDev* __restrict__ G, double* __restrict__ part, int e_alt,
                                             int which, int vb) {
    const Tile t = ldg_struct(&tiles[vb]);
    const InstDev& in = I[t.inst];
    const LevelDev& L = LV[t.lev];  // finest-level tiles
    if (!tile_live0(t, L, in, S)) return;
    const T* z = (const T*)(e_alt ? L.e2 : L.e);
    T* zo = (T*)(which == 0 ? in.kph : in.ksh);
    T* y = (T*)(which == 0 ? in.kv : in.kt);
    const T* w2 = (const T*)(which == 0 ? in.krh : in.ks);
    Rows0<R> q;
    rows0<R>(L, t, q);
    T acc[R][2];
#pragma unroll
    for (int r = 0; r < R; r++) {
        T Lz, D;
        lap_p<T, T, true>(L, z, q.ic, q.jc[r], q.id[r], L.pitch, q.bt[r], G, in.gidx, Lz, D);
        const T zc = z[q.id[r]], wv = w2[q.id[r]];
        acc[r][0] = acc[r][1] = (T)0;
        if (q.bt[r] & 0x0F) {
            zo[q.id[r]] = zc;
            y[q.id[r]] = Lz;
            if (which == 0) {
                acc[r][0] = wv * Lz;
            } else {
                acc[r][0] = Lz * wv;
                acc[r][1] = Lz * Lz;
            }
        }
    }
    write_sub_partials<2, T, R>(in, L, t, acc, part);
}

// alpha = rho / (rh, v)   (which = 0)   or   omega = (t, s) / (t, t)   (which = 1)
template <bool WIDE = false>
__device__ __forceinline__ void b_bicg_scalar(const InstDev* __restrict__ I, InstState* __restrict__ S,
                              const double* __restrict__ part, int which, int vb) {
    const int k = vb;
    const InstDev& in = I[k];
    if (S[k].ppe_state != ST_ACTIVE) return;
    const int beg = in.tile_beg, cnt = in.tile_cnt;
    pdl_wait();  // the operator apply's partials
    double r[2];
    inst_sum<2, WIDE>(part, beg, cnt, r);
    if (threadIdx.x == 0) {
        if (which == 0) S[k].alpha = r[0] != 0.0 ? S[k].rho / r[0] : 0.0;
        else S[k].omega = r[1] != 0.0 ? r[0] / r[1] : 0.0;
    }
}

// s = r - alpha v; preconditioner input.
template <typename T, int R = 1>
__device__ __forceinline__ void b_bicg_s(const Tile* __restrict__ tiles, const LevelDev* __restrict__ LV,
                                         const InstDev* __restrict__ I, const InstState* __restrict__ S, int vb) {
    const Tile t = ldg_struct(&tiles[vb]);
    const InstDev& in = I[t.inst];
    const InstState& st = S[t.inst];
    const LevelDev& L = LV[t.lev];  // finest-level tiles
    if (!tile_live0(t, L, in, S)) return;
    Rows0<R> q;
    rows0<R>(L, t, q);
    const T alpha = (T)st.alpha;
    T sv[R];
#pragma unroll
    for (int r = 0; r < R; r++) sv[r] = ((const T*)in.kr)[q.id[r]] - alpha * ((const T*)in.kv)[q.id[r]];
#pragma unroll
    for (int r = 0; r < R; r++)
        if (q.bt[r] & 0x0F) {
            ((T*)in.ks)[q.id[r]] = sv[r];
            ((T*)L.r)[q.id[r]] = sv[r];
        }
}

// p += alpha ph + omega sh (FP64) ; r = s - omega t (T).
// partials: 0 (r,r)  1 unused  2 (rh,r)  3 (p,area)
template <typename T, int R = 1>
__device__ __forceinline__ void b_bicg_x(const Tile* __restrict__ tiles, const LevelDev* __restrict__ LV,
                                         const InstDev* __restrict__ I, const InstState* __restrict__ S,
                                         double* __restrict__ part, int vb) {
    const Tile t = ldg_struct(&tiles[vb]);
    const InstDev& in = I[t.inst];
    const InstState& st = S[t.inst];
    const LevelDev& L = LV[t.lev];  // finest-level tiles
    if (!tile_live0(t, L, in, S)) return;
    Rows0<R> q;
    rows0<R>(L, t, q);
    const double alpha = st.alpha, omega = st.omega;
    const T omf = (T)omega;
    const double dxi = __ldg(&in.dx[q.ic]);
    const bool sing = in.singular;  // the area-weighted sum of p serves the nullspace projection only
    T acc[R][4];
#pragma unroll
    for (int r = 0; r < R; r++) {
        const int id = q.id[r];
        const double pn = in.p[id] + alpha * (double)((const T*)in.kph)[id] + omega * (double)((const T*)in.ksh)[id];
        const T rv = ((const T*)in.ks)[id] - omf * ((const T*)in.kt)[id];
        const T rh = ((const T*)in.krh)[id];
        acc[r][0] = acc[r][1] = acc[r][2] = acc[r][3] = (T)0;
        if (q.bt[r] & 0x0F) {
            in.p[id] = pn;
            ((T*)in.kr)[id] = rv;
            acc[r][0] = rv * rv;
            acc[r][2] = rh * rv;
            if (sing) acc[r][3] = (T)(pn * (dxi * __ldg(&in.dy[q.jc[r]])));
        }
    }
    write_sub_partials<4, T, R>(in, L, t, acc, part);
}

// Multigrid tile phases.  A tile is 32 columns by 8R rows of one level of
// one instance.  In the phases without reductions (smoothing, restriction)
// thread (w, lane) handles column i0+lane of the R consecutive rows from
// j0+R*w: it loads its column once on rows j0+R*w-1 .. j0+R*w+R and takes
// the north and south values from there.  Every load uses indices clamped
// into the level's rows (ghost rows included) and columns, so all of a
// thread's loads issue together (no load waits on the stencil byte);
// results are stored for live cells only, each from the same operands and
// arithmetic whatever R and the row assignment.

// Weighted-Jacobi sweep.  flags: 1 = start from e = 0.
template <typename T, int R = 1>
__device__ __forceinline__ void smooth_tile(const Tile& t, const LevelDev& L, const T om, const int* gidx,
                                            const GhostDev* __restrict__ G, int flags, int src_alt, int state) {
    const T* src = (const T*)(src_alt ? L.e2 : L.e);
    T* dst = (T*)(src_alt ? L.e : L.e2);
    const T* rr = (const T*)L.r;
    const int P = L.pitch;
    const int i = t.i0 + (int)(threadIdx.x & 31), jb = t.j0 + R * (int)(threadIdx.x >> 5);
    const int ic = clampi(i, 1, L.NX);
    T col[R + 2];  // column ic on rows jb-1 .. jb+R
#pragma unroll
    for (int k = 0; k < R + 2; k++) col[k] = src[ic + clampi(jb - 1 + k, 0, L.NY + 1) * P];
    int id[R];
    uint8_t bt[R];
    T val[R];
#pragma unroll
    for (int r = 0; r < R; r++) {
        const int j = jb + r, jc = clampi(j, 1, L.NY);
        id[r] = ic + jc * P;
        bt[r] = (i == ic && j == jc) ? __ldg(&L.bits[id[r]]) : (uint8_t)0;
    }
    auto fetch = [src](int q) { return (T)src[q]; };
#pragma unroll
    for (int r = 0; r < R; r++) {
        const int jc = clampi(jb + r, 1, L.NY);
        const T eE = src[id[r] + 1], eW = src[id[r] - 1];
        T Le, D;
        if (L.depth == 0)
            lap_vals<T, true>(L, ic, jc, id[r], P, bt[r], G, gidx, eE, eW, col[r + 2], col[r], col[r + 1], fetch, Le, D);
        else
            lap_vals<T, false>(L, ic, jc, id[r], P, bt[r], G, nullptr, eE, eW, col[r + 2], col[r], col[r + 1], fetch,
                               Le, D);
        val[r] = (flags & 1) ? jacobi_from_zero<T>(rr[id[r]], D, om) : jacobi_update<T>(col[r + 1], rr[id[r]], Le, D, om);
    }
    if (state != ST_ACTIVE) return;
#pragma unroll
    for (int r = 0; r < R; r++)
        if (bt[r] & 0x0F) dst[id[r]] = val[r];
}
template <typename T, int R = 1>
__device__ __forceinline__ void b_smooth(const Tile* __restrict__ tiles, const LevelDev* __restrict__ LV,
                                         const InstDev* __restrict__ I, const InstState* __restrict__ S,
                                         const GhostDev* __restrict__ G, int flags, int src_alt, int vb) {
    const Tile t = ldg_struct(&tiles[vb]);
    const LevelDev& L = LV[t.lev];
    if (!tile_live(t, L, S)) return;
    smooth_tile<T, R>(t, L, (T)I[t.inst].omega, L.depth == 0 ? I[t.inst].gidx : nullptr, G, flags, src_alt, ST_ACTIVE);
}
// The same sweep with the tile staged in shared memory by the tensor memory
// accelerator: one thread issues three 2-D tile loads on an mbarrier (the
// correction with a one-cell halo, from 16 bytes left of the tile so that the
// box start is aligned; the right-hand side; the stencil bytes), and the
// block computes from shared memory.  The loads of a tile no longer cost
// registers, so more of them are in flight.  Out-of-range box parts read
// zero; every stored cell (stencil byte non-zero, so inside the level) takes
// the same operands and arithmetic as smooth_tile.  A copy that does not
// complete within the wait limit sets *err and the block leaves.
template <typename T, int R>
struct SmoothStage {
    static constexpr int PAD = 16 / (int)sizeof(T);
    static constexpr int BX = TILE_X + 2 * PAD, BY = TILE_Y * R + 2;
    alignas(128) T e[BY][BX];
    alignas(128) T r[TILE_Y * R][TILE_X];
    alignas(128) uint8_t b[TILE_Y * R][TILE_X];
    unsigned long long bar;
};
// state: the instance's pressure-solve state (stores only while active).
template <typename T, int R>
__device__ __forceinline__ void smooth_tile_tma(const Tile& t, const LevelDev& L, const T om, const int* gidx,
                                                const GhostDev* __restrict__ G, const CUtensorMap* __restrict__ tm,
                                                int flags, int src_alt, unsigned* err, int state) {
    using St = SmoothStage<T, R>;
    __shared__ St sm;
    const bool zero = (flags & 1) != 0;
    const CUtensorMap* m = tm + (size_t)t.lev * TMA_MAPS_PER_LEVEL + (R == 1 ? 0 : 4);
    if (threadIdx.x == 0) {
        mbar_init(&sm.bar, 1);
        const unsigned bytes = (zero ? 0u : (unsigned)sizeof(sm.e)) + (unsigned)sizeof(sm.r) + (unsigned)sizeof(sm.b);
        mbar_expect_tx(&sm.bar, bytes);
        if (!zero) tma_load_2d(&sm.e[0][0], &m[src_alt ? 1 : 0], t.i0 - St::PAD, t.j0 - 1, &sm.bar);
        tma_load_2d(&sm.r[0][0], &m[2], t.i0, t.j0, &sm.bar);
        tma_load_2d(&sm.b[0][0], &m[3], t.i0, t.j0, &sm.bar);
    }
    __syncthreads();
    if (!mbar_wait(&sm.bar, 0)) {
        if (threadIdx.x == 0) atomicExch(err, 1u);
        mbar_wait(&sm.bar, 0);  // the copies in flight, bounded again
        return;
    }
    if (state != ST_ACTIVE) return;
    const T* src = (const T*)(src_alt ? L.e2 : L.e);
    T* dst = (T*)(src_alt ? L.e : L.e2);
    const int P = L.pitch, lane = (int)(threadIdx.x & 31), w = (int)(threadIdx.x >> 5);
    const int ic = clampi(t.i0 + lane, 1, L.NX);
    auto fetch = [src](int q) { return (T)src[q]; };
#pragma unroll
    for (int r = 0; r < R; r++) {
        const int row = R * w + r;
        const int jc = clampi(t.j0 + row, 1, L.NY), id = ic + jc * P;
        const uint8_t bt = sm.b[row][lane];
        const int x = lane + St::PAD;
        const T eP = sm.e[row + 1][x], eN = sm.e[row + 2][x], eS = sm.e[row][x];
        const T eE = sm.e[row + 1][x + 1], eW = sm.e[row + 1][x - 1];
        T Le, D;
        if (L.depth == 0) lap_vals<T, true>(L, ic, jc, id, P, bt, G, gidx, eE, eW, eN, eS, eP, fetch, Le, D);
        else lap_vals<T, false>(L, ic, jc, id, P, bt, G, nullptr, eE, eW, eN, eS, eP, fetch, Le, D);
        const T rv = sm.r[row][lane];
        const T val = zero ? jacobi_from_zero<T>(rv, D, om) : jacobi_update<T>(eP, rv, Le, D, om);
        if (bt & 0x0F) dst[id] = val;
    }
}
template <typename T, int R>
__device__ __forceinline__ void b_smooth_tma(const Tile* __restrict__ tiles, const LevelDev* __restrict__ LV,
                                             const InstDev* __restrict__ I, const InstState* __restrict__ S,
                                             const GhostDev* __restrict__ G, const CUtensorMap* __restrict__ tm,
                                             int flags, int src_alt, unsigned* err, int vb) {
    const Tile t = ldg_struct(&tiles[vb]);
    const LevelDev& L = LV[t.lev];
    if (!tile_live(t, L, S)) return;
    smooth_tile_tma<T, R>(t, L, (T)I[t.inst].omega, L.depth == 0 ? I[t.inst].gidx : nullptr, G, tm, flags, src_alt,
                          err, ST_ACTIVE);
}
// One level of a one-instance solver (tiles from the block index, x0 = 0).
template <typename T, int R>
__device__ __forceinline__ void b_smooth_grid_tma(const GridTiles& g, const InstState* __restrict__ S,
                                                  const GhostDev* __restrict__ G, const CUtensorMap* __restrict__ tm,
                                                  int flags, int src_alt, unsigned* err, int vb) {
    const int state = S[g.inst].ppe_state;
    smooth_tile_tma<T, R>(g.tile(vb), g.L, (T)g.omega, g.L.depth == 0 ? g.gidx : nullptr, G, tm, flags, src_alt, err,
                          state);
}

template <typename T, int R = 1>
__device__ __forceinline__ void b_smooth_grid(const GridTiles& g, const InstState* __restrict__ S,
                                              const GhostDev* __restrict__ G, int flags, int src_alt, int vb) {
    const int state = S[g.inst].ppe_state;
    smooth_tile<T, R>(g.tile(vb), g.L, (T)g.omega, g.L.depth == 0 ? g.gidx : nullptr, G, flags, src_alt, state);
}

// Restriction of the fine residual (area weighted) onto the coarse level,
// fused with the first (zero-start) smoothing sweep of a middle coarse level.
// One thread per FINE cell: tiles of the fine level start at (1, 1), so the
// fine cells of a coarse cell share a tile (lanes 2k, 2k+1 when x is
// coarsened; when y is, rows 2J-1, 2J are a thread's consecutive rows for
// R > 1 and warps 2w, 2w+1 for R = 1); each thread forms (r - L e) dA of its
// cells, pairs are summed in x by shuffle and then in y (in registers, or
// through shared memory for R = 1) in the order (t00 + t10) + (t01 + t11), as
// the oracle, and the thread of the first child writes the coarse cell.
template <typename T, int R = 1>
__device__ __forceinline__ void b_restrict(const Tile* __restrict__ tiles, const LevelDev* __restrict__ LV,
                                           const InstDev* __restrict__ I, const InstState* __restrict__ S,
                                           const GhostDev* __restrict__ G, int fine_alt, int vb) {
    static_assert(R == 1 || R % 2 == 0, "rows per thread: 1 or even");
    __shared__ T rows[TILE_Y][TILE_X];
    const Tile t = ldg_struct(&tiles[vb]);
    const LevelDev& F = LV[t.lev];
    if (!tile_live(t, F, S)) return;
    const LevelDev& C = LV[F.child];
    const T* fe = (const T*)(fine_alt ? F.e2 : F.e);
    const T* fr = (const T*)F.r;
    const int* gidx = F.depth == 0 ? I[t.inst].gidx : nullptr;
    const int FP = F.pitch, cx = C.cx, cy = C.cy;
    const int lane = (int)(threadIdx.x & 31), w = (int)(threadIdx.x >> 5);
    const int i = t.i0 + lane, jb = t.j0 + R * w;
    const int ic = clampi(i, 1, F.NX);
    T col[R + 2];  // column ic on rows jb-1 .. jb+R
#pragma unroll
    for (int k = 0; k < R + 2; k++) col[k] = fe[ic + clampi(jb - 1 + k, 0, F.NY + 1) * FP];
    bool in[R];
    int id[R];
    uint8_t fb[R];
    T term[R];
#pragma unroll
    for (int r = 0; r < R; r++) {
        const int j = jb + r;
        in[r] = i <= F.NX && j <= F.NY;
        id[r] = ic + clampi(j, 1, F.NY) * FP;
        fb[r] = in[r] ? __ldg(&F.bits[id[r]]) : (uint8_t)0;
    }
    auto fetch = [fe](int q) { return (T)fe[q]; };
#pragma unroll
    for (int r = 0; r < R; r++) {
        const int jc = clampi(jb + r, 1, F.NY);
        const T eE = fe[id[r] + 1], eW = fe[id[r] - 1];
        T Le, D;
        if (F.depth == 0)
            lap_vals<T, true>(F, ic, jc, id[r], FP, fb[r], G, gidx, eE, eW, col[r + 2], col[r], col[r + 1], fetch, Le, D);
        else
            lap_vals<T, false>(F, ic, jc, id[r], FP, fb[r], G, nullptr, eE, eW, col[r + 2], col[r], col[r + 1], fetch,
                               Le, D);
        term[r] = (fb[r] & 0x0F) ? (fr[id[r]] - Le) * (__ldg(&LvA<T>::dw(F)[ic]) * __ldg(&LvA<T>::dh(F)[jc])) : (T)0;
    }
    // x pairs: (2I-1, 2I) are lanes (2k, 2k+1); the even lane keeps t0 + t1
    if (cx == 2) {
#pragma unroll
        for (int r = 0; r < R; r++) term[r] = term[r] + __shfl_xor_sync(0xffffffffu, term[r], 1);
    }
    // y pairs: rows (2J-1, 2J)
    bool first[R];  // this row is the first child row of its coarse cell
    if (R == 1) {
        // warps (2m, 2m+1)
        if (cy == 2) {
            if (w & 1) rows[w][lane] = term[0];
            __syncthreads();
            if (!(w & 1)) term[0] = term[0] + rows[w + 1][lane];
        }
        first[0] = cy != 2 || !(w & 1);
    } else {
        // the thread's rows (2m, 2m+1)
#pragma unroll
        for (int r = 0; r < R; r++) {
            first[r] = cy != 2 || !(r & 1);
            if (cy == 2 && !(r & 1)) term[r] = term[r] + term[r + 1];
        }
    }
    if (cx == 2 && (lane & 1)) return;
    T* rc = (T*)C.r;
    const T om = (T)I[t.inst].omega;
#pragma unroll
    for (int r = 0; r < R; r++) {
        if (!in[r] || !first[r]) continue;
        const int j = jb + r;
        const int I0 = cx == 2 ? (i + 1) >> 1 : i, J0 = cy == 2 ? (j + 1) >> 1 : j;
        const int cid = I0 + J0 * C.pitch;
        const uint8_t cb = __ldg(&C.bits[cid]);
        if (!(cb & 0x0F)) {
            rc[cid] = (T)0;
            continue;
        }
        const T rv = term[r] / (__ldg(&LvA<T>::dw(C)[I0]) * __ldg(&LvA<T>::dh(C)[J0]));
        rc[cid] = rv;
        if (C.child >= 0) ((T*)C.e)[cid] = jacobi_from_zero<T>(rv, lap_diag<T>(C, I0, J0, cb), om);
    }
}

// Bilinear correction at fine cell (i, j) from the next coarser level; ce(I, J)
// returns a coarse value, cb(I, J) a coarse stencil byte.
template <typename T, typename FE, typename FB>
__device__ __forceinline__ T prolong_corr(const LevelDev& F, int i, int j, FE ce, FB cb) {
    const int I0 = __ldg(&F.pI[i]), In = __ldg(&F.pIn[i]), J0 = __ldg(&F.pJ[j]), Jn = __ldg(&F.pJn[j]);
    const T wx = __ldg(&LvA<T>::pwx(F)[i]), wy = __ldg(&LvA<T>::pwy(F)[j]);
    const T sx = (T)__ldg(&F.psx[i]), sy = (T)__ldg(&F.psy[j]);
    T w00 = ((T)1 - wx) * ((T)1 - wy), w10 = wx * ((T)1 - wy), w01 = ((T)1 - wx) * wy, w11 = wx * wy;
    w00 = (cb(I0, J0) & 0x0F) ? w00 : (T)0;
    w10 = (cb(In, J0) & 0x0F) ? w10 : (T)0;
    w01 = (cb(I0, Jn) & 0x0F) ? w01 : (T)0;
    w11 = (cb(In, Jn) & 0x0F) ? w11 : (T)0;
    const T sw = w00 + w10 + w01 + w11;
    return (w00 * ce(I0, J0) + sx * w10 * ce(In, J0) + sy * w01 * ce(I0, Jn) + (sx * sy) * w11 * ce(In, Jn)) / sw;
}

// Bilinear prolongation of the coarse correction, added on the fine level.
template <typename T, int R = 1>
__device__ __forceinline__ void b_prolong(const Tile* __restrict__ tiles, const LevelDev* __restrict__ LV,
                                          const InstState* __restrict__ S, int fine_alt, int coarse_alt, int vb) {
    const Tile t = ldg_struct(&tiles[vb]);
    const LevelDev& F = LV[t.lev];
    if (!tile_live(t, F, S)) return;
    const LevelDev& C = LV[F.child];
    // the coarsest level's solution is always in e; a middle level's in the buffer its sweeps ended on
    const T* ce = (const T*)((coarse_alt && C.child >= 0) ? C.e2 : C.e);
    T* fe = (T*)(fine_alt ? F.e2 : F.e);
    const int P = F.pitch, CP = C.pitch;
    const uint8_t* cbits = C.bits;
    auto fce = [ce, CP](int I, int J) { return ce[I + J * CP]; };
    auto fcb = [cbits, CP](int I, int J) { return __ldg(&cbits[I + J * CP]); };
    const int i = t.i0 + (int)(threadIdx.x & 31), jb = t.j0 + (int)(threadIdx.x >> 5);
    const int ic = clampi(i, 1, F.NX);
    int id[R], jcs[R];
    uint8_t bt[R];
    T val[R];
#pragma unroll
    for (int r = 0; r < R; r++) {
        const int j = jb + 8 * r, jc = clampi(j, 1, F.NY);
        jcs[r] = jc;
        id[r] = ic + jc * P;
        bt[r] = (i == ic && j == jc) ? __ldg(&F.bits[id[r]]) : (uint8_t)0;
    }
#pragma unroll
    for (int r = 0; r < R; r++) val[r] = fe[id[r]] + prolong_corr<T>(F, ic, jcs[r], fce, fcb);
#pragma unroll
    for (int r = 0; r < R; r++)
        if (bt[r] & 0x0F) fe[id[r]] = val[r];
}

// Prolongation of the coarse correction fused with the first post-smoothing
// sweep, for a coarse level (no IBM ghosts) with 32x8 tiles (graph and
// host-loop modes).  The tile and a one-cell halo of buffer cur (the
// pre-smoothed correction, which no block writes in this phase) are staged in
// shared memory, the prolongation is added on the staged cells, and one
// weighted-Jacobi sweep of the tile is written to buffer cur ^ 1.  Same values
// as b_prolong (in place on cur) followed by b_smooth from cur into cur ^ 1;
// buffer cur keeps its pre-prolongation values, which the next sweep (from
// cur ^ 1 back into cur) overwrites on every live cell.
constexpr int PS_W = TILE_X + 2, PS_H = TILE_Y + 2, PS_N = PS_W * PS_H;

template <typename T>
__device__ __forceinline__ void b_prolong_sweep(const Tile* __restrict__ tiles, const LevelDev* __restrict__ LV,
                                                const InstDev* __restrict__ I, const InstState* __restrict__ S,
                                                int cur, int coarse_alt, int vb) {
    __shared__ T ea[PS_N];
    __shared__ uint8_t bs[PS_N];
    const Tile t = ldg_struct(&tiles[vb]);
    const LevelDev& F = LV[t.lev];
    if (!tile_live(t, F, S)) return;
    const LevelDev& C = LV[F.child];
    const T* ce = (const T*)((coarse_alt && C.child >= 0) ? C.e2 : C.e);
    const T* fe = (const T*)(cur ? F.e2 : F.e);
    T* fo = (T*)(cur ? F.e : F.e2);
    const T* fr = (const T*)F.r;
    const T om = (T)I[t.inst].omega;
    const int P = F.pitch, CP = C.pitch, ib = t.i0 - 1, jb = t.j0 - 1;
    const uint8_t* cbits = C.bits;
    auto fce = [ce, CP](int I0, int J0) { return ce[I0 + J0 * CP]; };
    auto fcb = [cbits, CP](int I0, int J0) { return __ldg(&cbits[I0 + J0 * CP]); };
    // stage the tile and its halo; add the correction on the live cells
    for (int q = threadIdx.x; q < PS_N; q += blockDim.x) {
        const int rj = q / PS_W, ri = q - rj * PS_W, i = ib + ri, j = jb + rj;
        const bool inside = i >= 0 && i < F.nx && j >= 0 && j < F.ny;
        const int id = inside ? i + j * P : 0;
        const uint8_t bt = (inside && i >= 1 && i <= F.NX && j >= 1 && j <= F.NY) ? __ldg(&F.bits[id]) : (uint8_t)0;
        T v = inside ? fe[id] : (T)0;
        if (bt & 0x0F) v = v + prolong_corr<T>(F, i, j, fce, fcb);
        ea[q] = v;
        bs[q] = bt;
    }
    __syncthreads();
    // one sweep of the tile
    const int ri = 1 + (int)(threadIdx.x & 31), rj = 1 + (int)(threadIdx.x >> 5), q = ri + rj * PS_W;
    const int i = ib + ri, j = jb + rj;
    if (bs[q] & 0x0F) {
        const int id = i + j * P;
        T Le, D;
        lap_p<T, T, false>(F, ea, i, j, q, PS_W, bs[q], nullptr, nullptr, Le, D);
        fo[id] = jacobi_update<T>(ea[q], fr[id], Le, D, om);
    }
}

// ------------------------------------------------- small levels (sub-cycle)
//
// The coarse levels of one instance with at most SUB_MAX_CELLS cells are run
// by one block in shared memory.  The restriction into the first of them
// (with its zero-start sweep) is an ordinary tile phase; the block then
// stages, for every small level, e, e2, r and the stencil bytes (compact rows
// of nx cells, ghost ring included), the 1-D metric arrays and the
// prolongation tables, and runs the rest of the V-cycle on them.  The
// per-cell arithmetic is that of b_restrict / b_smooth / b_prolong.

// View of a staged level; the pointers are formed from the dynamic shared
// memory base and the offsets of its SubHdr, so accesses compile to
// shared-memory loads and stores.
template <typename T> struct SubPair;
template <> struct SubPair<float> { using type = float2; };
template <> struct SubPair<double> { using type = double2; };

template <typename T>
struct SubGeo {
    using T2 = typename SubPair<T>::type;
    T *e, *e2, *r, *dw, *pwx, *dh, *pwy;
    T2 *cew, *cns;
    int *pI, *pIn, *pJ, *pJn;
    uint8_t* b;
    signed char *psx, *psy;
    int NX, NY, nx, ny, dirmask, child, depth, cx, cy;
};

template <typename T>
__device__ __forceinline__ SubGeo<T> sub_geo(unsigned char* sm, const SubHdr& h) {
    unsigned char* p = sm + h.base;
    const SubLayout& o = h.o;
    SubGeo<T> g;
    g.e = (T*)(p + o.e); g.e2 = (T*)(p + o.e2); g.r = (T*)(p + o.r);
    g.cew = (typename SubGeo<T>::T2*)(p + o.cew); g.dw = (T*)(p + o.dw); g.pwx = (T*)(p + o.pwx);
    g.cns = (typename SubGeo<T>::T2*)(p + o.cns); g.dh = (T*)(p + o.dh); g.pwy = (T*)(p + o.pwy);
    g.pI = (int*)(p + o.pI); g.pIn = (int*)(p + o.pIn); g.pJ = (int*)(p + o.pJ); g.pJn = (int*)(p + o.pJn);
    g.b = p + o.b;
    g.psx = (signed char*)(p + o.psx); g.psy = (signed char*)(p + o.psy);
    g.NX = h.NX; g.NY = h.NY; g.nx = h.nx; g.ny = h.ny;
    g.dirmask = h.dirmask; g.child = h.child; g.depth = h.depth;
    g.cx = h.cx; g.cy = h.cy;
    return g;
}

// dst[q] = src[row-major q with row pitch `pitch`], q < n, rows of nx; eight
// loads in flight per thread.
template <typename U>
__device__ __forceinline__ void sub_load_rows(U* dst, const U* src, int nx, int n, int pitch) {
    for (int base = threadIdx.x; base < n; base += 8 * blockDim.x) {
        U v[8];
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const int q = base + k * (int)blockDim.x;
            if (q < n) {
                const int j = q / nx;
                v[k] = src[q + j * (pitch - nx)];
            }
        }
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const int q = base + k * (int)blockDim.x;
            if (q < n) dst[q] = v[k];
        }
    }
}

template <typename U>
__device__ __forceinline__ void sub_load_ro(U* dst, const U* src, int n) {
    for (int q = threadIdx.x; q < n; q += blockDim.x) dst[q] = __ldg(&src[q]);
}

template <typename T>
__device__ __forceinline__ LapCoef<T> sub_coef(const SubGeo<T>& g, int i, int j, uint8_t bt) {
    const auto ew = g.cew[i], ns = g.cns[j];
    const T cE = ew.x, cW = ew.y, cN = ns.x, cS = ns.y;
    LapCoef<T> c;
    c.ce = (bt & B_E) ? cE : (T)0;
    c.cw = (bt & B_W) ? cW : (T)0;
    c.cn = (bt & B_N) ? cN : (T)0;
    c.cs = (bt & B_S) ? cS : (T)0;
    T dd = c.ce + c.cw + c.cn + c.cs;
    if (g.dirmask) {
        if (i == g.NX && (g.dirmask & (1 << 1))) dd += (T)2 * cE;
        if (i == 1 && (g.dirmask & (1 << 0))) dd += (T)2 * cW;
        if (j == g.NY && (g.dirmask & (1 << 3))) dd += (T)2 * cN;
        if (j == 1 && (g.dirmask & (1 << 2))) dd += (T)2 * cS;
    }
    c.dd = dd;
    return c;
}

template <typename T>
__device__ __forceinline__ T sub_lap(const SubGeo<T>& g, const T* e, int i, int j, int id, uint8_t bt, T& D) {
    const LapCoef<T> c = sub_coef<T>(g, i, j, bt);
    const int P = g.nx;
    D = c.dd;
    return c.ce * e[id + 1] + c.cw * e[id - 1] + c.cn * e[id + P] + c.cs * e[id - P] - c.dd * e[id];
}

// Loops over the interior cells of a staged level: warps take rows, lanes
// take columns (no integer division per cell).
#define SUB_FOR_CELLS(g, i, j)                                                                   \
    for (int j = 1 + (int)(threadIdx.x >> 5); j <= (g).NY; j += (int)(blockDim.x >> 5))          \
        for (int i = 1 + (int)(threadIdx.x & 31); i <= (g).NX; i += 32)

// Weighted-Jacobi sweep of a staged level (src -> dst by parity).
template <typename T>
__device__ __forceinline__ void sub_smooth(const SubGeo<T>& g, int src_alt, T om) {
    const T* src = src_alt ? g.e2 : g.e;
    T* dst = src_alt ? g.e : g.e2;
    const int nx = g.nx;
    SUB_FOR_CELLS(g, i, j) {
        const int id = i + j * nx;
        const uint8_t bt = g.b[id];
        if (!(bt & 0x0F)) continue;
        T D;
        const T Le = sub_lap<T>(g, src, i, j, id, bt, D);
        dst[id] = jacobi_update<T>(src[id], g.r[id], Le, D, om);
    }
}

// Area-weighted restriction of the fine residual r - L e (buffer fine_alt of
// staged level f) onto staged level c; a middle level also takes its first
// sweep from zero (e = -om r / D).
template <typename T>
__device__ __forceinline__ void sub_restrict(const SubGeo<T>& c, const SubGeo<T>& f, int fine_alt, T om) {
    const T* fe = fine_alt ? f.e2 : f.e;
    SUB_FOR_CELLS(c, I0, J0) {
        const int cid = I0 + J0 * c.nx;
        const uint8_t cb = c.b[cid];
        if (!(cb & 0x0F)) {
            c.r[cid] = (T)0;
            continue;
        }
        T rowsum[2] = {(T)0, (T)0};  // (t00 + t10) + (t01 + t11), as the tile phase
#pragma unroll
        for (int dj = 0; dj < 2; dj++)
#pragma unroll
            for (int di = 0; di < 2; di++) {
                const int i = c.cx * (I0 - 1) + 1 + di, j = c.cy * (J0 - 1) + 1 + dj;
                if (di >= c.cx || dj >= c.cy || i > f.NX || j > f.NY) continue;
                const int id = i + j * f.nx;
                const uint8_t bt = f.b[id];
                if (!(bt & 0x0F)) continue;
                T D;
                const T Le = sub_lap<T>(f, fe, i, j, id, bt, D);
                const T term = (f.r[id] - Le) * (f.dw[i] * f.dh[j]);
                rowsum[dj] = di == 0 ? term : rowsum[dj] + term;
            }
        const T acc = c.cy == 2 ? rowsum[0] + rowsum[1] : rowsum[0];
        const T rv = acc / (c.dw[I0] * c.dh[J0]);
        c.r[cid] = rv;
        if (c.child >= 0) c.e[cid] = jacobi_from_zero<T>(rv, sub_coef<T>(c, I0, J0, cb).dd, om);
    }
}

// Bilinear prolongation of staged level c's correction onto staged level f.
template <typename T>
__device__ __forceinline__ void sub_prolong(const SubGeo<T>& f, const SubGeo<T>& c, int fine_alt, int coarse_alt) {
    const T* ce = (coarse_alt && c.child >= 0) ? c.e2 : c.e;
    T* fe = fine_alt ? f.e2 : f.e;
    const int nx = f.nx, CP = c.nx;
    SUB_FOR_CELLS(f, i, j) {
        const int id = i + j * nx;
        if (!(f.b[id] & 0x0F)) continue;
        const int I0 = f.pI[i], In = f.pIn[i], J0 = f.pJ[j], Jn = f.pJn[j];
        const T wx = f.pwx[i], wy = f.pwy[j];
        const T sx = (T)f.psx[i], sy = (T)f.psy[j];
        T w00 = ((T)1 - wx) * ((T)1 - wy), w10 = wx * ((T)1 - wy), w01 = ((T)1 - wx) * wy, w11 = wx * wy;
        const int c00 = I0 + J0 * CP, c10 = In + J0 * CP, c01 = I0 + Jn * CP, c11 = In + Jn * CP;
        w00 = (c.b[c00] & 0x0F) ? w00 : (T)0;
        w10 = (c.b[c10] & 0x0F) ? w10 : (T)0;
        w01 = (c.b[c01] & 0x0F) ? w01 : (T)0;
        w11 = (c.b[c11] & 0x0F) ? w11 : (T)0;
        const T sw = w00 + w10 + w01 + w11;
        const T val = (w00 * ce[c00] + sx * w10 * ce[c10] + sy * w01 * ce[c01] + (sx * sy) * w11 * ce[c11]) / sw;
        fe[id] += val;
    }
}

// Synchronises the first n threads of the block (n a multiple of 32).
__device__ __forceinline__ void sub_sync(int n) {
    if (n == 32) __syncwarp();
    else if (n == (int)blockDim.x) __syncthreads();
    else asm volatile("bar.sync 1, %0;" ::"r"(n) : "memory");
}

// Coarsest level: e = 0, then red-black SOR sweeps.  Each thread keeps the
// operator of its cells (at most SUB_COARSE_PER_THREAD) in registers; only
// the warps that own cells take part.
template <typename T>
__device__ __forceinline__ void sub_coarse_solve(const SubGeo<T>& g, int sweeps) {
    const T om = (T)COARSE_OMEGA;
    const int NX = g.NX, nx = g.nx, NXY = g.NX * g.NY;
    const int nthr = min((int)blockDim.x, (NXY + 31) & ~31);
    for (int q = threadIdx.x; q < nx * g.ny; q += blockDim.x) g.e[q] = (T)0;
    __syncthreads();
    if (NXY <= 32) {
        // one warp, one cell per lane: neighbours by shuffle (cells beyond the
        // interior hold e = 0, like the ghost ring)
        if (threadIdx.x < 32) {
            const int lane = threadIdx.x;
            const bool own = lane < NXY;
            const int j = 1 + (own ? lane / NX : 0), i = 1 + (own ? lane - (j - 1) * NX : 0);
            const int c = i + j * nx;
            const uint8_t bt = own ? g.b[c] : (uint8_t)0;
            const bool live = bt & 0x0F;
            const LapCoef<T> lc = sub_coef<T>(g, i, j, bt);
            const T rd = live ? rcpa(lc.dd) : (T)0, rr = own ? g.r[c] : (T)0;
            const int col = (i + j) & 1;
            const bool hasE = i < NX, hasW = i > 1, hasN = j < g.NY, hasS = j > 1;
            T e = (T)0;
            for (int it = 0; it < sweeps; it++) {
#pragma unroll
                for (int cc = 0; cc < 2; cc++) {
                    const T vE = __shfl_down_sync(0xffffffffu, e, 1), vW = __shfl_up_sync(0xffffffffu, e, 1);
                    const T vN = __shfl_sync(0xffffffffu, e, min(lane + NX, 31));
                    const T vS = __shfl_sync(0xffffffffu, e, max(lane - NX, 0));
                    const T eE = hasE ? vE : (T)0, eW = hasW ? vW : (T)0;
                    const T eN = hasN ? vN : (T)0, eS = hasS ? vS : (T)0;
                    const T Le = lc.ce * eE + lc.cw * eW + lc.cn * eN + lc.cs * eS - lc.dd * e;
                    if (live && col == cc) e = e + om * (Le - rr) * rd;
                }
            }
            if (live) g.e[c] = e;
        }
        __syncthreads();
        return;
    }
    if ((int)threadIdx.x < nthr) {
        int id[SUB_COARSE_PER_THREAD], col[SUB_COARSE_PER_THREAD];
        T ce[SUB_COARSE_PER_THREAD], cw[SUB_COARSE_PER_THREAD], cn[SUB_COARSE_PER_THREAD],
            cs[SUB_COARSE_PER_THREAD], dd[SUB_COARSE_PER_THREAD], rd[SUB_COARSE_PER_THREAD],
            rr[SUB_COARSE_PER_THREAD];
#pragma unroll
        for (int k = 0; k < SUB_COARSE_PER_THREAD; k++) {
            const int q = threadIdx.x + k * nthr;
            id[k] = -1;
            col[k] = 2;
            ce[k] = cw[k] = cn[k] = cs[k] = dd[k] = rd[k] = rr[k] = (T)0;
            if (q < NXY) {
                const int j = 1 + q / NX, i = 1 + q - (j - 1) * NX, c = i + j * nx;
                const uint8_t bt = g.b[c];
                if (bt & 0x0F) {
                    const LapCoef<T> lc = sub_coef<T>(g, i, j, bt);
                    id[k] = c;
                    col[k] = (i + j) & 1;
                    ce[k] = lc.ce; cw[k] = lc.cw; cn[k] = lc.cn; cs[k] = lc.cs; dd[k] = lc.dd;
                    rd[k] = rcpa(lc.dd);
                    rr[k] = g.r[c];
                }
            }
        }
        T* e = g.e;
        for (int it = 0; it < sweeps; it++) {
#pragma unroll
            for (int cc = 0; cc < 2; cc++) {
#pragma unroll
                for (int k = 0; k < SUB_COARSE_PER_THREAD; k++) {
                    if (col[k] != cc) continue;
                    const int c = id[k];
                    const T ec = e[c];
                    const T Le = ce[k] * e[c + 1] + cw[k] * e[c - 1] + cn[k] * e[c + nx] + cs[k] * e[c - nx] - dd[k] * ec;
                    e[c] = ec + om * (Le - rr[k]) * rd[k];
                }
                sub_sync(nthr);
            }
        }
    }
    __syncthreads();
}

// Stages the geometry of instance k's small levels (headers, metric arrays,
// prolongation tables, stencil bytes, zero fields) in the block's dynamic
// shared memory: one contiguous copy of the instance's image, 16 B per load,
// four loads in flight per thread.
template <typename T>
__device__ __forceinline__ void sub_stage_geometry(const int* __restrict__ sub, const LevelDev* __restrict__ LV,
                                                   const InstDev* __restrict__ I, int k, unsigned char* sm) {
    (void)sub;
    (void)LV;
    const uint4* src = (const uint4*)I[k].sub_img;
    uint4* dst = (uint4*)sm;
    const int n16 = I[k].sub_img_bytes >> 4, nt = (int)blockDim.x;
    for (int q0 = threadIdx.x; q0 < n16; q0 += 4 * nt) {
        uint4 v[4];
#pragma unroll
        for (int u = 0; u < 4; u++)
            if (q0 + u * nt < n16) v[u] = __ldg(&src[q0 + u * nt]);
#pragma unroll
        for (int u = 0; u < 4; u++)
            if (q0 + u * nt < n16) dst[q0 + u * nt] = v[u];
    }
    __syncthreads();
}

// Asynchronous global -> shared copies (cp.async) of 4, 8 or 16 bytes, and
// the wait for all of this thread's.
template <int N>
__device__ __forceinline__ void cp_async(unsigned dst, const void* src) {
    static_assert(N == 4 || N == 8 || N == 16, "cp.async size");
    if constexpr (N == 16) asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(src) : "memory");
    else if constexpr (N == 8) asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(dst), "l"(src) : "memory");
    else asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Stages instance `in`'s small levels for one V-cycle in one round of
// asynchronous copies: the image (headers, geometry, zero fields) except the
// first level's e and r, which come from that level's global buffers (e: the
// zero-start sweep of the tile phase; when the first level is the coarsest,
// the image's zero e is kept).  The same shared-memory contents as staging
// the image and then loading e and r, without the round trip in between.
template <typename T>
__device__ __forceinline__ void sub_stage_all(const InstDev& in, unsigned char* sm) {
    const unsigned char* img = in.sub_img;
    const T* ge = (const T*)in.sub_ge;
    const T* gr = (const T*)in.sub_gr;
    const int n16 = in.sub_img_bytes >> 4, nx = in.sub_nx, n = nx * in.sub_ny, gp = in.sub_gpitch;
    const int oe = in.sub_oe, orr = in.sub_or, span = (int)sub_al16((size_t)n * sizeof(T));
    const bool load_e = in.sub_child >= 0;
    const unsigned sb = (unsigned)__cvta_generic_to_shared(sm);
    for (int q = threadIdx.x; q < n16; q += blockDim.x) {
        const int b = q << 4;
        if ((load_e && b >= oe && b < oe + span) || (b >= orr && b < orr + span)) continue;
        cp_async<16>(sb + b, img + b);
    }
    // The first level's e and r are the output of the phase before (the
    // restriction into it): a programmatic launch of this kernel starts while
    // that phase runs and waits here, after the geometry copies are issued.
    pdl_wait();
    for (int q = threadIdx.x; q < n; q += blockDim.x) {
        const int g = q + (q / nx) * (gp - nx);
        if (load_e) cp_async<(int)sizeof(T)>(sb + oe + q * (int)sizeof(T), ge + g);
        cp_async<(int)sizeof(T)>(sb + orr + q * (int)sizeof(T), gr + g);
    }
    cp_async_wait_all();
    __syncthreads();
}

// Small coarse levels of one instance (vb = instance) in one block, from the
// first small level (restricted by the tile phase before) down to the RB-SOR
// solve and back up; the first small level's correction is written back to
// its global buffer for the prolongation above it.  sm: dynamic shared
// memory of at least the instance's staged bytes; geometry_staged: the block
// staged this instance's geometry there before (persistent kernel).
template <typename T>
__device__ __forceinline__ void b_subcycle(const int* __restrict__ sub, const LevelDev* __restrict__ LV,
                                           const InstDev* __restrict__ I, const InstState* __restrict__ S,
                                           int pre, int post, unsigned char* sm, bool geometry_staged, int vb) {
    (void)sub;
    (void)LV;
    const int k = vb;
    if (S[k].ppe_state != ST_ACTIVE) return;
    const InstDev& in = I[k];
    const SubHdr* hdr = (const SubHdr*)sm;
    if (!geometry_staged) {
        sub_stage_all<T>(in, sm);
    } else {
        // geometry resident from an earlier V-cycle: the first level's e and
        // r from global memory, every other field zeroed
        const SubGeo<T> g = sub_geo<T>(sm, hdr[0]);
        const int n = g.nx * g.ny;
        if (g.child >= 0) sub_load_rows<T>(g.e, (const T*)in.sub_ge, g.nx, n, in.sub_gpitch);  // zero-start sweep of the tile phase
        else
            for (int q = threadIdx.x; q < n; q += blockDim.x) g.e[q] = (T)0;
        sub_load_rows<T>(g.r, (const T*)in.sub_gr, g.nx, n, in.sub_gpitch);
        for (int q = threadIdx.x; q < n; q += blockDim.x) g.e2[q] = (T)0;
        for (int s = 1; s < hdr[0].ns; s++) {
            const SubGeo<T> c = sub_geo<T>(sm, hdr[s]);
            const int m = c.nx * c.ny;
            for (int q = threadIdx.x; q < m; q += blockDim.x) {
                c.e[q] = (T)0;
                c.e2[q] = (T)0;
            }
        }
        __syncthreads();
    }
    const int ns = hdr[0].ns;
    const T om = (T)in.omega;
    // descend
    for (int s = 0; s < ns; s++) {
        const SubGeo<T> g = sub_geo<T>(sm, hdr[s]);
        if (s > 0) {
            const SubGeo<T> f = sub_geo<T>(sm, hdr[s - 1]);
            sub_restrict<T>(g, f, parity_after_pre(f.depth, pre), om);
            __syncthreads();
        }
        if (g.child < 0) {
            sub_coarse_solve<T>(g, in.coarse_sweeps);
            break;
        }
        int cur = 0;
        for (int q = 1; q < pre; q++) {
            sub_smooth<T>(g, cur, om);
            __syncthreads();
            cur ^= 1;
        }
    }
    // ascend
    for (int s = ns - 2; s >= 0; s--) {
        const SubGeo<T> f = sub_geo<T>(sm, hdr[s]);
        const SubGeo<T> c = sub_geo<T>(sm, hdr[s + 1]);
        int cur = parity_after_pre(f.depth, pre);
        sub_prolong<T>(f, c, cur, parity_after_post(f.depth + 1, pre, post));
        __syncthreads();
        for (int q = 0; q < post; q++) {
            sub_smooth<T>(f, cur, om);
            __syncthreads();
            cur ^= 1;
        }
    }
    // write back the first small level's correction (the buffer its last sweep ended on)
    const SubGeo<T> g = sub_geo<T>(sm, hdr[0]);
    const int res = (g.child < 0) ? 0 : parity_after_post(g.depth, pre, post);
    const T* src = res ? g.e2 : g.e;
    T* dst = (T*)(res ? in.sub_ge2 : in.sub_ge);
    const int n = g.nx * g.ny, gp = in.sub_gpitch;
    for (int q = threadIdx.x; q < n; q += blockDim.x) {
        const int j = q / g.nx;
        dst[q + j * (gp - g.nx)] = src[q];
    }
    __syncthreads();  // the block may stage another instance in the same memory
}

// ------------------------------------------------------------ projection

__device__ __forceinline__ void b_p_finalize(const Tile* __restrict__ tiles, const InstDev* __restrict__ I,
                             const InstState* __restrict__ S, int vb) {
    const Tile t = ldg_struct(&tiles[vb]);
    const InstDev& in = I[t.inst];
    if (in.retired) return;
    if (!in.singular) return;
    int i, j;
    tile_ij(t, i, j);
    if (i < 1 || i > in.NX || j < 1 || j > in.NY) return;
    const int id = i + j * in.pitch;
    const uint8_t ty = __ldg(&in.type[id]);
    if (ty == T_FLUID || ty == T_GHOST) in.p[id] -= S[t.inst].pmean;
}

__device__ __forceinline__ double corr_u(const InstDev& in, int i, int id) {
    const bool act = __ldg(&in.type[id]) == T_FLUID || __ldg(&in.type[id + 1]) == T_FLUID;
    if (!act) return in.Us[id];
    if (i == 0 && !(in.dirmask & 1)) return in.Us[id];
    if (i == in.nx - 2 && !(in.dirmask & 2)) return in.Us[id];
    return in.Us[id] - in.dt * __ldg(&in.kx[i]) * (in.p[id + 1] - in.p[id]);
}
__device__ __forceinline__ double corr_v(const InstDev& in, int j, int id) {
    const int P = in.pitch;
    const bool act = __ldg(&in.type[id]) == T_FLUID || __ldg(&in.type[id + P]) == T_FLUID;
    if (!act) return in.Vs[id];
    if (j == 0 && !(in.dirmask & 4)) return in.Vs[id];
    if (j == in.ny - 2 && !(in.dirmask & 8)) return in.Vs[id];
    return in.Vs[id] - in.dt * __ldg(&in.ky[j]) * (in.p[id + P] - in.p[id]);
}

// Largest |d| of a block (thread 0), with NaN counted as 0 like fmax: the
// absolute values are compared as 64-bit integers, which order non-negative
// doubles as their values do, with no FP64 operation.
__device__ __forceinline__ double block_max_abs(double d) {
    __shared__ unsigned long long sh[32];
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    unsigned long long v = (unsigned long long)__double_as_longlong(d) & 0x7FFFFFFFFFFFFFFFull;
    if (v > 0x7FF0000000000000ull) v = 0ull;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long x = __shfl_xor_sync(0xffffffffu, v, o);
        v = x > v ? x : v;
    }
    if (l == 0) sh[w] = v;
    __syncthreads();
    unsigned long long m = 0ull;
    if (threadIdx.x == 0)
        for (int q = 0; q < nw; q++) m = sh[q] > m ? sh[q] : m;
    __syncthreads();
    return __longlong_as_double((long long)m);
}

// Projection of cell and face velocities; divergence and boundary fluxes.
// Every face value is formed once: thread (w, lane) forms the east face U
// and the north face V of its cell and the interpolated pressures there;
// warp 0 forms the south faces of the tile's first row, warp 1 the west faces
// of its first column; the cells take their west and south values from
// shared memory.  The operands and operations of each value are those of the
// cell-by-cell form, so the results are the same.
__device__ __forceinline__ void b_correct(const Tile* __restrict__ tiles, const InstDev* __restrict__ I,
                          double* __restrict__ part, int vb) {
    const Tile t = ldg_struct(&tiles[vb]);
    const InstDev& in = I[t.inst];
    if (in.retired) return;
    TileFaces& F = tile_faces();
    auto& sU = F.x[0];   // U and the interpolated pressure on the x faces
    auto& sPe = F.x[1];
    auto& sV = F.y[0];   // V and the interpolated pressure on the y faces
    auto& sPn = F.y[1];
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    int i, j;
    tile_ij(t, i, j);
    const int P = in.pitch, id = i + j * P, NX = in.NX, NY = in.NY;
    const double* p = in.p;
    const bool row = j >= 1 && j <= NY, col = i >= 1 && i <= NX;
    double fl[2] = {0.0, 0.0};
    {
        double Un = 0.0, pe = 0.0;
        if (row && i <= NX) {
            Un = corr_u(in, i, id);
            in.U[id] = Un;
            if (i == 0) fl[0] += Un * __ldg(&in.dy[j]);
            if (i == NX) fl[1] += Un * __ldg(&in.dy[j]);
            pe = p[id] * __ldg(&in.gx[i]) + p[id + 1] * __ldg(&in.fx[i]);
        }
        sU[w][l + 1] = Un;
        sPe[w][l + 1] = pe;
    }
    {
        double Vn = 0.0, pn = 0.0;
        if (col && j <= NY) {
            Vn = corr_v(in, j, id);
            in.V[id] = Vn;
            if (j == 0) fl[0] += Vn * __ldg(&in.dx[i]);
            if (j == NY) fl[1] += Vn * __ldg(&in.dx[i]);
            pn = p[id] * __ldg(&in.gy[j]) + p[id + P] * __ldg(&in.fy[j]);
        }
        sV[w + 1][l] = Vn;
        sPn[w + 1][l] = pn;
    }
    if (w == 0) {  // south faces of the first row
        const int js = t.j0 - 1, ids = i + js * P;
        double Vs = 0.0, ps = 0.0;
        if (js >= 0 && col) {
            Vs = corr_v(in, js, ids);
            ps = p[ids] * __ldg(&in.gy[js]) + p[ids + P] * __ldg(&in.fy[js]);
        }
        sV[0][l] = Vs;
        sPn[0][l] = ps;
    } else if (w == 1 && l < TILE_Y) {  // west faces of the first column
        const int iw = t.i0 - 1, jw = t.j0 + l, idw = iw + jw * P;
        double Uw = 0.0, pw = 0.0;
        if (iw >= 0 && jw >= 1 && jw <= NY) {
            Uw = corr_u(in, iw, idw);
            pw = p[idw] * __ldg(&in.gx[iw]) + p[idw + 1] * __ldg(&in.fx[iw]);
        }
        sU[l][0] = Uw;
        sPe[l][0] = pw;
    }
    __syncthreads();
    double d = 0.0;
    if (row && col) {
        if (__ldg(&in.type[id]) == T_FLUID) {
            const double ixi = __ldg(&in.ix[i]), iyj = __ldg(&in.iy[j]);
            in.u[id] -= in.dt * (sPe[w][l + 1] - sPe[w][l]) * ixi;
            in.v[id] -= in.dt * (sPn[w + 1][l] - sPn[w][l]) * iyj;
            d = (sU[w][l + 1] - sU[w][l]) * ixi + (sV[w + 1][l] - sV[w][l]) * iyj;
            in.div[id] = d;
        } else {
            in.div[id] = 0.0;
        }
    }
    const double m = block_max_abs(d);
    // boundary mass fluxes: tiles that hold a boundary face only
    const bool edge = t.i0 == 0 || t.i0 + TILE_X > NX || t.j0 == 0 || t.j0 + TILE_Y > NY;
    __shared__ double out[2];
    if (edge) block_sum<2>(fl, out);
    if (threadIdx.x == 0) {
        part[(size_t)vb * NPART] = m;
        part[(size_t)vb * NPART + 1] = edge ? out[0] : 0.0;
        part[(size_t)vb * NPART + 2] = edge ? out[1] : 0.0;
    }
}

__device__ __forceinline__ void b_correct_reduce(const InstDev* __restrict__ I, InstState* __restrict__ S,
                                 const double* __restrict__ part, int vb) {
    const int k = vb;
    const InstDev& in = I[k];
    if (in.retired) return;
    double m = 0.0, a[2] = {0.0, 0.0};
    for (int t = threadIdx.x; t < in.tile_cnt; t += blockDim.x) {
        const double* q = part + (size_t)(in.tile_beg + t) * NPART;
        m = fmax(m, q[0]);
        a[0] += q[1];
        a[1] += q[2];
    }
    const double mm = block_max(m);
    __shared__ double out[2];
    block_sum<2>(a, out);
    if (threadIdx.x == 0) {
        S[k].max_div = mm;
        S[k].flux_in = out[0];
        S[k].flux_out = out[1];
        S[k].have_nold = 1;
    }
}

// ---------------------------------------------------------------- forces

__device__ __forceinline__ int locate(const double* c, int n, double x) {
    // last index in [1, n-2] with c[idx] <= x, minus nothing; 0 when x < c[1]; clamp to [0, n-2]
    int lo = 1, hi = n - 1;  // search [1, n-1)
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (c[mid] <= x) lo = mid + 1;
        else hi = mid;
    }
    int i0 = lo - 1;
    if (i0 < 0) i0 = 0;
    if (i0 > n - 2) i0 = n - 2;
    return i0;
}

__device__ __forceinline__ double sample(const InstDev& in, const double* q, double x, double y) {
    const int i0 = locate(in.xc, in.nx, x), j0 = locate(in.yc, in.ny, y);
    const double xi = (x - __ldg(&in.xc[i0])) / (__ldg(&in.xc[i0 + 1]) - __ldg(&in.xc[i0]));
    const double et = (y - __ldg(&in.yc[j0])) / (__ldg(&in.yc[j0 + 1]) - __ldg(&in.yc[j0]));
    const int P = in.pitch, id = i0 + j0 * P;
    return (1 - xi) * (1 - et) * q[id] + xi * (1 - et) * q[id + 1] + (1 - xi) * et * q[id + P] +
           xi * et * q[id + P + 1];
}

// Drag and lift from body-surface samples: pressure by bilinear sampling of
// the ghost-filled field, wall shear from a probe 1.5 cells along the normal
// (sample geometry precomputed once; the body does not move).
__device__ __forceinline__ double bil(const double* q, int c, int P, double xi, double et) {
    return (1 - xi) * (1 - et) * q[c] + xi * (1 - et) * q[c + 1] + (1 - xi) * et * q[c + P] + xi * et * q[c + P + 1];
}

// vb = instance * FORCE_BLOCKS + b: block b sums its share of the samples
// into fpart; the last of the instance's blocks to finish (ticket ftick)
// sums the FORCE_BLOCKS partials in block order and writes the forces and the
// time-history record.
__device__ __forceinline__ void b_forces(const InstDev* __restrict__ I, InstState* __restrict__ S,
                                         double* __restrict__ fpart, unsigned* __restrict__ ftick, int vb) {
    const int k = vb / FORCE_BLOCKS, fb = vb - k * FORCE_BLOCKS;
    const InstDev& in = I[k];
    if (in.retired) return;
    constexpr int per = FORCE_SAMPLES / FORCE_BLOCKS;
    if (in.body) {
        const double mu = 1.0 / in.re;
        const int P = in.pitch;
        double F[2] = {0.0, 0.0};
        for (int q = fb * per + threadIdx.x; q < (fb + 1) * per; q += blockDim.x) {
            const ForceSample f = ldg_struct(&in.fs[q]);
            const double ps = bil(in.p, f.c0, P, f.xi0, f.et0);
            double up = bil(in.u, f.c1, P, f.xi1, f.et1);
            double vp = bil(in.v, f.c1, P, f.xi1, f.et1);
            if (in.moving) {
                // velocity relative to the wall at the sample point
                const double* b = in.fsb + 5 * (size_t)q;
                const double rx = b[0] * in.bcs - b[1] * in.bsn, ry = b[0] * in.bsn + b[1] * in.bcs;
                up = up - (in.bu - in.bw * ry);
                vp = vp - (in.bv + in.bw * rx);
            }
            F[0] += (-ps * f.nx + mu * up / f.del) * f.ds;
            F[1] += (-ps * f.ny + mu * vp / f.del) * f.ds;
        }
        __shared__ double out[2];
        block_sum<2>(F, out);
        if (threadIdx.x == 0) {
            fpart[2 * (size_t)vb] = out[0];
            fpart[2 * (size_t)vb + 1] = out[1];
        }
    }
    __shared__ bool last;
    if (threadIdx.x == 0) {
        __threadfence();
        last = atomicAdd(&ftick[k], 1u) == FORCE_BLOCKS - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double cd = 0.0, cl = 0.0;  // valid in thread 0
    if (threadIdx.x == 0) {
        if (in.body) {
            double fx = 0.0, fy = 0.0;
            const volatile double* fp = fpart + 2 * (size_t)k * FORCE_BLOCKS;
            for (int b = 0; b < FORCE_BLOCKS; b++) {
                fx += fp[2 * b];
                fy += fp[2 * b + 1];
            }
            cd = fx / in.fref;
            cl = fy / in.fref;
        }
        S[k].cd = cd;
        S[k].cl = cl;
        ftick[k] = 0u;
    }
    // time-history record of this step: step count, forces, probe values
    if (in.hist_cap > 0) {
        const long long hn = S[k].hist_n;
        double* rec = in.hist + (size_t)(hn % in.hist_cap) * in.hist_w;
        if (threadIdx.x == 0) {
            rec[0] = (double)S[k].nstep;
            rec[1] = cd;
            rec[2] = cl;
        }
        for (int q = threadIdx.x; q < in.nprobe; q += blockDim.x) {
            const int c = in.probe_cell[q];
            rec[3 + 3 * q] = in.u[c];
            rec[4 + 3 * q] = in.v[c];
            rec[5 + 3 * q] = in.p[c];
        }
        __syncthreads();
        if (threadIdx.x == 0) S[k].hist_n = hn + 1;
    }
}

}  // namespace ifx
