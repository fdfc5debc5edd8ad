// kernels_cluster.cu -- the pressure preconditioner's V-cycle on one
// thread-block cluster per instance (graph and host-loop execution).
//
// A cluster of CMG_CTAS CTAs x CMG_THREADS threads holds every multigrid level
// above the instance's sub-cycle in distributed shared memory: each CTA owns
// a block of rows of each level (e, e2, r, stencil bytes), and a table of row
// pointers per level (generic addresses of the owning CTA's rows, obtained
// with cluster.map_shared_rank) gives every CTA direct loads of rows owned by
// the others, so neighbour rows need no exchange.  Phases are separated by
// hardware cluster barriers instead of grid-wide ones.  The restriction into
// the first small level writes it to global memory, CTA 0 runs the sub-cycle
// there (b_subcycle, all CMG_THREADS threads), and the prolongation reads the
// result back.  Per-cell arithmetic is that of the tile phases (lap_vals,
// jacobi_update, the (t00 + t10) + (t01 + t11) restriction order,
// prolong_corr), so the result equals the tile path's bit for bit.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <mutex>

#include "method_body.cuh"

namespace cg = cooperative_groups;

namespace ifx {
namespace {

template <typename T>
struct CView {
    T** pe;   // row pointer tables (whole level, ring rows -> a zero row)
    T** pe2;
    T** pr;
    uint8_t** pb;
    T* e;     // this CTA's rows
    T* e2;
    T* r;
    uint8_t* b;
    int r0, r1;  // own level rows [r0, r1] (1-based), empty when r1 < r0
};

template <typename T>
__device__ __forceinline__ CView<T> cview(unsigned char* sm, const CmgLevel& c, int rank, int NY) {
    CView<T> v;
    v.pe = (T**)(sm + c.pe);
    v.pe2 = (T**)(sm + c.pe2);
    v.pr = (T**)(sm + c.pr);
    v.pb = (uint8_t**)(sm + c.pb);
    v.e = (T*)(sm + c.e);
    v.e2 = (T*)(sm + c.e2);
    v.r = (T*)(sm + c.r);
    v.b = sm + c.b;
    v.r0 = 1 + rank * c.m;
    v.r1 = min(NY, (rank + 1) * c.m);
    return v;
}

// f(i, j, local row) over this CTA's interior cells: warps take (row, 32-column
// chunk) items.
template <typename F>
__device__ __forceinline__ void for_own(int NX, int r0, int r1, F f) {
    const int nrows = r1 - r0 + 1;
    if (nrows <= 0) return;
    const int lane = (int)(threadIdx.x & 31), warp = (int)(threadIdx.x >> 5), nw = (int)(blockDim.x >> 5);
    const int nch = (NX + 31) >> 5, items = nrows * nch;
    for (int it = warp; it < items; it += nw) {
        const int rr = it / nch, ch = it - rr * nch;
        const int i = 1 + ch * 32 + lane;
        if (i <= NX) f(i, r0 + rr, rr);
    }
}

// Weighted-Jacobi sweep of a distributed level (src buffer by parity).
template <typename T, bool L0>
__device__ __forceinline__ void c_sweep(const LevelDev& L, const CView<T>& v, int src_alt, bool zero, T om,
                                        const GhostDev* G, const int* gidx) {
    T** ps = src_alt ? v.pe2 : v.pe;
    T* dst = src_alt ? v.e : v.e2;
    const int P = L.pitch, nx = L.nx;
    for_own(L.NX, v.r0, v.r1, [&](int i, int j, int rr) {
        const int lid = rr * nx + i;
        const uint8_t bt = v.b[lid];
        if (!(bt & 0x0F)) return;
        const T* rc = ps[j];
        const T* rn = ps[j + 1];
        const T* rs = ps[j - 1];
        T Le, D;
        lap_vals<T, L0>(L, i, j, i + j * P, P, bt, G, gidx, rc[i + 1], rc[i - 1], rn[i], rs[i], rc[i],
                        [ps, P](int q) {
                            const int jj = q / P;
                            return ps[jj][q - jj * P];
                        },
                        Le, D);
        dst[lid] = zero ? jacobi_from_zero<T>(v.r[lid], D, om) : jacobi_update<T>(rc[i], v.r[lid], Le, D, om);
    });
}

// Restriction of the residual of distributed fine level F (buffer fine_alt)
// onto coarse cell (I0, J0); returns false for a dead coarse cell.
template <typename T, bool F0>
__device__ __forceinline__ T c_restrict_cell(const LevelDev& F, const CView<T>& vf, int fine_alt, const LevelDev& C,
                                             int I0, int J0, const GhostDev* G, const int* gidx) {
    T** pf = fine_alt ? vf.pe2 : vf.pe;
    const int FP = F.pitch, cx = C.cx, cy = C.cy;
    T rows[2] = {(T)0, (T)0};
#pragma unroll
    for (int dj = 0; dj < 2; dj++)
#pragma unroll
        for (int di = 0; di < 2; di++) {
            if (di >= cx || dj >= cy) continue;
            const int i = cx * (I0 - 1) + 1 + di, j = cy * (J0 - 1) + 1 + dj;
            T term = (T)0;
            if (i <= F.NX && j <= F.NY) {
                const uint8_t fb = vf.pb[j][i];
                if (fb & 0x0F) {
                    const T* rc = pf[j];
                    const T* rn = pf[j + 1];
                    const T* rs = pf[j - 1];
                    T Le, D;
                    lap_vals<T, F0>(F, i, j, i + j * FP, FP, fb, G, gidx, rc[i + 1], rc[i - 1], rn[i], rs[i], rc[i],
                                    [pf, FP](int q) {
                                        const int jj = q / FP;
                                        return pf[jj][q - jj * FP];
                                    },
                                    Le, D);
                    term = (vf.pr[j][i] - Le) * (__ldg(&LvA<T>::dw(F)[i]) * __ldg(&LvA<T>::dh(F)[j]));
                }
            }
            rows[dj] = di == 0 ? term : rows[dj] + term;
        }
    return cy == 2 ? rows[0] + rows[1] : rows[0];
}

template <typename T, bool F0>
__device__ __forceinline__ void c_restrict(const LevelDev& F, const CView<T>& vf, int fine_alt, const LevelDev& C,
                                           const CView<T>* vc, T om, const GhostDev* G, const int* gidx, int rank) {
    auto store = [&](int I0, int J0, T* rc, T* ec, uint8_t cb) {
        if (!(cb & 0x0F)) {
            *rc = (T)0;
            return;
        }
        const T acc = c_restrict_cell<T, F0>(F, vf, fine_alt, C, I0, J0, G, gidx);
        const T rv = acc / (__ldg(&LvA<T>::dw(C)[I0]) * __ldg(&LvA<T>::dh(C)[J0]));
        *rc = rv;
        if (C.child >= 0) *ec = jacobi_from_zero<T>(rv, lap_diag<T>(C, I0, J0, cb), om);
    };
    if (vc) {
        const int nx = C.nx;
        for_own(C.NX, vc->r0, vc->r1, [&](int I0, int J0, int rr) {
            const int lid = rr * nx + I0;
            store(I0, J0, &vc->r[lid], &vc->e[lid], vc->b[lid]);
        });
    } else {  // the first small level, in global memory: cells spread over the cluster
        T* rc = (T*)C.r;
        T* ec = (T*)C.e;
        const int n = C.NX * C.NY, stride = CMG_CTAS * (int)blockDim.x;
        for (int q = rank * (int)blockDim.x + (int)threadIdx.x; q < n; q += stride) {
            const int J0 = 1 + q / C.NX, I0 = 1 + q - (J0 - 1) * C.NX, cid = I0 + J0 * C.pitch;
            store(I0, J0, &rc[cid], &ec[cid], __ldg(&C.bits[cid]));
        }
    }
}

// Prolongation into distributed fine level F (buffer fine_alt) from a
// distributed coarse level (vc, buffer coarse_buf) or from global memory.
template <typename T>
__device__ __forceinline__ void c_prolong(const LevelDev& F, const CView<T>& vf, int fine_alt, const LevelDev& C,
                                          const CView<T>* vc, int coarse_buf) {
    T* fe = fine_alt ? vf.e2 : vf.e;
    const int nx = F.nx;
    if (vc) {
        T** pc = coarse_buf ? vc->pe2 : vc->pe;
        uint8_t** pcb = vc->pb;
        auto fce = [pc](int I, int J) { return pc[J][I]; };
        auto fcb = [pcb](int I, int J) { return pcb[J][I]; };
        for_own(F.NX, vf.r0, vf.r1, [&](int i, int j, int rr) {
            const int lid = rr * nx + i;
            if (vf.b[lid] & 0x0F) fe[lid] = fe[lid] + prolong_corr<T>(F, i, j, fce, fcb);
        });
    } else {
        const T* ce = (const T*)(coarse_buf ? C.e2 : C.e);
        const uint8_t* cbits = C.bits;
        const int CP = C.pitch;
        auto fce = [ce, CP](int I, int J) { return ce[I + J * CP]; };
        auto fcb = [cbits, CP](int I, int J) { return __ldg(&cbits[I + J * CP]); };
        for_own(F.NX, vf.r0, vf.r1, [&](int i, int j, int rr) {
            const int lid = rr * nx + i;
            if (vf.b[lid] & 0x0F) fe[lid] = fe[lid] + prolong_corr<T>(F, i, j, fce, fcb);
        });
    }
}

template <typename T>
__global__ void __launch_bounds__(CMG_THREADS, 1)
    k_vcycle_cluster(const int* __restrict__ sub, const LevelDev* __restrict__ LV, const InstDev* __restrict__ I,
                     const InstState* __restrict__ S, const GhostDev* __restrict__ G, int pre, int post) {
    extern __shared__ __align__(16) unsigned char sm[];
    cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank();
    const int k = (int)(blockIdx.x / CMG_CTAS);
    if (S[k].ppe_state != ST_ACTIVE) return;  // the whole cluster (one instance)
    const InstDev& in = I[k];
    const int lb = sub[k], nd = lb - in.lev0;
    int nxs[CMG_MAX_LEVELS], nys[CMG_MAX_LEVELS];
#pragma unroll
    for (int l = 0; l < CMG_MAX_LEVELS; l++) {
        nxs[l] = l < nd ? LV[in.lev0 + l].nx : 0;
        nys[l] = l < nd ? LV[in.lev0 + l].ny : 0;
    }
    const CmgLayout lay = cmg_layout(nd, nxs, nys, (int)sizeof(T), 0);
    const T om = (T)in.omega;
    const int* gidx = in.gidx;
    // ---- stage: zero rows, own rows (e, e2 = 0; r of the finest level; stencil bytes), row pointer tables
    T* zero = (T*)(sm + lay.zero);
    uint8_t* zerob = sm + lay.zerob;
    for (int q = threadIdx.x; q < nxs[0]; q += blockDim.x) {
        zero[q] = (T)0;
        zerob[q] = 0;
    }
    for (int l = 0; l < nd; l++) {
        const LevelDev& L = LV[in.lev0 + l];
        const CmgLevel& c = lay.lv[l];
        const CView<T> v = cview<T>(sm, c, rank, L.NY);
        const int nrows = v.r1 - v.r0 + 1, nx = L.nx;
        const T* gr = (const T*)L.r;
        for (int q = threadIdx.x; q < nrows * nx; q += blockDim.x) {
            const int rr = q / nx, i = q - rr * nx, gid = i + (v.r0 + rr) * L.pitch;
            v.e[q] = (T)0;
            v.e2[q] = (T)0;
            v.r[q] = l == 0 ? gr[gid] : (T)0;
            v.b[q] = __ldg(&L.bits[gid]);
        }
        for (int j = threadIdx.x; j < L.ny; j += blockDim.x) {
            if (j >= 1 && j <= L.NY) {
                const int owner = (j - 1) / c.m, lr = (j - 1) - owner * c.m;
                v.pe[j] = cl.map_shared_rank((T*)(sm + c.e) + lr * nx, owner);
                v.pe2[j] = cl.map_shared_rank((T*)(sm + c.e2) + lr * nx, owner);
                v.pr[j] = cl.map_shared_rank((T*)(sm + c.r) + lr * nx, owner);
                v.pb[j] = cl.map_shared_rank(sm + c.b + lr * nx, owner);
            } else {
                v.pe[j] = zero;
                v.pe2[j] = zero;
                v.pr[j] = zero;
                v.pb[j] = zerob;
            }
        }
    }
    cl.sync();
    // ---- descend
    const LevelDev& L0 = LV[in.lev0];
    const CView<T> v0 = cview<T>(sm, lay.lv[0], rank, L0.NY);
    c_sweep<T, true>(L0, v0, 0, true, om, G, gidx);
    cl.sync();
    int cur0 = 1;
    for (int q = 1; q < pre; q++) {
        c_sweep<T, true>(L0, v0, cur0, false, om, G, gidx);
        cl.sync();
        cur0 ^= 1;
    }
    for (int l = 1; l < nd; l++) {
        const LevelDev& F = LV[in.lev0 + l - 1];
        const LevelDev& C = LV[in.lev0 + l];
        const CView<T> vf = cview<T>(sm, lay.lv[l - 1], rank, F.NY);
        const CView<T> vc = cview<T>(sm, lay.lv[l], rank, C.NY);
        if (l == 1) c_restrict<T, true>(F, vf, parity_after_pre(0, pre), C, &vc, om, G, gidx, rank);
        else c_restrict<T, false>(F, vf, parity_after_pre(l - 1, pre), C, &vc, om, G, gidx, rank);
        cl.sync();
        int cur = 0;
        for (int q = 1; q < pre; q++) {
            c_sweep<T, false>(C, vc, cur, false, om, G, gidx);
            cl.sync();
            cur ^= 1;
        }
    }
    {   // restriction into the first small level (global memory)
        const LevelDev& F = LV[lb - 1];
        const LevelDev& C = LV[lb];
        const CView<T> vf = cview<T>(sm, lay.lv[nd - 1], rank, F.NY);
        if (nd == 1) c_restrict<T, true>(F, vf, parity_after_pre(0, pre), C, nullptr, om, G, gidx, rank);
        else c_restrict<T, false>(F, vf, parity_after_pre(nd - 1, pre), C, nullptr, om, G, gidx, rank);
    }
    cl.sync();
    if (rank == 0) b_subcycle<T>(sub, LV, I, S, pre, post, sm + lay.sub, false, k);
    cl.sync();
    // ---- ascend
    for (int l = nd - 1; l >= 0; l--) {
        const LevelDev& F = LV[in.lev0 + l];
        const LevelDev& C = LV[in.lev0 + l + 1];
        const CView<T> vf = cview<T>(sm, lay.lv[l], rank, F.NY);
        const int coarse_alt = parity_after_post(l + 1, pre, post);
        int cur = parity_after_pre(l, pre);
        if (l + 1 < nd) {
            const CView<T> vc = cview<T>(sm, lay.lv[l + 1], rank, C.NY);
            c_prolong<T>(F, vf, cur, C, &vc, coarse_alt && C.child >= 0);
        } else {
            c_prolong<T>(F, vf, cur, C, nullptr, coarse_alt && C.child >= 0);
        }
        cl.sync();
        for (int q = 0; q < post; q++) {
            if (l == 0) c_sweep<T, true>(F, vf, cur, false, om, G, gidx);
            else c_sweep<T, false>(F, vf, cur, false, om, G, gidx);
            cl.sync();
            cur ^= 1;
        }
        if (l == 0) cur0 = cur;
    }
    // ---- the finest level's correction back to global memory
    {
        T* ge = (T*)(cur0 ? L0.e2 : L0.e);
        const T* src = cur0 ? v0.e2 : v0.e;
        const int nrows = v0.r1 - v0.r0 + 1, nx = L0.nx;
        for (int q = threadIdx.x; q < nrows * nx; q += blockDim.x) {
            const int rr = q / nx, i = q - rr * nx;
            ge[i + (v0.r0 + rr) * L0.pitch] = src[q];
        }
    }
    cl.sync();  // no CTA leaves while others may still read its rows
}

}  // namespace

// Bytes of dynamic shared memory the cluster V-cycle needs for one instance
// (distributed levels lev0 .. lb-1 plus its sub-cycle area of sub_bytes).
size_t cluster_vcycle_bytes(int nd, const int* nx, const int* ny, int tsize, size_t sub_bytes) {
    if (nd < 1 || nd > CMG_MAX_LEVELS) return (size_t)-1;
    return cmg_layout(nd, nx, ny, tsize, sub_bytes).bytes;
}

template <typename T>
cudaError_t cluster_vcycle_setup(int smem_bytes, int ninst, int* ok) {
    *ok = 0;
    // the attributes belong to the kernel, shared by every solver on the
    // device: the shared-memory limit is only raised (a smaller solver set up
    // after a larger one must not lower it under the larger one's launches)
    static std::mutex mu;
    static int cur[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    dev = dev >= 0 && dev < 64 ? dev : 0;
    std::lock_guard<std::mutex> g(mu);
    cudaError_t e = cudaFuncSetAttribute(k_vcycle_cluster<T>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
    if (smem_bytes > cur[dev]) {
        e = cudaFuncSetAttribute(k_vcycle_cluster<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes);
        if (e != cudaSuccess) return e;
        cur[dev] = smem_bytes;
    }
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = CMG_CTAS;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(CMG_CTAS);
    cfg.blockDim = dim3(CMG_THREADS);
    cfg.dynamicSmemBytes = (size_t)smem_bytes;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int nclusters = 0;
    e = cudaOccupancyMaxActiveClusters(&nclusters, (const void*)k_vcycle_cluster<T>, &cfg);
    if (e != cudaSuccess) return e;
    *ok = nclusters >= ninst ? 1 : 0;
    return cudaSuccess;
}

template <typename T>
cudaError_t launch_vcycle_cluster(const int* sub, int ninst, const LevelDev* LV, const InstDev* I, const InstState* S,
                                  const GhostDev* G, int pre, int post, int smem_bytes, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = CMG_CTAS;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(CMG_CTAS * ninst);
    cfg.blockDim = dim3(CMG_THREADS);
    cfg.dynamicSmemBytes = (size_t)smem_bytes;
    cfg.stream = s;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_vcycle_cluster<T>, sub, LV, I, S, G, pre, post);
}

template cudaError_t cluster_vcycle_setup<double>(int, int, int*);
template cudaError_t cluster_vcycle_setup<float>(int, int, int*);
template cudaError_t launch_vcycle_cluster<double>(const int*, int, const LevelDev*, const InstDev*, const InstState*,
                                                   const GhostDev*, int, int, int, cudaStream_t);
template cudaError_t launch_vcycle_cluster<float>(const int*, int, const LevelDev*, const InstDev*, const InstState*,
                                                  const GhostDev*, int, int, int, cudaStream_t);

}  // namespace ifx
