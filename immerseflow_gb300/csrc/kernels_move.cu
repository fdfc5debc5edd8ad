// kernels_move.cu -- geometry of bodies in prescribed rigid motion, redone on
// the device at the start of every time step (no reference counterpart: the
// reference claims moving boundaries, README.md:7,11, without code).
//
// One block per moving instance.  The body's new pose (motion.h) moves it
// within the box of cells around its old and new positions; only that region
// changes, and the block redoes there, in this order with a block barrier
// between the phases:
//   A  tagging (the static rule of k_tag) and the fresh cells (not fluid in
//      the previous step, fluid now; they keep the ghost value they had and
//      are stamped with the step number);
//   B  ghost marking (solid cells with a fluid cell among their 8 neighbours);
//   C  finest-level stencil bytes, the ghost index map cleared, and the face
//      velocities of the fresh cells interpolated from the cell values;
//   D  the IBM ghost list: the region's ghosts in row-major order into the
//      instance's ghost slots (a block prefix sum, so the order is that of the
//      static set-up), slots left over emptied;
//   E  every coarser level's cells in use (any child in use) and stencil bytes,
//      also in the sub-cycle's image of the small levels.
// The image-point weights of the new ghosts (k_ghost_weights) and the force
// samples at the new pose (k_move_forces) follow as kernels of their own.  The
// CPU restatement rebuilds the same tables on the whole grid; the rules are
// local, so the results are the same.
//
// Compiled with -fmad=false: the pose, the predicate and the sample positions
// round every operation on its own, like the CPU restatement.
#include <cuda_runtime.h>

#include "ibm_geom.cuh"
#include "ifx_dev.h"
#include "ifx_kernels.h"
#include "motion.h"

namespace ifx {

constexpr int MOVE_THREADS = 1024;

struct Box {
    int i0, i1, j0, j1;
};

// Cells (i0..i1, j0..j1) around the ellipse of semi-axes a, b at the pose:
// every cell centre inside the body lies strictly within.
__device__ Box body_box(const InstDev& in) {
    const double c = in.bcs, s = in.bsn, a = in.ba, b = in.bb;
    const double hx = sqrt(a * a * (c * c) + b * b * (s * s));
    const double hy = sqrt(a * a * (s * s) + b * b * (c * c));
    Box r;
    r.i0 = ub_index(in.xc, in.nx, in.bcx - hx);
    r.i1 = ub_index(in.xc, in.nx, in.bcx + hx) + 1;
    r.j0 = ub_index(in.yc, in.ny, in.bcy - hy);
    r.j1 = ub_index(in.yc, in.ny, in.bcy + hy) + 1;
    return r;
}

// Deterministic block-wide exclusive prefix count of flag; returns the total.
__device__ __forceinline__ int block_scan(bool flag, int* wsum, int& before) {
    const int lane = (int)(threadIdx.x & 31), w = (int)(threadIdx.x >> 5), nw = (int)(blockDim.x >> 5);
    const unsigned bal = __ballot_sync(0xffffffffu, flag);
    before = __popc(bal & ((1u << lane) - 1u));
    if (lane == 0) wsum[w] = __popc(bal);
    __syncthreads();
    if (w == 0) {
        const int v = lane < nw ? wsum[lane] : 0;
        int incl = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane < nw) wsum[lane] = incl - v;
        if (lane == 31) wsum[32] = incl;
    }
    __syncthreads();
    before += wsum[w];
    return wsum[32];
}

__global__ void __launch_bounds__(MOVE_THREADS) k_move_geometry(InstDev* __restrict__ I, InstState* __restrict__ S,
                                                                const LevelDev* __restrict__ LV, GhostDev* __restrict__ G,
                                                                const int* __restrict__ mv) {
    const int k = mv[blockIdx.x];
    InstDev& in = I[k];
    if (in.retired || S[k].geo_err) return;
    __shared__ Box reg;    // cells whose type may change
    __shared__ int ok;
    __shared__ int wsum[33];
    __shared__ int base;
    __shared__ int nprev;  // ghost slots in use before this step
    const int P = in.pitch, tid = (int)threadIdx.x, nt = (int)blockDim.x;
    const int stamp = (int)S[k].nstep;
    if (tid == 0) {
        nprev = S[k].n_ibm;
        const double t = (double)S[k].nstep * in.dt;
        const Pose p = pose_at(in.mo_x0, in.mo_y0, in.mo_th0, in.mo_u, in.mo_v, in.mo_ax, in.mo_ay, in.mo_ath, in.mo_f,
                               in.mo_w, in.mo_phx, in.mo_phy, in.mo_pha, t);
        const double ox = in.bcx, oy = in.bcy, oc = in.bcs, os = in.bsn;
        in.bcx = p.x;
        in.bcy = p.y;
        in.bcs = p.c;
        in.bsn = p.s;
        const Box nb = body_box(in);
        const Box ob{S[k].bb[0], S[k].bb[1], S[k].bb[2], S[k].bb[3]};
        Box r;
        r.i0 = min(nb.i0, ob.i0) - 1;
        r.i1 = max(nb.i1, ob.i1) + 1;
        r.j0 = min(nb.j0, ob.j0) - 1;
        r.j1 = max(nb.j1, ob.j1) + 1;
        // the body, its ghosts' image points and their interpolation cells
        // stay three cells inside the domain
        ok = r.i0 >= 3 && r.j0 >= 3 && r.i1 <= in.NX - 2 && r.j1 <= in.NY - 2;
        if (ok) {
            in.bu = p.u;
            in.bv = p.v;
            in.bw = p.w;
            S[k].bb[0] = nb.i0;
            S[k].bb[1] = nb.i1;
            S[k].bb[2] = nb.j0;
            S[k].bb[3] = nb.j1;
            reg = r;
        } else {
            in.bcx = ox;  // keep the last valid geometry
            in.bcy = oy;
            in.bcs = oc;
            in.bsn = os;
            S[k].geo_err = 1;
        }
    }
    __syncthreads();
    if (!ok) return;
    const double cx = in.bcx, cy = in.bcy, cs = in.bcs, sn = in.bsn;
    uint8_t* type = const_cast<uint8_t*>(in.type);
    int* gidx = const_cast<int*>(in.gidx);
    const int W = reg.i1 - reg.i0 + 1, H = reg.j1 - reg.j0 + 1, ncell = W * H;
    // A: tagging, fresh cells
    for (int q = tid; q < ncell; q += nt) {
        const int i = reg.i0 + q % W, j = reg.j0 + q / W, id = i + j * P;
        const uint8_t old = type[id];
        const int ins = inside_ellipse(in.xc[i], in.yc[j], cx, cy, cs, sn, in.bia2, in.bib2);
        const uint8_t nw = ins ? T_SOLID : T_FLUID;
        type[id] = nw;
        in.iblank[id] = ins ? 0.0 : 1.0;
        if (old != T_FLUID && nw == T_FLUID) in.fresh[id] = stamp;
    }
    __syncthreads();
    // B: ghost marking (a cell that becomes a ghost is not fluid, so the
    // concurrent tests for fluid neighbours are unaffected)
    for (int q = tid; q < ncell; q += nt) {
        const int i = reg.i0 + q % W, j = reg.j0 + q / W, id = i + j * P;
        if (type[id] != T_SOLID) continue;
        bool g = false;
        for (int dj = -1; dj <= 1; dj++)
            for (int di = -1; di <= 1; di++)
                if (type[(i + di) + (j + dj) * P] == T_FLUID) g = true;
        if (g) type[id] = T_GHOST;
    }
    __syncthreads();
    // C: finest-level stencil bytes (the region grown by one cell: the
    // neighbours of changed cells), ghost map cleared, fresh faces
    {
        const LevelDev& L0 = LV[in.lev0];
        uint8_t* bits = const_cast<uint8_t*>(L0.bits);
        const int W1 = W + 2, H1 = H + 2;
        for (int q = tid; q < W1 * H1; q += nt) {
            const int i = reg.i0 - 1 + q % W1, j = reg.j0 - 1 + q / W1, id = i + j * P;
            uint8_t bt = 0;
            if (type[id] == T_FLUID) {
                auto probe = [&](int nid, uint8_t ob, uint8_t gb) {
                    const uint8_t t = type[nid];
                    if (t == T_FLUID) bt |= ob;
                    if (t == T_GHOST) bt |= (uint8_t)(ob | gb);
                };
                probe(id + 1, B_E, G_E);
                probe(id - 1, B_W, G_W);
                probe(id + P, B_N, G_N);
                probe(id - P, B_S, G_S);
            }
            bits[id] = bt;
        }
        for (int q = tid; q < ncell; q += nt) {
            const int i = reg.i0 + q % W, j = reg.j0 + q / W, id = i + j * P;
            gidx[id] = -1;
            if (in.fresh[id] != stamp) continue;
            // the faces of a fresh cell, as the initial face interpolation
            in.U[id] = in.u[id] * in.gx[i] + in.u[id + 1] * in.fx[i];
            in.U[id - 1] = in.u[id - 1] * in.gx[i - 1] + in.u[id] * in.fx[i - 1];
            in.V[id] = in.v[id] * in.gy[j] + in.v[id + P] * in.fy[j];
            in.V[id - P] = in.v[id - P] * in.gy[j - 1] + in.v[id] * in.fy[j - 1];
        }
    }
    __syncthreads();
    // D: IBM ghost list in row-major order
    if (tid == 0) base = 0;
    __syncthreads();
    for (int q0 = 0; q0 < ncell; q0 += nt) {
        const int q = q0 + tid;
        int id = -1;
        if (q < ncell) id = (reg.i0 + q % W) + (reg.j0 + q / W) * P;
        const bool g = id >= 0 && type[id] == T_GHOST;
        int before;
        const int total = block_scan(g, wsum, before);
        const int slot = base + before;
        if (g && slot < in.ibm_cap) {
            GhostDev e;
            e.cell = id;
            e.inst = k;
            e.side = -1;
            e.adj = -1;
            for (int m = 0; m < 4; m++) {
                e.nb[m] = id;
                e.wu[m] = e.wv[m] = e.wp[m] = 0.0;
            }
            e.cu = e.cv = 0.0;
            e.qi[0] = e.qi[1] = -1;
            e.qf[0] = e.qf[1] = 0.0;
            e.qown = -1;
            e.qh = 0.0;
            G[in.ibm_beg + slot] = e;
            gidx[id] = in.ibm_beg + slot;
        }
        __syncthreads();
        if (tid == 0) base += total;
        __syncthreads();
    }
    const int nnew = min(base, in.ibm_cap);
    for (int s = nnew + tid; s < nprev; s += nt) G[in.ibm_beg + s].cell = -1;
    if (tid == 0) {
        S[k].n_ibm = nnew;
        if (base > in.ibm_cap) S[k].geo_err = 2;
    }
    // E: coarser levels (cells in use: any child in use; stencil bytes: open
    // towards neighbours in use), mirrored into the sub-cycle image
    Box f{reg.i0, reg.i1, reg.j0, reg.j1};  // finer-level cells whose use may have changed
    for (int l = 1; l < in.nlev; l++) {
        __syncthreads();
        const LevelDev& F = LV[in.lev0 + l - 1];
        const LevelDev& C = LV[in.lev0 + l];
        Box c;
        c.i0 = (f.i0 - 1) / C.cx + 1;
        c.i1 = (f.i1 - 1) / C.cx + 1;
        c.j0 = (f.j0 - 1) / C.cy + 1;
        c.j1 = (f.j1 - 1) / C.cy + 1;
        const int cw = c.i1 - c.i0 + 1, ch = c.j1 - c.j0 + 1;
        for (int q = tid; q < cw * ch; q += nt) {
            const int Ic = c.i0 + q % cw, J = c.j0 + q / cw;
            uint8_t a = 0;
            for (int dj = 0; dj < C.cy; dj++)
                for (int di = 0; di < C.cx; di++) {
                    const int i = C.cx * (Ic - 1) + 1 + di, j = C.cy * (J - 1) + 1 + dj;
                    if (i <= F.NX && j <= F.NY)
                        a |= l == 1 ? (uint8_t)(type[i + j * P] == T_FLUID) : F.act[i + j * F.pitch];
                }
            C.act[Ic + J * C.pitch] = a;
        }
        __syncthreads();
        uint8_t* cb = const_cast<uint8_t*>(C.bits);
        const int b0 = max(c.i0 - 1, 1), b1 = min(c.i1 + 1, C.NX), d0 = max(c.j0 - 1, 1), d1 = min(c.j1 + 1, C.NY);
        const int bw = b1 - b0 + 1, bh = d1 - d0 + 1;
        unsigned char* img = nullptr;
        int inx = 0;
        size_t ob = 0;
        if (in.sub_lb > 0 && l >= in.sub_lb) {
            const SubHdr* hd = (const SubHdr*)in.sub_img;
            const SubHdr& h = hd[l - in.sub_lb];
            img = const_cast<unsigned char*>(in.sub_img);
            inx = h.nx;
            ob = (size_t)h.base + h.o.b;
        }
        for (int q = tid; q < bw * bh; q += nt) {
            const int i = b0 + q % bw, j = d0 + q / bw, id = i + j * C.pitch;
            uint8_t bt = 0;
            if (C.act[id]) {
                if (i + 1 <= C.NX && C.act[id + 1]) bt |= B_E;
                if (i - 1 >= 1 && C.act[id - 1]) bt |= B_W;
                if (j + 1 <= C.NY && C.act[id + C.pitch]) bt |= B_N;
                if (j - 1 >= 1 && C.act[id - C.pitch]) bt |= B_S;
            }
            cb[id] = bt;
            if (img) img[ob + i + (size_t)j * inx] = bt;
        }
        f = c;
    }
}

// The body-surface force samples at the new pose (the static table's
// formulas), one thread per sample over many small blocks: the binary
// searches and FP64 divisions are latency chains, and GB300's FP64 pipe is
// narrow, so the work is spread over the SMs.
__global__ void k_move_forces(const InstDev* __restrict__ I, const InstState* __restrict__ S, const int* __restrict__ mv) {
    const int k = mv[blockIdx.y];
    const InstDev& in = I[k];
    if (in.retired || S[k].geo_err) return;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= FORCE_SAMPLES) return;
    const int P = in.pitch;
    const double cx = in.bcx, cy = in.bcy, cs = in.bcs, sn = in.bsn;
    const double* b = in.fsb + 5 * (size_t)q;
    const double lx = b[0], ly = b[1], nlx = b[2], nly = b[3];
    const double xs = cx + lx * cs - ly * sn;
    const double ys = cy + lx * sn + ly * cs;
    const double nxw = nlx * cs - nly * sn, nyw = nlx * sn + nly * cs;
    const int i0 = min(max(ub_index(in.xc, in.nx, xs), 0), in.nx - 2);
    const int j0 = min(max(ub_index(in.yc, in.ny, ys), 0), in.ny - 2);
    const double h = fmax(fmax(in.dx[i0], in.dx[i0 + 1]), fmax(in.dy[j0], in.dy[j0 + 1]));
    const double del = 1.5 * h;
    ForceSample e;
    e.c0 = i0 + j0 * P;
    e.xi0 = (xs - in.xc[i0]) / (in.xc[i0 + 1] - in.xc[i0]);
    e.et0 = (ys - in.yc[j0]) / (in.yc[j0 + 1] - in.yc[j0]);
    const double xq = xs + del * nxw, yq = ys + del * nyw;
    const int i1 = min(max(ub_index(in.xc, in.nx, xq), 0), in.nx - 2);
    const int j1 = min(max(ub_index(in.yc, in.ny, yq), 0), in.ny - 2);
    e.c1 = i1 + j1 * P;
    e.xi1 = (xq - in.xc[i1]) / (in.xc[i1 + 1] - in.xc[i1]);
    e.et1 = (yq - in.yc[j1]) / (in.yc[j1 + 1] - in.yc[j1]);
    e.nx = nxw;
    e.ny = nyw;
    e.ds = b[4];
    e.del = del;
    const_cast<ForceSample*>(in.fs)[q] = e;
}

// Body box of every moving instance at its current pose (set-up).
__global__ void k_move_init(InstDev* __restrict__ I, InstState* __restrict__ S, const int* __restrict__ mv, int nmv,
                            const int* __restrict__ n_ibm) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nmv) return;
    const int k = mv[q];
    const Box b = body_box(I[k]);
    S[k].bb[0] = b.i0;
    S[k].bb[1] = b.i1;
    S[k].bb[2] = b.j0;
    S[k].bb[3] = b.j1;
    S[k].n_ibm = n_ibm[q];
    S[k].geo_err = 0;
}

cudaError_t launch_move_geometry(InstDev* I, InstState* S, const LevelDev* LV, GhostDev* G, const int* mv, int nmv,
                                 cudaStream_t s) {
    if (nmv == 0) return cudaSuccess;
    k_move_geometry<<<nmv, MOVE_THREADS, 0, s>>>(I, S, LV, G, mv);
    return cudaGetLastError();
}
cudaError_t launch_move_forces(const InstDev* I, const InstState* S, const int* mv, int nmv, cudaStream_t s) {
    if (nmv == 0) return cudaSuccess;
    k_move_forces<<<dim3((FORCE_SAMPLES + 31) / 32, nmv), 32, 0, s>>>(I, S, mv);
    return cudaGetLastError();
}
cudaError_t launch_move_init(InstDev* I, InstState* S, const int* mv, int nmv, const int* n_ibm, cudaStream_t s) {
    if (nmv == 0) return cudaSuccess;
    k_move_init<<<(nmv + 127) / 128, 128, 0, s>>>(I, S, mv, nmv, n_ibm);
    return cudaGetLastError();
}

}  // namespace ifx
