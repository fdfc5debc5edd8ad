// solver.cu -- host orchestration behind the C ABI (include/immerseflow_gb300.h).
//
// Replaces the reference's ImmerseFlow object (src/header/globalVariables.cuh:70-88):
// allocation() + readGridData() + initializeData() become ifx_create*, the
// per-step ADsolver() becomes ifx_step.  Differences by design:
//  - all device memory is allocated once at creation (the reference does 11
//    cudaMalloc/cudaFree per step and 2 per residual reduction);
//  - one stream per solver, no cudaDeviceSynchronize after each launch;
//  - convergence loops run on the device: reduce kernels vote and a CUDA
//    graph with conditional WHILE nodes repeats the loop body, so a time step
//    is one graph launch with no host round trip (a host-driven loop with the
//    same semantics is kept for debugging, IFX_NO_GRAPH=1);
//  - any number of instances of uneven size are advanced together.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <exception>
#include <vector>

#include "ifx_host.h"
#include "ifx_kernels.h"
#include "motion.h"

using namespace ifx;

namespace {

ifx_status cuerr(cudaError_t e, const char* what) {
    if (e == cudaErrorMemoryAllocation) return set_error(IFX_ERR_NOMEM, std::string(what) + ": " + cudaGetErrorString(e));
    return set_error(IFX_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CUDA_TRY(x)                                        \
    do {                                                   \
        cudaError_t e_ = (x);                              \
        if (e_ != cudaSuccess) return cuerr(e_, #x);       \
    } while (0)

#define IFX_TRY(x)                                         \
    do {                                                   \
        ifx_status s_ = (x);                               \
        if (s_ != IFX_OK) return s_;                       \
    } while (0)

template <typename T>
ifx_status dalloc(ifx_solver* S, T** out, size_t n) {
    void* p = nullptr;
    size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
    CUDA_TRY(cudaMalloc(&p, bytes));
    S->allocs.push_back(p);
    S->device_bytes += bytes;
    CUDA_TRY(cudaMemsetAsync(p, 0, bytes, S->stream));
    *out = (T*)p;
    return IFX_OK;
}

template <typename T>
ifx_status dupload(ifx_solver* S, T** out, const std::vector<T>& h) {
    IFX_TRY(dalloc(S, out, h.size()));
    if (!h.empty()) CUDA_TRY(cudaMemcpyAsync(*out, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, S->stream));
    return IFX_OK;
}

// Shared-memory image of the sub-cycle's levels lb.. of instance I, laid out
// as the device code reads it (SubHdr table, then per level the arrays of
// sub_layout): metric arrays in T, prolongation tables (levels with a coarser
// one), dense stencil bytes, and zero e, e2, r.
template <typename T>
std::vector<unsigned char> sub_image(const Instance& I, int lb) {
    const int nl = (int)I.lev.size(), ns = nl - lb, ts = (int)sizeof(T);
    size_t total = SUB_HDR_BYTES;
    for (int s = 0; s < ns; s++) total += sub_level_bytes(I.lev[lb + s].nx, I.lev[lb + s].ny, ts);
    std::vector<unsigned char> img(total, 0);
    size_t off = SUB_HDR_BYTES;
    for (int s = 0; s < ns; s++) {
        const int l = lb + s;
        const HostLevel& L = I.lev[l];
        SubHdr h;
        std::memset(&h, 0, sizeof(h));
        h.o = sub_layout(L.nx, L.ny, ts);
        h.base = (unsigned)off;
        h.NX = L.NX; h.NY = L.NY; h.nx = L.nx; h.ny = L.ny;
        h.dirmask = I.dirmask;
        h.child = l + 1 < nl ? I.lev_base + l + 1 : -1;
        h.depth = l;
        h.ns = ns;
        h.cx = L.cx; h.cy = L.cy;
        std::memcpy(img.data() + s * sizeof(SubHdr), &h, sizeof(h));
        unsigned char* b = img.data() + off;
        auto put_t = [&](size_t o, const std::vector<double>& v, int n) {
            T* d = (T*)(b + o);
            for (int q = 0; q < n && q < (int)v.size(); q++) d[q] = (T)v[q];
        };
        auto put_i = [&](size_t o, const std::vector<int>& v, int n) {
            int* d = (int*)(b + o);
            for (int q = 0; q < n && q < (int)v.size(); q++) d[q] = v[q];
        };
        auto put_c = [&](size_t o, const std::vector<signed char>& v, int n) {
            signed char* d = (signed char*)(b + o);
            for (int q = 0; q < n && q < (int)v.size(); q++) d[q] = v[q];
        };
        // face coefficient pairs: the products of the T copies, as the tile phases form them
        auto put_pairs = [&](size_t o, const std::vector<double>& k, const std::vector<double>& inv, int n) {
            T* d = (T*)(b + o);
            for (int q = 0; q < n && q < (int)k.size(); q++) {
                const T iq = (T)inv[q];
                d[2 * q] = (T)k[q] * iq;
                d[2 * q + 1] = q > 0 ? (T)k[q - 1] * iq : (T)0;
            }
        };
        put_pairs(h.o.cew, L.kx, L.ix, L.nx); put_t(h.o.dw, L.dw, L.nx);
        put_pairs(h.o.cns, L.ky, L.iy, L.ny); put_t(h.o.dh, L.dh, L.ny);
        if (h.child >= 0) {
            put_t(h.o.pwx, L.pwx, L.nx); put_t(h.o.pwy, L.pwy, L.ny);
            put_i(h.o.pI, L.pI, L.nx); put_i(h.o.pIn, L.pIn, L.nx);
            put_i(h.o.pJ, L.pJ, L.ny); put_i(h.o.pJn, L.pJn, L.ny);
            put_c(h.o.psx, L.psx, L.nx); put_c(h.o.psy, L.psy, L.ny);
        }
        for (int j = 0; j < L.ny; j++)
            for (int i = 0; i < L.nx; i++) b[h.o.b + i + (size_t)j * L.nx] = L.bits[i + (size_t)j * L.pitch];
        off += h.o.bytes;
    }
    return img;
}

std::vector<float> to_f(const std::vector<double>& v) {
    std::vector<float> r(v.size());
    for (size_t k = 0; k < v.size(); k++) r[k] = (float)v[k];
    return r;
}

// TMA tensor maps of every multigrid level for the staged smoothing sweep
// (launch_smooth_tma): per level e, e2, r (type T) and the stencil bytes, for
// 32x8 tiles and for wide tiles; the box of e carries a one-cell halo and
// starts 16 bytes left of the tile.  Returns false when the driver cannot
// encode them (the plain tile kernels are used then).
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
bool tensor_maps(const std::vector<LevelDev>& lv, int ts, std::vector<CUtensorMap>& out) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !p) {
        cudaGetLastError();
        return false;
    }
    const EncodeTiledFn enc = (EncodeTiledFn)p;
    const CUtensorMapDataType dt = ts == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    out.assign(lv.size() * TMA_MAPS_PER_LEVEL, CUtensorMap{});
    for (size_t v = 0; v < lv.size(); v++) {
        const LevelDev& L = lv[v];
        const cuuint64_t dims[2] = {(cuuint64_t)L.pitch, (cuuint64_t)L.ny};
        const cuuint64_t st_t[1] = {(cuuint64_t)L.pitch * ts}, st_b[1] = {(cuuint64_t)L.pitch};
        const cuuint32_t es[2] = {1, 1};
        for (int w = 0; w < 2; w++) {
            const int rows = w ? MG_ROWS_WIDE : 1, pad = 16 / ts;
            const cuuint32_t be[2] = {(cuuint32_t)(TILE_X + 2 * pad), (cuuint32_t)(TILE_Y * rows + 2)};
            const cuuint32_t bt[2] = {(cuuint32_t)TILE_X, (cuuint32_t)(TILE_Y * rows)};
            CUtensorMap* m = &out[v * TMA_MAPS_PER_LEVEL + 4 * w];
            void* arr[3] = {L.e, L.e2, L.r};
            for (int a = 0; a < 3; a++)
                if (enc(&m[a], dt, 2, arr[a], dims, st_t, a < 2 ? be : bt, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
                    return false;
            if (enc(&m[3], CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, (void*)L.bits, dims, st_b, bt, es,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
                return false;
        }
    }
    return true;
}

// Face-coefficient pairs of one direction: (k[i] inv[i], k[i-1] inv[i]) with
// both factors first rounded to T, so that each product is the one the
// kernels would form from the T copies of k and inv.
template <typename T, typename V2>
std::vector<V2> face_pairs(const std::vector<double>& k, const std::vector<double>& inv) {
    std::vector<V2> r(k.size());
    for (size_t i = 0; i < k.size(); i++) {
        const T ii = (T)inv[i];
        r[i].x = (T)k[i] * ii;
        r[i].y = i > 0 ? (T)k[i - 1] * ii : (T)0;
    }
    return r;
}

int round_up(int a, int b) { return (a + b - 1) / b * b; }

// ------------------------------------------------------------- grid

// Face coordinates -> centres and widths (readGridData, src/include/preSim.cu:293-355;
// widths are stored 1-D because they are separable).
void build_grid(Instance& I, const double* xf, const double* yf) {
    const int nx = I.nx, ny = I.ny;
    I.xf.assign(xf, xf + I.NX + 1);
    I.yf.assign(yf, yf + I.NY + 1);
    I.xc.assign(nx, 0.0);
    I.yc.assign(ny, 0.0);
    for (int i = 1; i < nx - 1; i++) I.xc[i] = (xf[i - 1] + xf[i]) / 2.0;
    for (int j = 1; j < ny - 1; j++) I.yc[j] = (yf[j - 1] + yf[j]) / 2.0;
    I.xc[0] = -1 * I.xc[1];
    I.yc[0] = -1 * I.yc[1];
    I.xc[nx - 1] = xf[nx - 2] + (xf[nx - 2] - I.xc[nx - 2]);
    I.yc[ny - 1] = yf[ny - 2] + (yf[ny - 2] - I.yc[ny - 2]);
    I.dx.assign(nx, 0.0);
    I.dy.assign(ny, 0.0);
    for (int i = 1; i < nx - 1; i++) I.dx[i] = xf[i] - xf[i - 1];
    for (int j = 1; j < ny - 1; j++) I.dy[j] = yf[j] - yf[j - 1];
    I.dx[0] = I.dx[1];
    I.dx[nx - 1] = I.dx[nx - 2];
    I.dy[0] = I.dy[1];
    I.dy[ny - 1] = I.dy[ny - 2];
    I.fx.assign(nx, 0.0);
    I.gx.assign(nx, 0.0);
    I.fy.assign(ny, 0.0);
    I.gy.assign(ny, 0.0);
    for (int i = 0; i < nx - 1; i++) {
        I.fx[i] = I.dx[i] / (I.dx[i] + I.dx[i + 1]);
        I.gx[i] = I.dx[i + 1] / (I.dx[i] + I.dx[i + 1]);
    }
    for (int j = 0; j < ny - 1; j++) {
        I.fy[j] = I.dy[j] / (I.dy[j] + I.dy[j + 1]);
        I.gy[j] = I.dy[j + 1] / (I.dy[j] + I.dy[j + 1]);
    }
}

// Multigrid hierarchy from the tagged finest level.  Coarse cells merge 2x2
// children (ceil at odd sizes); a coarse cell is active when any child is.
// Coarsening of a multigrid level with NX x NY cells on an lx x ly domain: by
// 2 in a direction that has at least 4 cells, except that while the mean
// spacings differ by more than sqrt(2) only the finer direction is coarsened
// (semi-coarsening: point smoothing leaves errors that are rough along the
// weakly coupled, coarsely spaced direction).  The finest level is always
// coarsened when possible; coarser ones while they have more than 64 cells.
// Returns false for the coarsest level.  The oracle uses the same rule.
bool mg_coarsening(int NX, int NY, double lx, double ly, bool finest, int* cx, int* cy) {
    if (!finest && NX * NY <= 64) return false;
    const double hx = lx / NX, hy = ly / NY, r = 1.4142135623730951;
    const bool x_coarse = hx > r * hy, y_coarse = hy > r * hx;  // that direction is already coarser
    *cx = (NX >= 4 && !x_coarse) ? 2 : 1;
    *cy = (NY >= 4 && !y_coarse) ? 2 : 1;
    return *cx == 2 || *cy == 2;
}

void build_levels(Instance& I) {
    I.lev.clear();
    HostLevel l0;
    l0.NX = I.NX;
    l0.NY = I.NY;
    l0.nx = I.nx;
    l0.ny = I.ny;
    l0.pitch = I.pitch;
    l0.dw = I.dx;
    l0.dh = I.dy;
    l0.xc.assign(I.nx, 0.0);
    l0.yc.assign(I.ny, 0.0);
    for (int i = 1; i < I.nx - 1; i++) l0.xc[i] = 0.5 * (I.xf[i - 1] + I.xf[i]);
    for (int j = 1; j < I.ny - 1; j++) l0.yc[j] = 0.5 * (I.yf[j - 1] + I.yf[j]);
    l0.xc[0] = I.xf[0] - 0.5 * l0.dw[0];
    l0.xc[I.nx - 1] = I.xf[I.NX] + 0.5 * l0.dw[I.nx - 1];
    l0.yc[0] = I.yf[0] - 0.5 * l0.dh[0];
    l0.yc[I.ny - 1] = I.yf[I.NY] + 0.5 * l0.dh[I.ny - 1];
    I.lev.push_back(l0);
    const double lx = I.xf[I.NX] - I.xf[0], ly = I.yf[I.NY] - I.yf[0];
    while (true) {
        const HostLevel& f = I.lev.back();
        int cx, cy;
        if (!mg_coarsening(f.NX, f.NY, lx, ly, I.lev.size() == 1, &cx, &cy)) break;
        HostLevel c;
        c.cx = cx;
        c.cy = cy;
        c.NX = cx == 2 ? (f.NX + 1) / 2 : f.NX;
        c.NY = cy == 2 ? (f.NY + 1) / 2 : f.NY;
        c.nx = c.NX + 2;
        c.ny = c.NY + 2;
        c.pitch = round_up(c.nx, 32);
        c.dw.assign(c.nx, 0.0);
        c.dh.assign(c.ny, 0.0);
        for (int Ic = 1; Ic <= c.NX; Ic++) {
            int i = cx * (Ic - 1) + 1;
            c.dw[Ic] = f.dw[i] + (cx == 2 && i + 1 <= f.NX ? f.dw[i + 1] : 0.0);
        }
        for (int Jc = 1; Jc <= c.NY; Jc++) {
            int j = cy * (Jc - 1) + 1;
            c.dh[Jc] = f.dh[j] + (cy == 2 && j + 1 <= f.NY ? f.dh[j + 1] : 0.0);
        }
        c.dw[0] = c.dw[1];
        c.dw[c.nx - 1] = c.dw[c.nx - 2];
        c.dh[0] = c.dh[1];
        c.dh[c.ny - 1] = c.dh[c.ny - 2];
        c.xc.assign(c.nx, 0.0);
        c.yc.assign(c.ny, 0.0);
        double x0 = I.xf[0];
        for (int Ic = 1; Ic <= c.NX; Ic++) {
            c.xc[Ic] = x0 + 0.5 * c.dw[Ic];
            x0 += c.dw[Ic];
        }
        double y0 = I.yf[0];
        for (int Jc = 1; Jc <= c.NY; Jc++) {
            c.yc[Jc] = y0 + 0.5 * c.dh[Jc];
            y0 += c.dh[Jc];
        }
        c.xc[0] = I.xf[0] - 0.5 * c.dw[0];
        c.xc[c.nx - 1] = x0 + 0.5 * c.dw[c.nx - 1];
        c.yc[0] = I.yf[0] - 0.5 * c.dh[0];
        c.yc[c.ny - 1] = y0 + 0.5 * c.dh[c.ny - 1];
        I.lev.push_back(c);
    }
    for (size_t l = 0; l < I.lev.size(); l++) {
        HostLevel& v = I.lev[l];
        v.kx.assign(v.nx, 0.0);
        v.ky.assign(v.ny, 0.0);
        v.ix.assign(v.nx, 0.0);
        v.iy.assign(v.ny, 0.0);
        for (int i = 0; i < v.nx - 1; i++) v.kx[i] = 2.0 / (v.dw[i] + v.dw[i + 1]);
        for (int j = 0; j < v.ny - 1; j++) v.ky[j] = 2.0 / (v.dh[j] + v.dh[j + 1]);
        for (int i = 0; i < v.nx; i++) v.ix[i] = 1.0 / v.dw[i];
        for (int j = 0; j < v.ny; j++) v.iy[j] = 1.0 / v.dh[j];
        const size_t nn = (size_t)v.pitch * v.ny;
        v.act.assign(nn, 0);
        v.bits.assign(nn, 0);
        if (l == 0) {
            for (int j = 0; j < v.ny; j++)
                for (int i = 0; i < v.nx; i++) v.act[i + j * v.pitch] = I.type[i + j * I.pitch] == T_FLUID;
        } else {
            const HostLevel& f = I.lev[l - 1];
            for (int J = 1; J <= v.NY; J++)
                for (int Ic = 1; Ic <= v.NX; Ic++) {
                    uint8_t a = 0;
                    for (int dj = 0; dj < v.cy; dj++)
                        for (int di = 0; di < v.cx; di++) {
                            int i = v.cx * (Ic - 1) + 1 + di, j = v.cy * (J - 1) + 1 + dj;
                            if (i <= f.NX && j <= f.NY) a |= f.act[i + j * f.pitch];
                        }
                    v.act[Ic + J * v.pitch] = a;
                }
        }
        for (int j = 1; j <= v.NY; j++)
            for (int i = 1; i <= v.NX; i++) {
                const int id = i + j * v.pitch;
                if (!v.act[id]) continue;
                uint8_t bt = 0;
                auto probe = [&](int ni, int nj, uint8_t ob, uint8_t gb) {
                    if (ni < 1 || ni > v.NX || nj < 1 || nj > v.NY) return;
                    const int nid = ni + nj * v.pitch;
                    if (l == 0) {
                        const uint8_t t = I.type[nid];
                        if (t == T_FLUID) bt |= ob;
                        if (t == T_GHOST) bt |= (uint8_t)(ob | gb);
                    } else if (v.act[nid]) {
                        bt |= ob;
                    }
                };
                probe(i + 1, j, B_E, G_E);
                probe(i - 1, j, B_W, G_W);
                probe(i, j + 1, B_N, G_N);
                probe(i, j - 1, B_S, G_S);
                v.bits[id] = bt;
            }
        if (l > 0) {
            HostLevel& f = I.lev[l - 1];
            f.pI.assign(f.nx, 0);
            f.pIn.assign(f.nx, 0);
            f.pwx.assign(f.nx, 0.0);
            f.psx.assign(f.nx, 1);
            f.pJ.assign(f.ny, 0);
            f.pJn.assign(f.ny, 0);
            f.pwy.assign(f.ny, 0.0);
            f.psy.assign(f.ny, 1);
            // ring centres are the mirror images of the first/last interior
            // centres: the neighbour beyond a domain side is the cell itself
            // with sign +1 (Neumann) or -1 (Dirichlet)
            for (int i = 1; i <= f.NX; i++) {
                if (v.cx == 1) {  // not coarsened in x: the coarse column of the same index
                    f.pI[i] = i;
                    f.pIn[i] = i;
                    f.pwx[i] = 0.0;
                    f.psx[i] = 1;
                    continue;
                }
                int Ic = (i + 1) / 2;
                int In = f.xc[i] < v.xc[Ic] ? Ic - 1 : Ic + 1;
                double w = (f.xc[i] - v.xc[Ic]) / (v.xc[In] - v.xc[Ic]);
                signed char sg = 1;
                if (In < 1) { sg = (I.dirmask & (1 << IFX_SIDE_W)) ? -1 : 1; In = Ic; }
                if (In > v.NX) { sg = (I.dirmask & (1 << IFX_SIDE_E)) ? -1 : 1; In = Ic; }
                f.pI[i] = Ic;
                f.pIn[i] = In;
                f.pwx[i] = w;
                f.psx[i] = sg;
            }
            for (int j = 1; j <= f.NY; j++) {
                if (v.cy == 1) {
                    f.pJ[j] = j;
                    f.pJn[j] = j;
                    f.pwy[j] = 0.0;
                    f.psy[j] = 1;
                    continue;
                }
                int Jc = (j + 1) / 2;
                int Jn = f.yc[j] < v.yc[Jc] ? Jc - 1 : Jc + 1;
                double w = (f.yc[j] - v.yc[Jc]) / (v.yc[Jn] - v.yc[Jc]);
                signed char sg = 1;
                if (Jn < 1) { sg = (I.dirmask & (1 << IFX_SIDE_S)) ? -1 : 1; Jn = Jc; }
                if (Jn > v.NY) { sg = (I.dirmask & (1 << IFX_SIDE_N)) ? -1 : 1; Jn = Jc; }
                f.pJ[j] = Jc;
                f.pJn[j] = Jn;
                f.pwy[j] = w;
                f.psy[j] = sg;
            }
        }
    }
}

// IBM ghost stub of cell id (weights follow on the device).
GhostDev ibm_stub(int id, int inst) {
    GhostDev g;
    std::memset(&g, 0, sizeof(g));
    g.cell = id;
    g.inst = inst;
    g.side = -1;
    g.qi[0] = g.qi[1] = -1;
    g.qown = -1;
    g.adj = -1;
    for (int k = 0; k < 4; k++) g.nb[k] = id;
    return g;
}

// Domain ghost relations (wall/inflow/slip/outflow per side, corners from the
// diagonal interior cell) and IBM ghost stubs, in row-major cell order.  A
// moving body's instance instead gets its IBM ghosts after the domain ghosts,
// in a fixed number of slots (the current ghosts in row-major order, then
// empty slots, cell -1) that the device refills every step.
void build_ghosts(Instance& I, int inst, std::vector<GhostDev>& out, std::vector<int>& ibm_list) {
    const int nx = I.nx, ny = I.ny, P = I.pitch;
    const ifx_config& c = I.cfg;
    I.ghost_beg = (int)out.size();
    I.n_ibm = 0;
    std::vector<int> ibm_cells;
    auto rule = [&](int side, int k_along, double* wu, double* wv, double* wp, double* cu, double* cv, int* qi,
                    double* qf) {
        const int bt = c.bc_type[side];
        const bool normal_is_u = (side == IFX_SIDE_W || side == IFX_SIDE_E);
        *qi = -1;
        *qf = 0.0;
        if (bt == IFX_BC_WALL || bt == IFX_BC_INFLOW) {
            *wu = -1.0; *cu = 2.0 * c.bc_u[side];
            *wv = -1.0; *cv = 2.0 * c.bc_v[side];
            *wp = 1.0;
        } else if (bt == IFX_BC_SLIP) {
            if (normal_is_u) { *wu = -1.0; *wv = 1.0; }
            else { *wu = 1.0; *wv = -1.0; }
            *cu = *cv = 0.0;
            *wp = 1.0;
        } else {
            *wu = -1.0; *wv = -1.0;
            *cu = *cv = 0.0;
            *qi = side * I.qstride + k_along;
            *qf = 2.0;
            *wp = -1.0;
        }
    };
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            const int id = i + j * P;
            const uint8_t t = I.type[id];
            if (t != T_DOMAIN && t != T_GHOST) continue;
            GhostDev g;
            std::memset(&g, 0, sizeof(g));
            g.cell = id;
            g.inst = inst;
            g.qi[0] = g.qi[1] = -1;
            g.qown = -1;
            g.adj = -1;
            for (int k = 0; k < 4; k++) g.nb[k] = id;
            if (t == T_GHOST) {
                if (I.moving) {
                    ibm_cells.push_back(id);
                    continue;
                }
                g.side = -1;
                ibm_list.push_back((int)out.size());
                I.n_ibm++;
                out.push_back(g);
                continue;
            }
            const bool W = i == 0, E = i == nx - 1, So = j == 0, N = j == ny - 1;
            int sd;
            if ((W || E) && (So || N)) sd = 4;
            else if (W) sd = IFX_SIDE_W;
            else if (E) sd = IFX_SIDE_E;
            else if (So) sd = IFX_SIDE_S;
            else sd = IFX_SIDE_N;
            g.side = sd;
            if (sd == 4) {
                const int di = (i == 0) ? 1 : nx - 2, dj = (j == 0) ? 1 : ny - 2;
                const int sa = (i == 0) ? IFX_SIDE_W : IFX_SIDE_E;
                const int sb = (j == 0) ? IFX_SIDE_S : IFX_SIDE_N;
                double wua, wva, wpa, cua, cva, qfa, wub, wvb, wpb, cub, cvb, qfb;
                int qia, qib;
                rule(sa, dj, &wua, &wva, &wpa, &cua, &cva, &qia, &qfa);
                rule(sb, di, &wub, &wvb, &wpb, &cub, &cvb, &qib, &qfb);
                g.nb[0] = di + dj * P;
                g.wu[0] = 0.5 * (wua + wub);
                g.wv[0] = 0.5 * (wva + wvb);
                g.wp[0] = 0.5 * (wpa + wpb);
                g.cu = 0.5 * (cua + cub);
                g.cv = 0.5 * (cva + cvb);
                g.qi[0] = qia;
                g.qf[0] = 0.5 * qfa;
                g.qi[1] = qib;
                g.qf[1] = 0.5 * qfb;
            } else {
                int ai = i, aj = j;
                if (sd == IFX_SIDE_W) ai = 1;
                if (sd == IFX_SIDE_E) ai = nx - 2;
                if (sd == IFX_SIDE_S) aj = 1;
                if (sd == IFX_SIDE_N) aj = ny - 2;
                const int k_along = (sd <= 1) ? j : i;
                g.nb[0] = ai + aj * P;
                g.adj = g.nb[0];
                rule(sd, k_along, &g.wu[0], &g.wv[0], &g.wp[0], &g.cu, &g.cv, &g.qi[0], &g.qf[0]);
                if (c.bc_type[sd] == IFX_BC_OUTFLOW) {
                    g.qown = g.qi[0];
                    g.qh = (sd <= 1) ? I.dx[ai] : I.dy[aj];
                }
            }
            out.push_back(g);
        }
    if (I.moving) {
        // slots: four times the ghosts now, and at least four per finest cell
        // width along the body's perimeter (Ramanujan's approximation)
        double h = 1e300;
        for (int i = 1; i <= I.NX; i++) h = std::min(h, I.dx[i]);
        for (int j = 1; j <= I.NY; j++) h = std::min(h, I.dy[j]);
        const double a = c.body_a, b = c.body_b;
        const double per = M_PI * (3.0 * (a + b) - std::sqrt((3.0 * a + b) * (a + 3.0 * b)));
        I.ibm_cap = (int)std::min(4.0 * I.NX * (double)I.NY,
                                  std::max(4.0 * (double)ibm_cells.size(), 4.0 * per / h)) + 64;
        I.ibm_beg = (int)out.size();
        I.n_ibm = (int)ibm_cells.size();
        for (int s = 0; s < I.ibm_cap; s++) {
            GhostDev g = ibm_stub(s < I.n_ibm ? ibm_cells[s] : -1, inst);
            ibm_list.push_back((int)out.size());
            out.push_back(g);
        }
    }
    I.ghost_cnt = (int)out.size() - I.ghost_beg;
}

// Body-surface samples in the body frame: parametric point on the ellipse,
// outward unit normal and arc-length weight (lx, ly, nlx, nly, ds) each.
std::vector<double> force_body_frame(const Instance& I) {
    const double a = I.cfg.body_a, b = I.cfg.body_b;
    const double dth = 2.0 * M_PI / FORCE_SAMPLES;
    std::vector<double> out(5 * (size_t)FORCE_SAMPLES);
    for (int k = 0; k < FORCE_SAMPLES; k++) {
        double t = dth * (k + 0.5);
        double ct = std::cos(t), st = std::sin(t);
        double nlx = ct / a, nly = st / b;
        double nl = std::sqrt(nlx * nlx + nly * nly);
        double* o = out.data() + 5 * (size_t)k;
        o[0] = a * ct;
        o[1] = b * st;
        o[2] = nlx / nl;
        o[3] = nly / nl;
        o[4] = std::sqrt(a * a * st * st + b * b * ct * ct) * dth;
    }
    return out;
}

// Body-surface samples for drag/lift at the current pose: the body-frame
// samples placed on the grid, with the bilinear bases/weights of the pressure
// sample and of the velocity probe (same formulas as the oracle; the device
// redoes them every step for a moving body).
std::vector<ForceSample> build_force_table(const Instance& I) {
    std::vector<ForceSample> out;
    if (I.cfg.body != IFX_BODY_ELLIPSE) return out;
    const int nx = I.nx, ny = I.ny, P = I.pitch;
    auto locate = [](const std::vector<double>& cc, int n, double x) {
        int i0 = (int)(std::upper_bound(cc.begin() + 1, cc.begin() + n - 1, x) - cc.begin()) - 1;
        return std::min(std::max(i0, 0), n - 2);
    };
    const std::vector<double> bf = force_body_frame(I);
    out.resize(FORCE_SAMPLES);
    for (int k = 0; k < FORCE_SAMPLES; k++) {
        const double* o = bf.data() + 5 * (size_t)k;
        double lx = o[0], ly = o[1], nlx = o[2], nly = o[3], ds = o[4];
        double xs = I.cfg.body_cx + lx * I.cs - ly * I.sn;
        double ys = I.cfg.body_cy + lx * I.sn + ly * I.cs;
        double nxw = nlx * I.cs - nly * I.sn, nyw = nlx * I.sn + nly * I.cs;
        int i0 = locate(I.xc, nx, xs), j0 = locate(I.yc, ny, ys);
        // the larger width of the two bracketing cells per direction: the same
        // for a surface point and its mirror image on a symmetric grid
        double h = std::max(std::max(I.dx[i0], I.dx[i0 + 1]), std::max(I.dy[j0], I.dy[j0 + 1]));
        double del = 1.5 * h;
        ForceSample f;
        f.c0 = i0 + j0 * P;
        f.xi0 = (xs - I.xc[i0]) / (I.xc[i0 + 1] - I.xc[i0]);
        f.et0 = (ys - I.yc[j0]) / (I.yc[j0 + 1] - I.yc[j0]);
        double xq = xs + del * nxw, yq = ys + del * nyw;
        int i1 = locate(I.xc, nx, xq), j1 = locate(I.yc, ny, yq);
        f.c1 = i1 + j1 * P;
        f.xi1 = (xq - I.xc[i1]) / (I.xc[i1 + 1] - I.xc[i1]);
        f.et1 = (yq - I.yc[j1]) / (I.yc[j1 + 1] - I.yc[j1]);
        f.nx = nxw;
        f.ny = nyw;
        f.ds = ds;
        f.del = del;
        out[k] = f;
    }
    return out;
}

// Host initial condition (same formulas as initializeKernel for the vortex,
// src/include/preSim.cu:70-73).
void initial_field(const Instance& I, std::vector<double>& u, std::vector<double>& v) {
    const int nx = I.nx, ny = I.ny, P = I.pitch;
    u.assign(I.ncell, 0.0);
    v.assign(I.ncell, 0.0);
    const ifx_config& c = I.cfg;
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            const int id = i + j * P;
            const uint8_t t = I.type[id];
            if (c.init == IFX_INIT_VORTEX) {
                if (t == T_SOLID || t == T_GHOST) continue;
                double r = std::sqrt(std::pow(I.xc[i] - 0.5, 2.0) + std::pow(I.yc[j] - 0.5, 2.0));
                double r0 = 0.1;
                u[id] = 1.0 - 0.25 * (I.yc[j] - 0.5) * std::exp((1.0 - std::pow(r / r0, 2.0)) / 2.0);
                v[id] = 0.25 * (I.xc[i] - 0.5) * std::exp((1.0 - std::pow(r / r0, 2.0)) / 2.0);
            } else if (c.init == IFX_INIT_UNIFORM) {
                if (t == T_FLUID || t == T_DOMAIN) u[id] = c.bc_u[IFX_SIDE_W];
            }
        }
}

ifx_status validate(const ifx_config* c) {
    if (c->nx < 4 || c->ny < 4) return set_error(IFX_ERR_ARG, "method mode needs nx, ny >= 4");
    if (IFX_PADDED_CELLS(c->nx, c->ny) > IFX_MAX_CELLS)
        return set_error(IFX_ERR_ARG, "nx, ny give more than IFX_MAX_CELLS cells (rows padded to 32)");
    if (!(c->dt > 0) || !(c->re > 0)) return set_error(IFX_ERR_ARG, "dt and Re must be positive");
    if (c->mg_pre < 1 || c->mg_post < 1) return set_error(IFX_ERR_ARG, "multigrid sweeps must be >= 1");
    if (!(c->mg_omega > 0 && c->mg_omega < 2)) return set_error(IFX_ERR_ARG, "multigrid omega must lie in (0, 2)");
    if (c->coarse_sweeps < 1 || c->coarse_sweeps > 10000) return set_error(IFX_ERR_ARG, "coarse sweeps must lie in 1..10000");
    if (c->mixed_inner < 2) return set_error(IFX_ERR_ARG, "mixed_inner must be >= 2");
    if (!(c->restart_drop > 0 && c->restart_drop < 1) || c->restart_every < 1)
        return set_error(IFX_ERR_ARG, "defect correction: restart_drop in (0, 1), restart_every >= 1");
    if (c->ad_itermax < 1 || c->ppe_itermax < 0) return set_error(IFX_ERR_ARG, "bad iteration caps");
    if (c->body == IFX_BODY_ELLIPSE && !(c->body_a > 0 && c->body_b > 0))
        return set_error(IFX_ERR_ARG, "body semi-axes must be positive");
    for (int s = 0; s < 4; s++)
        if (c->bc_type[s] < 0 || c->bc_type[s] > 3) return set_error(IFX_ERR_ARG, "bad boundary type");
    bool outflow = false;
    for (int s = 0; s < 4; s++) outflow = outflow || c->bc_type[s] == IFX_BC_OUTFLOW;
    // Without an outflow side the pressure is fixed only up to a constant, and
    // the solve makes the right-hand side compatible by removing its
    // area-weighted mean.  With a body the eliminated ghost rows make the
    // operator non-symmetric: its compatibility condition is no longer the
    // area-weighted mean, and the solve stalls at its iteration cap.
    if (c->body != IFX_BODY_NONE && !outflow)
        return set_error(IFX_ERR_ARG, "a body needs an outflow side (Dirichlet pressure) in method mode");
    if (c->ppe_method != IFX_PPE_JACOBI)
        return set_error(IFX_ERR_ARG, "PPE-Method point-gs / line-sor selects the REFERENCE-mode pressure solve; "
                                      "method mode solves the pressure with multigrid-preconditioned BiCGSTAB");
    if (c->motion != IFX_MOTION_NONE) {
        if (c->motion != IFX_MOTION_PRESCRIBED) return set_error(IFX_ERR_ARG, "bad motion type");
        if (c->body != IFX_BODY_ELLIPSE) return set_error(IFX_ERR_ARG, "body motion needs a body");
        const double m[9] = {c->motion_u, c->motion_v, c->motion_amp_x, c->motion_amp_y, c->motion_amp_deg,
                             c->motion_freq, c->motion_phase_x, c->motion_phase_y, c->motion_phase_deg};
        for (double x : m)
            if (!std::isfinite(x)) return set_error(IFX_ERR_ARG, "motion parameters must be finite");
    }
    return IFX_OK;
}

// -------------------------------------------------------- method: create

template <typename T>
ifx_status alloc_level_fields(ifx_solver* S, HostLevel& L) {
    const size_t nn = (size_t)L.pitch * L.ny;
    T *e = nullptr, *e2 = nullptr, *r = nullptr;
    IFX_TRY(dalloc(S, &e, nn));
    IFX_TRY(dalloc(S, &e2, nn));
    IFX_TRY(dalloc(S, &r, nn));
    L.d_e = e;
    L.d_e2 = e2;
    L.d_r = r;
    return IFX_OK;
}

int max_pred_pairs(const ifx_solver* S);
int max_ppe_bodies(const ifx_solver* S);

// Plan and grid of the persistent per-step kernel (co-resident blocks only).
ifx_status setup_persistent(ifx_solver* S) {
    if (S->lmax > kMaxLevels) return IFX_OK;
    int coop = 0, sms = 0, bps = 0;
    CUDA_TRY(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, S->device));
    CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, S->device));
    if (!coop) return IFX_OK;
    if (S->prec == IFX_PREC_FP64) CUDA_TRY(persist_occupancy<double>(&bps, S->sub_bytes));
    else CUDA_TRY(persist_occupancy<float>(&bps, S->sub_bytes));
    if (bps < 1) return IFX_OK;
    S->persist_grid = sms * std::min(bps, 4);
    if (S->persist_grid > 64 * 32) S->persist_grid = 64 * 32;
    S->persist_full = S->persist_grid;
    S->persist_sms = sms;
    IFX_TRY(dalloc(S, &S->dBar, 1));
    PersistPlan& P = S->plan;
    std::memset(&P, 0, sizeof(P));
    P.I = S->dI;
    P.S = S->dS;
    P.LV = S->dLV;
    P.G = S->dG;
    P.gval = S->dGval;
    P.part = S->dPart;
    P.fpart = S->dFpart;
    P.ftick = S->dFtick;
    P.t0 = S->dT0;
    P.nt0 = S->nt0;
    for (int l = 1; l < S->lmax; l++) {
        P.tsm[l] = S->dTsm[l];
        P.ntsm[l] = S->ntsm[l];
        P.tre[l] = S->dTre[l];
        P.ntre[l] = S->ntre[l];
    }
    P.tall = S->dTall;
    P.sub = S->dSub;
    P.bar = S->dBar;
    P.ng = S->ng;
    P.ninst = (int)S->inst.size();
    P.lmax = S->lmax;
    P.mg_pre = S->mg_pre;
    P.mg_post = S->mg_post;
    P.sub_bytes = S->sub_bytes;
    P.spin_limit = kSpinLimit;
    P.withhold_arrival = 0;
    P.pred_pairs = max_pred_pairs(S);
    P.ppe_bodies = max_ppe_bodies(S);
    CUDA_TRY(cudaStreamSynchronize(S->stream));
    return IFX_OK;
}

ifx_status create_method(ifx_solver* S, int n, const ifx_config* cfgs, const double* const* xfs,
                         const double* const* yfs) {
    S->mode = IFX_MODE_METHOD;
    S->prec = cfgs[0].precision;
    S->mg_pre = cfgs[0].mg_pre;
    S->mg_post = cfgs[0].mg_post;
    for (int k = 0; k < n; k++) {
        IFX_TRY(validate(&cfgs[k]));
        if (cfgs[k].mode != IFX_MODE_METHOD) return set_error(IFX_ERR_ARG, "a batch holds method-mode instances only");
        if (cfgs[k].precision != S->prec || cfgs[k].mg_pre != S->mg_pre || cfgs[k].mg_post != S->mg_post)
            return set_error(IFX_ERR_ARG, "instances of one batch share precision and multigrid sweeps");
    }
    S->inst.resize(n);
    std::vector<InstDev> hI(n);
    for (int k = 0; k < n; k++) {
        Instance& I = S->inst[k];
        I.cfg = cfgs[k];
        I.NX = I.cfg.nx;
        I.NY = I.cfg.ny;
        I.nx = I.NX + 2;
        I.ny = I.NY + 2;
        I.pitch = round_up(I.nx, 32);
        I.ncell = (size_t)I.pitch * I.ny;
        I.qstride = std::max(I.nx, I.ny);
        build_grid(I, xfs[k], yfs[k]);
        for (int s = 0; s < 4; s++)
            if (I.cfg.bc_type[s] == IFX_BC_OUTFLOW) I.dirmask |= 1 << s;
        I.singular = I.dirmask == 0;
        if (I.cfg.body == IFX_BODY_ELLIPSE) {
            const double th = I.cfg.body_angle_deg * M_PI / 180.0;
            I.cs = std::cos(th);
            I.sn = std::sin(th);
            I.ia2 = 1.0 / (I.cfg.body_a * I.cfg.body_a);
            I.ib2 = 1.0 / (I.cfg.body_b * I.cfg.body_b);
        }
        I.moving = I.cfg.motion == IFX_MOTION_PRESCRIBED;
        MotionDef mo{};
        Pose p0{};
        if (I.moving) {
            // the pose at t = 0 from the same function as every later step
            mo = motion_def(I.cfg);
            p0 = pose_at(mo.x0, mo.y0, mo.th0, mo.u, mo.v, mo.ax, mo.ay, mo.ath, mo.f, mo.w, mo.phx, mo.phy, mo.pha, 0.0);
            I.cs = p0.c;
            I.sn = p0.s;
        }
        InstDev& d = I.dev;
        std::memset(&d, 0, sizeof(d));
        d.NX = I.NX; d.NY = I.NY; d.nx = I.nx; d.ny = I.ny; d.pitch = I.pitch;
        d.singular = I.singular;
        d.dirmask = I.dirmask;
        d.body = I.cfg.body == IFX_BODY_ELLIPSE;
        d.dt = I.cfg.dt;
        d.re = I.cfg.re;
        d.dtre = I.cfg.dt / I.cfg.re;
        d.idt = 1.0 / I.cfg.dt;
        d.omega = I.cfg.mg_omega;
        d.ppe_tol = I.cfg.ppe_tol;
        d.ad_itermax = I.cfg.ad_itermax;
        d.ppe_itermax = I.cfg.ppe_itermax;
        d.mixed_inner = I.cfg.mixed_inner;
        d.coarse_sweeps = I.cfg.coarse_sweeps;
        d.restart_drop = I.cfg.restart_drop;
        d.restart_every = I.cfg.restart_every;
        d.uc = I.cfg.outflow_uc;
        d.bcx = I.cfg.body_cx; d.bcy = I.cfg.body_cy; d.ba = I.cfg.body_a; d.bb = I.cfg.body_b;
        d.bcs = I.cs; d.bsn = I.sn; d.bia2 = I.ia2; d.bib2 = I.ib2;
        if (I.moving) {
            d.moving = 1;
            d.mo_x0 = mo.x0; d.mo_y0 = mo.y0; d.mo_th0 = mo.th0; d.mo_u = mo.u; d.mo_v = mo.v;
            d.mo_ax = mo.ax; d.mo_ay = mo.ay; d.mo_ath = mo.ath; d.mo_f = mo.f; d.mo_w = mo.w;
            d.mo_phx = mo.phx; d.mo_phy = mo.phy; d.mo_pha = mo.pha;
            d.bu = p0.u; d.bv = p0.v; d.bw = p0.w;  // the initial ghosts see the wall velocity at t = 0
            int* fresh = nullptr;
            IFX_TRY(dalloc(S, &fresh, I.ncell));
            d.fresh = fresh;
        }
        d.fref = 0.5 * I.cfg.force_ref_u * I.cfg.force_ref_u * I.cfg.force_ref_len;
        const size_t nc = I.ncell;
        IFX_TRY(dalloc(S, &d.u, nc)); IFX_TRY(dalloc(S, &d.v, nc));
        IFX_TRY(dalloc(S, &d.u2, nc)); IFX_TRY(dalloc(S, &d.v2, nc));
        IFX_TRY(dalloc(S, &d.Us, nc)); IFX_TRY(dalloc(S, &d.Vs, nc));
        IFX_TRY(dalloc(S, &d.U, nc)); IFX_TRY(dalloc(S, &d.V, nc));
        IFX_TRY(dalloc(S, &d.Nu, nc)); IFX_TRY(dalloc(S, &d.Nv, nc));
        IFX_TRY(dalloc(S, &d.ru, nc)); IFX_TRY(dalloc(S, &d.rv, nc));
        IFX_TRY(dalloc(S, &d.p, nc)); IFX_TRY(dalloc(S, &d.b, nc));
        IFX_TRY(dalloc(S, &d.pold, nc)); IFX_TRY(dalloc(S, &d.pold2, nc));
        IFX_TRY(dalloc(S, &d.dup, nc)); IFX_TRY(dalloc(S, &d.dvp, nc));
        IFX_TRY(dalloc(S, &d.div, nc)); IFX_TRY(dalloc(S, &d.iblank, nc));
        if (S->prec == IFX_PREC_MIXED)
            for (float** a : {&d.du, &d.dv, &d.du2, &d.dv2, &d.rfu, &d.rfv}) IFX_TRY(dalloc(S, a, nc));
        for (void** kv : {&d.kr, &d.krh, &d.kp, &d.kv, &d.ks, &d.kt, &d.kph, &d.ksh}) {
            if (S->prec == IFX_PREC_FP64) {
                double* a = nullptr;
                IFX_TRY(dalloc(S, &a, nc));
                *kv = a;
            } else {
                float* a = nullptr;
                IFX_TRY(dalloc(S, &a, nc));
                *kv = a;
            }
        }
        double *xf_d = nullptr, *yf_d = nullptr, *xc_d = nullptr, *yc_d = nullptr, *dx_d = nullptr,
               *dy_d = nullptr, *fx_d = nullptr, *gx_d = nullptr, *fy_d = nullptr, *gy_d = nullptr;
        IFX_TRY(dupload(S, &xf_d, I.xf)); IFX_TRY(dupload(S, &yf_d, I.yf));
        IFX_TRY(dupload(S, &xc_d, I.xc)); IFX_TRY(dupload(S, &yc_d, I.yc));
        IFX_TRY(dupload(S, &dx_d, I.dx)); IFX_TRY(dupload(S, &dy_d, I.dy));
        IFX_TRY(dupload(S, &fx_d, I.fx)); IFX_TRY(dupload(S, &gx_d, I.gx));
        IFX_TRY(dupload(S, &fy_d, I.fy)); IFX_TRY(dupload(S, &gy_d, I.gy));
        d.xf = xf_d; d.yf = yf_d; d.xc = xc_d; d.yc = yc_d; d.dx = dx_d; d.dy = dy_d;
        d.fx = fx_d; d.gx = gx_d; d.fy = fy_d; d.gy = gy_d;
        uint8_t* type_d = nullptr;
        IFX_TRY(dalloc(S, &type_d, nc));
        d.type = type_d;
        IFX_TRY(dalloc(S, &d.qbu, 4 * (size_t)I.qstride));
        IFX_TRY(dalloc(S, &d.qbv, 4 * (size_t)I.qstride));
        hI[k] = d;
    }
    IFX_TRY(dalloc(S, &S->dI, n));
    CUDA_TRY(cudaMemcpyAsync(S->dI, hI.data(), n * sizeof(InstDev), cudaMemcpyHostToDevice, S->stream));
    // tagging on the device, then the type arrays back to the host
    for (int k = 0; k < n; k++) {
        Instance& I = S->inst[k];
        uint8_t* type_d = const_cast<uint8_t*>(I.dev.type);
        CUDA_TRY(launch_tag(S->dI, k, I.nx * I.ny, type_d, S->stream));
        CUDA_TRY(launch_mark_ghosts(S->dI, k, I.NX * I.NY, type_d, S->stream));
        S->launches += 2;
        I.type.assign(I.ncell, 0);
        CUDA_TRY(cudaMemcpyAsync(I.type.data(), type_d, I.ncell, cudaMemcpyDeviceToHost, S->stream));
    }
    CUDA_TRY(cudaStreamSynchronize(S->stream));
    // ghost tables, hierarchy, tiles
    std::vector<GhostDev> hG;
    std::vector<int> hIbm;
    std::vector<LevelDev> hLV;
    std::vector<Tile> hT0;
    int lmax = 0;
    for (int k = 0; k < n; k++) {
        Instance& I = S->inst[k];
        I.n_fluid = 0;
        I.area = 0.0;
        for (int j = 1; j <= I.NY; j++)
            for (int i = 1; i <= I.NX; i++)
                if (I.type[i + j * I.pitch] == T_FLUID) {
                    I.n_fluid++;
                    I.area += I.dx[i] * I.dy[j];
                }
        build_ghosts(I, k, hG, hIbm);
        build_levels(I);
        lmax = std::max(lmax, (int)I.lev.size());
    }
    S->lmax = lmax;
    S->ng = (int)hG.size();
    S->nibm = (int)hIbm.size();
    IFX_TRY(dupload(S, &S->dG, hG));
    IFX_TRY(dupload(S, &S->dIbm, hIbm));
    IFX_TRY(dalloc(S, &S->dGval, 3 * (size_t)std::max(1, S->ng)));
    IFX_TRY(dalloc(S, &S->dBiIp, 4 * (size_t)std::max(1, S->nibm)));
    std::vector<std::vector<Tile>> tsm(lmax), tre(lmax), tsmW(lmax), treW(lmax);
    std::vector<Tile> hT0W;
    std::vector<Tile> hTall;
    std::vector<int> hSub;
    for (int k = 0; k < n; k++) {
        Instance& I = S->inst[k];
        InstDev& d = I.dev;
        I.lev_base = (int)hLV.size();
        std::vector<int> gidx(I.ncell, -1);
        for (int g = I.ghost_beg; g < I.ghost_beg + I.ghost_cnt; g++)
            if (hG[g].side < 0 && hG[g].cell >= 0) gidx[hG[g].cell] = g;
        int* gidx_d = nullptr;
        IFX_TRY(dupload(S, &gidx_d, gidx));
        d.gidx = gidx_d;
        const int nl = (int)I.lev.size();
        // first level handled inside one block per instance (>= 1, <= coarsest): at
        // most SUB_MAX_CELLS (FP64: SUB_MAX_CELLS_FP64) cells, and it and every
        // coarser level staged in shared memory within SUB_SMEM_MAX bytes
        const int tsz = S->prec == IFX_PREC_FP64 ? 8 : 4;
        const long long sub_max = S->prec == IFX_PREC_FP64 ? SUB_MAX_CELLS_FP64 : SUB_MAX_CELLS;
        auto staged = [&](int from) {
            size_t b = SUB_HDR_BYTES;
            for (int l = from; l < nl; l++) b += sub_level_bytes(I.lev[l].nx, I.lev[l].ny, tsz);
            return b;
        };
        int lb = nl - 1;
        for (int l = 1; l < nl; l++)
            if ((long long)I.lev[l].NX * I.lev[l].NY <= sub_max && staged(l) <= (size_t)SUB_SMEM_MAX) {
                lb = l;
                break;
            }
        if (nl < 2 || nl - lb > kSubLevels || staged(lb) > (size_t)SUB_SMEM_MAX ||
            (long long)I.lev[nl - 1].NX * I.lev[nl - 1].NY > (long long)TILE_THREADS * SUB_COARSE_PER_THREAD)
            return set_error(IFX_ERR_ARG, "grid too small or too elongated for the multigrid hierarchy");
        S->sub_bytes = std::max(S->sub_bytes, (int)staged(lb));
        {   // cluster V-cycle: levels 0 .. lb-1 distributed, then the sub-cycle area
            const int nd = lb;
            size_t cb = (size_t)-1;
            if (nd <= CMG_MAX_LEVELS) {
                int nxs[CMG_MAX_LEVELS], nys[CMG_MAX_LEVELS];
                for (int l = 0; l < nd; l++) {
                    nxs[l] = I.lev[l].nx;
                    nys[l] = I.lev[l].ny;
                }
                cb = cluster_vcycle_bytes(nd, nxs, nys, tsz, staged(lb));
            }
            S->cmg_bytes = std::max(S->cmg_bytes, cb);
        }
        for (int l = 0; l < nl; l++) {
            HostLevel& L = I.lev[l];
            IFX_TRY(dupload(S, &L.d_kx, L.kx)); IFX_TRY(dupload(S, &L.d_ky, L.ky));
            IFX_TRY(dupload(S, &L.d_ix, L.ix)); IFX_TRY(dupload(S, &L.d_iy, L.iy));
            IFX_TRY(dupload(S, &L.d_dw, L.dw)); IFX_TRY(dupload(S, &L.d_dh, L.dh));
            IFX_TRY(dupload(S, &L.d_kxf, to_f(L.kx))); IFX_TRY(dupload(S, &L.d_kyf, to_f(L.ky)));
            IFX_TRY(dupload(S, &L.d_ixf, to_f(L.ix))); IFX_TRY(dupload(S, &L.d_iyf, to_f(L.iy)));
            IFX_TRY(dupload(S, &L.d_dwf, to_f(L.dw))); IFX_TRY(dupload(S, &L.d_dhf, to_f(L.dh)));
            IFX_TRY(dupload(S, &L.d_cew, face_pairs<double, double2>(L.kx, L.ix)));
            IFX_TRY(dupload(S, &L.d_cns, face_pairs<double, double2>(L.ky, L.iy)));
            IFX_TRY(dupload(S, &L.d_cewf, face_pairs<float, float2>(L.kx, L.ix)));
            IFX_TRY(dupload(S, &L.d_cnsf, face_pairs<float, float2>(L.ky, L.iy)));
            IFX_TRY(dupload(S, &L.d_bits, L.bits));
            if (I.moving && l > 0) IFX_TRY(dupload(S, &L.d_act, L.act));
            if (S->prec == IFX_PREC_FP64) IFX_TRY(alloc_level_fields<double>(S, L));
            else IFX_TRY(alloc_level_fields<float>(S, L));
            if (l + 1 < nl) {
                IFX_TRY(dupload(S, &L.d_pI, L.pI)); IFX_TRY(dupload(S, &L.d_pIn, L.pIn));
                IFX_TRY(dupload(S, &L.d_pJ, L.pJ)); IFX_TRY(dupload(S, &L.d_pJn, L.pJn));
                IFX_TRY(dupload(S, &L.d_pwx, L.pwx)); IFX_TRY(dupload(S, &L.d_pwy, L.pwy));
                IFX_TRY(dupload(S, &L.d_pwxf, to_f(L.pwx))); IFX_TRY(dupload(S, &L.d_pwyf, to_f(L.pwy)));
                IFX_TRY(dupload(S, &L.d_psx, L.psx)); IFX_TRY(dupload(S, &L.d_psy, L.psy));
            }
            LevelDev ld;
            std::memset(&ld, 0, sizeof(ld));
            ld.NX = L.NX; ld.NY = L.NY; ld.nx = L.nx; ld.ny = L.ny; ld.pitch = L.pitch;
            ld.inst = k;
            ld.depth = l;
            ld.dirmask = I.dirmask;
            ld.kx = L.d_kx; ld.ky = L.d_ky; ld.ix = L.d_ix; ld.iy = L.d_iy; ld.dw = L.d_dw; ld.dh = L.d_dh;
            ld.kxf = L.d_kxf; ld.kyf = L.d_kyf; ld.ixf = L.d_ixf; ld.iyf = L.d_iyf; ld.dwf = L.d_dwf; ld.dhf = L.d_dhf;
            ld.cew = L.d_cew; ld.cns = L.d_cns; ld.cewf = L.d_cewf; ld.cnsf = L.d_cnsf;
            ld.bits = L.d_bits;
            ld.act = L.d_act;
            ld.e = L.d_e; ld.e2 = L.d_e2; ld.r = L.d_r;
            ld.pI = L.d_pI; ld.pIn = L.d_pIn; ld.pJ = L.d_pJ; ld.pJn = L.d_pJn;
            ld.pwx = L.d_pwx; ld.pwy = L.d_pwy; ld.pwxf = L.d_pwxf; ld.pwyf = L.d_pwyf;
            ld.psx = L.d_psx; ld.psy = L.d_psy;
            ld.cx = L.cx;
            ld.cy = L.cy;
            ld.child = (l + 1 < nl) ? I.lev_base + l + 1 : -1;
            ld.parent = (l > 0) ? I.lev_base + l - 1 : -1;
            // tiles
            const int lv = I.lev_base + l;
            std::vector<Tile> tl;
            std::vector<Tile> tw;  // wide tiles of the multigrid phases
            for (int j0 = 0; j0 < L.ny; j0 += TILE_Y)
                for (int i0 = 0; i0 < L.nx; i0 += TILE_X) tl.push_back(Tile{k, lv, i0, j0});
            for (int j0 = 0; j0 < L.ny; j0 += TILE_Y * MG_ROWS_WIDE)
                for (int i0 = 0; i0 < L.nx; i0 += TILE_X) tw.push_back(Tile{k, lv, i0, j0});
            ld.tbeg = (int)hTall.size();
            ld.tcnt = (int)tl.size();
            hTall.insert(hTall.end(), tl.begin(), tl.end());
            hLV.push_back(ld);
            if (l == 0) {
                I.tile_beg = (int)hT0.size();
                I.tile_cnt = (int)tl.size();
                if (I.tile_cnt >= 4 * 256) S->wide_sums = 1;  // four rows per thread of a 256-thread reduction
                hT0.insert(hT0.end(), tl.begin(), tl.end());
                hT0W.insert(hT0W.end(), tw.begin(), tw.end());
            } else {
                // tile phases: restriction into every level down to the first
                // small one (tiles of the finer level starting at (1, 1), so that
                // the children of a coarse cell share a tile), smoothing and
                // prolongation above it
                if (l <= lb) {
                    const HostLevel& f = I.lev[l - 1];
                    for (int j0 = 1; j0 <= f.NY; j0 += TILE_Y)
                        for (int i0 = 1; i0 <= f.NX; i0 += TILE_X) tre[l].push_back(Tile{k, lv - 1, i0, j0});
                    for (int j0 = 1; j0 <= f.NY; j0 += TILE_Y * MG_ROWS_WIDE)
                        for (int i0 = 1; i0 <= f.NX; i0 += TILE_X) treW[l].push_back(Tile{k, lv - 1, i0, j0});
                }
                if (l < lb) tsm[l].insert(tsm[l].end(), tl.begin(), tl.end());
                if (l < lb) tsmW[l].insert(tsmW[l].end(), tw.begin(), tw.end());
            }
        }
        hSub.push_back(I.lev_base + lb);
        d.lev0 = I.lev_base;
        d.nlev = nl;
        d.tile_beg = I.tile_beg;
        d.tile_cnt = I.tile_cnt;
        d.ghost_beg = I.ghost_beg;
        d.ghost_cnt = I.ghost_cnt;
        d.n_fluid = I.n_fluid;
        d.area = I.area;
        d.ad_lim = I.cfg.ad_tol * std::max(1, I.n_fluid);
        {
            std::vector<ForceSample> fs = build_force_table(I);
            ForceSample* fs_d = nullptr;
            if (!fs.empty()) IFX_TRY(dupload(S, &fs_d, fs));
            d.fs = fs_d;
            if (I.moving) {
                double* fsb = nullptr;
                IFX_TRY(dupload(S, &fsb, force_body_frame(I)));
                d.fsb = fsb;
            }
        }
        d.ibm_beg = I.ibm_beg;
        d.ibm_cap = I.ibm_cap;
        d.sub_lb = (lb >= 1 && lb < nl) ? lb : 0;
        d.kx = I.lev[0].d_kx; d.ky = I.lev[0].d_ky; d.ix = I.lev[0].d_ix; d.iy = I.lev[0].d_iy;
        {   // the implicit predictor's coefficients, each formed as the kernels formed it per cell
            const HostLevel& L0 = I.lev[0];
            const double dtre = d.dtre;
            std::vector<double2> ax(L0.kx.size()), ay(L0.ky.size());
            std::vector<double> cs(L0.kx.size());
            for (size_t i = 0; i < ax.size(); i++) {
                ax[i].x = dtre * (L0.kx[i] * L0.ix[i]);
                ax[i].y = i > 0 ? dtre * (L0.kx[i - 1] * L0.ix[i]) : 0.0;
                cs[i] = (1.0 + ax[i].x) + ax[i].y;
            }
            for (size_t j = 0; j < ay.size(); j++) {
                ay[j].x = dtre * (L0.ky[j] * L0.iy[j]);
                ay[j].y = j > 0 ? dtre * (L0.ky[j - 1] * L0.iy[j]) : 0.0;
            }
            double2 *ax_d = nullptr, *ay_d = nullptr;
            double* cs_d = nullptr;
            IFX_TRY(dupload(S, &ax_d, ax));
            IFX_TRY(dupload(S, &ay_d, ay));
            IFX_TRY(dupload(S, &cs_d, cs));
            d.pax = ax_d; d.pay = ay_d; d.pcs = cs_d;
        }
        hI[k] = d;
    }
    IFX_TRY(dupload(S, &S->dLV, hLV));
    S->hLV = hLV;
    {   // staged smoothing (TMA) on the mixed path, where it measured faster
        // (FP64 32x8 tiles: no gain); IFX_TMA=0 keeps the plain tile loads
        const char* e = std::getenv("IFX_TMA");
        std::vector<CUtensorMap> maps;
        if (S->prec == IFX_PREC_MIXED && !(e && e[0] == '0') && tensor_maps(hLV, 4, maps)) {
            IFX_TRY(dupload(S, &S->dTmap, maps));
            IFX_TRY(dalloc(S, &S->dErr, 1));
        }
    }
    IFX_TRY(dupload(S, &S->dT0, hT0));
    S->nt0 = (int)hT0.size();
    S->dTsm.assign(lmax, nullptr);
    S->dTre.assign(lmax, nullptr);
    S->ntsm.assign(lmax, 0);
    S->ntre.assign(lmax, 0);
    for (int l = 1; l < lmax; l++) {
        IFX_TRY(dupload(S, &S->dTsm[l], tsm[l]));
        IFX_TRY(dupload(S, &S->dTre[l], tre[l]));
        S->ntsm[l] = (int)tsm[l].size();
        S->ntre[l] = (int)tre[l].size();
    }
    IFX_TRY(dupload(S, &S->dT0W, hT0W));
    S->nt0W = (int)hT0W.size();
    S->dTsmW.assign(lmax, nullptr);
    S->dTreW.assign(lmax, nullptr);
    S->ntreW.assign(lmax, 0);
    S->ntsmW.assign(lmax, 0);
    for (int l = 1; l < lmax; l++) {
        IFX_TRY(dupload(S, &S->dTsmW[l], tsmW[l]));
        IFX_TRY(dupload(S, &S->dTreW[l], treW[l]));
        S->ntreW[l] = (int)treW[l].size();
        S->ntsmW[l] = (int)tsmW[l].size();
    }
    S->hT0full = hT0;
    S->hT0Wfull = hT0W;
    S->hTsmFull = tsm;
    S->hTreFull = tre;
    S->hTsmWFull = tsmW;
    S->hTreWFull = treW;
    S->in_lists.assign(n, 1);
    S->listed = n;
    IFX_TRY(dupload(S, &S->dTall, hTall));
    IFX_TRY(dupload(S, &S->dSub, hSub));
    {   // shared-memory images of the small levels, one buffer for all instances
        std::vector<unsigned char> all;
        std::vector<size_t> at(n);
        for (int k = 0; k < n; k++) {
            const Instance& I = S->inst[k];
            const std::vector<unsigned char> img = S->prec == IFX_PREC_FP64 ? sub_image<double>(I, hSub[k] - I.lev_base)
                                                                            : sub_image<float>(I, hSub[k] - I.lev_base);
            at[k] = all.size();
            all.insert(all.end(), img.begin(), img.end());
            hI[k].sub_img_bytes = (int)img.size();
        }
        unsigned char* d_img = nullptr;
        IFX_TRY(dupload(S, &d_img, all));
        for (int k = 0; k < n; k++) {
            hI[k].sub_img = d_img + at[k];
            const LevelDev& L = hLV[hSub[k]];  // the first small level
            SubHdr h0;
            std::memcpy(&h0, all.data() + at[k], sizeof(h0));
            hI[k].sub_ge = L.e;
            hI[k].sub_ge2 = L.e2;
            hI[k].sub_gr = L.r;
            hI[k].sub_gpitch = L.pitch;
            hI[k].sub_oe = (int)(h0.base + h0.o.e);
            hI[k].sub_or = (int)(h0.base + h0.o.r);
            hI[k].sub_nx = h0.nx;
            hI[k].sub_ny = h0.ny;
            hI[k].sub_child = h0.child;
            InstDev& dv = S->inst[k].dev;
            dv.sub_img = hI[k].sub_img;
            dv.sub_img_bytes = hI[k].sub_img_bytes;
            dv.sub_ge = L.e; dv.sub_ge2 = L.e2; dv.sub_gr = L.r; dv.sub_gpitch = L.pitch;
            dv.sub_oe = hI[k].sub_oe; dv.sub_or = hI[k].sub_or;
            dv.sub_nx = h0.nx; dv.sub_ny = h0.ny; dv.sub_child = h0.child;
        }
    }
    if (S->prec == IFX_PREC_FP64) CUDA_TRY(subcycle_smem_limit<double>(S->sub_bytes));
    else CUDA_TRY(subcycle_smem_limit<float>(S->sub_bytes));
    S->cmg_ok = 0;
    if (S->cmg_bytes <= CMG_SMEM_MAX) {
        int ok = 0;
        cudaError_t e = S->prec == IFX_PREC_FP64 ? cluster_vcycle_setup<double>((int)S->cmg_bytes, n, &ok)
                                                 : cluster_vcycle_setup<float>((int)S->cmg_bytes, n, &ok);
        S->cmg_ok = e == cudaSuccess && ok;
        if (e != cudaSuccess) cudaGetLastError();  // cluster launches unavailable: tile V-cycle only
    }
    IFX_TRY(dalloc(S, &S->dPart, (size_t)S->nt0 * NPART));
    IFX_TRY(dalloc(S, &S->dFpart, (size_t)n * 2 * FORCE_BLOCKS));
    IFX_TRY(dalloc(S, &S->dFtick, (size_t)n));
    IFX_TRY(dalloc(S, &S->dS, n));
    IFX_TRY(dalloc(S, &S->dCtl, 1));
    CUDA_TRY(cudaMallocHost((void**)&S->hS, n * sizeof(InstState)));
    CUDA_TRY(cudaMallocHost((void**)&S->hCtl, sizeof(LoopCtl)));
    CUDA_TRY(cudaMallocHost((void**)&S->h_flag, sizeof(unsigned int)));
    *S->h_flag = 0;
    if (!S->ev2) CUDA_TRY(cudaEventCreateWithFlags(&S->ev2, cudaEventDisableTiming));
    std::memset(S->hS, 0, n * sizeof(InstState));
    CUDA_TRY(cudaMemcpyAsync(S->dI, hI.data(), n * sizeof(InstDev), cudaMemcpyHostToDevice, S->stream));
    // image-point weights of the IBM ghosts
    CUDA_TRY(launch_ghost_weights(S->dG, S->dIbm, S->nibm, S->dI, S->dBiIp, S->stream));
    S->launches++;
    {   // moving bodies: their instances, their IBM ghost slots, body boxes
        std::vector<int> mv, slots, nibm;
        for (int k = 0; k < n; k++) {
            const Instance& I = S->inst[k];
            if (!I.moving) continue;
            mv.push_back(k);
            nibm.push_back(I.n_ibm);
            // the slots in use are the first ones: listed column-wise over
            // 32-wide rows, consecutive slots land in different blocks of the
            // per-step weight kernel (32 threads each), i.e. on different SMs
            const int nb = (I.ibm_cap + 31) / 32;
            for (int b = 0; b < nb; b++)
                for (int l = 0; l < 32; l++) {
                    const int s = b + l * nb;
                    if (s < I.ibm_cap) slots.push_back(I.ibm_beg + s);
                }
        }
        S->nmv = (int)mv.size();
        S->nmvslots = (int)slots.size();
        if (S->nmv) {
            int* dn = nullptr;
            IFX_TRY(dupload(S, &S->dMv, mv));
            IFX_TRY(dupload(S, &S->dMvSlots, slots));
            IFX_TRY(dupload(S, &dn, nibm));
            CUDA_TRY(launch_move_init(S->dI, S->dS, S->dMv, S->nmv, dn, S->stream));
            S->launches++;
        }
    }
    // initial field, outflow face values, ghosts and faces
    for (int k = 0; k < n; k++) {
        Instance& I = S->inst[k];
        std::vector<double> u, v;
        initial_field(I, u, v);
        std::vector<double> qbu(4 * (size_t)I.qstride, 0.0), qbv(4 * (size_t)I.qstride, 0.0);
        for (int g = I.ghost_beg; g < I.ghost_beg + I.ghost_cnt; g++)
            if (hG[g].qown >= 0) {
                qbu[hG[g].qown] = u[hG[g].adj];
                qbv[hG[g].qown] = v[hG[g].adj];
            }
        CUDA_TRY(cudaMemcpyAsync(I.dev.u, u.data(), I.ncell * 8, cudaMemcpyHostToDevice, S->stream));
        CUDA_TRY(cudaMemcpyAsync(I.dev.v, v.data(), I.ncell * 8, cudaMemcpyHostToDevice, S->stream));
        CUDA_TRY(cudaMemcpyAsync(I.dev.u2, u.data(), I.ncell * 8, cudaMemcpyHostToDevice, S->stream));
        CUDA_TRY(cudaMemcpyAsync(I.dev.v2, v.data(), I.ncell * 8, cudaMemcpyHostToDevice, S->stream));
        CUDA_TRY(cudaMemcpyAsync(I.dev.qbu, qbu.data(), qbu.size() * 8, cudaMemcpyHostToDevice, S->stream));
        CUDA_TRY(cudaMemcpyAsync(I.dev.qbv, qbv.data(), qbv.size() * 8, cudaMemcpyHostToDevice, S->stream));
        CUDA_TRY(cudaStreamSynchronize(S->stream));  // host vectors go out of scope
    }
    CUDA_TRY(launch_ghost_fill(S->dG, S->ng, S->dI, 3, S->dGval, S->stream));
    CUDA_TRY(launch_face_rhs(S->dT0, S->nt0, S->dI, S->dS, S->dPart, 1, S->stream));
    S->launches += 3;
    CUDA_TRY(cudaStreamSynchronize(S->stream));
    IFX_TRY(setup_persistent(S));
    return IFX_OK;
}

// ------------------------------------------------------- method: step

struct Seq {
    ifx_solver* S;
    long long n = 0;  // launches issued through this sequence
    cudaError_t err = cudaSuccess;
    void add(cudaError_t e) {
        n++;
        if (e != cudaSuccess && err == cudaSuccess) err = e;
    }
};

// One V-cycle on the correction equation; returns which buffer (0: e,
// 1: e2) holds the finest-level result.
// The FP32 (mixed) path restarts its Krylov recursion from FP64 true residuals.
template <typename T>
constexpr int mixed_of() { return sizeof(T) == 4 ? 1 : 0; }

// first_done: the finest level's zero-start sweep already ran (fused with
// the Krylov direction update).
// Tile grid of level l of a one-instance solver (the layout of its tile
// lists: rows of tiles of TILE_X x 8 rows cells from (0, 0)).
GridTiles grid_of(const ifx_solver* S, int l, int rows) {
    const Instance& I = S->inst[0];
    GridTiles g;
    g.L = S->hLV[I.lev_base + l];
    g.gidx = I.dev.gidx;
    g.omega = I.dev.omega;
    g.inst = 0;
    g.lev = I.lev_base + l;
    g.x0 = 0;
    g.y0 = 0;
    g.th = TILE_Y * rows;
    g.ntx = (g.L.nx + TILE_X - 1) / TILE_X;
    return g;
}

template <typename T>
int seq_vcycle(Seq& q, bool first_done = false) {
    ifx_solver* S = q.S;
    cudaStream_t st = S->stream;
    const int L = S->lmax, pre = S->mg_pre, post = S->mg_post;
    if (S->cmg_use) {  // the whole V-cycle on one thread-block cluster per instance
        q.add(launch_vcycle_cluster<T>(S->dSub, (int)S->inst.size(), S->dLV, S->dI, S->dS, S->dG, pre, post,
                                       (int)S->cmg_bytes, st));
        return parity_after_post(0, pre, post);
    }
    // multigrid tile lists: 32x8 tiles, or wide tiles with MG_ROWS_WIDE rows per thread
    const int R = S->mg_rows;
    const bool one = S->inst.size() == 1;  // one instance: tiles from the block index
    auto smooth = [&](const Tile* tl, int nt, int l, int flags, int src_alt) {
        if (one && S->dTmap)
            return launch_smooth_grid_tma<T>(grid_of(S, l, R), nt, S->dS, S->dG, S->dTmap, flags, src_alt, R, S->dErr, st);
        if (one) return launch_smooth_grid<T>(grid_of(S, l, R), nt, S->dS, S->dG, flags, src_alt, R, st);
        if (S->dTmap)
            return launch_smooth_tma<T>(tl, nt, S->dLV, S->dI, S->dS, S->dG, S->dTmap, flags, src_alt, R, S->dErr, st);
        return launch_smooth<T>(tl, nt, S->dLV, S->dI, S->dS, S->dG, flags, src_alt, R, st);
    };
    const bool W = R == MG_ROWS_WIDE;
    const Tile* t0 = W ? S->dT0W : S->dT0;
    const int nt0 = W ? S->nt0W : S->nt0;
    auto tsm = [&](int l) { return W ? S->dTsmW[l] : S->dTsm[l]; };
    auto ntsm = [&](int l) { return W ? S->ntsmW[l] : S->ntsm[l]; };
    auto tre = [&](int l) { return W ? S->dTreW[l] : S->dTre[l]; };
    auto ntre = [&](int l) { return W ? S->ntreW[l] : S->ntre[l]; };
    // finest level: first sweep from zero, then the rest of the pre-smoothing
    if (!first_done) q.add(smooth(t0, nt0, 0, 1, 0));
    int cur0 = 1;
    for (int k = 1; k < pre; k++) {
        q.add(smooth(t0, nt0, 0, 0, cur0));
        cur0 ^= 1;
    }
    // large coarse levels: one launch per phase
    for (int l = 1; l < L; l++) {
        if (ntre(l) == 0) break;
        q.add(launch_restrict<T>(tre(l), ntre(l), S->dLV, S->dI, S->dS, S->dG, parity_after_pre(l - 1, pre), R, st));
        if (ntsm(l) == 0) continue;
        int cur = 0;
        for (int k = 1; k < pre; k++) {
            q.add(smooth(tsm(l), ntsm(l), l, 0, cur));
            cur ^= 1;
        }
    }
    // small levels of every instance: one block each
    q.add(launch_subcycle<T>(S->dSub, (int)S->inst.size(), S->dLV, S->dI, S->dS, pre, post, S->sub_bytes, st));
    for (int l = L - 2; l >= 0; l--) {
        const Tile* tl = l == 0 ? t0 : tsm(l);
        const int nt = l == 0 ? nt0 : ntsm(l);
        if (nt == 0) continue;
        int cur = parity_after_pre(l, pre);
        int k = 0;
        if (l >= 1) {  // prolongation fused with the first sweep (32x8 tiles in either shape): cur -> cur ^ 1
            q.add(launch_prolong_sweep<T>(S->dTsm[l], S->ntsm[l], S->dLV, S->dI, S->dS, cur,
                                          parity_after_post(l + 1, pre, post), st));
            cur ^= 1;
            k = 1;
        } else {
            q.add(launch_prolong<T>(tl, nt, S->dLV, S->dS, cur, parity_after_post(l + 1, pre, post), R, st));
        }
        for (; k < post; k++) {
            q.add(smooth(tl, nt, l, 0, cur));
            cur ^= 1;
        }
        if (l == 0) cur0 = cur;
    }
    return cur0;
}

void seq_pre(Seq& q) {
    ifx_solver* S = q.S;
    cudaStream_t st = S->stream;
    const int n = (int)S->inst.size();
    q.add(launch_step_begin(S->dI, S->dS, n, S->dCtl, st));
    if (S->nmv) {
        // moving bodies: geometry at the new pose, then the new ghosts' weights
        q.add(launch_move_geometry(S->dI, S->dS, S->dLV, S->dG, S->dMv, S->nmv, st));
        q.add(launch_ghost_weights(S->dG, S->dMvSlots, S->nmvslots, S->dI, nullptr, st, 32));
        q.add(launch_move_forces(S->dI, S->dS, S->dMv, S->nmv, st));
    }
    q.add(launch_outflow(S->dG, S->ng, S->dI, st));
    q.add(launch_ghost_fill(S->dG, S->ng, S->dI, 3, S->dGval, st));
    q.n++;  // ghost fill is two kernels
    q.add(launch_conv_rhs(S->dT0, S->nt0, S->dI, S->dS, st));
    q.add(launch_pred_guess(S->dT0, S->nt0, S->dI, st));
}

template <typename T>
void seq_pred_body(Seq& q, unsigned long long h) {
    ifx_solver* S = q.S;
    cudaStream_t st = S->stream;
    const int n = (int)S->inst.size();
    if (mixed_of<T>()) {
        // on the multigrid tile shape
        const int R = S->mg_rows;
        const Tile* t0 = R == MG_ROWS_WIDE ? S->dT0W : S->dT0;
        const int nt0 = R == MG_ROWS_WIDE ? S->nt0W : S->nt0;
        // the FP64 refresh of each inner cycle runs inside the sweeps that start and end it
        for (int par = 0; par < 2; par++) {
            q.add(launch_pred_sweep32(t0, nt0, S->dG, S->ng, S->dLV, S->dI, S->dS, S->dPart, par, R, st));
            q.add(launch_pred_reduce(S->dI, S->dS, S->dPart, n, par, S->dCtl, h, st, S->wide_sums));
        }
        return;
    }
    q.add(launch_pred_sweep(S->dT0, S->nt0, S->dG, S->ng, S->dI, S->dS, S->dPart, 0, st));
    q.add(launch_pred_reduce(S->dI, S->dS, S->dPart, n, 0, S->dCtl, h, st, S->wide_sums));
    q.add(launch_pred_sweep(S->dT0, S->nt0, S->dG, S->ng, S->dI, S->dS, S->dPart, 1, st));
    q.add(launch_pred_reduce(S->dI, S->dS, S->dPart, n, 1, S->dCtl, h, st, S->wide_sums));
}

template <typename T>
void seq_mid(Seq& q) {
    ifx_solver* S = q.S;
    cudaStream_t st = S->stream;
    const int n = (int)S->inst.size();
    if (mixed_of<T>())
        q.add(launch_pred_refresh(S->mg_rows == MG_ROWS_WIDE ? S->dT0W : S->dT0,
                                  S->mg_rows == MG_ROWS_WIDE ? S->nt0W : S->nt0, S->dG, S->ng, S->dI, S->dS, 0, 1,
                                  nullptr, S->mg_rows, st));
    q.add(launch_ghost_fill(S->dG, S->ng, S->dI, 3, S->dGval, st));
    q.n++;
    q.add(launch_face_rhs(S->dT0, S->nt0, S->dI, S->dS, S->dPart, 0, st));
    q.add(launch_rhs_reduce(S->dI, S->dS, S->dPart, n, st, S->wide_sums));
    q.add(launch_bicg_start<T>(S->dT0, S->nt0, S->dLV, S->dI, S->dS, S->dG, S->dPart, 0, nullptr, n, st));
    q.add(launch_bicg_reduce_r(S->dI, S->dS, S->dPart, n, 1, mixed_of<T>(), S->dCtl, 0ull, st, S->wide_sums));
}

// One BiCGSTAB iteration with two V-cycle preconditioner applications.
template <typename T>
void seq_ppe_body(Seq& q, unsigned long long h) {
    ifx_solver* S = q.S;
    cudaStream_t st = S->stream;
    const int n = (int)S->inst.size();
    // finest-level Krylov phases on the multigrid tile shape
    const int R = S->mg_rows;
    const Tile* t0 = R == MG_ROWS_WIDE ? S->dT0W : S->dT0;
    const int nt0 = R == MG_ROWS_WIDE ? S->nt0W : S->nt0;
    if (mixed_of<T>()) {
        // FP64 true residual and restart for the instances whose FP32 recursion ran its course
        q.add(launch_bicg_start<T>(S->dT0, S->nt0, S->dLV, S->dI, S->dS, S->dG, S->dPart, 1, S->dCtl, n, st));
        q.add(launch_bicg_reduce_r(S->dI, S->dS, S->dPart, n, 2, 1, S->dCtl, 0ull, st, S->wide_sums));
    }
    // direction updates fused with the first sweep of the tile V-cycle
    const bool fuse = !S->cmg_use;
    if (fuse) q.add(launch_bicg_dir_smooth<T>(t0, nt0, S->dLV, S->dI, S->dS, S->dG, 0, R, st));
    else q.add(launch_bicg_p<T>(t0, nt0, S->dLV, S->dI, S->dS, R, st));
    int e1 = seq_vcycle<T>(q, fuse);
    q.add(launch_bicg_apply<T>(t0, nt0, S->dLV, S->dI, S->dS, S->dG, S->dPart, e1, 0, R, st));
    q.add(launch_bicg_scalar(S->dI, S->dS, S->dPart, n, 0, st, S->wide_sums));
    if (fuse) q.add(launch_bicg_dir_smooth<T>(t0, nt0, S->dLV, S->dI, S->dS, S->dG, 1, R, st));
    else q.add(launch_bicg_s<T>(t0, nt0, S->dLV, S->dI, S->dS, R, st));
    int e2 = seq_vcycle<T>(q, fuse);
    q.add(launch_bicg_apply<T>(t0, nt0, S->dLV, S->dI, S->dS, S->dG, S->dPart, e2, 1, R, st));
    q.add(launch_bicg_scalar(S->dI, S->dS, S->dPart, n, 1, st, S->wide_sums));
    q.add(launch_bicg_x<T>(t0, nt0, S->dLV, S->dI, S->dS, S->dPart, R, st));
    q.add(launch_bicg_reduce_r(S->dI, S->dS, S->dPart, n, 0, mixed_of<T>(), S->dCtl, h, st, S->wide_sums));
}

void seq_post(Seq& q) {
    ifx_solver* S = q.S;
    cudaStream_t st = S->stream;
    const int n = (int)S->inst.size();
    q.add(launch_p_finalize(S->dT0, S->nt0, S->dI, S->dS, st));
    q.add(launch_ghost_fill(S->dG, S->ng, S->dI, 4, S->dGval, st));
    q.n++;
    q.add(launch_correct(S->dT0, S->nt0, S->dI, S->dPart, st));
    q.add(launch_correct_reduce(S->dI, S->dS, S->dPart, n, st));
    q.add(launch_ghost_fill(S->dG, S->ng, S->dI, 3, S->dGval, st));
    q.n++;
    q.add(launch_forces(S->dI, S->dS, S->dFpart, S->dFtick, n, st));
}

int max_pred_pairs(const ifx_solver* S) {
    int m = 1;
    for (auto& I : S->inst) m = std::max(m, (I.cfg.ad_itermax + 1) / 2);
    return m;
}
int max_ppe_bodies(const ifx_solver* S) {
    int m = 1;
    for (auto& I : S->inst) m = std::max(m, I.cfg.ppe_itermax + 1);
    return m;
}

// Host-driven loop: run the body, read the vote, repeat.
template <class F>
ifx_status host_loop(ifx_solver* S, Seq& q, int maxit, F body) {
    for (int k = 0; k < maxit; k++) {
        body(q, 0ull);
        if (q.err != cudaSuccess) return cuerr(q.err, "kernel launch");
        CUDA_TRY(cudaMemcpyAsync(S->hCtl, S->dCtl, sizeof(LoopCtl), cudaMemcpyDeviceToHost, S->stream));
        CUDA_TRY(cudaStreamSynchronize(S->stream));
        if (S->hCtl->result == 0) break;
    }
    return IFX_OK;
}

template <typename T>
ifx_status step_method_host(ifx_solver* S) {
    Seq q{S};
    seq_pre(q);
    IFX_TRY(host_loop(S, q, max_pred_pairs(S), [](Seq& qq, unsigned long long h) { seq_pred_body<T>(qq, h); }));
    seq_mid<T>(q);
    CUDA_TRY(cudaMemcpyAsync(S->hCtl, S->dCtl, sizeof(LoopCtl), cudaMemcpyDeviceToHost, S->stream));
    CUDA_TRY(cudaStreamSynchronize(S->stream));
    if (S->hCtl->result != 0)
        IFX_TRY(host_loop(S, q, max_ppe_bodies(S), [](Seq& qq, unsigned long long h) { seq_ppe_body<T>(qq, h); }));
    seq_post(q);
    if (q.err != cudaSuccess) return cuerr(q.err, "kernel launch");
    S->launches += q.n;
    return IFX_OK;
}

// ---- CUDA graph of one time step: linear segments captured to the graph,
//      the two convergence loops as conditional WHILE nodes.
struct GraphBuilder {
    ifx_solver* S;
    cudaGraph_t g;
    std::vector<cudaGraphNode_t> frontier;
    cudaError_t err = cudaSuccess;

    template <class F>
    long long segment(F fn) {
        Seq q{S};
        if (err != cudaSuccess) return 0;
        err = cudaStreamBeginCaptureToGraph(S->stream, g, frontier.empty() ? nullptr : frontier.data(), nullptr,
                                            frontier.size(), cudaStreamCaptureModeThreadLocal);
        if (err != cudaSuccess) return 0;
        fn(q);
        const cudaGraphNode_t* deps = nullptr;
        size_t nd = 0;
        cudaStreamCaptureStatus cs;
        cudaError_t e2 = cudaStreamGetCaptureInfo(S->stream, &cs, nullptr, nullptr, &deps, nullptr, &nd);
        std::vector<cudaGraphNode_t> nf;
        if (e2 == cudaSuccess)
            for (size_t k = 0; k < nd; k++) nf.push_back(deps[k]);
        cudaGraph_t out = nullptr;
        cudaError_t e3 = cudaStreamEndCapture(S->stream, &out);
        if (q.err != cudaSuccess) err = q.err;
        else if (e2 != cudaSuccess) err = e2;
        else if (e3 != cudaSuccess) err = e3;
        frontier = nf;
        return q.n;
    }

    template <class F>
    long long loop(F body) {
        if (err != cudaSuccess) return 0;
        cudaGraphConditionalHandle h;
        err = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault);
        if (err != cudaSuccess) return 0;
        cudaGraphNodeParams p = {cudaGraphNodeTypeConditional};
        p.conditional.handle = h;
        p.conditional.type = cudaGraphCondTypeWhile;
        p.conditional.size = 1;
        cudaGraphNode_t node;
        err = cudaGraphAddNode(&node, g, frontier.empty() ? nullptr : frontier.data(), nullptr, frontier.size(), &p);
        if (err != cudaSuccess) return 0;
        cudaGraph_t body_g = p.conditional.phGraph_out[0];
        Seq q{S};
        err = cudaStreamBeginCaptureToGraph(S->stream, body_g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
        if (err != cudaSuccess) return 0;
        body(q, (unsigned long long)h);
        cudaGraph_t out = nullptr;
        cudaError_t e3 = cudaStreamEndCapture(S->stream, &out);
        if (q.err != cudaSuccess) err = q.err;
        else if (e3 != cudaSuccess) err = e3;
        frontier.assign(1, node);
        return q.n;
    }
};

template <typename T>
ifx_status build_graph(ifx_solver* S) {
    GraphBuilder b{S, nullptr, {}, cudaSuccess};
    CUDA_TRY(cudaGraphCreate(&b.g, 0));
    S->graph = b.g;
    S->graph_nodes_pre = b.segment([](Seq& q) { seq_pre(q); });
    S->graph_nodes_pred = b.loop([](Seq& q, unsigned long long h) { seq_pred_body<T>(q, h); });
    S->graph_nodes_mid = b.segment([](Seq& q) { seq_mid<T>(q); });
    S->graph_nodes_ppe = b.loop([](Seq& q, unsigned long long h) { seq_ppe_body<T>(q, h); });
    S->graph_nodes_post = b.segment([](Seq& q) { seq_post(q); });
    if (b.err != cudaSuccess) return cuerr(b.err, "graph capture");
    CUDA_TRY(cudaGraphInstantiate(&S->gexec, S->graph, 0));
    return IFX_OK;
}

// Per-instance outcome of the steps just finished.  An instance whose state
// became non-finite is marked IFX_ERR_DIVERGED and retired (later steps leave
// it unchanged while the other instances go on); the call reports
// IFX_ERR_DIVERGED once, when that happens.  An instance whose pressure solve
// stopped at its iteration cap above the tolerance is marked
// IFX_ERR_NOT_CONVERGED (a warning: its steps continue).
ifx_status check_states(ifx_solver* S) {
    const int n = (int)S->inst.size();
    if ((int)S->inst_status.size() != n) S->inst_status.assign(n, IFX_OK);
    if (S->states_enqueued) {
        S->states_enqueued = false;  // copied behind the step, which the caller waited for
    } else {
        CUDA_TRY(cudaMemcpyAsync(S->hS, S->dS, n * sizeof(InstState), cudaMemcpyDeviceToHost, S->stream));
        CUDA_TRY(cudaStreamSynchronize(S->stream));
    }
    bool copies = false;
    ifx_status worst = IFX_OK;
    for (int k = 0; k < n; k++) {
        Instance& I = S->inst[k];
        if (I.dev.retired) continue;
        const InstState& s = S->hS[k];
        if (s.geo_err) {
            // a moving body left the domain or outgrew its ghost slots
            S->inst_status[k] = IFX_ERR_GEOMETRY;
            I.dev.retired = 1;
            CUDA_TRY(cudaMemcpyAsync(&S->dI[k].retired, &I.dev.retired, sizeof(int), cudaMemcpyHostToDevice, S->stream));
            copies = true;
            if (worst == IFX_OK) worst = IFX_ERR_GEOMETRY;
        } else if (!std::isfinite(s.ppe_rel) || !std::isfinite(s.max_div) || !std::isfinite(s.pred_metric)) {
            S->inst_status[k] = IFX_ERR_DIVERGED;
            I.dev.retired = 1;
            CUDA_TRY(cudaMemcpyAsync(&S->dI[k].retired, &I.dev.retired, sizeof(int), cudaMemcpyHostToDevice, S->stream));
            copies = true;
            worst = IFX_ERR_DIVERGED;
        } else if (s.ppe_iters >= I.cfg.ppe_itermax && s.ppe_rel > I.cfg.ppe_tol && S->inst_status[k] == IFX_OK) {
            S->inst_status[k] = IFX_ERR_NOT_CONVERGED;
        }
    }
    if (copies) CUDA_TRY(cudaStreamSynchronize(S->stream));  // the host sources of the copies above
    return worst;
}

// Execution mode from IFX_EXEC: "persistent" (default when cooperative
// launch is available), "graph", or "host" (IFX_NO_GRAPH=1 also selects host).
int exec_mode_selected(const ifx_solver* S) {
    if (S->exec_override == 0 && S->persist_grid > 0) return 0;
    if (S->exec_override == 1 || S->exec_override == 2) return S->exec_override;
    const char* e = std::getenv("IFX_EXEC");
    const char* ng = std::getenv("IFX_NO_GRAPH");
    if (ng && ng[0] == '1') return 2;
    if (e && std::strcmp(e, "host") == 0) return 2;
    if (e && std::strcmp(e, "graph") == 0) return 1;
    return S->persist_grid > 0 ? 0 : 1;
}
// The persistent kernel has no phase for moving bodies: their solvers run as
// a graph instead.
int exec_mode(const ifx_solver* S) {
    const int m = exec_mode_selected(S);
    return (m == 0 && S->nmv > 0) ? 1 : m;
}

// Issues nsteps time steps on the solver's stream.  The host-loop mode reads
// the convergence state after every loop body, so it completes the steps here.
template <typename T>
ifx_status step_launch(ifx_solver* S, int nsteps) {
    if (S->poisoned) return set_error(IFX_ERR_STATE, "a grid barrier timed out earlier; recreate the solver");
    const int mode = exec_mode(S);
    S->use_graph = mode == 1;
    S->pending_mode = mode;
    S->pending_steps = nsteps;
    CUDA_TRY(cudaEventRecord(S->ev0, S->stream));
    if (mode == 0) {
        S->plan.nsteps = nsteps;
        const cudaError_t e = launch_persist_step<T>(S->plan, S->persist_grid, S->stream);
        // a barrier fault set by ifx_set_barrier_fault applies to this launch only
        S->plan.spin_limit = kSpinLimit;
        S->plan.withhold_arrival = 0;
        CUDA_TRY(e);
        S->launches += 1;
    } else if (S->use_graph) {
        if (!S->gexec) IFX_TRY(build_graph<T>(S));
        for (int s = 0; s < nsteps; s++) CUDA_TRY(cudaGraphLaunch(S->gexec, S->stream));
    } else {
        for (int s = 0; s < nsteps; s++) IFX_TRY(step_method_host<T>(S));
    }
    CUDA_TRY(cudaEventRecord(S->ev1, S->stream));
    // the error flag and the instance states follow the steps in the stream,
    // so that step_finish waits once (ev2) and reads both from pinned memory
    const unsigned int* flag = mode == 0 ? &S->dBar->err : S->dErr;
    *S->h_flag = 0;
    if (flag) CUDA_TRY(cudaMemcpyAsync(S->h_flag, flag, sizeof(unsigned int), cudaMemcpyDeviceToHost, S->stream));
    CUDA_TRY(cudaMemcpyAsync(S->hS, S->dS, S->inst.size() * sizeof(InstState), cudaMemcpyDeviceToHost, S->stream));
    CUDA_TRY(cudaEventRecord(S->ev2, S->stream));
    S->states_enqueued = true;
    return IFX_OK;
}

// Waits for the steps issued by step_launch and checks the solver state.
ifx_status step_finish(ifx_solver* S) {
    const int nsteps = S->pending_steps, mode = S->pending_mode;
    if (nsteps == 0) return IFX_OK;
    S->pending_steps = 0;
    CUDA_TRY(cudaEventSynchronize(S->ev2));  // the steps (ev1), then their flag and state copies
    float ms = 0.f;
    CUDA_TRY(cudaEventElapsedTime(&ms, S->ev0, S->ev1));
    S->last_ms = ms;
    S->steps_done += nsteps;
    if (*S->h_flag) {
        S->poisoned = true;
        S->states_enqueued = false;
        return set_error(IFX_ERR_CUDA, mode == 0 ? "persistent step: grid barrier timed out"
                                                 : "a TMA tile copy did not complete");
    }
    ifx_status st = check_states(S);
    if (mode == 1) {
        // kernels executed by the graph: fixed segments plus loop bodies
        int pairs = 0, bodies = 0;
        for (size_t k = 0; k < S->inst.size(); k++) {
            pairs = std::max(pairs, (S->hS[k].pred_iters + 1) / 2);
            bodies = std::max(bodies, S->hS[k].ppe_iters);
        }
        bodies = std::max(bodies, 1);
        S->launches += (long long)nsteps * (S->graph_nodes_pre + pairs * S->graph_nodes_pred + S->graph_nodes_mid +
                                            bodies * S->graph_nodes_ppe + S->graph_nodes_post);
    }
    if (st == IFX_ERR_GEOMETRY)
        return set_error(st, "a moving body left the domain or outgrew its ghost slots (the instance is retired)");
    if (st != IFX_OK) return set_error(st, "non-finite value in the solver state (the instance is retired)");
    return IFX_OK;
}

// ---------------------------------------------------- reference mode

// Steps of one cooperative REFERENCE-mode launch (the per-step iteration counts fit a fixed buffer).
constexpr int kRefStepsPerLaunch = 1024;

ifx_status create_reference(ifx_solver* S, const ifx_config* c, const double* xf, const double* yf) {
    S->mode = IFX_MODE_REFERENCE;
    S->inst.resize(1);
    Instance& I = S->inst[0];
    I.cfg = *c;
    I.NX = c->nx;
    I.NY = c->ny;
    I.nx = I.NX + 2;
    I.ny = I.NY + 2;
    I.pitch = I.nx;
    I.ncell = (size_t)I.nx * I.ny;
    if (c->ppe_method < IFX_PPE_JACOBI || c->ppe_method > IFX_PPE_LINE_SOR) return set_error(IFX_ERR_ARG, "bad PPE-Method");
    if (!(c->relax_ad < 2.0) || !(c->relax_ppe < 2.0)) return set_error(IFX_ERR_ARG, "relaxation factors must be below 2");
    if (I.NX < 2 || I.NY < 2) return set_error(IFX_ERR_ARG, "reference mode needs nx, ny >= 2");
    build_grid(I, xf, yf);
    const int nx = I.nx, ny = I.ny;
    const size_t n = I.ncell;
    // readGridData's full dx/dy arrays (src/include/preSim.cu:328-355)
    std::vector<double> dx(n), dy(n), ib(n, 1.0);
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            dx[i + j * nx] = I.dx[i];
            dy[i + j * nx] = I.dy[j];
        }
    if (c->body == IFX_BODY_ELLIPSE) {
        // extension: the reference's iBlank kernel is fixed to 1 (src/include/preSim.cu:133)
        const double th = c->body_angle_deg * M_PI / 180.0, cs = std::cos(th), sn = std::sin(th);
        const double ia2 = 1.0 / (c->body_a * c->body_a), ib2 = 1.0 / (c->body_b * c->body_b);
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                // built with -ffp-contract=off: same rounding as the device predicate
                const double ddx = I.xc[i] - c->body_cx, ddy = I.yc[j] - c->body_cy;
                const double xr = ddx * cs + ddy * sn, yr = ddy * cs - ddx * sn;
                const double f = xr * xr * ia2 + yr * yr * ib2;
                ib[i + j * nx] = f < 1.0 ? 0.0 : 1.0;
            }
    }
    IFX_TRY(dalloc(S, &S->r_u, n)); IFX_TRY(dalloc(S, &S->r_v, n));
    IFX_TRY(dalloc(S, &S->r_ut, n)); IFX_TRY(dalloc(S, &S->r_vt, n));
    IFX_TRY(dalloc(S, &S->r_p, n)); IFX_TRY(dalloc(S, &S->r_pt, n));
    IFX_TRY(dupload(S, &S->r_dx, dx)); IFX_TRY(dupload(S, &S->r_dy, dy));
    IFX_TRY(dupload(S, &S->r_xc, I.xc)); IFX_TRY(dupload(S, &S->r_yc, I.yc));
    IFX_TRY(dupload(S, &S->r_ib, ib));
    IFX_TRY(dalloc(S, &S->r_coef, 5 * n));
    IFX_TRY(dalloc(S, &S->r_sx, n)); IFX_TRY(dalloc(S, &S->r_sy, n));
    IFX_TRY(dalloc(S, &S->r_uf, (size_t)(nx - 1) * (ny - 1)));
    IFX_TRY(dalloc(S, &S->r_vf, (size_t)(nx - 1) * (ny - 1)));
    IFX_TRY(dalloc(S, &S->r_res, 2 * ((n + 255) / 256) + 2));
    IFX_TRY(dalloc(S, &S->r_out, 4));
    if (c->ppe_method == IFX_PPE_LINE_SOR) IFX_TRY(dalloc(S, &S->r_line, n));
    S->r_grid = ref_steps_grid(nx, ny);
    if (S->r_grid > 0) {
        IFX_TRY(dalloc(S, &S->r_bar, 1));
        IFX_TRY(dalloc(S, &S->r_iters_d, kRefStepsPerLaunch));
        CUDA_TRY(cudaMallocHost((void**)&S->r_iters_h, kRefStepsPerLaunch * sizeof(int)));
    }
    CUDA_TRY(cudaMallocHost((void**)&S->h_out, 4 * sizeof(double)));
    // initializeData (src/include/preSim.cu:201-217)
    CUDA_TRY(launch_ref_init(nx, ny, S->r_xc, S->r_yc, S->r_u, S->r_v, S->r_p, S->stream));
    CUDA_TRY(cudaMemcpyAsync(S->r_ut, S->r_u, n * 8, cudaMemcpyDeviceToDevice, S->stream));
    CUDA_TRY(cudaMemcpyAsync(S->r_vt, S->r_v, n * 8, cudaMemcpyDeviceToDevice, S->stream));
    S->launches++;
    CUDA_TRY(cudaStreamSynchronize(S->stream));
    return IFX_OK;
}

// A relaxation factor as read from w-AD / w-PPE: 0 (unset) and 1 mean none.
double relax_factor(double w) { return w > 0.0 ? w : 1.0; }

RefDev refdev(ifx_solver* S) {
    const Instance& I = S->inst[0];
    const size_t n = I.ncell;
    RefDev R;
    R.nx = I.nx;
    R.ny = I.ny;
    R.dt = I.cfg.dt;
    R.re = I.cfg.re;
    R.dx = S->r_dx;
    R.dy = S->r_dy;
    R.iblank = S->r_ib;
    R.aP = S->r_coef;
    R.aE = S->r_coef + n;
    R.aW = S->r_coef + 2 * n;
    R.aN = S->r_coef + 3 * n;
    R.aS = S->r_coef + 4 * n;
    R.sx = S->r_sx;
    R.sy = S->r_sy;
    R.uf = S->r_uf;
    R.vf = S->r_vf;
    R.res = S->r_res;
    R.w_ad = relax_factor(I.cfg.relax_ad);
    return R;
}

// nsteps x ADsolver (src/include/ADSolver.cu:268-395).
ifx_status step_reference(ifx_solver* S, int nsteps) {
    const Instance& I = S->inst[0];
    RefDev R = refdev(S);
    cudaStream_t st = S->stream;
    CUDA_TRY(cudaEventRecord(S->ev0, st));
    CUDA_TRY(launch_ref_coeffs(R, st));
    S->launches++;
    if (S->r_grid > 0 && !S->poisoned) {
        // the whole step on the device: one cooperative launch per kRefStepsPerLaunch steps
        for (int s0 = 0; s0 < nsteps; s0 += kRefStepsPerLaunch) {
            const int k = std::min(kRefStepsPerLaunch, nsteps - s0);
            double* cu = S->r_cur ? S->r_ut : S->r_u;
            double* cv = S->r_cur ? S->r_vt : S->r_v;
            double* tu = S->r_cur ? S->r_u : S->r_ut;
            double* tv = S->r_cur ? S->r_v : S->r_vt;
            CUDA_TRY(launch_ref_steps(R, cu, cv, tu, tv, S->r_bar, I.cfg.ad_itermax, k, S->r_iters_d, S->r_grid, st));
            S->launches += 2;
            CUDA_TRY(cudaMemcpyAsync(S->r_iters_h, S->r_iters_d, k * sizeof(int), cudaMemcpyDeviceToHost, st));
            unsigned int err = 0;
            CUDA_TRY(cudaMemcpyAsync(S->h_out, &S->r_bar->err, sizeof(unsigned int), cudaMemcpyDeviceToHost, st));
            CUDA_TRY(cudaStreamSynchronize(st));
            std::memcpy(&err, S->h_out, sizeof(err));
            if (err) {
                S->poisoned = true;
                return set_error(IFX_ERR_CUDA, "reference step: grid barrier timed out");
            }
            for (int q = 0; q < k; q++) {
                S->r_iters.push_back(S->r_iters_h[q]);
                S->r_cur ^= (S->r_iters_h[q] & 1);
            }
        }
        CUDA_TRY(cudaEventRecord(S->ev1, st));
        CUDA_TRY(cudaEventSynchronize(S->ev1));
        float ms = 0.f;
        CUDA_TRY(cudaEventElapsedTime(&ms, S->ev0, S->ev1));
        S->last_ms = ms;
        S->steps_done += nsteps;
        return IFX_OK;
    }
    for (int s = 0; s < nsteps; s++) {
        double* cu = S->r_cur ? S->r_ut : S->r_u;
        double* cv = S->r_cur ? S->r_vt : S->r_v;
        CUDA_TRY(launch_ref_velf(R, cu, cv, st));
        CUDA_TRY(launch_ref_bc(R, cu, cv, st));
        CUDA_TRY(launch_ref_source(R, cu, cv, st));
        S->launches += 3;
        double ures = 1.0, vres = 1.0;
        int it = 0;
        // pow(10.0, -6.0) at src/include/ADSolver.cu:315
        while (ures + vres > 1e-6 && it < I.cfg.ad_itermax) {
            double* tu = S->r_cur ? S->r_u : S->r_ut;
            double* tv = S->r_cur ? S->r_v : S->r_vt;
            CUDA_TRY(launch_ref_bc(R, cu, cv, st));
            CUDA_TRY(launch_ref_velf(R, cu, cv, st));
            CUDA_TRY(launch_ref_jacobi(R, cu, cv, tu, tv, st));
            CUDA_TRY(launch_ref_bc(R, cu, cv, st));
            CUDA_TRY(launch_ref_resid(R, cu, tu, cv, tv, S->r_out, st));
            S->launches += 5;
            S->r_cur ^= 1;
            cu = tu;
            cv = tv;
            CUDA_TRY(cudaMemcpyAsync(S->h_out, S->r_out, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
            CUDA_TRY(cudaStreamSynchronize(st));
            ures = S->h_out[0];
            vres = S->h_out[1];
            it++;
        }
        S->r_iters.push_back(it);
    }
    CUDA_TRY(cudaEventRecord(S->ev1, st));
    CUDA_TRY(cudaEventSynchronize(S->ev1));
    float ms = 0.f;
    CUDA_TRY(cudaEventElapsedTime(&ms, S->ev0, S->ev1));
    S->last_ms = ms;
    S->steps_done += nsteps;
    return IFX_OK;
}

ifx_status ppe_reference(ifx_solver* S, int* iters) {
    const Instance& I = S->inst[0];
    RefDev R = refdev(S);
    cudaStream_t st = S->stream;
    CUDA_TRY(launch_ref_ppe_coeffs(R, st));
    CUDA_TRY(launch_ref_ppe_bc(R, S->r_p, st));
    S->launches += 2;
    double* cur = S->r_p;
    double* tmp = S->r_pt;
    double residual = 1.0;
    int it = 0;
    const int method = I.cfg.ppe_method;
    const double w = relax_factor(I.cfg.relax_ppe);
    // pow(10.0, -6.0) at src/include/PPESolver.cu:172
    while (residual > 1e-6 && it < I.cfg.ppe_itermax) {
        if (method == IFX_PPE_POINT_GS) {
            CUDA_TRY(launch_ref_ppe_rbgs(R, cur, w, S->r_out, st));
            S->launches += 3;
        } else if (method == IFX_PPE_LINE_SOR) {
            CUDA_TRY(launch_ref_ppe_lines(R, cur, S->r_pt, S->r_line, w, S->r_out, st));
            S->launches += 3;
        } else {
            CUDA_TRY(launch_ref_ppe_sweep(R, cur, tmp, S->r_out, st));
            S->launches += 2;
            std::swap(cur, tmp);
        }
        CUDA_TRY(cudaMemcpyAsync(S->h_out, S->r_out, sizeof(double), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        residual = S->h_out[0];
        it++;
    }
    CUDA_TRY(launch_ref_ppe_bc(R, cur, st));
    S->launches++;
    if (cur != S->r_p) CUDA_TRY(cudaMemcpyAsync(S->r_p, cur, I.ncell * 8, cudaMemcpyDeviceToDevice, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    if (iters) *iters = it;
    return IFX_OK;
}

// ------------------------------------------------------------ fields

ifx_status field_size(const Instance& I, int field, size_t* n) {
    switch (field) {
        case IFX_FIELD_U: case IFX_FIELD_V: case IFX_FIELD_P: case IFX_FIELD_IBLANK:
        case IFX_FIELD_CELLTYPE: case IFX_FIELD_DIV:
            *n = (size_t)I.nx * I.ny; return IFX_OK;
        case IFX_FIELD_UF: *n = (size_t)(I.nx - 1) * (I.ny - 2); return IFX_OK;
        case IFX_FIELD_VF: *n = (size_t)(I.nx - 2) * (I.ny - 1); return IFX_OK;
        case IFX_FIELD_XC: *n = I.nx; return IFX_OK;
        case IFX_FIELD_YC: *n = I.ny; return IFX_OK;
    }
    return set_error(IFX_ERR_ARG, "unknown field id");
}

ifx_status get_pitched(ifx_solver* S, const Instance& I, const double* src, double* host) {
    CUDA_TRY(cudaMemcpy2DAsync(host, I.nx * sizeof(double), src, I.pitch * sizeof(double), I.nx * sizeof(double),
                               I.ny, cudaMemcpyDeviceToHost, S->stream));
    CUDA_TRY(cudaStreamSynchronize(S->stream));
    return IFX_OK;
}

}  // namespace

// ================================================================== C ABI

namespace ifx {
ifx_status finish_pending(ifx_solver* S) { return S->pending_steps ? step_finish(S) : IFX_OK; }
ifx_status validate_method_config(const ifx_config* c) { return validate(c); }
}  // namespace ifx

static ifx_status new_solver(ifx_solver** out) {
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) return set_error(IFX_ERR_NODEVICE, "no CUDA device available");
    ifx_solver* S = new ifx_solver();
    CUDA_TRY(cudaGetDevice(&S->device));
    CUDA_TRY(cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking));
    CUDA_TRY(cudaEventCreate(&S->ev0));
    CUDA_TRY(cudaEventCreate(&S->ev1));
    *out = S;
    return IFX_OK;
}

extern "C" ifx_status ifx_create_batch(int n, const ifx_config* cfgs, const double* const* xfs,
                                       const double* const* yfs, ifx_solver** out) {
    if (!out || n < 1 || !cfgs || !xfs || !yfs) return set_error(IFX_ERR_ARG, "ifx_create_batch: bad argument");
    *out = nullptr;
    for (int k = 0; k < n; k++) {
        if (!xfs[k] || !yfs[k]) return set_error(IFX_ERR_ARG, "ifx_create_batch: null grid");
        if (cfgs[k].nx < 1 || cfgs[k].ny < 1 || IFX_PADDED_CELLS(cfgs[k].nx, cfgs[k].ny) > IFX_MAX_CELLS)
            return set_error(IFX_ERR_ARG, "ifx_create_batch: nx, ny must be >= 1 and give at most IFX_MAX_CELLS cells");
    }
    ifx_solver* S = nullptr;
    IFX_TRY(new_solver(&S));
    ifx_status st;
    if (n == 1 && cfgs[0].mode == IFX_MODE_REFERENCE) st = create_reference(S, &cfgs[0], xfs[0], yfs[0]);
    else st = create_method(S, n, cfgs, xfs, yfs);
    if (st != IFX_OK) {
        std::string msg = ifx::g_last_error;
        ifx_destroy(S);
        return set_error(st, msg);
    }
    *out = S;
    return IFX_OK;
}

extern "C" ifx_status ifx_create(const ifx_config* cfg, const double* xf, const double* yf, ifx_solver** out) {
    if (!cfg) return set_error(IFX_ERR_ARG, "ifx_create: null config");
    const double* xs[1] = {xf};
    const double* ys[1] = {yf};
    return ifx_create_batch(1, cfg, xs, ys, out);
}

extern "C" ifx_status ifx_create_from_file(const char* inputs_path, ifx_solver** out) {
    ifx_config c;
    IFX_TRY(ifx_config_read(inputs_path, &c));  // bounds nx, ny by IFX_MAX_CELLS
    std::vector<double> xf, yf;
    try {
        xf.resize((size_t)c.nx + 1);
        yf.resize((size_t)c.ny + 1);
    } catch (const std::exception&) {
        return set_error(IFX_ERR_NOMEM, "ifx_create_from_file: host grid arrays");
    }
    IFX_TRY(ifx_grid_read(c.xgrid, c.nx + 1, xf.data()));
    IFX_TRY(ifx_grid_read(c.ygrid, c.ny + 1, yf.data()));
    return ifx_create(&c, xf.data(), yf.data(), out);
}

extern "C" int ifx_num_instances(const ifx_solver* s) { return s ? (int)s->inst.size() : 0; }

extern "C" ifx_status ifx_get_dims(const ifx_solver* S, int inst, int* nx, int* ny) {
    if (!S || !nx || !ny || inst < 0 || inst >= (int)S->inst.size()) return set_error(IFX_ERR_ARG, "ifx_get_dims: bad argument");
    *nx = S->inst[inst].nx;
    *ny = S->inst[inst].ny;
    return IFX_OK;
}

extern "C" ifx_status ifx_step(ifx_solver* S, int nsteps) {
    if (!S || nsteps < 0) return set_error(IFX_ERR_ARG, "ifx_step: bad argument");
    if (nsteps == 0) return IFX_OK;
    CUDA_TRY(cudaSetDevice(S->device));
    if (S->mode == IFX_MODE_REFERENCE) return step_reference(S, nsteps);
    IFX_TRY(step_finish(S));
    if (S->prec == IFX_PREC_FP64) IFX_TRY(step_launch<double>(S, nsteps));
    else IFX_TRY(step_launch<float>(S, nsteps));
    return step_finish(S);
}

extern "C" ifx_status ifx_step_async(ifx_solver* S, int nsteps) {
    if (!S || nsteps < 0) return set_error(IFX_ERR_ARG, "ifx_step_async: bad argument");
    if (nsteps == 0) return IFX_OK;
    CUDA_TRY(cudaSetDevice(S->device));
    if (S->mode == IFX_MODE_REFERENCE) return step_reference(S, nsteps);
    IFX_TRY(step_finish(S));
    if (S->prec == IFX_PREC_FP64) return step_launch<double>(S, nsteps);
    return step_launch<float>(S, nsteps);
}

extern "C" ifx_status ifx_step_wait(ifx_solver* S) {
    if (!S) return set_error(IFX_ERR_ARG, "ifx_step_wait: null solver");
    CUDA_TRY(cudaSetDevice(S->device));
    return step_finish(S);
}

extern "C" ifx_status ifx_set_exec_mode(ifx_solver* S, int mode) {
    if (!S || mode < IFX_EXEC_DEFAULT || mode > IFX_EXEC_HOST) return set_error(IFX_ERR_ARG, "ifx_set_exec_mode: bad argument");
    if (mode == IFX_EXEC_PERSISTENT && S->persist_grid == 0)
        return set_error(IFX_ERR_STATE, "persistent execution is not available for this solver");
    IFX_TRY(step_finish(S));
    S->exec_override = mode;
    return IFX_OK;
}

// Blocks of the persistent kernel: its phases stride over their tiles, so any
// grid up to the co-resident one gives the same results; fewer blocks make each
// grid barrier cheaper (fewer arrivals on its counter) and suit instances with
// few tiles.
extern "C" ifx_status ifx_set_persistent_grid(ifx_solver* S, int blocks) {
    if (!S || blocks < 0) return set_error(IFX_ERR_ARG, "ifx_set_persistent_grid: bad argument");
    if (S->persist_full == 0) return set_error(IFX_ERR_STATE, "persistent execution is not available for this solver");
    if (blocks > S->persist_full)
        return set_error(IFX_ERR_ARG, "ifx_set_persistent_grid: more blocks than can be co-resident (" +
                                          std::to_string(S->persist_full) + ")");
    IFX_TRY(step_finish(S));
    S->persist_grid = blocks == 0 ? S->persist_full : blocks;
    return IFX_OK;
}

extern "C" ifx_status ifx_get_persistent_grid(ifx_solver* S, int* blocks) {
    if (!S || !blocks) return set_error(IFX_ERR_ARG, "ifx_get_persistent_grid: bad argument");
    *blocks = S->persist_grid;
    return IFX_OK;
}

extern "C" ifx_status ifx_get_exec_mode(ifx_solver* S, int* mode) {
    if (!S || !mode) return set_error(IFX_ERR_ARG, "ifx_get_exec_mode: bad argument");
    *mode = S->mode == IFX_MODE_METHOD ? exec_mode(S) : IFX_EXEC_HOST;
    return IFX_OK;
}

// Tile lists of the instances still active, written over the device lists
// (which they never outgrow): a retired instance's tiles would only start
// blocks that leave at once.  Each listed instance's level-0 partial sums move
// with its tiles (tile_beg).  The step graph is rebuilt; the persistent
// kernel takes the new counts.  Results do not change.
static ifx_status compact_tiles(ifx_solver* S) {
    const int n = (int)S->inst.size();
    std::vector<char> keep(n);
    for (int k = 0; k < n; k++) keep[k] = S->inst[k].dev.retired ? 0 : 1;
    auto filt = [&](const std::vector<Tile>& v) {
        std::vector<Tile> o;
        for (const Tile& t : v)
            if (keep[t.inst]) o.push_back(t);
        return o;
    };
    auto put = [&](Tile* d, const std::vector<Tile>& v) -> cudaError_t {
        return v.empty() ? cudaSuccess
                         : cudaMemcpyAsync(d, v.data(), v.size() * sizeof(Tile), cudaMemcpyHostToDevice, S->stream);
    };
    const std::vector<Tile> t0 = filt(S->hT0full), t0w = filt(S->hT0Wfull);
    CUDA_TRY(put(S->dT0, t0));
    CUDA_TRY(put(S->dT0W, t0w));
    S->nt0 = (int)t0.size();
    S->nt0W = (int)t0w.size();
    for (int l = 1; l < S->lmax; l++) {
        const std::vector<Tile> a = filt(S->hTsmFull[l]), b = filt(S->hTreFull[l]);
        const std::vector<Tile> c = filt(S->hTsmWFull[l]), d = filt(S->hTreWFull[l]);
        CUDA_TRY(put(S->dTsm[l], a));
        CUDA_TRY(put(S->dTre[l], b));
        CUDA_TRY(put(S->dTsmW[l], c));
        CUDA_TRY(put(S->dTreW[l], d));
        S->ntsm[l] = (int)a.size();
        S->ntre[l] = (int)b.size();
        S->ntsmW[l] = (int)c.size();
        S->ntreW[l] = (int)d.size();
        S->plan.ntsm[l] = S->ntsm[l];
        S->plan.ntre[l] = S->ntre[l];
    }
    S->plan.nt0 = S->nt0;
    for (size_t q = 0; q < t0.size(); q++) {
        const int k = t0[q].inst;
        if (q > 0 && t0[q - 1].inst == k) continue;
        Instance& I = S->inst[k];
        I.tile_beg = (int)q;
        I.dev.tile_beg = (int)q;
        CUDA_TRY(cudaMemcpyAsync(&S->dI[k].tile_beg, &I.dev.tile_beg, sizeof(int), cudaMemcpyHostToDevice, S->stream));
    }
    CUDA_TRY(cudaStreamSynchronize(S->stream));
    S->in_lists = keep;
    S->listed = 0;
    for (char c : keep) S->listed += c;
    if (S->gexec) {
        cudaGraphExecDestroy(S->gexec);
        cudaGraphDestroy(S->graph);
        S->gexec = nullptr;
        S->graph = nullptr;
    }
    return IFX_OK;
}

extern "C" ifx_status ifx_set_instance_active(ifx_solver* S, int inst, int active) {
    if (!S || inst < 0 || inst >= (int)S->inst.size()) return set_error(IFX_ERR_ARG, "ifx_set_instance_active: bad argument");
    if (S->mode != IFX_MODE_METHOD) return set_error(IFX_ERR_STATE, "ifx_set_instance_active needs a METHOD-mode solver");
    CUDA_TRY(cudaSetDevice(S->device));
    IFX_TRY(step_finish(S));
    Instance& I = S->inst[inst];
    I.dev.retired = active ? 0 : 1;
    CUDA_TRY(cudaMemcpyAsync(&S->dI[inst].retired, &I.dev.retired, sizeof(int), cudaMemcpyHostToDevice, S->stream));
    CUDA_TRY(cudaStreamSynchronize(S->stream));
    // list the active instances only, once half of the listed ones are gone
    // (or when an instance that is not listed comes back)
    int nact = 0;
    for (const Instance& J : S->inst) nact += J.dev.retired ? 0 : 1;
    if ((active && !S->in_lists[inst]) || (!active && nact > 0 && S->inst.size() > 1 && 2 * nact <= S->listed))
        IFX_TRY(compact_tiles(S));
    return IFX_OK;
}

// Rows per thread of the multigrid tile phases, or the cluster V-cycle; the
// step graph is rebuilt on change.
static void drop_graph(ifx_solver* S) {
    if (S->gexec) cudaGraphExecDestroy(S->gexec);
    if (S->graph) cudaGraphDestroy(S->graph);
    S->gexec = nullptr;
    S->graph = nullptr;
}
static void set_mg_rows(ifx_solver* S, int rows) {
    if (rows == S->mg_rows) return;
    drop_graph(S);
    S->mg_rows = rows;
}
static void set_cluster_mg(ifx_solver* S, int on) {
    on = on && S->cmg_ok;
    if (on == S->cmg_use) return;
    drop_graph(S);
    S->cmg_use = on;
}

namespace {
// Device copy of the state a time step carries to the next one (cell and
// face velocities, convection history, pressure, outflow boundary values and
// the per-instance iteration state).
struct StateSnapshot {
    std::vector<std::pair<void*, size_t>> items;  // (source, bytes)
    std::vector<void*> copies;
    ifx_status take(ifx_solver* S) {
        for (const Instance& I : S->inst) {
            const InstDev& d = I.dev;
            const size_t nc = I.ncell * sizeof(double), nq = 4 * (size_t)I.qstride * sizeof(double);
            for (void* p : {(void*)d.u, (void*)d.v, (void*)d.U, (void*)d.V, (void*)d.Nu, (void*)d.Nv, (void*)d.p,
                            (void*)d.pold, (void*)d.pold2, (void*)d.dup, (void*)d.dvp})
                items.push_back({p, nc});
            items.push_back({(void*)d.qbu, nq});
            items.push_back({(void*)d.qbv, nq});
            if (d.hist_cap > 0) items.push_back({(void*)d.hist, (size_t)d.hist_cap * d.hist_w * sizeof(double)});
        }
        items.push_back({(void*)S->dS, S->inst.size() * sizeof(InstState)});
        for (auto& it : items) {
            void* c = nullptr;
            CUDA_TRY(cudaMalloc(&c, it.second));
            copies.push_back(c);
            CUDA_TRY(cudaMemcpyAsync(c, it.first, it.second, cudaMemcpyDeviceToDevice, S->stream));
        }
        CUDA_TRY(cudaStreamSynchronize(S->stream));
        return IFX_OK;
    }
    ifx_status restore(ifx_solver* S) {
        for (size_t k = 0; k < items.size(); k++)
            CUDA_TRY(cudaMemcpyAsync(items[k].first, copies[k], items[k].second, cudaMemcpyDeviceToDevice, S->stream));
        CUDA_TRY(cudaStreamSynchronize(S->stream));
        return IFX_OK;
    }
    ~StateSnapshot() {
        for (void* c : copies) cudaFree(c);
    }
};
}  // namespace

extern "C" ifx_status ifx_autotune(ifx_solver* S, int steps, int* chosen, double* ms_per_step) {
    if (!S || steps < 1) return set_error(IFX_ERR_ARG, "ifx_autotune: bad argument");
    if (S->mode != IFX_MODE_METHOD) return set_error(IFX_ERR_STATE, "ifx_autotune needs a METHOD-mode solver");
    // the trial steps of a moving body rewrite its geometry (cell types, ghost
    // slots, stencil bytes) for later poses, and the snapshot restores only the
    // flow state
    if (S->nmv > 0)
        return set_error(IFX_ERR_STATE, "ifx_autotune: a moving body's trial steps would move its geometry, which the "
                                        "restored state does not include; set the execution mode directly");
    CUDA_TRY(cudaSetDevice(S->device));
    IFX_TRY(step_finish(S));
    StateSnapshot snap;
    IFX_TRY(snap.take(S));
    const long long steps0 = S->steps_done;
    const int saved = S->exec_override, saved_rows = S->mg_rows, saved_cmg = S->cmg_use;
    const int saved_grid = S->persist_grid;
    // (execution mode, rows per thread of the multigrid tile phases, cluster
    // V-cycle, persistent grid); the persistent kernel always uses 32x8 tiles
    struct Cand {
        int mode, rows, cmg, grid;
    };
    std::vector<Cand> cand;
    if (S->persist_full > 0) {
        cand.push_back({IFX_EXEC_PERSISTENT, 1, 0, S->persist_full});
        // a few instances: also one block per SM (fewer arrivals per grid
        // barrier; fewer blocks than SMs measured slower on every workload)
        if (S->inst.size() <= 8 && S->persist_sms < S->persist_full)
            cand.push_back({IFX_EXEC_PERSISTENT, 1, 0, S->persist_sms});
    }
    cand.push_back({IFX_EXEC_GRAPH, 1, 0, saved_grid});
    cand.push_back({IFX_EXEC_GRAPH, MG_ROWS_WIDE, 0, saved_grid});
    if (S->cmg_ok) cand.push_back({IFX_EXEC_GRAPH, 1, 1, saved_grid});
    Cand best = cand[0];
    double best_ms = 1e300;
    ifx_status st = IFX_OK;
    for (const auto& c : cand) {
        S->exec_override = c.mode;
        set_mg_rows(S, c.rows);
        set_cluster_mg(S, c.cmg);
        S->persist_grid = c.grid;
        st = ifx_step(S, 1);  // warm-up (builds the graph on first use)
        if (st == IFX_OK) st = ifx_step(S, steps);
        if (st == IFX_OK) st = snap.restore(S);
        if (st != IFX_OK) break;
        const double ms = S->last_ms / steps;
        if (ms < best_ms) {
            best_ms = ms;
            best = c;
        }
    }
    S->steps_done = steps0;
    if (st != IFX_OK) {
        S->exec_override = saved;
        set_mg_rows(S, saved_rows);
        set_cluster_mg(S, saved_cmg);
        S->persist_grid = saved_grid;
        snap.restore(S);
        return st;
    }
    S->exec_override = best.mode;
    set_mg_rows(S, best.rows);
    set_cluster_mg(S, best.cmg);
    S->persist_grid = best.grid;
    if (chosen) *chosen = best.mode;
    if (ms_per_step) *ms_per_step = best_ms;
    return IFX_OK;
}

// ------------------------------------------------------------ sweep schedule

namespace {
ifx_schedule schedule_of(const ifx_config& c) {
    ifx_schedule s;
    s.mg_pre = c.mg_pre;
    s.mg_post = c.mg_post;
    s.mg_omega = c.mg_omega;
    s.coarse_sweeps = c.coarse_sweeps;
    s.mixed_inner = c.mixed_inner;
    s.restart_drop = c.restart_drop;
    s.restart_every = c.restart_every;
    return s;
}
bool same_schedule(const ifx_schedule& a, const ifx_schedule& b) {
    return a.mg_pre == b.mg_pre && a.mg_post == b.mg_post && a.mg_omega == b.mg_omega &&
           a.coarse_sweeps == b.coarse_sweeps && a.mixed_inner == b.mixed_inner && a.restart_drop == b.restart_drop &&
           a.restart_every == b.restart_every;
}
ifx_status check_schedule(const ifx_schedule* s) {
    if (!s) return set_error(IFX_ERR_ARG, "schedule: null");
    if (s->mg_pre < 1 || s->mg_post < 1 || s->mg_pre > 16 || s->mg_post > 16)
        return set_error(IFX_ERR_ARG, "schedule: multigrid sweeps must lie in 1..16");
    if (!(s->mg_omega > 0 && s->mg_omega < 2)) return set_error(IFX_ERR_ARG, "schedule: omega must lie in (0, 2)");
    if (s->coarse_sweeps < 1 || s->coarse_sweeps > 10000)
        return set_error(IFX_ERR_ARG, "schedule: coarse sweeps must lie in 1..10000");
    if (s->mixed_inner < 2) return set_error(IFX_ERR_ARG, "schedule: mixed_inner must be >= 2");
    if (!(s->restart_drop > 0 && s->restart_drop < 1) || s->restart_every < 1)
        return set_error(IFX_ERR_ARG, "schedule: restart_drop in (0, 1), restart_every >= 1");
    return IFX_OK;
}
// Every instance takes the schedule: host configuration, device descriptor
// (omega, coarse sweeps, restart rule, mixed_inner), the persistent plan's
// sweep counts; the step graph is rebuilt on next use (it holds the sweep
// counts and omega as launch parameters).  The descriptors are read back from
// the device first: a moving body's pose lives there.
ifx_status apply_schedule(ifx_solver* S, const ifx_schedule& s) {
    std::vector<InstDev> h(S->inst.size());
    CUDA_TRY(cudaMemcpyAsync(h.data(), S->dI, h.size() * sizeof(InstDev), cudaMemcpyDeviceToHost, S->stream));
    CUDA_TRY(cudaStreamSynchronize(S->stream));
    for (size_t k = 0; k < S->inst.size(); k++) {
        Instance& I = S->inst[k];
        I.cfg.mg_pre = s.mg_pre;
        I.cfg.mg_post = s.mg_post;
        I.cfg.mg_omega = s.mg_omega;
        I.cfg.coarse_sweeps = s.coarse_sweeps;
        I.cfg.mixed_inner = s.mixed_inner;
        I.cfg.restart_drop = s.restart_drop;
        I.cfg.restart_every = s.restart_every;
        I.dev.omega = s.mg_omega;
        I.dev.coarse_sweeps = s.coarse_sweeps;
        I.dev.mixed_inner = s.mixed_inner;
        I.dev.restart_drop = s.restart_drop;
        I.dev.restart_every = s.restart_every;
        h[k].omega = s.mg_omega;
        h[k].coarse_sweeps = s.coarse_sweeps;
        h[k].mixed_inner = s.mixed_inner;
        h[k].restart_drop = s.restart_drop;
        h[k].restart_every = s.restart_every;
        h[k].retired = I.dev.retired;
    }
    CUDA_TRY(cudaMemcpyAsync(S->dI, h.data(), h.size() * sizeof(InstDev), cudaMemcpyHostToDevice, S->stream));
    CUDA_TRY(cudaStreamSynchronize(S->stream));
    drop_graph(S);
    S->mg_pre = S->plan.mg_pre = s.mg_pre;
    S->mg_post = S->plan.mg_post = s.mg_post;
    return IFX_OK;
}
}  // namespace

extern "C" ifx_status ifx_set_schedule(ifx_solver* S, const ifx_schedule* sched) {
    if (!S) return set_error(IFX_ERR_ARG, "ifx_set_schedule: null solver");
    if (S->mode != IFX_MODE_METHOD) return set_error(IFX_ERR_STATE, "ifx_set_schedule needs a METHOD-mode solver");
    IFX_TRY(check_schedule(sched));
    CUDA_TRY(cudaSetDevice(S->device));
    IFX_TRY(step_finish(S));
    return apply_schedule(S, *sched);
}

extern "C" ifx_status ifx_get_schedule(const ifx_solver* S, int inst, ifx_schedule* out) {
    if (!S || !out || inst < 0 || inst >= (int)S->inst.size()) return set_error(IFX_ERR_ARG, "ifx_get_schedule: bad argument");
    *out = schedule_of(S->inst[inst].cfg);
    return IFX_OK;
}

extern "C" ifx_status ifx_autotune_schedule(ifx_solver* S, int steps, ifx_schedule* chosen, double* ms_per_step) {
    if (!S || steps < 1) return set_error(IFX_ERR_ARG, "ifx_autotune_schedule: bad argument");
    if (S->mode != IFX_MODE_METHOD) return set_error(IFX_ERR_STATE, "ifx_autotune_schedule needs a METHOD-mode solver");
    if (S->nmv > 0)
        return set_error(IFX_ERR_STATE, "ifx_autotune_schedule: a moving body's trial steps would move its geometry, "
                                        "which the restored state does not include; set the schedule directly");
    CUDA_TRY(cudaSetDevice(S->device));
    IFX_TRY(step_finish(S));
    StateSnapshot snap;
    IFX_TRY(snap.take(S));
    const long long steps0 = S->steps_done;
    const int n = (int)S->inst.size();
    std::vector<int> retired0(n), status0(S->inst_status.begin(), S->inst_status.end());
    for (int k = 0; k < n; k++) retired0[k] = S->inst[k].dev.retired;
    const ifx_schedule start = schedule_of(S->inst[0].cfg);
    // one candidate: a warm-up step (rebuilds the graph), `steps` timed steps
    // from the same state, then the state, the statuses and the retirements
    // are put back; a schedule is valid when every pressure solve of the timed
    // steps met its stop rule and no instance diverged
    auto trial = [&](const ifx_schedule& c, double* ms) -> ifx_status {
        IFX_TRY(apply_schedule(S, c));
        ifx_status st = ifx_step(S, 1);
        if (st == IFX_OK) st = ifx_step(S, steps);
        bool ok = st == IFX_OK;
        *ms = S->last_ms / steps;
        for (int k = 0; k < n && ok; k++)
            ok = retired0[k] || (S->inst_status[k] == status0[k] && S->hS[k].ppe_rel <= S->inst[k].cfg.ppe_tol);
        if (!ok) *ms = 1e300;
        if (S->poisoned) return set_error(IFX_ERR_CUDA, "ifx_autotune_schedule: a grid barrier timed out");
        IFX_TRY(snap.restore(S));
        for (int k = 0; k < n; k++) {
            S->inst[k].dev.retired = retired0[k];
            S->inst_status[k] = status0[k];
        }
        S->steps_done = steps0;
        return IFX_OK;  // apply_schedule of the next trial uploads the descriptors (retired flags included)
    };
    ifx_schedule best = start;
    double best_ms = 1e300;
    ifx_status st = trial(best, &best_ms);
    // coordinate search, one pass: a change is kept when it is faster by more
    // than 1 % (timing noise)
    auto consider = [&](ifx_schedule c) {
        if (st != IFX_OK || same_schedule(c, best)) return;
        double ms = 0;
        st = trial(c, &ms);
        if (st == IFX_OK && ms < 0.99 * best_ms) {
            best = c;
            best_ms = ms;
        }
    };
    const int pp[5][2] = {{1, 1}, {2, 2}, {1, 2}, {2, 1}, {3, 3}};
    const ifx_schedule b0 = best;
    for (auto& q : pp) {
        ifx_schedule c = b0;
        c.mg_pre = q[0];
        c.mg_post = q[1];
        consider(c);
    }
    const ifx_schedule b1 = best;
    for (double om : {0.6, 0.7, 0.8, 0.9}) {
        ifx_schedule c = b1;
        c.mg_omega = om;
        consider(c);
    }
    const ifx_schedule b2 = best;
    for (int cs : {10, 20, 40, 80}) {
        ifx_schedule c = b2;
        c.coarse_sweeps = cs;
        consider(c);
    }
    if (S->prec == IFX_PREC_MIXED) {
        const ifx_schedule b3 = best;
        for (int mi : {4, 8, 16}) {
            ifx_schedule c = b3;
            c.mixed_inner = mi;
            consider(c);
        }
        const ifx_schedule b4 = best;
        for (double rd : {1e-3, 1e-4, 1e-5}) {
            ifx_schedule c = b4;
            c.restart_drop = rd;
            consider(c);
        }
    }
    if (st != IFX_OK) {
        apply_schedule(S, start);
        return st;
    }
    if (best_ms >= 1e300) {
        IFX_TRY(apply_schedule(S, start));
        return set_error(IFX_ERR_NOT_CONVERGED, "ifx_autotune_schedule: no schedule met the stop rule");
    }
    IFX_TRY(apply_schedule(S, best));
    if (chosen) *chosen = best;
    if (ms_per_step) *ms_per_step = best_ms;
    return IFX_OK;
}

extern "C" ifx_status ifx_set_mg_tile_rows(ifx_solver* S, int rows) {
    if (!S || (rows != 1 && rows != MG_ROWS_WIDE)) return set_error(IFX_ERR_ARG, "ifx_set_mg_tile_rows: rows must be 1 or 4");
    if (S->mode != IFX_MODE_METHOD) return set_error(IFX_ERR_STATE, "ifx_set_mg_tile_rows needs a METHOD-mode solver");
    CUDA_TRY(cudaSetDevice(S->device));
    IFX_TRY(step_finish(S));
    set_mg_rows(S, rows);
    return IFX_OK;
}

extern "C" ifx_status ifx_set_cluster_vcycle(ifx_solver* S, int on) {
    if (!S) return set_error(IFX_ERR_ARG, "ifx_set_cluster_vcycle: null solver");
    if (S->mode != IFX_MODE_METHOD) return set_error(IFX_ERR_STATE, "ifx_set_cluster_vcycle needs a METHOD-mode solver");
    if (on && !S->cmg_ok) return set_error(IFX_ERR_STATE, "the cluster V-cycle does not fit these instances on this device");
    CUDA_TRY(cudaSetDevice(S->device));
    IFX_TRY(step_finish(S));
    set_cluster_mg(S, on);
    return IFX_OK;
}

extern "C" ifx_status ifx_get_cluster_vcycle(const ifx_solver* S, int* available, int* on) {
    if (!S) return set_error(IFX_ERR_ARG, "ifx_get_cluster_vcycle: null solver");
    if (available) *available = S->cmg_ok;
    if (on) *on = S->cmg_use;
    return IFX_OK;
}

extern "C" ifx_status ifx_get_mg_tile_rows(const ifx_solver* S, int* rows) {
    if (!S || !rows) return set_error(IFX_ERR_ARG, "ifx_get_mg_tile_rows: bad argument");
    *rows = S->mg_rows;
    return IFX_OK;
}

extern "C" ifx_status ifx_device_bytes(const ifx_solver* S, size_t* bytes) {
    if (!S || !bytes) return set_error(IFX_ERR_ARG, "ifx_device_bytes: bad argument");
    *bytes = S->device_bytes;
    return IFX_OK;
}

extern "C" ifx_status ifx_ppe_reference(ifx_solver* S, int* iters) {
    if (!S) return set_error(IFX_ERR_ARG, "ifx_ppe_reference: null solver");
    if (S->mode != IFX_MODE_REFERENCE) return set_error(IFX_ERR_STATE, "ifx_ppe_reference needs a REFERENCE-mode solver");
    CUDA_TRY(cudaSetDevice(S->device));
    return ppe_reference(S, iters);
}

extern "C" ifx_status ifx_get_field_i(ifx_solver* S, int inst, int field, double* host, size_t n) {
    if (!S || !host || inst < 0 || inst >= (int)S->inst.size()) return set_error(IFX_ERR_ARG, "ifx_get_field: bad argument");
    if (S->pending_steps) IFX_TRY(step_finish(S));
    const Instance& I = S->inst[inst];
    size_t need;
    IFX_TRY(field_size(I, field, &need));
    if (n != need) return set_error(IFX_ERR_ARG, "ifx_get_field: size mismatch, expected " + std::to_string(need));
    CUDA_TRY(cudaSetDevice(S->device));
    const int nx = I.nx, ny = I.ny;
    if (field == IFX_FIELD_XC) { std::memcpy(host, I.xc.data(), nx * 8); return IFX_OK; }
    if (field == IFX_FIELD_YC) { std::memcpy(host, I.yc.data(), ny * 8); return IFX_OK; }
    if (S->mode == IFX_MODE_REFERENCE) {
        const double* src = nullptr;
        if (field == IFX_FIELD_U) src = S->r_cur ? S->r_ut : S->r_u;
        else if (field == IFX_FIELD_V) src = S->r_cur ? S->r_vt : S->r_v;
        else if (field == IFX_FIELD_P) src = S->r_p;
        else if (field == IFX_FIELD_IBLANK) src = S->r_ib;
        else if (field == IFX_FIELD_UF) src = S->r_uf;
        else if (field == IFX_FIELD_VF) src = S->r_vf;
        else return set_error(IFX_ERR_ARG, "field not available in REFERENCE mode");
        CUDA_TRY(cudaMemcpyAsync(host, src, n * 8, cudaMemcpyDeviceToHost, S->stream));
        CUDA_TRY(cudaStreamSynchronize(S->stream));
        return IFX_OK;
    }
    const InstDev& d = I.dev;
    switch (field) {
        case IFX_FIELD_U: return get_pitched(S, I, d.u, host);
        case IFX_FIELD_V: return get_pitched(S, I, d.v, host);
        case IFX_FIELD_P: return get_pitched(S, I, d.p, host);
        case IFX_FIELD_IBLANK: return get_pitched(S, I, d.iblank, host);
        case IFX_FIELD_DIV: return get_pitched(S, I, d.div, host);
        case IFX_FIELD_CELLTYPE:
            for (int j = 0; j < ny; j++)
                for (int i = 0; i < nx; i++) host[i + j * nx] = I.type[i + j * I.pitch];
            return IFX_OK;
        case IFX_FIELD_UF:
        case IFX_FIELD_VF: {
            std::vector<double> full((size_t)nx * ny);
            IFX_TRY(get_pitched(S, I, field == IFX_FIELD_UF ? d.U : d.V, full.data()));
            if (field == IFX_FIELD_UF) {
                for (int j = 1; j < ny - 1; j++)
                    for (int i = 0; i < nx - 1; i++) host[i + (j - 1) * (nx - 1)] = full[i + j * nx];
            } else {
                for (int j = 0; j < ny - 1; j++)
                    for (int i = 1; i < nx - 1; i++) host[(i - 1) + j * (nx - 2)] = full[i + j * nx];
            }
            return IFX_OK;
        }
    }
    return set_error(IFX_ERR_ARG, "unknown field");
}

extern "C" ifx_status ifx_get_field(ifx_solver* S, int field, double* host, size_t n) {
    return ifx_get_field_i(S, 0, field, host, n);
}

extern "C" ifx_status ifx_set_field_i(ifx_solver* S, int inst, int field, const double* host, size_t n) {
    if (!S || !host || inst < 0 || inst >= (int)S->inst.size()) return set_error(IFX_ERR_ARG, "ifx_set_field: bad argument");
    if (S->pending_steps) IFX_TRY(step_finish(S));
    const Instance& I = S->inst[inst];
    if (field != IFX_FIELD_U && field != IFX_FIELD_V && field != IFX_FIELD_P)
        return set_error(IFX_ERR_ARG, "ifx_set_field: only u, v, p can be set");
    if (n != (size_t)I.nx * I.ny) return set_error(IFX_ERR_ARG, "ifx_set_field: size mismatch");
    CUDA_TRY(cudaSetDevice(S->device));
    double* dst;
    size_t pitch = I.pitch;
    if (S->mode == IFX_MODE_REFERENCE) {
        dst = field == IFX_FIELD_U ? (S->r_cur ? S->r_ut : S->r_u) : field == IFX_FIELD_V ? (S->r_cur ? S->r_vt : S->r_v) : S->r_p;
    } else {
        dst = field == IFX_FIELD_U ? I.dev.u : field == IFX_FIELD_V ? I.dev.v : I.dev.p;
    }
    CUDA_TRY(cudaMemcpy2DAsync(dst, pitch * 8, host, I.nx * 8, I.nx * 8, I.ny, cudaMemcpyHostToDevice, S->stream));
    CUDA_TRY(cudaStreamSynchronize(S->stream));
    return IFX_OK;
}

extern "C" ifx_status ifx_set_field(ifx_solver* S, int field, const double* host, size_t n) {
    return ifx_set_field_i(S, 0, field, host, n);
}

namespace {
// The dense staging buffer of the state calls (three fields of the largest
// instance), allocated on first use in either mode.
ifx_status state_stage(ifx_solver* S, double** out) {
    if (!S->dStage) {
        size_t most = 0;
        for (const Instance& I : S->inst) most = std::max(most, (size_t)I.nx * I.ny);
        IFX_TRY(dalloc(S, &S->dStage, 3 * most));
    }
    *out = S->dStage;
    return IFX_OK;
}

// Host copies of u, v, p (n values each; NULL: skip that field) to or from the
// dense staging buffer: one copy when the three lie back to back in one host
// allocation (v = u + n, p = v + n), as in the staging buffer, else one each.
cudaError_t copy_state_in(double* stage, const double* const h[3], size_t n, cudaStream_t st) {
    if (h[0] && h[1] == h[0] + n && h[2] == h[1] + n)
        return cudaMemcpyAsync(stage, h[0], 3 * n * 8, cudaMemcpyHostToDevice, st);
    for (int k = 0; k < 3; k++)
        if (h[k]) {
            const cudaError_t e = cudaMemcpyAsync(stage + k * n, h[k], n * 8, cudaMemcpyHostToDevice, st);
            if (e != cudaSuccess) return e;
        }
    return cudaSuccess;
}
cudaError_t copy_state_out(double* const h[3], const double* stage, size_t n, cudaStream_t st) {
    if (h[0] && h[1] == h[0] + n && h[2] == h[1] + n)
        return cudaMemcpyAsync(h[0], stage, 3 * n * 8, cudaMemcpyDeviceToHost, st);
    for (int k = 0; k < 3; k++)
        if (h[k]) {
            const cudaError_t e = cudaMemcpyAsync(h[k], stage + k * n, n * 8, cudaMemcpyDeviceToHost, st);
            if (e != cudaSuccess) return e;
        }
    return cudaSuccess;
}

// The device arrays of u, v, p of one instance and their row pitch.
void state_arrays(ifx_solver* S, const Instance& I, double* (&f)[3], size_t& pitch) {
    if (S->mode == IFX_MODE_REFERENCE) {
        f[0] = S->r_cur ? S->r_ut : S->r_u;
        f[1] = S->r_cur ? S->r_vt : S->r_v;
        f[2] = S->r_p;
        pitch = I.nx;
    } else {
        f[0] = I.dev.u;
        f[1] = I.dev.v;
        f[2] = I.dev.p;
        pitch = I.pitch;
    }
}
}  // namespace

extern "C" ifx_status ifx_set_state(ifx_solver* S, int inst, const double* u, const double* v, const double* p,
                                    size_t n) {
    if (!S || inst < 0 || inst >= (int)S->inst.size() || (!u && !v && !p))
        return set_error(IFX_ERR_ARG, "ifx_set_state: bad argument");
    if (S->pending_steps) IFX_TRY(step_finish(S));
    const Instance& I = S->inst[inst];
    if (n != (size_t)I.nx * I.ny) return set_error(IFX_ERR_ARG, "ifx_set_state: size mismatch");
    CUDA_TRY(cudaSetDevice(S->device));
    double* f[3];
    size_t pitch;
    state_arrays(S, I, f, pitch);
    double* stage = nullptr;
    IFX_TRY(state_stage(S, &stage));
    const double* h[3] = {u, v, p};
    double* dst[3];
    for (int k = 0; k < 3; k++) dst[k] = h[k] ? f[k] : nullptr;
    CUDA_TRY(copy_state_in(stage, h, n, S->stream));
    CUDA_TRY(launch_state_unpack(stage, dst[0], dst[1], dst[2], I.nx, I.ny, (int)pitch, S->stream));
    S->launches++;
    CUDA_TRY(cudaStreamSynchronize(S->stream));
    return IFX_OK;
}

extern "C" ifx_status ifx_get_state(ifx_solver* S, int inst, double* u, double* v, double* p, size_t n) {
    if (!S || inst < 0 || inst >= (int)S->inst.size() || (!u && !v && !p))
        return set_error(IFX_ERR_ARG, "ifx_get_state: bad argument");
    if (S->pending_steps) IFX_TRY(step_finish(S));
    const Instance& I = S->inst[inst];
    if (n != (size_t)I.nx * I.ny) return set_error(IFX_ERR_ARG, "ifx_get_state: size mismatch");
    CUDA_TRY(cudaSetDevice(S->device));
    double* f[3];
    size_t pitch;
    state_arrays(S, I, f, pitch);
    double* stage = nullptr;
    IFX_TRY(state_stage(S, &stage));
    double* h[3] = {u, v, p};
    const double* src[3];
    for (int k = 0; k < 3; k++) src[k] = h[k] ? f[k] : nullptr;
    CUDA_TRY(launch_state_pack(src[0], src[1], src[2], stage, I.nx, I.ny, (int)pitch, S->stream));
    S->launches++;
    CUDA_TRY(copy_state_out(h, stage, n, S->stream));
    CUDA_TRY(cudaStreamSynchronize(S->stream));
    return IFX_OK;
}

// ifx_set_state, nsteps steps and ifx_get_state in one call: the copies, the
// layout kernels and the steps are issued back to back on the solver's stream
// and the call waits once, at the end.
extern "C" ifx_status ifx_step_state(ifx_solver* S, int inst, const double* u_in, const double* v_in,
                                     const double* p_in, int nsteps, double* u_out, double* v_out, double* p_out,
                                     size_t n) {
    if (!S || inst < 0 || inst >= (int)S->inst.size() || nsteps < 0)
        return set_error(IFX_ERR_ARG, "ifx_step_state: bad argument");
    if (S->mode == IFX_MODE_REFERENCE) {  // its step waits on the host every Jacobi sweep anyway
        if (u_in || v_in || p_in) IFX_TRY(ifx_set_state(S, inst, u_in, v_in, p_in, n));
        IFX_TRY(ifx_step(S, nsteps));
        return (u_out || v_out || p_out) ? ifx_get_state(S, inst, u_out, v_out, p_out, n) : IFX_OK;
    }
    if (S->pending_steps) IFX_TRY(step_finish(S));
    const Instance& I = S->inst[inst];
    if (n != (size_t)I.nx * I.ny) return set_error(IFX_ERR_ARG, "ifx_step_state: size mismatch");
    CUDA_TRY(cudaSetDevice(S->device));
    double* f[3];
    size_t pitch;
    state_arrays(S, I, f, pitch);
    double* stage = nullptr;
    IFX_TRY(state_stage(S, &stage));
    const double* hi[3] = {u_in, v_in, p_in};
    if (u_in || v_in || p_in) {
        double* dst[3];
        for (int k = 0; k < 3; k++) dst[k] = hi[k] ? f[k] : nullptr;
        CUDA_TRY(copy_state_in(stage, hi, n, S->stream));
        CUDA_TRY(launch_state_unpack(stage, dst[0], dst[1], dst[2], I.nx, I.ny, (int)pitch, S->stream));
        S->launches++;
    }
    ifx_status st = IFX_OK;
    if (nsteps > 0) {
        st = S->prec == IFX_PREC_FP64 ? step_launch<double>(S, nsteps) : step_launch<float>(S, nsteps);
        if (st != IFX_OK) {
            cudaStreamSynchronize(S->stream);  // the input copies read the caller's buffers
            return st;
        }
    }
    double* ho[3] = {u_out, v_out, p_out};
    if (u_out || v_out || p_out) {
        const double* src[3];
        for (int k = 0; k < 3; k++) src[k] = ho[k] ? f[k] : nullptr;
        CUDA_TRY(launch_state_pack(src[0], src[1], src[2], stage, I.nx, I.ny, (int)pitch, S->stream));
        S->launches++;
        CUDA_TRY(copy_state_out(ho, stage, n, S->stream));
    }
    CUDA_TRY(cudaStreamSynchronize(S->stream));
    return step_finish(S);  // the steps' status (its wait has already passed)
}

extern "C" ifx_status ifx_write_results(ifx_solver* S, const char* dir) {
    if (!S || !dir) return set_error(IFX_ERR_ARG, "ifx_write_results: bad argument");
    if (S->pending_steps) IFX_TRY(step_finish(S));
    const Instance& I = S->inst[0];
    const size_t n = (size_t)I.nx * I.ny;
    std::vector<double> q(n);
    const std::string d(dir);
    struct { int f; const char* name; } outs[4] = {
        {IFX_FIELD_P, "/p.dat"}, {IFX_FIELD_U, "/uc.dat"}, {IFX_FIELD_V, "/vc.dat"}, {IFX_FIELD_IBLANK, "/final_results.dat"}};
    for (auto& o : outs) {
        IFX_TRY(ifx_get_field(S, o.f, q.data(), n));
        IFX_TRY(ifx_write_tecplot((d + o.name).c_str(), I.nx, I.ny, I.xc.data(), I.yc.data(), q.data()));
    }
    return IFX_OK;
}

// IBM ghosts of an instance now: a moving body's count is kept on the device.
static int current_ibm(const ifx_solver* S, int inst) {
    const Instance& I = S->inst[inst];
    return (I.moving && S->hS && S->hS[inst].nstep > 0) ? S->hS[inst].n_ibm : I.n_ibm;
}

extern "C" ifx_status ifx_get_stats(ifx_solver* S, int inst, ifx_stats* out) {
    if (!S || !out || inst < 0 || inst >= (int)S->inst.size()) return set_error(IFX_ERR_ARG, "ifx_get_stats: bad argument");
    if (S->pending_steps) IFX_TRY(step_finish(S));
    std::memset(out, 0, sizeof(*out));
    out->steps = S->steps_done;
    out->kernel_launches = S->launches;
    const Instance& I = S->inst[inst];
    if (S->mode == IFX_MODE_REFERENCE) {
        out->last_ad_iters = S->r_iters.empty() ? 0 : S->r_iters.back();
        for (int it : S->r_iters) out->ad_iters_total += it;
        out->n_fluid = I.NX * I.NY;
        return IFX_OK;
    }
    CUDA_TRY(cudaSetDevice(S->device));
    CUDA_TRY(cudaMemcpyAsync(S->hS, S->dS, S->inst.size() * sizeof(InstState), cudaMemcpyDeviceToHost, S->stream));
    CUDA_TRY(cudaStreamSynchronize(S->stream));
    const InstState& s = S->hS[inst];
    out->last_ad_iters = s.pred_iters;
    out->last_ppe_iters = s.ppe_iters;
    out->last_ad_metric = s.pred_metric;
    out->last_ppe_residual = s.ppe_rel;
    out->max_div = s.max_div;
    out->cd = s.cd;
    out->cl = s.cl;
    out->mass_flux_in = s.flux_in;
    out->mass_flux_out = s.flux_out;
    out->n_fluid = I.n_fluid;
    out->n_ibm_ghost = current_ibm(S, inst);
    out->mg_levels = (int)I.lev.size();
    out->status = inst < (int)S->inst_status.size() ? S->inst_status[inst] : IFX_OK;
    return IFX_OK;
}

extern "C" ifx_status ifx_forces(ifx_solver* S, double* cd, double* cl) {
    ifx_stats st;
    IFX_TRY(ifx_get_stats(S, 0, &st));
    if (cd) *cd = st.cd;
    if (cl) *cl = st.cl;
    return IFX_OK;
}

extern "C" ifx_status ifx_get_ibm_ghosts(ifx_solver* S, int inst, int cap, int* cells, int* nb, double* wu,
                                         double* wp, double* bi_ip, int* count) {
    if (!S || !count || inst < 0 || inst >= (int)S->inst.size()) return set_error(IFX_ERR_ARG, "ifx_get_ibm_ghosts: bad argument");
    if (S->pending_steps) IFX_TRY(step_finish(S));
    const Instance& I = S->inst[inst];
    *count = (S->mode == IFX_MODE_METHOD) ? current_ibm(S, inst) : 0;
    if (*count == 0 || cap <= 0) return IFX_OK;
    CUDA_TRY(cudaSetDevice(S->device));
    std::vector<GhostDev> g(I.ghost_cnt);
    std::vector<double> bip(4 * (size_t)std::max(1, S->nibm));
    CUDA_TRY(cudaMemcpyAsync(g.data(), S->dG + I.ghost_beg, g.size() * sizeof(GhostDev), cudaMemcpyDeviceToHost, S->stream));
    CUDA_TRY(cudaMemcpyAsync(bip.data(), S->dBiIp, bip.size() * sizeof(double), cudaMemcpyDeviceToHost, S->stream));
    CUDA_TRY(cudaStreamSynchronize(S->stream));
    // position of this instance's first IBM ghost in the global IBM list
    int ibase = 0;
    for (int k = 0; k < inst; k++) ibase += S->inst[k].moving ? S->inst[k].ibm_cap : S->inst[k].n_ibm;
    auto dense = [&](int c) { return (c % I.pitch) + (c / I.pitch) * I.nx; };
    int q = 0;
    for (const GhostDev& e : g) {
        if (e.side >= 0 || e.cell < 0) continue;
        if (q >= cap) break;
        if (cells) cells[q] = dense(e.cell);
        for (int k = 0; k < 4; k++) {
            if (nb) nb[4 * q + k] = dense(e.nb[k]);
            if (wu) wu[4 * q + k] = e.wu[k];
            if (wp) wp[4 * q + k] = e.wp[k];
        }
        if (bi_ip)  // recorded at creation: not kept for a moving body
            for (int k = 0; k < 4; k++)
                bi_ip[4 * q + k] = I.moving ? std::nan("") : bip[4 * (size_t)(ibase + q) + k];
        q++;
    }
    return IFX_OK;
}

extern "C" ifx_status ifx_last_step_ms(ifx_solver* S, double* ms) {
    if (!S || !ms) return set_error(IFX_ERR_ARG, "ifx_last_step_ms: bad argument");
    if (S->pending_steps) IFX_TRY(step_finish(S));
    *ms = S->last_ms;
    return IFX_OK;
}

template <typename T>
static ifx_status profile_kernel(ifx_solver* S, int kernel, int reps, double* ms) {
    cudaStream_t st = S->stream;
    const int n = (int)S->inst.size();
    CUDA_TRY(launch_step_begin(S->dI, S->dS, n, S->dCtl, st));
    auto one = [&]() -> cudaError_t {
        switch (kernel) {
            case 0: {  // the finest-level sweep as the step launches it (the handle's tile shape)
                const int R = S->mg_rows;
                const Tile* t0 = R == MG_ROWS_WIDE ? S->dT0W : S->dT0;
                const int nt0 = R == MG_ROWS_WIDE ? S->nt0W : S->nt0;
                if (S->inst.size() == 1 && S->dTmap)
                    return launch_smooth_grid_tma<T>(grid_of(S, 0, R), nt0, S->dS, S->dG, S->dTmap, 0, 0, R, S->dErr, st);
                if (S->inst.size() == 1) return launch_smooth_grid<T>(grid_of(S, 0, R), nt0, S->dS, S->dG, 0, 0, R, st);
                if (S->dTmap)
                    return launch_smooth_tma<T>(t0, nt0, S->dLV, S->dI, S->dS, S->dG, S->dTmap, 0, 0, R, S->dErr, st);
                return launch_smooth<T>(t0, nt0, S->dLV, S->dI, S->dS, S->dG, 0, 0, R, st);
            }
            case 1: return launch_bicg_apply<T>(S->dT0, S->nt0, S->dLV, S->dI, S->dS, S->dG, S->dPart, 0, 0, 1, st);
            case 2: return launch_pred_sweep(S->dT0, S->nt0, S->dG, S->ng, S->dI, S->dS, S->dPart, 0, st);
            case 4: return launch_barrier_bench(S->dBar, S->persist_grid, 1000, st);
            case 5: return launch_subcycle<T>(S->dSub, n, S->dLV, S->dI, S->dS, S->mg_pre, S->mg_post, S->sub_bytes, st);
            default: return launch_conv_rhs(S->dT0, S->nt0, S->dI, S->dS, st);
        }
    };
    CUDA_TRY(one());  // warm
    CUDA_TRY(cudaEventRecord(S->ev0, st));
    for (int k = 0; k < reps; k++) CUDA_TRY(one());
    CUDA_TRY(cudaEventRecord(S->ev1, st));
    CUDA_TRY(cudaEventSynchronize(S->ev1));
    float t = 0.f;
    CUDA_TRY(cudaEventElapsedTime(&t, S->ev0, S->ev1));
    *ms = kernel == 4 ? t / reps / 1000.0 : t / reps;
    S->launches += reps + 2;
    return IFX_OK;
}

extern "C" ifx_status ifx_profile_kernel(ifx_solver* S, int kernel, int reps, double* ms_per_launch,
                                         long long* cells) {
    if (!S || !ms_per_launch || reps < 1 || kernel < 0 || kernel > 5) return set_error(IFX_ERR_ARG, "ifx_profile_kernel: bad argument");
    if (S->pending_steps) IFX_TRY(step_finish(S));
    if (kernel == 4 && S->persist_grid == 0) return set_error(IFX_ERR_STATE, "cooperative launch unavailable");
    if (S->mode != IFX_MODE_METHOD) return set_error(IFX_ERR_STATE, "ifx_profile_kernel needs a METHOD-mode solver");
    CUDA_TRY(cudaSetDevice(S->device));
    long long c = 0;
    for (auto& I : S->inst) c += (long long)I.NX * I.NY;
    if (cells) *cells = c;
    if (S->prec == IFX_PREC_FP64) return profile_kernel<double>(S, kernel, reps, ms_per_launch);
    return profile_kernel<float>(S, kernel, reps, ms_per_launch);
}

extern "C" ifx_status ifx_set_barrier_fault(ifx_solver* S, long long spin_limit, int withhold_arrival) {
    if (!S) return set_error(IFX_ERR_ARG, "ifx_set_barrier_fault: bad argument");
    if (S->mode != IFX_MODE_METHOD || S->persist_grid == 0)
        return set_error(IFX_ERR_STATE, "ifx_set_barrier_fault needs the persistent kernel");
    S->plan.spin_limit = spin_limit > 0 ? spin_limit : kSpinLimit;
    S->plan.withhold_arrival = withhold_arrival != 0;
    return IFX_OK;
}

extern "C" ifx_status ifx_trace_step(ifx_solver* S, int cap, double* us, int* n) {
    if (!S || !us || !n || cap < 1) return set_error(IFX_ERR_ARG, "ifx_trace_step: bad argument");
    if (S->pending_steps) IFX_TRY(step_finish(S));
    if (S->mode != IFX_MODE_METHOD || S->persist_grid == 0) return set_error(IFX_ERR_STATE, "ifx_trace_step needs the persistent kernel");
    CUDA_TRY(cudaSetDevice(S->device));
    long long* d = nullptr;
    IFX_TRY(dalloc(S, &d, (size_t)cap + 1));
    CUDA_TRY(cudaMemsetAsync(d, 0, sizeof(long long) * (cap + 1), S->stream));
    S->plan.trace = d;
    S->plan.trace_cap = cap + 1;
    S->plan.nsteps = 1;
    cudaError_t e = S->prec == IFX_PREC_FP64 ? launch_persist_step<double>(S->plan, S->persist_grid, S->stream)
                                             : launch_persist_step<float>(S->plan, S->persist_grid, S->stream);
    S->plan.trace = nullptr;
    S->plan.trace_cap = 0;
    S->plan.spin_limit = kSpinLimit;
    S->plan.withhold_arrival = 0;
    if (e != cudaSuccess) return cuerr(e, "ifx_trace_step");
    std::vector<long long> h(cap + 1);
    CUDA_TRY(cudaMemcpyAsync(h.data(), d, sizeof(long long) * (cap + 1), cudaMemcpyDeviceToHost, S->stream));
    CUDA_TRY(cudaStreamSynchronize(S->stream));
    int khz = 0;
    CUDA_TRY(cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, S->device));
    int k = 0;
    while (k < cap && h[k + 1] != 0) {
        us[k] = (double)(h[k + 1] - h[k]) / (khz * 1e-3);
        k++;
    }
    *n = k;
    S->steps_done += 1;
    S->launches += 1;
    return check_states(S);
}

extern "C" ifx_status ifx_synchronize(ifx_solver* S) {
    if (!S) return set_error(IFX_ERR_ARG, "ifx_synchronize: null solver");
    if (S->pending_steps) IFX_TRY(step_finish(S));
    CUDA_TRY(cudaStreamSynchronize(S->stream));
    return IFX_OK;
}

extern "C" void ifx_destroy(ifx_solver* S) {
    if (!S) return;
    cudaSetDevice(S->device);
    if (S->stream) cudaStreamSynchronize(S->stream);
    if (S->gexec) cudaGraphExecDestroy(S->gexec);
    if (S->graph) cudaGraphDestroy(S->graph);
    for (void* p : S->allocs) cudaFree(p);
    if (S->hS) cudaFreeHost(S->hS);
    if (S->hCtl) cudaFreeHost(S->hCtl);
    if (S->h_flag) cudaFreeHost(S->h_flag);
    if (S->h_out) cudaFreeHost(S->h_out);
    if (S->r_iters_h) cudaFreeHost(S->r_iters_h);
    if (S->ev0) cudaEventDestroy(S->ev0);
    if (S->ev1) cudaEventDestroy(S->ev1);
    if (S->ev2) cudaEventDestroy(S->ev2);
    if (S->stream) cudaStreamDestroy(S->stream);
    delete S;
}
