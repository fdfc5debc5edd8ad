// kernels_ibm.cu -- immersed-boundary set-up on the device: iBlank tagging,
// ghost-cell marking and image-point interpolation weights.
//
// The reference tags cells with an FP32 circle test that is commented out
// (src/include/preSim.cu:110-136) and has no ghost-cell code at all; this is
// the ghost-cell method of Mittal et al. (J. Comput. Phys. 227, 2008):
// ghost cell G (solid, with a fluid cell among its 8 neighbours) -> body
// intercept BI (closest boundary point) -> image point IP = 2 BI - G ->
// bilinear stencil of the 4 cell centres around IP.  When G itself is one of
// the 4 nodes its row is replaced by the boundary condition at BI
// (Dirichlet for velocity, zero normal derivative for pressure), and the 4x4
// system is solved in FP64.
//
// This file is compiled with -fmad=false: every product and sum is rounded
// separately, like the oracle built with -ffp-contract=off, so iBlank, the
// ghost list and the weights match the CPU restatement bit for bit.
#include <cuda_runtime.h>

#include "ibm_geom.cuh"
#include "ifx_dev.h"
#include "ifx_kernels.h"

namespace ifx {

__global__ void k_tag(const InstDev* __restrict__ I, int inst, uint8_t* __restrict__ type) {
    const InstDev& in = I[inst];
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= in.nx * in.ny) return;
    const int i = q % in.nx, j = q / in.nx;
    const int id = i + j * in.pitch;
    const int ins = in.body ? inside_body(in, in.xc[i], in.yc[j]) : 0;
    in.iblank[id] = ins ? 0.0 : 1.0;
    const bool ring = i == 0 || j == 0 || i == in.nx - 1 || j == in.ny - 1;
    type[id] = ring ? T_DOMAIN : (ins ? T_SOLID : T_FLUID);
}

__global__ void k_mark_ghosts(const InstDev* __restrict__ I, int inst, uint8_t* __restrict__ type) {
    const InstDev& in = I[inst];
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= in.NX * in.NY) return;
    const int i = 1 + q % in.NX, j = 1 + q / in.NX;
    const int id = i + j * in.pitch;
    if (type[id] != T_SOLID) return;
    bool g = false;
    for (int dj = -1; dj <= 1; dj++)
        for (int di = -1; di <= 1; di++) {
            const int a = i + di, b = j + dj;
            if (a < 1 || a > in.NX || b < 1 || b > in.NY) continue;
            if (type[a + b * in.pitch] == T_FLUID) g = true;  // fluid cells never change here
        }
    if (g) type[id] = T_GHOST;
}

// Closest point on x^2/e0^2 + y^2/e1^2 = 1 (e0 >= e1) to (y0, y1) >= 0, after
// D. Eberly, "Distance from a point to an ellipse, an ellipsoid, or a
// hyperellipsoid" (Geometric Tools, 2013): the root s of
// G(s) = (r0 z0 / (s + r0))^2 + (z1 / (s + 1))^2 - 1 in Eberly's bracket, by
// Newton's method from s = 0 (G convex and decreasing: monotone from the left
// of the root, one step from the right lands left of it), a step outside the
// bracket replaced by bisection.  A few steps with three divisions each instead
// of ~60 halvings with two; the same operations as the CPU restatement.
__device__ double ell_root(double r0, double z0, double z1, double g) {
    const double n0 = r0 * z0;
    double s0 = z1 - 1.0;
    double s1 = (g < 0.0 ? 0.0 : sqrt(n0 * n0 + z1 * z1) - 1.0);
    double s = 0.0;
    for (int k = 0; k < 200; k++) {
        const double i0 = 1.0 / (s + r0), i1 = 1.0 / (s + 1.0);
        const double ra = n0 * i0, rb = z1 * i1;
        const double gg = ra * ra + rb * rb - 1.0;
        if (gg > 0.0) s0 = s;
        else if (gg < 0.0) s1 = s;
        else break;
        const double dg = -2.0 * (ra * ra * i0 + rb * rb * i1);
        double sn = s - gg / dg;
        if (!(sn > s0 && sn < s1)) sn = 0.5 * (s0 + s1);  // outside the bracket (or not a number)
        if (sn == s || sn == s0 || sn == s1) break;
        s = sn;
    }
    return s;
}

__device__ void ell_closest_q1(double e0, double e1, double y0, double y1, double* x0, double* x1) {
    if (y1 > 0.0) {
        if (y0 > 0.0) {
            const double z0 = y0 / e0, z1 = y1 / e1;
            const double g = z0 * z0 + z1 * z1 - 1.0;
            if (g != 0.0) {
                const double r0 = (e0 / e1) * (e0 / e1);
                const double sb = ell_root(r0, z0, z1, g);
                *x0 = r0 * y0 / (sb + r0);
                *x1 = y1 / (sb + 1.0);
            } else {
                *x0 = y0;
                *x1 = y1;
            }
        } else {
            *x0 = 0.0;
            *x1 = e1;
        }
    } else {
        const double numer0 = e0 * y0, denom0 = e0 * e0 - e1 * e1;
        if (numer0 < denom0) {
            const double xde0 = numer0 / denom0;
            *x0 = e0 * xde0;
            *x1 = e1 * sqrt(fmax(0.0, 1.0 - xde0 * xde0));
        } else {
            *x0 = e0;
            *x1 = 0.0;
        }
    }
}

__device__ void ellipse_closest(double a, double b, double px, double py, double* bx, double* by, double* nxo,
                                double* nyo) {
    const bool sw = a < b;
    const double e0 = sw ? b : a, e1 = sw ? a : b;
    const double q0 = sw ? py : px, q1 = sw ? px : py;
    const double s0 = q0 < 0.0 ? -1.0 : 1.0, s1 = q1 < 0.0 ? -1.0 : 1.0;
    double x0, x1;
    ell_closest_q1(e0, e1, fabs(q0), fabs(q1), &x0, &x1);
    x0 *= s0;
    x1 *= s1;
    double g0 = x0 / (e0 * e0), g1 = x1 / (e1 * e1);
    const double gl = sqrt(g0 * g0 + g1 * g1);
    g0 /= gl;
    g1 /= gl;
    if (sw) {
        *bx = x1; *by = x0; *nxo = g1; *nyo = g0;
    } else {
        *bx = x0; *by = x1; *nxo = g0; *nyo = g1;
    }
}

// Solve m w = rhs (4x4, partial pivoting); false when singular.
__device__ bool solve4(double m[4][4], const double rhs[4], double out[4]) {
    double a[4][5];
    for (int r = 0; r < 4; r++) {
        for (int c = 0; c < 4; c++) a[r][c] = m[r][c];
        a[r][4] = rhs[r];
    }
    for (int c = 0; c < 4; c++) {
        int piv = c;
        for (int r = c + 1; r < 4; r++)
            if (fabs(a[r][c]) > fabs(a[piv][c])) piv = r;
        if (fabs(a[piv][c]) < 1e-12) return false;
        if (piv != c)
            for (int k = 0; k < 5; k++) {
                const double tmp = a[c][k];
                a[c][k] = a[piv][k];
                a[piv][k] = tmp;
            }
        for (int r = c + 1; r < 4; r++) {
            const double f = a[r][c] / a[c][c];
            for (int k = c; k < 5; k++) a[r][k] -= f * a[c][k];
        }
    }
    for (int r = 3; r >= 0; r--) {
        double s = a[r][4];
        for (int k = r + 1; k < 4; k++) s -= a[r][k] * out[k];
        out[r] = s / a[r][r];
    }
    return true;
}

__global__ void k_ghost_weights(GhostDev* __restrict__ G, const int* __restrict__ ibm, int nibm,
                                const InstDev* __restrict__ I, double* __restrict__ bi_ip) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nibm) return;
    GhostDev& g = G[ibm[q]];
    if (g.cell < 0) return;  // an unused slot of a moving body's instance
    const InstDev& in = I[g.inst];
    const int P = in.pitch, nx = in.nx, ny = in.ny;
    const int i = g.cell % P, j = g.cell / P;
    const double px = in.xc[i] - in.bcx, py = in.yc[j] - in.bcy;
    const double lx = px * in.bcs + py * in.bsn, ly = -px * in.bsn + py * in.bcs;
    double bx, by, nlx, nly;
    ellipse_closest(in.ba, in.bb, lx, ly, &bx, &by, &nlx, &nly);
    const double BIx = in.bcx + bx * in.bcs - by * in.bsn;
    const double BIy = in.bcy + bx * in.bsn + by * in.bcs;
    const double nwx = nlx * in.bcs - nly * in.bsn, nwy = nlx * in.bsn + nly * in.bcs;
    const double IPx = 2.0 * BIx - in.xc[i], IPy = 2.0 * BIy - in.yc[j];
    if (bi_ip) {
        bi_ip[4 * (size_t)q] = BIx;
        bi_ip[4 * (size_t)q + 1] = BIy;
        bi_ip[4 * (size_t)q + 2] = IPx;
        bi_ip[4 * (size_t)q + 3] = IPy;
    }
    int i0 = ub_index(in.xc, nx, IPx), j0 = ub_index(in.yc, ny, IPy);
    i0 = min(max(i0, 1), nx - 3);
    j0 = min(max(j0, 1), ny - 3);
    const double hx = in.xc[i0 + 1] - in.xc[i0], hy = in.yc[j0 + 1] - in.yc[j0];
    const double xi = (IPx - in.xc[i0]) / hx, eta = (IPy - in.yc[j0]) / hy;
    const double xb = (BIx - in.xc[i0]) / hx, eb = (BIy - in.yc[j0]) / hy;
    const int ci[4] = {0, 1, 0, 1}, cj[4] = {0, 0, 1, 1};
    double mD[4][4], mN[4][4];
    int gk = -1;
    for (int k = 0; k < 4; k++) {
        g.nb[k] = (i0 + ci[k]) + (j0 + cj[k]) * P;
        if (g.nb[k] == g.cell) gk = k;
    }
    for (int k = 0; k < 4; k++) {
        double bD[4], bN[4];
        if (k == gk) {
            bD[0] = xb * eb; bD[1] = xb; bD[2] = eb; bD[3] = 1.0;
            const double nxi = nwx / hx, net = nwy / hy;
            const double sc = fmin(hx, hy);
            bN[0] = (nxi * eb + net * xb) * sc; bN[1] = nxi * sc; bN[2] = net * sc; bN[3] = 0.0;
        } else {
            const double x = ci[k], y = cj[k];
            bD[0] = bN[0] = x * y; bD[1] = bN[1] = x; bD[2] = bN[2] = y; bD[3] = bN[3] = 1.0;
        }
        for (int r = 0; r < 4; r++) {
            mD[r][k] = bD[r];
            mN[r][k] = bN[r];
        }
    }
    const double bip[4] = {xi * eta, xi, eta, 1.0};
    double wD[4], wN[4];
    const bool okD = solve4(mD, bip, wD), okN = solve4(mN, bip, wN);
    if (!okD || !okN) {
        const double wb[4] = {(1 - xi) * (1 - eta), xi * (1 - eta), (1 - xi) * eta, xi * eta};
        double sum = 0;
        for (int k = 0; k < 4; k++)
            if (k != gk) sum += wb[k];
        for (int k = 0; k < 4; k++) {
            const double w = (k == gk || sum <= 0) ? 0.0 : wb[k] / sum;
            wD[k] = w;
            wN[k] = w;
        }
    }
    // pressure: nodes that are IBM ghosts themselves are dropped so that every
    // ghost pressure is a linear function of fluid cells
    double keep = 0.0;
    for (int k = 0; k < 4; k++)
        if (k != gk && in.type[g.nb[k]] != T_GHOST) keep += wN[k];
    if (!(keep > 0.05)) {
        const double wb[4] = {(1 - xi) * (1 - eta), xi * (1 - eta), (1 - xi) * eta, xi * eta};
        keep = 0.0;
        for (int k = 0; k < 4; k++) {
            wN[k] = wb[k];
            if (k != gk && in.type[g.nb[k]] != T_GHOST) keep += wb[k];
        }
    }
    for (int k = 0; k < 4; k++) {
        if (k == gk) {
            g.wu[k] = g.wv[k] = g.wp[k] = 0.0;
            continue;
        }
        g.wu[k] = -wD[k];
        g.wv[k] = -wD[k];
        g.wp[k] = (in.type[g.nb[k]] != T_GHOST) ? wN[k] / keep : 0.0;
    }
    // Dirichlet value at BI: the wall velocity (zero for a body at rest).  The
    // ghost is q_G = 2 q_BI - q_IP with q_IP = w_G q_BI + sum_k w_k q_k when G
    // is a node of the image-point cell (w_G = 0 otherwise), so its constant is
    // (2 - w_G) q_BI.
    g.cu = g.cv = 0.0;
    if (in.moving) {
        const double wg = 2.0 - (gk >= 0 ? wD[gk] : 0.0);
        const double ub = in.bu - in.bw * (BIy - in.bcy), vb = in.bv + in.bw * (BIx - in.bcx);
        g.cu = wg * ub;
        g.cv = wg * vb;
    }
}

cudaError_t launch_tag(const InstDev* I, int inst, int n_cells, uint8_t* type, cudaStream_t s) {
    k_tag<<<(n_cells + 255) / 256, 256, 0, s>>>(I, inst, type);
    return cudaGetLastError();
}
cudaError_t launch_mark_ghosts(const InstDev* I, int inst, int n_interior, uint8_t* type, cudaStream_t s) {
    k_mark_ghosts<<<(n_interior + 255) / 256, 256, 0, s>>>(I, inst, type);
    return cudaGetLastError();
}
cudaError_t launch_ghost_weights(GhostDev* G, const int* ibm, int nibm, const InstDev* I, double* bi_ip,
                                 cudaStream_t s, int threads) {
    if (nibm == 0) return cudaSuccess;
    k_ghost_weights<<<(nibm + threads - 1) / threads, threads, 0, s>>>(G, ibm, nibm, I, bi_ip);
    return cudaGetLastError();
}

}  // namespace ifx
