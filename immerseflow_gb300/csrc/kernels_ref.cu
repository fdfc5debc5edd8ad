// kernels_ref.cu -- the reference's own algorithm (REFERENCE mode) on sm_103a.
//
// ImmerseFlow::ADsolver (src/include/ADSolver.cu:268-395) and the Jacobi
// Laplace solve that PPESolver intends (src/include/PPESolver.cu:13-71,
// 137-205), one instance, dense rows (index i + j*nx as in the reference).
// The arithmetic of every kernel follows the reference expression by
// expression; what changes is the launch structure: one thread per cell
// (no grid-stride loop), no cudaMalloc/cudaFree per step, residual sums
// reduced on the device in a fixed order (no per-iteration allocation), and
// the whole step in one cooperative launch (k_ref_steps).
#include <cuda_runtime.h>

#include <algorithm>

#include "grid_barrier.cuh"
#include "ifx_kernels.h"

namespace ifx {

#define RIDX(i, j) ((i) + (j) * R.nx)

__global__ void k_ref_coeffs(RefDev R) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= R.nx * R.ny) return;
    const int i = q % R.nx, j = q / R.nx, id = q, nx = R.nx;
    double aP = 1, aW = 1, aE = 1, aS = 1, aN = 1;
    if (i > 0 && i < R.nx - 1 && j > 0 && j < R.ny - 1) {
        const double dt = R.dt, Re = R.re;
        const double dx_i = R.dx[id], dx_ip1 = R.dx[id + 1], dx_im1 = R.dx[id - 1];
        const double dy_j = R.dy[id], dy_jp1 = R.dy[id + nx], dy_jm1 = R.dy[id - nx];
        aP = 1.0 + (dt / Re) * ((2 / (dx_i * (dx_i + dx_ip1))) + (2 / (dx_i * (dx_i + dx_im1)))) +
             (dt / Re) * ((2 / (dy_j * (dy_j + dy_jp1))) + (2 / (dy_j * (dy_j + dy_jm1))));
        aW = (dt / Re) * (2 / (dx_i * (dx_i + dx_im1)));
        aE = (dt / Re) * (2 / (dx_i * (dx_i + dx_ip1)));
        aS = (dt / Re) * (2 / (dy_j * (dy_j + dy_jm1)));
        aN = (dt / Re) * (2 / (dy_j * (dy_j + dy_jp1)));
    }
    R.aP[id] = aP; R.aW[id] = aW; R.aE[id] = aE; R.aS[id] = aS; R.aN[id] = aN;
}

// Compute_velf with its loop structure: uf for every index, vf only for
// indices in [(nx-1)(ny-2), (nx-2)(ny-1)) (the second grid-stride loop of
// src/include/ADSolver.cu:179 starts from the exhausted index).
__device__ __forceinline__ void velf_cell(const RefDev& R, const double* __restrict__ u,
                                          const double* __restrict__ v, int id) {
    const int nx = R.nx, ny = R.ny;
    const int nu = (nx - 1) * (ny - 2), nv = (nx - 2) * (ny - 1);
    if (id < nu) {
        const int i = id % (nx - 1), j = id / (nx - 1), idc = j * nx + i;
        R.uf[id] = 1.0 / (R.dx[idc + nx] + R.dx[idc + nx + 1]) *
                   (u[idc + nx + 1] * R.dx[idc + nx] + u[idc + nx] * R.dx[idc + nx + 1]);
    } else if (id < nv) {
        const int i = id % (nx - 2), j = id / (nx - 2), idc = j * nx + i;
        R.vf[id] = 1.0 / (R.dy[idc + nx + 1] + R.dy[idc + 1]) *
                   (v[idc + nx + 1] * R.dy[idc + 1] + v[idc + 1] * R.dy[idc + nx + 1]);
    }
}
__global__ void k_ref_velf(RefDev R, const double* __restrict__ u, const double* __restrict__ v) {
    velf_cell(R, u, v, blockIdx.x * blockDim.x + threadIdx.x);
}

// set_velocity_BC (src/include/ADSolver.cu:195-217): ghost = 2*wall - adjacent,
// u_wall = 1, v_wall = 0.  The reference's corner cells race on a
// neighbouring ghost; here edges use the interior neighbour and a corner
// applies the rule twice to its diagonal interior cell (edge first, then
// corner), which is one of the orders the reference can produce.
__device__ __forceinline__ void bc_cell(const RefDev& R, double* __restrict__ u, double* __restrict__ v, int q) {
    const int nx = R.nx, ny = R.ny;
    if (q >= nx * ny) return;
    const int i = q % nx, j = q / nx;
    const bool ei = (i == 0 || i == nx - 1), ej = (j == 0 || j == ny - 1);
    if (!ei && !ej) return;
    int ai = i, aj = j;
    if (i == 0) ai = 1;
    if (i == nx - 1) ai = nx - 2;
    if (j == 0) aj = 1;
    if (j == ny - 1) aj = ny - 2;
    const int a = RIDX(ai, aj);
    if (ei && ej) {
        const double ue = -u[a] + 1.0 * 2.0, ve = -v[a] + 0.0 * 2.0;
        u[q] = -ue + 1.0 * 2.0;
        v[q] = -ve + 0.0 * 2.0;
    } else {
        u[q] = -u[a] + 1.0 * 2.0;
        v[q] = -v[a] + 0.0 * 2.0;
    }
}
__global__ void k_ref_bc(RefDev R, double* __restrict__ u, double* __restrict__ v) {
    bc_cell(R, u, v, blockIdx.x * blockDim.x + threadIdx.x);
}

// ADSource (src/include/ADSolver.cu:46-79), including its 0.5 factor.
__device__ __forceinline__ void source_cell(const RefDev& R, const double* __restrict__ u,
                                            const double* __restrict__ v, int id) {
    const int nx = R.nx, ny = R.ny;
    if (id >= nx * ny) return;
    const int i = id % nx, j = id / nx;
    double sx = 0.0, sy = 0.0;
    if (i > 0 && i < nx - 1 && j > 0 && j < ny - 1) {
        const double dt = R.dt;
        const double dx_i = R.dx[id], dx_ip1 = R.dx[id + 1], dx_im1 = R.dx[id - 1];
        const double dy_j = R.dy[id], dy_jp1 = R.dy[id + nx], dy_jm1 = R.dy[id - nx];
        const double ufe = R.uf[i + (j - 1) * (nx - 1)], ufw = R.uf[i - 1 + (j - 1) * (nx - 1)];
        const double vfn = R.vf[i - 1 + j * (nx - 2)], vfs = R.vf[i - 1 + (j - 1) * (nx - 2)];
        sx = (u[id] - (dt / dx_i) * 0.5 * (((1 / (dx_i + dx_ip1)) * (u[id + 1] * dx_i + u[id] * dx_ip1) * ufe) -
                                           ((1 / (dx_i + dx_im1)) * (u[id] * dx_im1 + u[id - 1] * dx_i) * ufw)) -
              (dt / dy_j) * 0.5 * (((1 / (dy_j + dy_jp1)) * (u[id + nx] * dy_j + u[id] * dy_jp1) * vfn) -
                                   ((1 / (dy_j + dy_jm1)) * (u[id] * dy_jm1 + u[id - nx] * dy_j) * vfs)));
        sy = (v[id] - (dt / dx_i) * 0.5 * (((1 / (dx_i + dx_ip1)) * (v[id + 1] * dx_i + v[id] * dx_ip1) * ufe) -
                                           ((1 / (dx_i + dx_im1)) * (v[id] * dx_im1 + v[id - 1] * dx_i) * ufw)) -
              (dt / dy_j) * 0.5 * (((1 / (dy_j + dy_jp1)) * (v[id + nx] * dy_j + v[id] * dy_jp1) * vfn) -
                                   ((1 / (dy_j + dy_jm1)) * (v[id] * dy_jm1 + v[id - nx] * dy_j) * vfs)));
    }
    R.sx[id] = sx;
    R.sy[id] = sy;
}
__global__ void k_ref_source(RefDev R, const double* __restrict__ u, const double* __restrict__ v) {
    source_cell(R, u, v, blockIdx.x * blockDim.x + threadIdx.x);
}

// ADusolver_kernel / ADvsolver_kernel (src/include/ADSolver.cu:81-120), fused.
__device__ __forceinline__ void jacobi_cell(const RefDev& R, const double* __restrict__ u,
                                            const double* __restrict__ v, double* __restrict__ un,
                                            double* __restrict__ vn, int id) {
    const int nx = R.nx, ny = R.ny;
    if (id >= nx * ny) return;
    const int i = id % nx, j = id / nx;
    if (!(i > 0 && i < nx - 1 && j > 0 && j < ny - 1)) return;
    const double a = R.sx[id] + R.aE[id] * u[id + 1] + R.aW[id] * u[id - 1] + R.aN[id] * u[id + nx] +
                     R.aS[id] * u[id - nx];
    un[id] = R.iblank[id] * a / R.aP[id];
    const double b = R.sy[id] + R.aE[id] * v[id + 1] + R.aW[id] * v[id - 1] + R.aN[id] * v[id + nx] +
                     R.aS[id] * v[id - nx];
    vn[id] = R.iblank[id] * b / R.aP[id];
    // under-relaxation, the reference's commented-out lines (src/include/ADSolver.cu:95,116)
    if (R.w_ad != 1.0) {
        un[id] = (1.0 - R.w_ad) * u[id] + R.w_ad * un[id];
        vn[id] = (1.0 - R.w_ad) * v[id] + R.w_ad * vn[id];
    }
}
__global__ void k_ref_jacobi(RefDev R, const double* __restrict__ u, const double* __restrict__ v,
                             double* __restrict__ un, double* __restrict__ vn) {
    jacobi_cell(R, u, v, un, vn, blockIdx.x * blockDim.x + threadIdx.x);
}

// Fixed-order two-level sum: each block writes its partial, the last block
// to finish adds the partials in block order.
// Partial sums of a block of 256 cells (warp sums, then warps in order),
// written by thread 0 to scratch[slot * NV + k].
template <int NV>
__device__ __forceinline__ void block_partial(double (&v)[NV], double* scratch, int slot) {
    __shared__ double sh[NV][32];
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++) {
        double x = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (l == 0) sh[k][w] = x;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 0; k < NV; k++) {
            double s = 0.0;
            for (int q = 0; q < nw; q++) s += sh[k][q];
            scratch[slot * NV + k] = s;
        }
    }
    __syncthreads();
}

template <int NV>
__device__ void blocks_sum(double (&v)[NV], double* scratch, unsigned int* ticket, double* out) {
    __shared__ bool last;
    block_partial<NV>(v, scratch, blockIdx.x);
    if (threadIdx.x == 0) {
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        for (int k = 0; k < NV; k++) {
            double s = 0.0;
            for (unsigned int b = 0; b < gridDim.x; b++) s += ((volatile double*)scratch)[b * NV + k];
            out[k] = s;
        }
        *ticket = 0u;
    }
}

// Compute_{u,v}Residual_AD + Reduction (src/include/ADSolver.cu:122-160,
// src/include/preSim.cu:376-445): L1 of the update over fluid interior cells.
__device__ __forceinline__ void resid_cell(const RefDev& R, const double* __restrict__ uo,
                                           const double* __restrict__ un, const double* __restrict__ vo,
                                           const double* __restrict__ vn, int id, double (&r)[2]) {
    const int nx = R.nx, ny = R.ny;
    r[0] = r[1] = 0.0;
    if (id < nx * ny) {
        const int i = id % nx, j = id / nx;
        if (i > 0 && i < nx - 1 && j > 0 && j < ny - 1 && R.iblank[id] == 1) {
            r[0] = fabs(un[id] - uo[id]);
            r[1] = fabs(vn[id] - vo[id]);
        }
    }
}
__global__ void k_ref_resid(RefDev R, const double* __restrict__ uo, const double* __restrict__ un,
                            const double* __restrict__ vo, const double* __restrict__ vn, double* out,
                            unsigned int* ticket) {
    double r[2];
    resid_cell(R, uo, un, vo, vn, blockIdx.x * blockDim.x + threadIdx.x, r);
    blocks_sum<2>(r, R.res, ticket, out);
}

// nsteps ADsolver steps in one cooperative launch: the phases of
// launch_ref_velf / _bc / _source / _jacobi / _resid over 256-cell chunks
// (chunk c is the block c of those launches), separated by grid barriers; the
// L1 residual is summed chunk by chunk in the same order as blocks_sum, by
// every block, so all blocks take the same loop decision without another
// barrier.  iters[s] receives step s's Jacobi iterations.  The state starts
// in (u, v) and ends in (u, v) after an even total of iterations, in
// (ut, vt) after an odd one (the reference's buffer swaps).
__global__ void __launch_bounds__(256) k_ref_steps(RefDev R, double* u, double* v, double* ut, double* vt,
                                                   GridBar* bar, int itermax, int nsteps, int* iters) {
    const int n = R.nx * R.ny, nc = (n + 255) / 256, nf = ((R.nx - 1) * (R.ny - 1) + 255) / 256;
    unsigned long long ep = 0;
    __shared__ double tot[2];
    double *cu = u, *cv = v, *tu = ut, *tv = vt;
    for (int s = 0; s < nsteps; s++) {
        for (int c = blockIdx.x; c < nf; c += gridDim.x) velf_cell(R, cu, cv, c * 256 + threadIdx.x);
        if (!grid_barrier(bar, ep)) return;
        for (int c = blockIdx.x; c < nc; c += gridDim.x) bc_cell(R, cu, cv, c * 256 + threadIdx.x);
        if (!grid_barrier(bar, ep)) return;
        for (int c = blockIdx.x; c < nc; c += gridDim.x) source_cell(R, cu, cv, c * 256 + threadIdx.x);
        if (!grid_barrier(bar, ep)) return;
        double res = 1.0 + 1.0;  // ures + vres start at 1 (src/include/ADSolver.cu:313)
        int it = 0;
        while (res > 1e-6 && it < itermax) {
            for (int c = blockIdx.x; c < nc; c += gridDim.x) bc_cell(R, cu, cv, c * 256 + threadIdx.x);
            if (!grid_barrier(bar, ep)) return;
            for (int c = blockIdx.x; c < nf; c += gridDim.x) velf_cell(R, cu, cv, c * 256 + threadIdx.x);
            if (!grid_barrier(bar, ep)) return;
            for (int c = blockIdx.x; c < nc; c += gridDim.x) jacobi_cell(R, cu, cv, tu, tv, c * 256 + threadIdx.x);
            if (!grid_barrier(bar, ep)) return;
            for (int c = blockIdx.x; c < nc; c += gridDim.x) bc_cell(R, cu, cv, c * 256 + threadIdx.x);
            for (int c = blockIdx.x; c < nc; c += gridDim.x) {
                double r[2];
                resid_cell(R, cu, tu, cv, tv, c * 256 + threadIdx.x, r);
                block_partial<2>(r, R.res, c);
            }
            if (!grid_barrier(bar, ep)) return;
            if (threadIdx.x == 0) {
                double a = 0.0, b = 0.0;
                for (int c = 0; c < nc; c++) {
                    a += ((volatile double*)R.res)[c * 2];
                    b += ((volatile double*)R.res)[c * 2 + 1];
                }
                tot[0] = a;
                tot[1] = b;
            }
            __syncthreads();
            res = tot[0] + tot[1];
            __syncthreads();
            double* x = cu; cu = tu; tu = x;
            x = cv; cv = tv; tv = x;
            it++;
        }
        if (blockIdx.x == 0 && threadIdx.x == 0) iters[s] = it;
    }
}

// initializeKernel (src/include/preSim.cu:57-76): vortex in uniform flow.
__global__ void k_ref_init(int nx, int ny, const double* __restrict__ xc, const double* __restrict__ yc,
                           double* __restrict__ u, double* __restrict__ v, double* __restrict__ p) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= nx * ny) return;
    const int ix = id % nx, iy = id / nx;
    const double r = sqrt(pow(xc[ix] - 0.5, 2.0) + pow(yc[iy] - 0.5, 2.0));
    const double r0 = 0.1;
    u[id] = 1.0 - 0.25 * (yc[iy] - 0.5) * exp((1.0 - pow(r / r0, 2.0)) / 2.0);
    v[id] = 0.25 * (xc[ix] - 0.5) * exp((1.0 - pow(r / r0, 2.0)) / 2.0);
    if (p) p[id] = 0.0;
}

// calculatePPECoefficients as intended (src/include/PPESolver.cu:73-104).
__global__ void k_ref_ppe_coeffs(RefDev R) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= R.nx * R.ny) return;
    const int i = q % R.nx, j = q / R.nx, id = q, nx = R.nx;
    double aP = 1, aW = 1, aE = 1, aS = 1, aN = 1;
    if (i > 0 && i < R.nx - 1 && j > 0 && j < R.ny - 1) {
        const double dx_i = R.dx[id], dx_ip1 = R.dx[id + 1], dx_im1 = R.dx[id - 1];
        const double dy_j = R.dy[id], dy_jp1 = R.dy[id + nx], dy_jm1 = R.dy[id - nx];
        aP = -1 * (((2 / (dx_i * (dx_i + dx_ip1))) + (2 / (dx_i * (dx_i + dx_im1)))) +
                   ((2 / (dy_j * (dy_j + dy_jp1))) + (2 / (dy_j * (dy_j + dy_jm1)))));
        aW = (2 / (dx_i * (dx_i + dx_im1)));
        aE = (2 / (dx_i * (dx_i + dx_ip1)));
        aS = (2 / (dy_j * (dy_j + dy_jm1)));
        aN = (2 / (dy_j * (dy_j + dy_jp1)));
    }
    R.aP[id] = aP; R.aW[id] = aW; R.aE[id] = aE; R.aS[id] = aS; R.aN[id] = aN;
}

// set_pressure_BC (src/include/PPESolver.cu:54-71).
__global__ void k_ref_ppe_bc(RefDev R, double* __restrict__ p) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= R.nx * R.ny) return;
    const int i = q % R.nx, j = q / R.nx;
    if (i == 0 || j == 0) p[q] = 100.0;
}

// jacobiIteration (src/include/PPESolver.cu:13-31).
__global__ void k_ref_ppe_jacobi(RefDev R, const double* __restrict__ p, double* __restrict__ pn) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    const int nx = R.nx, ny = R.ny;
    if (id >= nx * ny) return;
    const int i = id % nx, j = id / nx;
    double val = p[id];
    if (i > 0 && i < nx - 1 && j > 0 && j < ny - 1)
        val = -(p[id + 1] * R.aE[id] + p[id - 1] * R.aW[id] + p[id + nx] * R.aN[id] + p[id - nx] * R.aS[id]) /
              R.aP[id];
    pn[id] = val;
}

// Compute_Residual + Reduction (src/include/PPESolver.cu:33-50,185): signed sum.
__global__ void k_ref_ppe_resid(RefDev R, const double* __restrict__ p, double* out, unsigned int* ticket) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    const int nx = R.nx, ny = R.ny;
    double r[1] = {0.0};
    if (id < nx * ny) {
        const int i = id % nx, j = id / nx;
        if (i > 0 && i < nx - 1 && j > 0 && j < ny - 1)
            r[0] = p[id] * R.aP[id] + p[id + 1] * R.aE[id] + p[id - 1] * R.aW[id] + p[id + nx] * R.aN[id] +
                   p[id - nx] * R.aS[id];
    }
    blocks_sum<1>(r, R.res, ticket, out);
}

// Point Gauss-Seidel / SOR on one colour of the red-black ordering, in place:
// the jacobiIteration update (src/include/PPESolver.cu:21-25) of the cells
// with (i + j) % 2 == colour, relaxed as (1 - w) p + w p_new when w != 1.
// Cells of one colour only read the other colour, so a launch is race-free.
__global__ void k_ref_ppe_rb(RefDev R, double* __restrict__ p, int colour, double w) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    const int nx = R.nx, ny = R.ny;
    if (id >= nx * ny) return;
    const int i = id % nx, j = id / nx;
    if (!(i > 0 && i < nx - 1 && j > 0 && j < ny - 1) || ((i + j) & 1) != colour) return;
    const double g =
        -(p[id + 1] * R.aE[id] + p[id - 1] * R.aW[id] + p[id + nx] * R.aN[id] + p[id - nx] * R.aS[id]) / R.aP[id];
    p[id] = w == 1.0 ? g : (1.0 - w) * p[id] + w * g;
}

// Line SOR along x for the rows j = first, first + 2, ... (one thread per row):
//   aW p[i-1] + aP p[i] + aE p[i+1] = -(aN p[i,j+1] + aS p[i,j-1])
// for i = 1..nx-2, ghost values at i = 0 and nx-1 moved to the right-hand
// side, solved by the Thomas algorithm (forward elimination into cp, dp, back
// substitution), then relaxed as (1 - w) p + w x when w != 1.  Rows of one
// parity only read rows of the other, so a launch is race-free.
__global__ void k_ref_ppe_line(RefDev R, double* __restrict__ p, double* __restrict__ cp, double* __restrict__ dp,
                               int first, double w) {
    const int j = first + 2 * (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int nx = R.nx, ny = R.ny;
    if (j > ny - 2) return;
    const int b = j * nx, last = nx - 2;
    for (int i = 1; i <= last; i++) {
        const int id = b + i;
        double rhs = -(R.aN[id] * p[id + nx] + R.aS[id] * p[id - nx]);
        if (i == 1) rhs -= R.aW[id] * p[id - 1];
        if (i == last) rhs -= R.aE[id] * p[id + 1];
        const double m = i == 1 ? R.aP[id] : R.aP[id] - R.aW[id] * cp[id - 1];
        cp[id] = i == last ? 0.0 : R.aE[id] / m;
        dp[id] = i == 1 ? rhs / m : (rhs - R.aW[id] * dp[id - 1]) / m;
    }
    double x = 0.0;
    for (int i = last; i >= 1; i--) {
        const int id = b + i;
        x = i == last ? dp[id] : dp[id] - cp[id] * x;
        p[id] = w == 1.0 ? x : (1.0 - w) * p[id] + w * x;
    }
}

static inline int nb256(int n) { return (n + 255) / 256; }

cudaError_t launch_ref_coeffs(const RefDev& R, cudaStream_t s) {
    k_ref_coeffs<<<nb256(R.nx * R.ny), 256, 0, s>>>(R);
    return cudaGetLastError();
}
cudaError_t launch_ref_velf(const RefDev& R, const double* u, const double* v, cudaStream_t s) {
    const int n = (R.nx - 1) * (R.ny - 1);
    k_ref_velf<<<nb256(n), 256, 0, s>>>(R, u, v);
    return cudaGetLastError();
}
cudaError_t launch_ref_bc(const RefDev& R, double* u, double* v, cudaStream_t s) {
    k_ref_bc<<<nb256(R.nx * R.ny), 256, 0, s>>>(R, u, v);
    return cudaGetLastError();
}
cudaError_t launch_ref_source(const RefDev& R, const double* u, const double* v, cudaStream_t s) {
    k_ref_source<<<nb256(R.nx * R.ny), 256, 0, s>>>(R, u, v);
    return cudaGetLastError();
}
cudaError_t launch_ref_jacobi(const RefDev& R, const double* u, const double* v, double* un, double* vn,
                              cudaStream_t s) {
    k_ref_jacobi<<<nb256(R.nx * R.ny), 256, 0, s>>>(R, u, v, un, vn);
    return cudaGetLastError();
}
cudaError_t launch_ref_resid(const RefDev& R, const double* uo, const double* un, const double* vo,
                             const double* vn, double* out, cudaStream_t s) {
    // out[0..1]: sums; out[2] holds the block ticket (zeroed at allocation)
    k_ref_resid<<<nb256(R.nx * R.ny), 256, 0, s>>>(R, uo, un, vo, vn, out, (unsigned int*)(out + 2));
    return cudaGetLastError();
}
int ref_steps_grid(int nx, int ny) {
    static int per_sm = -1, sms = 0;
    if (per_sm < 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        int coop = 0;
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
        if (!coop || cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_ref_steps, 256, 0) != cudaSuccess) per_sm = 0;
        cudaGetLastError();
    }
    const int nc = std::max((nx * ny + 255) / 256, ((nx - 1) * (ny - 1) + 255) / 256);
    const int cap = per_sm * sms;
    return cap <= 0 ? 0 : std::min(nc, cap);
}
cudaError_t launch_ref_steps(const RefDev& R, double* u, double* v, double* ut, double* vt, GridBar* bar,
                             int itermax, int nsteps, int* iters, int grid, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(bar, 0, sizeof(GridBar), s);
    if (e != cudaSuccess) return e;
    RefDev r = R;
    void* args[] = {&r, &u, &v, &ut, &vt, &bar, &itermax, &nsteps, &iters};
    return cudaLaunchCooperativeKernel((const void*)k_ref_steps, dim3(grid), dim3(256), args, 0, s);
}
cudaError_t launch_ref_init(int nx, int ny, const double* xc, const double* yc, double* u, double* v, double* p,
                            cudaStream_t s) {
    k_ref_init<<<nb256(nx * ny), 256, 0, s>>>(nx, ny, xc, yc, u, v, p);
    return cudaGetLastError();
}
cudaError_t launch_ref_ppe_coeffs(const RefDev& R, cudaStream_t s) {
    k_ref_ppe_coeffs<<<nb256(R.nx * R.ny), 256, 0, s>>>(R);
    return cudaGetLastError();
}
cudaError_t launch_ref_ppe_bc(const RefDev& R, double* p, cudaStream_t s) {
    k_ref_ppe_bc<<<nb256(R.nx * R.ny), 256, 0, s>>>(R, p);
    return cudaGetLastError();
}
cudaError_t launch_ref_ppe_rbgs(const RefDev& R, double* p, double w, double* out, cudaStream_t s) {
    for (int colour = 0; colour < 2; colour++) {
        k_ref_ppe_rb<<<nb256(R.nx * R.ny), 256, 0, s>>>(R, p, colour, w);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    k_ref_ppe_resid<<<nb256(R.nx * R.ny), 256, 0, s>>>(R, p, out, (unsigned int*)(out + 2));
    return cudaGetLastError();
}
cudaError_t launch_ref_ppe_lines(const RefDev& R, double* p, double* cp, double* dp, double w, double* out,
                                 cudaStream_t s) {
    const int rows = (R.ny - 2 + 1) / 2;  // rows of the larger parity
    for (int first = 1; first <= 2; first++) {
        k_ref_ppe_line<<<(rows + 63) / 64, 64, 0, s>>>(R, p, cp, dp, first, w);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    k_ref_ppe_resid<<<nb256(R.nx * R.ny), 256, 0, s>>>(R, p, out, (unsigned int*)(out + 2));
    return cudaGetLastError();
}
cudaError_t launch_ref_ppe_sweep(const RefDev& R, const double* p, double* pn, double* out, cudaStream_t s) {
    k_ref_ppe_jacobi<<<nb256(R.nx * R.ny), 256, 0, s>>>(R, p, pn);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_ref_ppe_resid<<<nb256(R.nx * R.ny), 256, 0, s>>>(R, pn, out, (unsigned int*)(out + 2));
    return cudaGetLastError();
}

}  // namespace ifx
