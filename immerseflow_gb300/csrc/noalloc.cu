// noalloc.cu -- a pressure solve that allocates nothing.
//
// Some callers cannot call cudaMalloc: a plug-in running inside a host
// application that owns every device allocation through its own pool, a
// service that accounts every byte of device memory up front and forbids
// allocation on its request path, or a latency-bound loop that cannot afford
// the device-wide synchronisation that cudaFree implies.
// ifx_ppe_reference_noalloc serves them: the caller passes its own device
// buffers for the inputs and the output, and the solver's scratch (second
// pressure buffer, stencil coefficients, reduction partials) lives in the
// file-scope array below, which exists on every GPU that loads this library
// until the process exits.
//
// Host code must not pass g_noalloc_scratch to a kernel: on the host that
// name is only a stand-in for the device symbol.  The device address is
// obtained once per device with cudaGetSymbolAddress (first call on that
// device) and cached.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>

#include "ifx_host.h"
#include "ifx_kernels.h"

namespace {

constexpr int kMaxCells = IFX_NOALLOC_MAX_CELLS;
constexpr int kMaxBlocks = (kMaxCells + 255) / 256;
// 5 coefficient arrays, 1 pressure buffer, 2 partials per block, 4 result slots
constexpr size_t kScratchDoubles = 6 * (size_t)kMaxCells + 2 * (size_t)kMaxBlocks + 4;

__device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double* g_addr[kMaxDevices] = {nullptr};

ifx_status scratch_address(int dev, double** out) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess)
            return ifx::set_error(IFX_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        g_addr[dev] = (double*)p;
    }
    *out = g_addr[dev];
    return IFX_OK;
}

}  // namespace

#define NA_TRY(x)                                                                                 \
    do {                                                                                          \
        cudaError_t e_ = (x);                                                                     \
        if (e_ != cudaSuccess) return ifx::set_error(IFX_ERR_CUDA, std::string(#x ": ") + cudaGetErrorString(e_)); \
    } while (0)

extern "C" ifx_status ifx_ppe_reference_noalloc(const double* d_dx, const double* d_dy, int nx, int ny,
                                                double* d_p, int itermax, double tol, int* iters,
                                                void* stream) {
    // a NaN tolerance would end the loop before the first sweep and report a
    // converged solve, so it is refused with the other bad arguments
    if (!d_dx || !d_dy || !d_p || nx < 3 || ny < 3 || itermax < 0 || !(tol == tol))
        return ifx::set_error(IFX_ERR_ARG, "ifx_ppe_reference_noalloc: bad argument");
    if ((long long)nx * ny > kMaxCells)
        return ifx::set_error(IFX_ERR_ARG, "ifx_ppe_reference_noalloc: nx*ny = " + std::to_string((long long)nx * ny) +
                                               " exceeds the fixed scratch of " + std::to_string(kMaxCells) +
                                               " cells (IFX_NOALLOC_MAX_CELLS)");
    int dev = 0;
    NA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return ifx::set_error(IFX_ERR_ARG, "ifx_ppe_reference_noalloc: device index");
    double* sc = nullptr;
    ifx_status st = scratch_address(dev, &sc);
    if (st != IFX_OK) return st;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t n = (size_t)nx * ny;
    ifx::RefDev R;
    std::memset(&R, 0, sizeof(R));
    R.nx = nx;
    R.ny = ny;
    R.dx = d_dx;
    R.dy = d_dy;
    R.aP = sc;
    R.aE = sc + n;
    R.aW = sc + 2 * n;
    R.aN = sc + 3 * n;
    R.aS = sc + 4 * n;
    double* ptmp = sc + 5 * n;
    R.res = sc + 6 * (size_t)kMaxCells;
    double* out = R.res + 2 * (size_t)kMaxBlocks;
    // the block-ticket and result slots must start at zero; the rest is overwritten
    NA_TRY(cudaMemsetAsync(out, 0, 4 * sizeof(double), s));
    NA_TRY(ifx::launch_ref_ppe_coeffs(R, s));
    NA_TRY(ifx::launch_ref_ppe_bc(R, d_p, s));
    double* cur = d_p;
    double* tmp = ptmp;
    double residual = 1.0;
    int it = 0;
    while (residual > tol && it < itermax) {
        NA_TRY(ifx::launch_ref_ppe_sweep(R, cur, tmp, out, s));
        double* t = cur;
        cur = tmp;
        tmp = t;
        NA_TRY(cudaMemcpyAsync(&residual, out, sizeof(double), cudaMemcpyDeviceToHost, s));
        NA_TRY(cudaStreamSynchronize(s));
        it++;
    }
    NA_TRY(ifx::launch_ref_ppe_bc(R, cur, s));
    if (cur != d_p) NA_TRY(cudaMemcpyAsync(d_p, cur, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    NA_TRY(cudaStreamSynchronize(s));
    if (iters) *iters = it;
    return IFX_OK;
}
