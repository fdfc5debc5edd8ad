"""The no-allocation pressure solve gives the same answer as the solver's own.

ifx_ppe_reference_noalloc exists for callers that cannot allocate device
memory themselves: a plug-in inside a host application that owns every device
allocation, a service with a fixed device-memory budget, or a latency-bound
loop that cannot afford the device synchronisation of cudaFree.  Here the
caller's buffers come from torch; the result is compared with
ifx_ppe_reference on a solver handle
(same kernels, so the tolerance of the other reference-mode tests, 1e-12
relative, holds) and with the reference's own result file p.dat (to its %f
print precision, 5e-7), on two calls in a row so that leftovers in the shared
scratch array cannot go unnoticed.  The file name sorts last, so a run that
stops at the first failure has run every other test first.
"""
import ctypes as C
import os

import numpy as np
import pytest

import immerseflow_gb300 as ifx
from immerseflow_gb300 import _capi as capi

pytestmark = pytest.mark.gpu


def _grid(golden_dir):
    c = ifx.config_read(os.path.join(golden_dir, "inputs", "inputs.txt"))
    xf = ifx.grid_read(c.xgrid.decode(), c.nx + 1)
    yf = ifx.grid_read(c.ygrid.decode(), c.ny + 1)
    return c, xf, yf


def _full_widths(xf, yf):
    # readGridData's full-size width arrays (src/include/preSim.cu:328-355)
    nx, ny = len(xf) + 1, len(yf) + 1
    dx = np.empty(nx)
    dy = np.empty(ny)
    dx[1:-1] = np.diff(xf)
    dy[1:-1] = np.diff(yf)
    dx[0], dx[-1], dy[0], dy[-1] = dx[1], dx[-2], dy[1], dy[-2]
    return np.tile(dx, (ny, 1)).ravel(), np.tile(dy[:, None], (1, nx)).ravel()


def test_noalloc_matches_solver_solve_twice(golden_dir, golden):
    torch = pytest.importorskip("torch")
    c, xf, yf = _grid(golden_dir)
    s = ifx.Solver.create(c, xf, yf)
    it_ref = s.ppe_reference()
    p_ref = s.get(capi.FIELD_P)
    s.close()
    nx, ny = c.nx + 2, c.ny + 2
    DX, DY = _full_widths(xf, yf)
    d_dx = torch.tensor(DX, dtype=torch.float64, device="cuda")
    d_dy = torch.tensor(DY, dtype=torch.float64, device="cuda")
    lib = ifx.lib()
    for call in range(2):
        d_p = torch.zeros(nx * ny, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        it = C.c_int(-1)
        st = lib.ifx_ppe_reference_noalloc(d_dx.data_ptr(), d_dy.data_ptr(), nx, ny, d_p.data_ptr(),
                                           c.ppe_itermax, 1e-6, C.byref(it), None)
        assert st == capi.IFX_OK, lib.ifx_last_error()
        torch.cuda.synchronize()
        p = d_p.cpu().numpy().reshape(ny, nx)
        assert it.value == it_ref, (call, it.value, it_ref)
        assert np.abs(p - p_ref).max() <= 1e-12 * np.abs(p_ref).max(), call
        # and on its own against the reference's result file p.dat (printed with %f)
        assert np.abs(p - golden["p"]).max() <= 5.0e-7 + 1e-12, call


def test_noalloc_rejects_grids_above_the_fixed_scratch():
    lib = ifx.lib()
    n = 200  # 200*200 cells > IFX_NOALLOC_MAX_CELLS; the size check precedes any device access
    dummy = C.c_void_p(16)
    st = lib.ifx_ppe_reference_noalloc(dummy, dummy, n, n, dummy, 10, 1e-6, None, None)
    assert st == capi.IFX_ERR_ARG
    assert b"IFX_NOALLOC_MAX_CELLS" in lib.ifx_last_error()
