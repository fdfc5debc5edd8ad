"""ctypes wrapper of the CPU oracle (oracle/liboracle.so) -- test infrastructure."""
import ctypes as C
import os

import numpy as np

from immerseflow_gb300 import _capi as capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
_dp = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")


class Oracle:
    def __init__(self):
        self.lib = L = C.CDLL(os.path.join(ROOT, "oracle", "liboracle.so"))
        L.orc_grid.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp, _dp]
        L.orc_ref_init.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp]
        L.orc_ref_ad_steps.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp, C.c_double, C.c_double, C.c_int,
                                       C.c_double, C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, _ip]
        L.orc_ref_ppe.argtypes = [C.c_int, C.c_int, _dp, _dp, C.c_int, C.c_double, _dp, C.POINTER(C.c_int)]
        L.orc_ref_ppe_opt.argtypes = [C.c_int, C.c_int, _dp, _dp, C.c_int, C.c_double, C.c_int, C.c_double, _dp,
                                      C.POINTER(C.c_int)]
        L.orc_ref_ad_steps_w.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp, C.c_double, C.c_double, C.c_int,
                                         C.c_double, C.c_double, C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, _ip]
        L.orc_inside.argtypes = [C.c_double] * 8
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.POINTER(capi.Config), _dp, _dp, C.c_int]
        L.orc_step.argtypes = [C.c_void_p, C.c_int]
        L.orc_get.argtypes = [C.c_void_p, C.c_int, _dp, C.c_long]
        L.orc_set.argtypes = [C.c_void_p, C.c_int, _dp, C.c_long]
        L.orc_stats.argtypes = [C.c_void_p, C.POINTER(capi.Stats)]
        L.orc_ghosts.argtypes = [C.c_void_p] + [C.c_void_p] * 6
        L.orc_mg_levels.argtypes = [C.c_void_p]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_sincos_turns.argtypes = [C.c_double, _dp, _dp]
        L.orc_body.argtypes = [C.c_void_p, _dp]

    def sincos_turns(self, x):
        """sin and cos of 2 pi x as the moving-body pose forms them."""
        s, c = np.zeros(1), np.zeros(1)
        self.lib.orc_sincos_turns(float(x), s, c)
        return s[0], c[0]

    # ---- reference primitives
    def grid(self, nx, ny, xf, yf):
        xc, yc = np.zeros(nx), np.zeros(ny)
        dx, dy = np.zeros(nx * ny), np.zeros(nx * ny)
        self.lib.orc_grid(nx, ny, np.ascontiguousarray(xf), np.ascontiguousarray(yf), xc, yc, dx, dy)
        return xc, yc, dx, dy

    def ref_ad(self, xf, yf, dt, re, itermax, nsteps, iblank=None, w_ad=1.0):
        nx, ny = len(xf) + 1, len(yf) + 1
        xc, yc, dx, dy = self.grid(nx, ny, xf, yf)
        u, v, p = np.zeros(nx * ny), np.zeros(nx * ny), np.zeros(nx * ny)
        self.lib.orc_ref_init(nx, ny, xc, yc, u, v, p)
        ut, vt = u.copy(), v.copy()
        uf, vf = np.zeros((nx - 1) * (ny - 2)), np.zeros((nx - 2) * (ny - 1))
        ib = np.ones(nx * ny) if iblank is None else np.ascontiguousarray(iblank, np.float64)
        iters = np.zeros(max(1, nsteps), np.int32)
        self.lib.orc_ref_ad_steps_w(nx, ny, dx, dy, ib, dt, re, itermax, 1e-6, w_ad, nsteps, u, v, ut, vt, uf, vf,
                                    iters)
        return u.reshape(ny, nx), v.reshape(ny, nx), iters[:nsteps], uf, vf

    def ref_ppe(self, xf, yf, itermax=100000, tol=1e-6, method=0, w=1.0):
        nx, ny = len(xf) + 1, len(yf) + 1
        _, _, dx, dy = self.grid(nx, ny, xf, yf)
        p = np.zeros(nx * ny)
        it = C.c_int(0)
        self.lib.orc_ref_ppe_opt(nx, ny, dx, dy, itermax, tol, method, w, p, C.byref(it))
        return p.reshape(ny, nx), it.value

    # ---- method solver
    def method(self, cfg, xf, yf, nthreads=4):
        return OracleSolver(self, cfg, xf, yf, nthreads)


class OracleSolver:
    def __init__(self, o, cfg, xf, yf, nthreads):
        self.o = o
        self.cfg = cfg
        self.nx, self.ny = cfg.nx + 2, cfg.ny + 2
        self.h = o.lib.orc_create(C.byref(cfg), np.ascontiguousarray(xf, np.float64),
                                  np.ascontiguousarray(yf, np.float64), nthreads)

    def step(self, n=1):
        self.o.lib.orc_step(self.h, n)

    def get(self, field):
        nx, ny = self.nx, self.ny
        shp = {capi.FIELD_UF: (ny - 2, nx - 1), capi.FIELD_VF: (ny - 1, nx - 2),
               capi.FIELD_XC: (nx,), capi.FIELD_YC: (ny,)}.get(field, (ny, nx))
        out = np.zeros(int(np.prod(shp)))
        r = self.o.lib.orc_get(self.h, field, out, out.size)
        assert r == 0
        return out.reshape(shp)

    def set(self, field, arr):
        a = np.ascontiguousarray(arr, np.float64).ravel()
        assert self.o.lib.orc_set(self.h, field, a, a.size) == 0

    def stats(self):
        st = capi.Stats()
        self.o.lib.orc_stats(self.h, C.byref(st))
        return st

    def ghosts(self):
        n = self.o.lib.orc_ghosts(self.h, None, None, None, None, None, None)
        cells = np.zeros(n, np.int32)
        nb = np.zeros(4 * n, np.int32)
        wu, wp = np.zeros(4 * n), np.zeros(4 * n)
        bi, ip = np.zeros(2 * n), np.zeros(2 * n)
        self.o.lib.orc_ghosts(self.h, cells.ctypes.data, nb.ctypes.data, wu.ctypes.data, wp.ctypes.data,
                              bi.ctypes.data, ip.ctypes.data)
        return cells, nb.reshape(n, 4), wu.reshape(n, 4), wp.reshape(n, 4), bi.reshape(n, 2), ip.reshape(n, 2)

    def levels(self):
        return self.o.lib.orc_mg_levels(self.h)

    def body(self):
        """Current body pose: x, y, cos, sin of the angle, u, v, rotation rate."""
        out = np.zeros(7)
        self.o.lib.orc_body(self.h, out)
        return out

    def __del__(self):
        try:
            self.o.lib.orc_destroy(self.h)
        except Exception:
            pass
