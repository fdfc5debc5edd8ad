"""GB300-native fractional-step / ghost-cell immersed-boundary solver.

Python side of the C ABI in include/immerseflow_gb300.h.  The compute path is
libimmerseflow_gb300.so (CUDA kernels for sm_103a + C++ host code); this
module only loads it with ctypes and converts arrays.  There is no CPU
fallback: if the library is missing or no GPU is present, the calls raise.
"""
import ctypes as C
import os

import numpy as np

from . import _capi as capi
from ._capi import Config, Schedule, Stats, default_config

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libimmerseflow_gb300.so")
_lib = None

# every entry point of include/immerseflow_gb300.h with (restype, argtypes)
_dp = C.POINTER(C.c_double)
_SIGS = {
    "ifx_status_string": (C.c_char_p, [C.c_int]),
    "ifx_last_error": (C.c_char_p, []),
    "ifx_version": (C.c_char_p, []),
    "ifx_config_default": (None, [C.POINTER(Config)]),
    "ifx_config_read": (C.c_int, [C.c_char_p, C.POINTER(Config)]),
    "ifx_grid_read": (C.c_int, [C.c_char_p, C.c_int, _dp]),
    "ifx_write_tecplot": (C.c_int, [C.c_char_p, C.c_int, C.c_int, _dp, _dp, _dp]),
    "ifx_create": (C.c_int, [C.POINTER(Config), _dp, _dp, C.POINTER(C.c_void_p)]),
    "ifx_create_from_file": (C.c_int, [C.c_char_p, C.POINTER(C.c_void_p)]),
    "ifx_create_batch": (C.c_int, [C.c_int, C.POINTER(Config), C.POINTER(_dp), C.POINTER(_dp),
                                   C.POINTER(C.c_void_p)]),
    "ifx_num_instances": (C.c_int, [C.c_void_p]),
    "ifx_get_dims": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "ifx_step": (C.c_int, [C.c_void_p, C.c_int]),
    "ifx_ppe_reference": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "ifx_ppe_reference_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int,
                                            C.c_double, C.POINTER(C.c_int), C.c_void_p]),
    "ifx_get_field": (C.c_int, [C.c_void_p, C.c_int, _dp, C.c_size_t]),
    "ifx_set_field": (C.c_int, [C.c_void_p, C.c_int, _dp, C.c_size_t]),
    "ifx_get_field_i": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _dp, C.c_size_t]),
    "ifx_set_field_i": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _dp, C.c_size_t]),
    "ifx_set_state": (C.c_int, [C.c_void_p, C.c_int, _dp, _dp, _dp, C.c_size_t]),
    "ifx_get_state": (C.c_int, [C.c_void_p, C.c_int, _dp, _dp, _dp, C.c_size_t]),
    "ifx_step_state": (C.c_int, [C.c_void_p, C.c_int, _dp, _dp, _dp, C.c_int, _dp, _dp, _dp, C.c_size_t]),
    "ifx_write_results": (C.c_int, [C.c_void_p, C.c_char_p]),
    "ifx_forces": (C.c_int, [C.c_void_p, _dp, _dp]),
    "ifx_get_stats": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(Stats)]),
    "ifx_last_step_ms": (C.c_int, [C.c_void_p, _dp]),
    "ifx_get_ibm_ghosts": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.c_void_p, C.c_void_p, C.POINTER(C.c_int)]),
    "ifx_synchronize": (C.c_int, [C.c_void_p]),
    "ifx_trace_step": (C.c_int, [C.c_void_p, C.c_int, _dp, C.POINTER(C.c_int)]),
    "ifx_profile_kernel": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _dp, C.POINTER(C.c_longlong)]),
    "ifx_set_barrier_fault": (C.c_int, [C.c_void_p, C.c_longlong, C.c_int]),
    "ifx_set_schedule": (C.c_int, [C.c_void_p, C.POINTER(Schedule)]),
    "ifx_get_schedule": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(Schedule)]),
    "ifx_autotune_schedule": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(Schedule), _dp]),
    "ifx_destroy": (None, [C.c_void_p]),
    "ifx_step_async": (C.c_int, [C.c_void_p, C.c_int]),
    "ifx_autotune": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int), _dp]),
    "ifx_set_mg_tile_rows": (C.c_int, [C.c_void_p, C.c_int]),
    "ifx_get_mg_tile_rows": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "ifx_set_cluster_vcycle": (C.c_int, [C.c_void_p, C.c_int]),
    "ifx_get_cluster_vcycle": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "ifx_step_wait": (C.c_int, [C.c_void_p]),
    "ifx_set_exec_mode": (C.c_int, [C.c_void_p, C.c_int]),
    "ifx_get_exec_mode": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "ifx_set_persistent_grid": (C.c_int, [C.c_void_p, C.c_int]),
    "ifx_get_persistent_grid": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "ifx_set_instance_active": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "ifx_device_bytes": (C.c_int, [C.c_void_p, C.POINTER(C.c_size_t)]),
    "ifx_checkpoint_bytes": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_size_t)]),
    "ifx_checkpoint_save": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_size_t]),
    "ifx_checkpoint_load": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_size_t]),
    "ifx_checkpoint_write": (C.c_int, [C.c_void_p, C.c_char_p]),
    "ifx_checkpoint_read": (C.c_int, [C.c_void_p, C.c_char_p]),
    "ifx_write_snapshot_ascii": (C.c_int, [C.c_void_p, C.c_int, C.c_char_p]),
    "ifx_read_snapshot_ascii": (C.c_int, [C.c_void_p, C.c_int, C.c_char_p]),
    "ifx_probes_read": (C.c_int, [C.c_char_p, C.c_int, _dp, C.POINTER(C.c_int)]),
    "ifx_set_history": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, _dp]),
    "ifx_get_probe_cells": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                      C.POINTER(C.c_int)]),
    "ifx_get_history": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _dp, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "ifx_write_probe_file": (C.c_int, [C.c_void_p, C.c_int, C.c_char_p]),
    "ifx_write_force_file": (C.c_int, [C.c_void_p, C.c_int, C.c_char_p]),
    "ifx_estimate_bytes": (C.c_int, [C.POINTER(Config), C.POINTER(C.c_size_t)]),
    "ifx_server_create": (C.c_int, [C.c_size_t, C.c_int, C.POINTER(C.c_void_p)]),
    "ifx_server_set_exec_mode": (C.c_int, [C.c_void_p, C.c_int]),
    "ifx_server_set_steps_per_tick": (C.c_int, [C.c_void_p, C.c_int]),
    "ifx_server_submit": (C.c_int, [C.c_void_p, C.POINTER(Config), _dp, _dp, C.c_int, C.POINTER(C.c_longlong)]),
    "ifx_server_tick": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "ifx_server_preempt": (C.c_int, [C.c_void_p, C.c_longlong, C.c_int]),
    "ifx_server_poll": (C.c_int, [C.c_void_p, C.POINTER(C.c_longlong), C.c_int, C.POINTER(C.c_int)]),
    "ifx_server_request_state": (C.c_int, [C.c_void_p, C.c_longlong, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                           C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "ifx_server_result": (C.c_int, [C.c_void_p, C.c_longlong, C.c_int, _dp, C.c_size_t]),
    "ifx_server_request_stats": (C.c_int, [C.c_void_p, C.c_longlong, C.POINTER(Stats)]),
    "ifx_server_release": (C.c_int, [C.c_void_p, C.c_longlong]),
    "ifx_server_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                  C.POINTER(C.c_size_t)]),
    "ifx_server_destroy": (None, [C.c_void_p]),
}

EXEC_DEFAULT, EXEC_PERSISTENT, EXEC_GRAPH, EXEC_HOST = -1, 0, 1, 2
REQ_WAITING, REQ_RUNNING, REQ_FINISHED, REQ_FAILED = 0, 1, 2, 3


class IFXError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"[{status}] {msg}")
        self.status = status


def lib():
    """The loaded CUDA library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m immerseflow_gb300.build`")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _check(st):
    if st != capi.IFX_OK:
        raise IFXError(st, lib().ifx_last_error().decode())


def _dptr(a):
    return a.ctypes.data_as(_dp)


def config_read(path):
    """readInputFile (src/main.cu:10-59) with the extension keywords."""
    c = Config()
    _check(lib().ifx_config_read(os.fsencode(path), C.byref(c)))
    return c


def grid_read(path, n):
    out = np.zeros(n)
    _check(lib().ifx_grid_read(os.fsencode(path), n, _dptr(out)))
    return out


def probes_read(path):
    """probe.dat (probe_init, test/UTIL_PRE_SIM.f90:172-202) -> (n, 2) array."""
    n = C.c_int()
    _check(lib().ifx_probes_read(os.fsencode(path), 0, None, C.byref(n)))
    xy = np.zeros(2 * max(n.value, 1))
    _check(lib().ifx_probes_read(os.fsencode(path), n.value, _dptr(xy), C.byref(n)))
    return xy[:2 * n.value].reshape(n.value, 2)


def write_tecplot(path, x, y, q):
    x = np.ascontiguousarray(x, np.float64)
    y = np.ascontiguousarray(y, np.float64)
    q = np.ascontiguousarray(q, np.float64)
    _check(lib().ifx_write_tecplot(os.fsencode(path), len(x), len(y), _dptr(x), _dptr(y), _dptr(q)))


class Solver:
    """One solver handle: a single instance, or a batch of instances."""

    def __init__(self, handle):
        self._h = C.c_void_p(handle)

    @classmethod
    def create(cls, cfg, xf, yf):
        xf = np.ascontiguousarray(xf, np.float64)
        yf = np.ascontiguousarray(yf, np.float64)
        h = C.c_void_p()
        _check(lib().ifx_create(C.byref(cfg), _dptr(xf), _dptr(yf), C.byref(h)))
        return cls(h.value)

    @classmethod
    def from_file(cls, inputs_path):
        h = C.c_void_p()
        _check(lib().ifx_create_from_file(os.fsencode(inputs_path), C.byref(h)))
        return cls(h.value)

    @classmethod
    def batch(cls, cfgs, xfs, yfs):
        n = len(cfgs)
        carr = (Config * n)(*cfgs)
        xs = [np.ascontiguousarray(x, np.float64) for x in xfs]
        ys = [np.ascontiguousarray(y, np.float64) for y in yfs]
        xp = (_dp * n)(*[_dptr(x) for x in xs])
        yp = (_dp * n)(*[_dptr(y) for y in ys])
        h = C.c_void_p()
        _check(lib().ifx_create_batch(n, carr, xp, yp, C.byref(h)))
        s = cls(h.value)
        s._keep = (xs, ys)
        return s

    @property
    def n_instances(self):
        return lib().ifx_num_instances(self._h)

    def step(self, n=1):
        _check(lib().ifx_step(self._h, n))

    def ppe_reference(self):
        it = C.c_int(0)
        _check(lib().ifx_ppe_reference(self._h, C.byref(it)))
        return it.value

    def get(self, field, inst=0, out=None):
        """Copy a field to the host; cell fields come back as [ny, nx].  With
        `out` (a C-contiguous float64 array of the field's size, e.g. a pinned
        buffer reused every step) the field is copied straight into it."""
        nx, ny = self.grid_dims(inst)
        shp = {capi.FIELD_UF: (ny - 2, nx - 1), capi.FIELD_VF: (ny - 1, nx - 2),
               capi.FIELD_XC: (nx,), capi.FIELD_YC: (ny,)}.get(field, (ny, nx))
        n = int(np.prod(shp))
        if out is None:
            out = np.zeros(n)
        elif out.dtype != np.float64 or not out.flags.c_contiguous or out.size != n:
            raise ValueError(f"out must be a C-contiguous float64 array of {n} values")
        _check(lib().ifx_get_field_i(self._h, inst, field, _dptr(out), out.size))
        return out.reshape(shp)

    def set(self, field, arr, inst=0):
        a = np.ascontiguousarray(arr, np.float64).ravel()
        _check(lib().ifx_set_field_i(self._h, inst, field, _dptr(a), a.size))

    def set_state(self, u, v, p, inst=0):
        """Set u, v and p of instance `inst` in one call (each nx*ny values in
        dense rows, or None to keep that field)."""
        nx, ny = self.grid_dims(inst)
        arrs = [None if a is None else np.ascontiguousarray(a, np.float64).ravel() for a in (u, v, p)]
        for a in arrs:
            if a is not None and a.size != nx * ny:
                raise ValueError(f"each field must hold {nx * ny} values")
        ptrs = [None if a is None else _dptr(a) for a in arrs]
        _check(lib().ifx_set_state(self._h, inst, *ptrs, nx * ny))

    def get_state(self, inst=0, out=None):
        """(u, v, p) of instance `inst` as [ny, nx] arrays in one call; with
        `out` (three C-contiguous float64 arrays of nx*ny values, e.g. pinned
        buffers reused every step) the fields are copied straight into them."""
        nx, ny = self.grid_dims(inst)
        if out is None:
            out = tuple(np.zeros(nx * ny) for _ in range(3))
        for a in out:
            if a.dtype != np.float64 or not a.flags.c_contiguous or a.size != nx * ny:
                raise ValueError(f"out must be three C-contiguous float64 arrays of {nx * ny} values")
        _check(lib().ifx_get_state(self._h, inst, *[_dptr(a) for a in out], nx * ny))
        return tuple(a.reshape(ny, nx) for a in out)

    def step_state(self, u, v, p, n=1, out=None, inst=0):
        """set_state(u, v, p), step(n) and get_state(out=out) in one call that
        waits once: each input nx*ny float64 values or None (keep), `out` three
        C-contiguous float64 arrays of nx*ny values (they may be the inputs) or
        None (no copy out).  Returns out reshaped to [ny, nx], or None."""
        nx, ny = self.grid_dims(inst)
        arrs = [None if a is None else np.ascontiguousarray(a, np.float64).ravel() for a in (u, v, p)]
        for a in arrs:
            if a is not None and a.size != nx * ny:
                raise ValueError(f"each field must hold {nx * ny} values")
        if out is not None:
            for a in out:
                if a.dtype != np.float64 or not a.flags.c_contiguous or a.size != nx * ny:
                    raise ValueError(f"out must be three C-contiguous float64 arrays of {nx * ny} values")
        ins = [None if a is None else _dptr(a) for a in arrs]
        outs = [None, None, None] if out is None else [_dptr(a) for a in out]
        _check(lib().ifx_step_state(self._h, inst, *ins, int(n), *outs, nx * ny))
        return None if out is None else tuple(a.reshape(ny, nx) for a in out)

    def grid_dims(self, inst=0):
        """(nx, ny) including the ghost ring."""
        nx = C.c_int()
        ny = C.c_int()
        _check(lib().ifx_get_dims(self._h, inst, C.byref(nx), C.byref(ny)))
        return nx.value, ny.value

    def stats(self, inst=0):
        st = Stats()
        _check(lib().ifx_get_stats(self._h, inst, C.byref(st)))
        return st

    def ibm_ghosts(self, inst=0):
        """IBM ghost table: cells, nb[4], Dirichlet weights, Neumann weights, BI/IP (dense indices)."""
        n = C.c_int()
        _check(lib().ifx_get_ibm_ghosts(self._h, inst, 0, None, None, None, None, None, C.byref(n)))
        k = n.value
        cells = np.zeros(k, np.int32)
        nb = np.zeros(4 * k, np.int32)
        wu, wp, bip = np.zeros(4 * k), np.zeros(4 * k), np.zeros(4 * k)
        _check(lib().ifx_get_ibm_ghosts(self._h, inst, k, cells.ctypes.data, nb.ctypes.data, wu.ctypes.data,
                                        wp.ctypes.data, bip.ctypes.data, C.byref(n)))
        return cells, nb.reshape(k, 4), wu.reshape(k, 4), wp.reshape(k, 4), bip.reshape(k, 4)

    def forces(self):
        cd = C.c_double()
        cl = C.c_double()
        _check(lib().ifx_forces(self._h, C.byref(cd), C.byref(cl)))
        return cd.value, cl.value

    def last_step_ms(self):
        ms = C.c_double()
        _check(lib().ifx_last_step_ms(self._h, C.byref(ms)))
        return ms.value

    def write_results(self, directory):
        _check(lib().ifx_write_results(self._h, os.fsencode(directory)))

    def profile_kernel(self, kernel, reps=50):
        """(mean ms per launch, interior cells per launch) of one step kernel."""
        ms = C.c_double()
        cells = C.c_longlong()
        _check(lib().ifx_profile_kernel(self._h, kernel, reps, C.byref(ms), C.byref(cells)))
        return ms.value, cells.value

    def trace_step(self, cap=4096):
        """One persistent time step; microseconds between consecutive grid barriers."""
        us = np.zeros(cap)
        n = C.c_int()
        _check(lib().ifx_trace_step(self._h, cap, _dptr(us), C.byref(n)))
        return us[:n.value]

    def synchronize(self):
        _check(lib().ifx_synchronize(self._h))

    def step_async(self, n=1):
        _check(lib().ifx_step_async(self._h, int(n)))

    def step_wait(self):
        _check(lib().ifx_step_wait(self._h))

    def set_exec_mode(self, mode):
        _check(lib().ifx_set_exec_mode(self._h, int(mode)))

    def exec_mode(self):
        m = C.c_int()
        _check(lib().ifx_get_exec_mode(self._h, C.byref(m)))
        return m.value

    def set_persistent_grid(self, blocks):
        """Blocks of the persistent mode's launch (0: all co-resident blocks)."""
        _check(lib().ifx_set_persistent_grid(self._h, int(blocks)))

    def persistent_grid(self):
        g = C.c_int()
        _check(lib().ifx_get_persistent_grid(self._h, C.byref(g)))
        return g.value

    def autotune(self, steps=2):
        """Pick the fastest execution mode by timing; state is restored.  Returns (mode, ms/step)."""
        m, ms = C.c_int(), C.c_double()
        _check(lib().ifx_autotune(self._h, int(steps), C.byref(m), C.byref(ms)))
        return m.value, ms.value

    def schedule(self, inst=0):
        """Sweep schedule of an instance (capi.Schedule)."""
        s = Schedule()
        _check(lib().ifx_get_schedule(self._h, int(inst), C.byref(s)))
        return s

    def set_schedule(self, sched):
        _check(lib().ifx_set_schedule(self._h, C.byref(sched)))

    def autotune_schedule(self, steps=2):
        """Pick the fastest valid sweep schedule by timing; state is restored.
        Returns (capi.Schedule, ms/step)."""
        s, ms = Schedule(), C.c_double()
        _check(lib().ifx_autotune_schedule(self._h, int(steps), C.byref(s), C.byref(ms)))
        return s, ms.value

    def set_mg_tile_rows(self, rows):
        _check(lib().ifx_set_mg_tile_rows(self._h, int(rows)))

    def mg_tile_rows(self):
        r = C.c_int()
        _check(lib().ifx_get_mg_tile_rows(self._h, C.byref(r)))
        return r.value

    def set_cluster_vcycle(self, on):
        _check(lib().ifx_set_cluster_vcycle(self._h, 1 if on else 0))

    def cluster_vcycle(self):
        """(available, on)"""
        a, o = C.c_int(), C.c_int()
        _check(lib().ifx_get_cluster_vcycle(self._h, C.byref(a), C.byref(o)))
        return bool(a.value), bool(o.value)

    # ---- restart / checkpoint
    def checkpoint(self, inst=0):
        """Binary checkpoint of one instance (bytes)."""
        n = C.c_size_t()
        _check(lib().ifx_checkpoint_bytes(self._h, int(inst), C.byref(n)))
        buf = C.create_string_buffer(n.value)
        _check(lib().ifx_checkpoint_save(self._h, int(inst), buf, n.value))
        return buf.raw

    def restore(self, blob, inst=0):
        """Loads a checkpoint made by checkpoint() into instance inst."""
        buf = C.create_string_buffer(bytes(blob), len(blob))
        _check(lib().ifx_checkpoint_load(self._h, int(inst), buf, len(blob)))

    def checkpoint_write(self, path):
        _check(lib().ifx_checkpoint_write(self._h, os.fsencode(path)))

    def checkpoint_read(self, path):
        _check(lib().ifx_checkpoint_read(self._h, os.fsencode(path)))

    def write_snapshot_ascii(self, path, inst=0):
        _check(lib().ifx_write_snapshot_ascii(self._h, int(inst), os.fsencode(path)))

    def read_snapshot_ascii(self, path, inst=0):
        _check(lib().ifx_read_snapshot_ascii(self._h, int(inst), os.fsencode(path)))

    # ---- time history
    def set_history(self, capacity, probes=(), inst=0):
        """Records step, cd, cl and u, v, p at each probe (x, y) every step."""
        xy = np.ascontiguousarray(np.asarray(probes, np.float64).reshape(-1))
        n = xy.size // 2
        _check(lib().ifx_set_history(self._h, int(inst), int(capacity), n, _dptr(xy) if n else None))

    def probe_cells(self, inst=0):
        n = C.c_int()
        _check(lib().ifx_get_probe_cells(self._h, int(inst), 0, None, None, C.byref(n)))
        i = (C.c_int * max(n.value, 1))()
        j = (C.c_int * max(n.value, 1))()
        _check(lib().ifx_get_probe_cells(self._h, int(inst), n.value, i, j, C.byref(n)))
        return [(i[k], j[k]) for k in range(n.value)]

    def history(self, cap=1 << 20, inst=0):
        """(records, 3 + 3*nprobes) array: step, cd, cl, then u, v, p per probe."""
        n, w = C.c_int(), C.c_int()
        _check(lib().ifx_get_history(self._h, int(inst), 0, None, C.byref(n), C.byref(w)))
        rows = np.zeros(max(cap, 1) * max(w.value, 1))
        _check(lib().ifx_get_history(self._h, int(inst), int(cap), _dptr(rows), C.byref(n), C.byref(w)))
        return rows[:n.value * w.value].reshape(n.value, w.value)

    def write_probe_file(self, path, inst=0):
        _check(lib().ifx_write_probe_file(self._h, int(inst), os.fsencode(path)))

    def write_force_file(self, path, inst=0):
        _check(lib().ifx_write_force_file(self._h, int(inst), os.fsencode(path)))

    def set_active(self, inst, active):
        _check(lib().ifx_set_instance_active(self._h, int(inst), 1 if active else 0))

    def device_bytes(self):
        b = C.c_size_t()
        _check(lib().ifx_device_bytes(self._h, C.byref(b)))
        return b.value

    def close(self):
        if self._h:
            lib().ifx_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def estimate_bytes(cfg):
    b = C.c_size_t()
    _check(lib().ifx_estimate_bytes(C.byref(cfg), C.byref(b)))
    return b.value


class Server:
    """Continuous-batching solve server (ifx_server_* in the C ABI)."""

    def __init__(self, hbm_budget_bytes, max_cohort=64, exec_mode=None, steps_per_tick=None):
        self._h = C.c_void_p()
        _check(lib().ifx_server_create(int(hbm_budget_bytes), int(max_cohort), C.byref(self._h)))
        if exec_mode is not None:
            _check(lib().ifx_server_set_exec_mode(self._h, int(exec_mode)))
        if steps_per_tick is not None:
            _check(lib().ifx_server_set_steps_per_tick(self._h, int(steps_per_tick)))

    def submit(self, cfg, xf, yf, nsteps):
        xf = np.ascontiguousarray(xf, dtype=np.float64)
        yf = np.ascontiguousarray(yf, dtype=np.float64)
        rid = C.c_longlong()
        _check(lib().ifx_server_submit(self._h, C.byref(cfg), _dptr(xf), _dptr(yf), int(nsteps), C.byref(rid)))
        return rid.value

    def tick(self):
        n = C.c_int()
        _check(lib().ifx_server_tick(self._h, C.byref(n)))
        return n.value

    def preempt(self, rid, front=True):
        """Takes a running request off the device (checkpoint in host memory)."""
        _check(lib().ifx_server_preempt(self._h, int(rid), 1 if front else 0))

    def poll(self, cap=1024):
        ids = (C.c_longlong * cap)()
        n = C.c_int()
        _check(lib().ifx_server_poll(self._h, ids, cap, C.byref(n)))
        return list(ids[:n.value])

    def state(self, rid):
        st, done, nx, ny = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        _check(lib().ifx_server_request_state(self._h, int(rid), C.byref(st), C.byref(done), C.byref(nx), C.byref(ny)))
        return st.value, done.value, nx.value, ny.value

    def result(self, rid, field):
        _, _, nx, ny = self.state(rid)
        out = np.empty(nx * ny)
        _check(lib().ifx_server_result(self._h, int(rid), int(field), _dptr(out), out.size))
        return out.reshape(ny, nx)

    def stats(self, rid):
        s = Stats()
        _check(lib().ifx_server_request_stats(self._h, int(rid), C.byref(s)))
        return s

    def release(self, rid):
        _check(lib().ifx_server_release(self._h, int(rid)))

    def info(self):
        w, r, c, b = C.c_int(), C.c_int(), C.c_int(), C.c_size_t()
        _check(lib().ifx_server_info(self._h, C.byref(w), C.byref(r), C.byref(c), C.byref(b)))
        return {"waiting": w.value, "running": r.value, "cohorts": c.value, "used_bytes": b.value}

    def close(self):
        if self._h:
            lib().ifx_server_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


from .interface import ImmerseFlow  # noqa: E402  (mirror of the reference object)

__all__ = ["Config", "Schedule", "Stats", "default_config", "Solver", "Server", "ImmerseFlow", "IFXError", "config_read",
           "grid_read", "write_tecplot", "probes_read", "estimate_bytes", "lib", "capi"]
