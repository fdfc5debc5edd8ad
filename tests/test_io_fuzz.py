"""Malformed input files never crash the parsers.

ifx_config_read (src/main.cu:10-59 grammar), ifx_grid_read
(src/include/preSim.cu:275-290) and ifx_probes_read (probe.dat) run on the host
without a GPU.  Fed seeded garbage built from their own keywords, numbers and
stray bytes, each must return a status code (OK or a parse error), never crash
the process or write past the caller's buffer.
"""
import ctypes as C
import os

import numpy as np
import pytest

import immerseflow_gb300 as ifx
from immerseflow_gb300 import _capi as capi

KEYWORDS = ["Restart", "nx ny", "Lx Ly", "w-AD w-PPE AD_itermax PPE_itermax AD_solver PPE_solver",
            "ErrorMax tmax dt Re mu", "Write Interval", "Solver-Mode", "Precision", "Initial-Field",
            "Boundary-Types", "Boundary-Velocity", "Outflow-Speed", "Body-Motion", "Body", "PPE-Tolerance",
            "Multigrid", "Mixed-Inner", "Force-Reference", "PPE-Method", "Grid-Files", "====", "____"]
WORDS = ["method", "reference", "mixed", "fp64", "vortex", "rest", "uniform", "wall", "inflow", "outflow",
         "slip", "circle", "ellipse", "none", "prescribed", "jacobi", "point-gs", "line-sor", "0", "1", "-1",
         "1e308", "-1e308", "nan", "inf", "2147483648", "0.5", "x", ",", "\t", "\x00", "\xff"]
OK_OR_PARSE = {capi.IFX_OK, capi.IFX_ERR_PARSE, capi.IFX_ERR_IO}


def _garbage(rng, nlines):
    out = []
    for _ in range(nlines):
        r = rng.random()
        if r < 0.4:
            out.append(KEYWORDS[rng.integers(len(KEYWORDS))])
        elif r < 0.8:
            out.append(" ".join(WORDS[k] for k in rng.integers(len(WORDS), size=rng.integers(0, 12))))
        else:
            out.append(bytes(rng.integers(0, 256, size=rng.integers(0, 40), dtype=np.uint8)).decode("latin-1"))
    return "\n".join(out)


def test_config_read_survives_garbage(tmp_path):
    lib = ifx.lib()
    rng = np.random.default_rng(0)
    p = tmp_path / "inputs.txt"
    for _ in range(400):
        p.write_bytes(_garbage(rng, int(rng.integers(0, 40))).encode("latin-1"))
        cfg = capi.Config()
        st = lib.ifx_config_read(str(p).encode(), C.byref(cfg))
        assert st in OK_OR_PARSE, (st, lib.ifx_last_error())


def test_grid_read_survives_garbage_and_keeps_to_its_buffer(tmp_path):
    lib = ifx.lib()
    rng = np.random.default_rng(1)
    p = tmp_path / "xgrid.dat2"
    for _ in range(300):
        n = int(rng.integers(2, 20))
        rows = []
        for i in range(int(rng.integers(0, 2 * n + 2))):
            rows.append(f"{i} {rng.normal():.6f}" if rng.random() < 0.7 else _garbage(rng, 1))
        p.write_bytes("\n".join(rows).encode("latin-1"))
        buf = np.full(n + 8, 12345.0)
        st = lib.ifx_grid_read(str(p).encode(), n, buf.ctypes.data_as(C.POINTER(C.c_double)))
        assert st in OK_OR_PARSE, (st, lib.ifx_last_error())
        assert np.all(buf[n:] == 12345.0)


def test_probes_read_survives_garbage_and_keeps_to_its_buffer(tmp_path):
    lib = ifx.lib()
    rng = np.random.default_rng(2)
    p = tmp_path / "probe.dat"
    for _ in range(300):
        cap = int(rng.integers(0, 6))
        head = str(int(rng.integers(-2, 10))) if rng.random() < 0.8 else _garbage(rng, 1)
        body = [f"{rng.normal():.4f}, {rng.normal():.4f}" if rng.random() < 0.7 else _garbage(rng, 1)
                for _ in range(int(rng.integers(0, 12)))]
        p.write_bytes("\n".join([head] + body).encode("latin-1"))
        xy = np.full(2 * cap + 8, 777.0)
        n = C.c_int(-5)
        st = lib.ifx_probes_read(str(p).encode(), cap, xy.ctypes.data_as(C.POINTER(C.c_double)), C.byref(n))
        assert st in OK_OR_PARSE, (st, lib.ifx_last_error())
        assert np.all(xy[2 * cap:] == 777.0)
        if st == capi.IFX_OK:
            assert n.value >= 0


@pytest.mark.parametrize("nxny", ["2147483647 50", "50 2147483647", "20000 20000", "2147483647 2147483647",
                                  "1 80000000"])
def test_oversized_grid_is_refused_before_any_allocation(golden_dir, tmp_path, nxny):
    # more than IFX_MAX_CELLS cells in the padded device layout (the last case
    # has 3 x 80000002 < 2^28 cells, but rows padded to 32 give 2.56e9): a parse
    # error from the file surface and an argument error from the create call,
    # both before any device access
    with open(os.path.join(golden_dir, "inputs", "inputs.txt")) as fh:
        lines = fh.read().splitlines()
    k = next(i for i, l in enumerate(lines) if "nx" in l)
    lines[k + 1] = nxny
    p = tmp_path / "inputs.txt"
    p.write_text("\n".join(lines) + "\n")
    lib = ifx.lib()
    cfg = capi.Config()
    assert lib.ifx_config_read(str(p).encode(), C.byref(cfg)) == capi.IFX_ERR_PARSE
    assert b"IFX_MAX_CELLS" in lib.ifx_last_error()
    h = C.c_void_p()
    assert lib.ifx_create_from_file(str(p).encode(), C.byref(h)) == capi.IFX_ERR_PARSE
    lib.ifx_config_default(C.byref(cfg))
    cfg.nx, cfg.ny = (int(v) for v in nxny.split())
    xf = np.linspace(0.0, 1.0, 8)
    xs = (C.POINTER(C.c_double) * 1)(xf.ctypes.data_as(C.POINTER(C.c_double)))
    st = lib.ifx_create_batch(1, C.byref(cfg), xs, xs, C.byref(h))
    assert st == capi.IFX_ERR_ARG, lib.ifx_last_error()
    assert b"IFX_MAX_CELLS" in lib.ifx_last_error()
