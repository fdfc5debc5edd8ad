"""The C-ABI library loads and exports every entry point declared in include/*.h."""
import ctypes as C
import glob
import os
import re
import subprocess

import immerseflow_gb300 as ifx
from immerseflow_gb300 import _capi as capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"\b(ifx_[a-z0-9_]+)\s*\(", src):
            names.add(m.group(1))
    return names


def test_every_declared_symbol_is_exported():
    lib = C.CDLL(ifx.LIB_PATH)
    names = declared_functions()
    assert len(names) >= 45
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_python_bindings_cover_the_header():
    assert declared_functions() <= set(ifx._SIGS)


def test_struct_layout_matches_header(tmp_path):
    src = tmp_path / "sz.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "immerseflow_gb300.h"\n'
                   'int main(void){printf("%zu %zu %zu %zu %d\\n", sizeof(ifx_config), sizeof(ifx_stats),'
                   ' offsetof(ifx_config, xgrid), offsetof(ifx_stats, status), IFX_MAX_CELLS); return 0;}\n')
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-I" + os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    assert int(out[0]) == C.sizeof(capi.Config)
    assert int(out[1]) == C.sizeof(capi.Stats)
    assert int(out[2]) == capi.Config.xgrid.offset
    assert int(out[3]) == capi.Stats.status.offset
    assert int(out[4]) == capi.MAX_CELLS


def test_config_default_matches_python_mirror():
    c = capi.Config()
    ifx.lib().ifx_config_default(C.byref(c))
    d = capi.default_config()
    for name, _ in capi.Config._fields_:
        a, b = getattr(c, name), getattr(d, name)
        if hasattr(a, "__len__") and not isinstance(a, bytes):
            a, b = list(a), list(b)
        assert a == b, name


def test_status_strings_and_no_device_error():
    L = ifx.lib()
    assert L.ifx_status_string(capi.IFX_ERR_PARSE) == b"parse error"
    assert L.ifx_version().startswith(b"immerseflow_gb300")


def test_noalloc_solve_refuses_bad_arguments_before_device_access():
    # null buffers, too-small grids and grids above IFX_NOALLOC_MAX_CELLS are
    # refused by the host checks that precede any CUDA call
    lib = ifx.lib()
    d = C.c_void_p(16)
    cases = [(None, d, 10, 10, d), (d, None, 10, 10, d), (d, d, 10, 10, None), (d, d, 2, 10, d), (d, d, 10, 2, d),
             (d, d, 200, 200, d), (d, d, 133, 132, d)]
    for dx, dy, nx, ny, p in cases:
        st = lib.ifx_ppe_reference_noalloc(dx, dy, nx, ny, p, 10, 1e-6, None, None)
        assert st == capi.IFX_ERR_ARG, (nx, ny)
    # a NaN tolerance would stop the loop before its first sweep
    st = lib.ifx_ppe_reference_noalloc(d, d, 10, 10, d, 10, float("nan"), None, None)
    assert st == capi.IFX_ERR_ARG
