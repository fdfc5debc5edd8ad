"""The reference's file surface: inputs.txt grammar, grid files, Tecplot writer."""
import hashlib
import os

import numpy as np
import pytest

import immerseflow_gb300 as ifx
from immerseflow_gb300 import _capi as capi


def reference_grammar(path):
    """Restatement of readInputFile (src/main.cu:10-59) for cross-checking."""
    out = {}
    lines = open(path).read().split("\n")
    k = 0
    while k < len(lines):
        line = lines[k]
        k += 1
        if not line or line[0] in "=_":
            continue
        nxt = lines[k].split() if k < len(lines) else []
        if "Restart" in line:
            out["restart"] = nxt[:2]; k += 1
        elif "nx" in line:
            out["nxny"] = nxt[:2]; k += 1
        elif "Lx" in line:
            out["lxly"] = nxt[:2]; k += 1
        elif "w-AD" in line:
            out["wad"] = nxt[:6]; k += 1
        elif "ErrorMax" in line:
            out["err"] = nxt[:5]; k += 1
        elif "Write Interval" in line:
            out["wi"] = nxt[:1]; k += 1
    return out


EXTENSION = """
___________________________| Method extensions |_______________________________
Solver-Mode
method
Precision
mixed
Initial-Field
uniform
Boundary-Types (W E S N)
inflow outflow slip slip
Boundary-Velocity (uW vW uE vE uS vS uN vN)
1 0 0 0 0 0 0 0
Outflow-Speed
1.0
Body (shape cx cy a b angle-deg)
ellipse 10 10 0.5 0.25 15
PPE-Tolerance AD-Tolerance
1e-9 1e-11
Multigrid (pre post omega)
3 2 0.7
Mixed-Inner
6
Force-Reference (U L)
1 1
Grid-Files (x y)
xgrid.dat ygrid.dat
"""


def test_reads_reference_inputs(golden_dir):
    c = ifx.config_read(os.path.join(golden_dir, "inputs", "inputs.txt"))
    assert (c.restart, c.restart_time, c.nx, c.ny) == (0, 9, 50, 50)
    assert (c.lx, c.ly) == (10.0, 5.0)
    assert (c.w_ad, c.w_ppe, c.ad_itermax, c.ppe_itermax, c.ad_solver, c.ppe_solver) == (1, 1, 25, 100000, 1, 1)
    assert (c.error_max, c.tmax, c.dt, c.re, c.mu) == (1e-6, 100.0, 0.001, 150.0, 0.01)
    assert c.write_interval == 1000
    assert c.mode == capi.MODE_REFERENCE
    assert c.xgrid.decode().endswith("inputs/xgrid.dat2")


def test_extension_keywords_invisible_to_reference_grammar(golden_dir, tmp_path):
    src = os.path.join(golden_dir, "inputs", "inputs.txt")
    ext = tmp_path / "inputs.txt"
    ext.write_text(open(src).read() + EXTENSION)
    assert reference_grammar(str(ext)) == reference_grammar(src)
    c = ifx.config_read(str(ext))
    assert (c.nx, c.ny, c.re, c.dt) == (50, 50, 150.0, 0.001)
    assert c.mode == capi.MODE_METHOD and c.precision == capi.PREC_MIXED and c.init == capi.INIT_UNIFORM
    assert list(c.bc_type) == [capi.BC_INFLOW, capi.BC_OUTFLOW, capi.BC_SLIP, capi.BC_SLIP]
    assert c.body == capi.BODY_ELLIPSE and (c.body_cx, c.body_b, c.body_angle_deg) == (10.0, 0.25, 15.0)
    assert (c.ppe_tol, c.ad_tol, c.mg_pre, c.mg_post, c.mg_omega, c.mixed_inner) == (1e-9, 1e-11, 3, 2, 0.7, 6)
    assert c.xgrid.decode() == str(tmp_path / "xgrid.dat")


@pytest.mark.parametrize("bad", ["nx ny\n50\n", "ErrorMax\n1e-6 abc\n", "Body\ntriangle 1 2 3\n",
                                 "Boundary-Types\ninflow outflow\n"])
def test_malformed_inputs_are_parse_errors(tmp_path, bad):
    p = tmp_path / "inputs.txt"
    p.write_text(bad)
    with pytest.raises(ifx.IFXError) as e:
        ifx.config_read(str(p))
    assert e.value.status == capi.IFX_ERR_PARSE


def test_relaxation_factors_and_ppe_method(golden_dir, tmp_path):
    """w-AD / w-PPE are ints in the reference (src/header/globalVariables.cuh:26):
    kept as ints, and as read in relax_ad / relax_ppe; PPE-Method selects the
    solver the PPE_Solver column names (1 point GS, 2 line SOR)."""
    src = open(os.path.join(golden_dir, "inputs", "inputs.txt")).read()
    c = ifx.config_read(os.path.join(golden_dir, "inputs", "inputs.txt"))
    assert (c.relax_ad, c.relax_ppe, c.ppe_method) == (1.0, 1.0, capi.PPE_JACOBI)
    p = tmp_path / "inputs.txt"
    p.write_text(src.replace("1       1       25          100000          1         1",
                             "0.8     1.5     25          100000          1         2") + "PPE-Method\nline-sor\n")
    c = ifx.config_read(str(p))
    assert (c.w_ad, c.w_ppe, c.relax_ad, c.relax_ppe) == (0, 1, 0.8, 1.5)
    assert (c.ppe_solver, c.ppe_method) == (2, capi.PPE_LINE_SOR)
    p.write_text(src + "PPE-Method\nmultigrid\n")
    with pytest.raises(ifx.IFXError) as e:
        ifx.config_read(str(p))
    assert e.value.status == capi.IFX_ERR_PARSE


def test_body_motion_keyword(golden_dir, tmp_path):
    """Body-Motion (extension): none, or prescribed with the nine motion
    parameters; it does not shadow the Body keyword."""
    src = open(os.path.join(golden_dir, "inputs", "inputs.txt")).read()
    p = tmp_path / "inputs.txt"
    p.write_text(src + "Body\ncircle 4 4 0.5\nBody-Motion\nprescribed 0.5 0 0 0.25 10 0.2 0 90 45\n")
    c = ifx.config_read(str(p))
    assert c.body == capi.BODY_ELLIPSE and (c.body_cx, c.body_cy, c.body_a) == (4.0, 4.0, 0.5)
    assert c.motion == capi.MOTION_PRESCRIBED
    assert (c.motion_u, c.motion_v, c.motion_amp_x, c.motion_amp_y, c.motion_amp_deg) == (0.5, 0.0, 0.0, 0.25, 10.0)
    assert (c.motion_freq, c.motion_phase_x, c.motion_phase_y, c.motion_phase_deg) == (0.2, 0.0, 90.0, 45.0)
    p.write_text(src + "Body-Motion\nprescribed 0.5 0\n")
    with pytest.raises(ifx.IFXError) as e:
        ifx.config_read(str(p))
    assert e.value.status == capi.IFX_ERR_PARSE
    p.write_text(src + "Body-Motion\nnone\n")
    assert ifx.config_read(str(p)).motion == capi.MOTION_NONE


def test_missing_inputs_is_io_error(tmp_path):
    with pytest.raises(ifx.IFXError) as e:
        ifx.config_read(str(tmp_path / "nope.txt"))
    assert e.value.status == capi.IFX_ERR_IO


def test_grid_files(golden_dir, tmp_path):
    x = ifx.grid_read(os.path.join(golden_dir, "inputs", "xgrid.dat"), 181)
    assert x[0] == 0.0 and abs(x[-1] - 10.0) < 1e-6 and np.all(np.diff(x) > 0)
    y = ifx.grid_read(os.path.join(golden_dir, "inputs", "ygrid.dat"), 129)
    assert abs(y[-1] - 5.0) < 1e-6
    t = tmp_path / "short.dat"
    t.write_text("1 0.0\n2 0.5\n")
    with pytest.raises(ifx.IFXError) as e:
        ifx.grid_read(str(t), 5)
    assert e.value.status == capi.IFX_ERR_PARSE


def test_tecplot_writer_is_byte_exact(golden, golden_dir, tmp_path):
    digests = dict(l.split() for l in open(os.path.join(golden_dir, "results_sha256.txt")))
    for name in ("uc", "vc", "p", "final_results"):
        out = tmp_path / f"{name}.dat"
        ifx.write_tecplot(str(out), golden["x"], golden["y"], golden[name])
        assert hashlib.sha256(out.read_bytes()).hexdigest() == digests[f"{name}.dat"], name


def test_grid_writer_roundtrip(tmp_path):
    from immerseflow_gb300 import cases

    f = cases.tanh_faces(96, 30.0, 10.0)
    cases.write_grid(str(tmp_path / "x.dat"), f)
    g = ifx.grid_read(str(tmp_path / "x.dat"), 97)
    assert np.abs(g - f).max() < 1e-6 * 30
    assert np.all(np.diff(f) > 0) and f[0] == 0.0 and f[-1] == 30.0
