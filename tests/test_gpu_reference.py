"""REFERENCE mode on the GPU against the golden files and the CPU oracle.

Floating-point tolerance: the CUDA kernels follow the reference expressions
but contract multiply-adds into FMAs, so they agree with the oracle (built
without contraction) to 1e-12 relative, and with the %f golden files to 5e-7.
"""
import os

import numpy as np
import pytest

import immerseflow_gb300 as ifx
from immerseflow_gb300 import _capi as capi

pytestmark = pytest.mark.gpu
PRINT_TOL = 5.0e-7 + 1e-12
FP_RTOL = 1e-12


def _solver(golden_dir, nsteps=0):
    c = ifx.config_read(os.path.join(golden_dir, "inputs", "inputs.txt"))
    c.tmax = 20
    xf = ifx.grid_read(c.xgrid.decode(), c.nx + 1)
    yf = ifx.grid_read(c.ygrid.decode(), c.ny + 1)
    s = ifx.Solver.create(c, xf, yf)
    if nsteps:
        s.step(nsteps)
    return s, xf, yf


def test_ad_20_steps_matches_golden_and_oracle(golden, golden_dir, oracle):
    s, xf, yf = _solver(golden_dir, 20)
    u, v = s.get(capi.FIELD_U), s.get(capi.FIELD_V)
    assert np.abs(u - golden["uc"]).max() <= PRINT_TOL
    assert np.abs(v - golden["vc"]).max() <= PRINT_TOL
    uo, vo, iters, _, _ = oracle.ref_ad(xf, yf, 1e-3, 150.0, 25, 20)
    assert np.abs(u - uo).max() <= FP_RTOL * np.abs(uo).max()
    assert np.abs(v - vo).max() <= FP_RTOL * max(np.abs(vo).max(), 1.0)
    st = s.stats()
    assert st.last_ad_iters == 5 and st.ad_iters_total == int(iters.sum())


def test_ad_step_by_step_equals_batched_steps(golden_dir):
    a, _, _ = _solver(golden_dir)
    for _ in range(6):
        a.step(1)
    b, _, _ = _solver(golden_dir, 6)
    assert np.array_equal(a.get(capi.FIELD_U), b.get(capi.FIELD_U))


def test_ad_nonsquare_grid_vs_oracle(oracle):
    # nx > ny: the reference's vf loop then writes a tail of vf (src/include/ADSolver.cu:179)
    c = ifx.default_config()
    c.nx, c.ny, c.re, c.dt = 64, 40, 150.0, 1e-3
    xf = np.linspace(0, 1.3, 65)
    yf = np.concatenate([[0.0], np.cumsum(np.linspace(0.02, 0.03, 40))])
    s = ifx.Solver.create(c, xf, yf)
    s.step(8)
    uo, vo, _, _, vfo = oracle.ref_ad(xf, yf, 1e-3, 150.0, 25, 8)
    u, v = s.get(capi.FIELD_U), s.get(capi.FIELD_V)
    assert np.abs(u - uo).max() <= FP_RTOL * np.abs(uo).max()
    assert np.abs(v - vo).max() <= FP_RTOL * max(np.abs(vo).max(), 1.0)
    assert np.abs(s.get(capi.FIELD_VF).ravel() - vfo).max() <= 1e-12


def test_ppe_reference_matches_golden_and_oracle(golden, golden_dir, oracle):
    s, xf, yf = _solver(golden_dir)
    it = s.ppe_reference()
    p = s.get(capi.FIELD_P)
    assert np.abs(p - golden["p"]).max() <= PRINT_TOL
    po, ito = oracle.ref_ppe(xf, yf)
    assert abs(it - ito) <= 2
    assert np.abs(p - po).max() <= 1e-9


def test_write_results_file_surface(golden, golden_dir, tmp_path):
    s, _, _ = _solver(golden_dir, 20)
    s.write_results(str(tmp_path))
    for name, key in (("uc.dat", "uc"), ("vc.dat", "vc"), ("final_results.dat", "final_results")):
        lines = (tmp_path / name).read_text().splitlines()
        assert lines[2] == 'ZONE T="BIG ZONE", I=52, J=52, DATAPACKING=POINT'
        vals = np.array([[float(t) for t in l.split(",")] for l in lines[3:]])
        assert np.abs(vals[:, 2].reshape(52, 52) - golden[key]).max() <= 2 * PRINT_TOL


def test_interface_mirror_runs_reference_main(golden, golden_dir, tmp_path):
    f = ifx.ImmerseFlow(results_dir=str(tmp_path))
    f.readInputFile(os.path.join(golden_dir, "inputs", "inputs.txt"))
    f.CUDAQuery()
    f.allocation()
    f.readGridData()
    f.initializeData()
    for _ in range(20):
        f.ADsolver()
    f.freeAllocation()
    lines = (tmp_path / "uc.dat").read_text().splitlines()[3:]
    u = np.array([float(l.split(",")[2]) for l in lines]).reshape(52, 52)
    assert np.abs(u - golden["uc"]).max() <= 2 * PRINT_TOL


@pytest.mark.parametrize("method,w", [(capi.PPE_POINT_GS, 1.0), (capi.PPE_POINT_GS, 1.8), (capi.PPE_LINE_SOR, 1.0),
                                      (capi.PPE_LINE_SOR, 1.6)])
def test_ppe_solver_options_vs_oracle(golden_dir, oracle, method, w):
    """PPE_Solver 1 (point GS) and 2 (line SOR) of inputs/inputs.txt:14, with
    w-PPE relaxation: a fixed number of iterations agrees with the oracle to
    1e-12, and the solve under the reference's stop rule to 1e-9 with the same
    iteration count (within 2: the signed residual sum is compared to 1e-6)."""
    c = ifx.config_read(os.path.join(golden_dir, "inputs", "inputs.txt"))
    c.ppe_method, c.relax_ppe = method, w
    xf = ifx.grid_read(c.xgrid.decode(), c.nx + 1)
    yf = ifx.grid_read(c.ygrid.decode(), c.ny + 1)
    c.ppe_itermax = 40
    s = ifx.Solver.create(c, xf, yf)
    assert s.ppe_reference() == 40
    po, ito = oracle.ref_ppe(xf, yf, itermax=40, method=method, w=w)
    assert ito == 40
    assert np.abs(s.get(capi.FIELD_P) - po).max() <= FP_RTOL * 100.0
    c.ppe_itermax = 100000
    s = ifx.Solver.create(c, xf, yf)
    it = s.ppe_reference()
    po, ito = oracle.ref_ppe(xf, yf, method=method, w=w)
    assert abs(it - ito) <= 2 and it < 14000
    assert np.abs(s.get(capi.FIELD_P) - po).max() <= 1e-9


def test_ad_relaxation_vs_oracle(golden_dir, oracle):
    """w-AD under-relaxation (the reference's commented-out src/include/ADSolver.cu:95,116)."""
    c = ifx.config_read(os.path.join(golden_dir, "inputs", "inputs.txt"))
    c.relax_ad = 0.8
    xf = ifx.grid_read(c.xgrid.decode(), c.nx + 1)
    yf = ifx.grid_read(c.ygrid.decode(), c.ny + 1)
    s = ifx.Solver.create(c, xf, yf)
    s.step(5)
    uo, vo, iters, _, _ = oracle.ref_ad(xf, yf, 1e-3, 150.0, 25, 5, w_ad=0.8)
    assert np.abs(s.get(capi.FIELD_U) - uo).max() <= FP_RTOL * np.abs(uo).max()
    assert np.abs(s.get(capi.FIELD_V) - vo).max() <= FP_RTOL * max(np.abs(vo).max(), 1.0)
    assert s.stats().ad_iters_total == int(iters.sum())


def test_method_mode_rejects_reference_ppe_options():
    from immerseflow_gb300 import cases

    cfg, xf, yf = cases.cavity(n=32)
    cfg.ppe_method = capi.PPE_LINE_SOR
    with pytest.raises(ifx.IFXError) as e:
        ifx.Solver.create(cfg, xf, yf)
    assert e.value.status == capi.IFX_ERR_ARG
