"""Pin the CPU oracle against the reference's own result files.

results/uc.dat, results/vc.dat: ADsolver after 20 steps on the 52x52 grid of
inputs/xgrid.dat2, ygrid.dat2 (vortex IC, Re=150, dt=1e-3, AD_itermax=25).
results/p.dat: the Jacobi Laplace solve PPESolver intends (p=100 on the W/S
ghosts).  The files are printed with %f, so agreement is to 5e-7.
"""
import os

import numpy as np

from immerseflow_gb300 import grid_read

PRINT_TOL = 5.0e-7 + 1e-12


def _grids(golden_dir):
    d = os.path.join(golden_dir, "inputs")
    return grid_read(os.path.join(d, "xgrid.dat2"), 51), grid_read(os.path.join(d, "ygrid.dat2"), 51)


def test_grid_centres_match_golden(oracle, golden, golden_dir):
    xf, yf = _grids(golden_dir)
    xc, yc, dx, dy = oracle.grid(52, 52, xf, yf)
    assert np.abs(xc - golden["x"]).max() <= PRINT_TOL
    assert np.abs(yc - golden["y"]).max() <= PRINT_TOL
    assert np.allclose(dx, 0.02) and np.allclose(dy, 0.02)


def test_reference_ad_matches_uc_vc(oracle, golden, golden_dir):
    xf, yf = _grids(golden_dir)
    u, v, iters, _, vf = oracle.ref_ad(xf, yf, dt=1e-3, re=150.0, itermax=25, nsteps=20)
    assert np.abs(u - golden["uc"]).max() <= PRINT_TOL
    assert np.abs(v - golden["vc"]).max() <= PRINT_TOL
    assert list(iters) == [5] * 20
    # the reference never computes vf on square grids (src/include/ADSolver.cu:179)
    assert np.all(vf == 0.0)


def test_golden_pins_reynolds_number(oracle, golden, golden_dir):
    xf, yf = _grids(golden_dir)
    u, _, _, _, _ = oracle.ref_ad(xf, yf, dt=1e-3, re=100.0, itermax=25, nsteps=20)
    assert np.abs(u - golden["uc"]).max() > 1e-4


def test_reference_ppe_matches_p(oracle, golden, golden_dir):
    xf, yf = _grids(golden_dir)
    p, it = oracle.ref_ppe(xf, yf)
    assert np.abs(p - golden["p"]).max() <= PRINT_TOL
    # the %f fixture pins the converged field, not the exact count (~1.48e4)
    assert 14000 < it < 15500


def test_iblank_golden_is_all_fluid(golden):
    assert np.all(golden["final_results"] == 1.0)
