"""The pressure solvers inputs/inputs.txt:14 advertises (PPE_Solver 1 point GS,
2 line SOR; parsed at src/main.cu:42, not implemented by the reference) and the
under-relaxation it comments out (src/include/ADSolver.cu:95,116), as restated
in the CPU oracle.

Pins, none of which needs a GPU:
  - the oracle's red-black Gauss-Seidel and zebra line SOR equal, bit for bit,
    an independent restatement here (numpy by colour; a plain Thomas loop per
    row) for a few iterations on a stretched grid;
  - run long enough, Jacobi, point GS and line SOR reach the same discrete
    solution as a direct sparse solve of the PPESolver system (p = 100 on the
    i = 0 and j = 0 ghosts, 0 on the others);
  - under the reference's stop rule (signed residual sum), Gauss-Seidel needs
    fewer iterations than Jacobi, line SOR fewer than point GS, and SOR with
    w = 1.8 fewer than w = 1;
  - w-AD = 1 leaves the AD step unchanged (golden uc.dat still reproduced).
"""
import os

import numpy as np
import pytest

from immerseflow_gb300 import grid_read


def coeffs(oracle, xf, yf):
    nx, ny = len(xf) + 1, len(yf) + 1
    _, _, dx, dy = oracle.grid(nx, ny, xf, yf)
    dx, dy = dx.reshape(ny, nx), dy.reshape(ny, nx)
    shp = (ny, nx)
    aP, aE, aW, aN, aS = (np.ones(shp) for _ in range(5))
    d, e = dx[1:-1, 1:-1], dy[1:-1, 1:-1]
    dE, dW = dx[1:-1, 2:], dx[1:-1, :-2]
    dN, dS = dy[2:, 1:-1], dy[:-2, 1:-1]
    aW[1:-1, 1:-1] = 2 / (d * (d + dW))
    aE[1:-1, 1:-1] = 2 / (d * (d + dE))
    aS[1:-1, 1:-1] = 2 / (e * (e + dS))
    aN[1:-1, 1:-1] = 2 / (e * (e + dN))
    aP[1:-1, 1:-1] = -1 * (((2 / (d * (d + dE))) + (2 / (d * (d + dW)))) + ((2 / (e * (e + dN))) + (2 / (e * (e + dS)))))
    return aP, aE, aW, aN, aS


def start(ny, nx):
    p = np.zeros((ny, nx))
    p[:, 0] = 100.0
    p[0, :] = 100.0
    return p


def rbgs_iter(p, a, w):
    aP, aE, aW, aN, aS = a
    ny, nx = p.shape
    jj, ii = np.mgrid[0:ny, 0:nx]
    for colour in (0, 1):
        m = ((ii + jj) % 2 == colour)
        m[0, :] = m[-1, :] = False
        m[:, 0] = m[:, -1] = False
        E, W = np.roll(p, -1, 1), np.roll(p, 1, 1)
        N, S = np.roll(p, -1, 0), np.roll(p, 1, 0)
        g = -(E * aE + W * aW + N * aN + S * aS) / aP
        p[m] = g[m] if w == 1.0 else ((1.0 - w) * p + w * g)[m]


def line_iter(p, a, w):
    aP, aE, aW, aN, aS = a
    ny, nx = p.shape
    last = nx - 2
    for first in (1, 2):
        for j in range(first, ny - 1, 2):
            cp, dp = [0.0] * nx, [0.0] * nx
            for i in range(1, last + 1):
                rhs = -(aN[j, i] * p[j + 1, i] + aS[j, i] * p[j - 1, i])
                if i == 1:
                    rhs -= aW[j, i] * p[j, 0]
                if i == last:
                    rhs -= aE[j, i] * p[j, nx - 1]
                m = aP[j, i] if i == 1 else aP[j, i] - aW[j, i] * cp[i - 1]
                cp[i] = 0.0 if i == last else aE[j, i] / m
                dp[i] = rhs / m if i == 1 else (rhs - aW[j, i] * dp[i - 1]) / m
            x = 0.0
            for i in range(last, 0, -1):
                x = dp[i] if i == last else dp[i] - cp[i] * x
                p[j, i] = x if w == 1.0 else (1.0 - w) * p[j, i] + w * x


def stretched(n, length, ratio):
    d = np.geomspace(1.0, ratio, n)
    return np.concatenate([[0.0], np.cumsum(d / d.sum() * length)])


@pytest.mark.parametrize("method,w", [(1, 1.0), (1, 1.6), (2, 1.0), (2, 1.3)])
def test_oracle_iterations_equal_independent_restatement(oracle, method, w):
    xf, yf = stretched(17, 1.0, 3.0), stretched(13, 0.7, 0.5)
    nx, ny = len(xf) + 1, len(yf) + 1
    a = coeffs(oracle, xf, yf)
    for k in (1, 2, 5):
        po, it = oracle.ref_ppe(xf, yf, itermax=k, tol=-np.inf, method=method, w=w)
        assert it == k
        p = start(ny, nx)
        for _ in range(k):
            (rbgs_iter if method == 1 else line_iter)(p, a, w)
        assert np.array_equal(po, p), (method, w, k, np.abs(po - p).max())


def test_all_methods_reach_the_direct_solution(oracle):
    sp = pytest.importorskip("scipy.sparse")
    spl = pytest.importorskip("scipy.sparse.linalg")
    xf, yf = stretched(24, 1.0, 2.0), stretched(20, 1.0, 1.0)
    nx, ny = len(xf) + 1, len(yf) + 1
    aP, aE, aW, aN, aS = coeffs(oracle, xf, yf)
    p0 = start(ny, nx)
    idx = -np.ones((ny, nx), int)
    idx[1:-1, 1:-1] = np.arange((nx - 2) * (ny - 2)).reshape(ny - 2, nx - 2)
    rows, cols, vals, rhs = [], [], [], np.zeros((nx - 2) * (ny - 2))
    for j in range(1, ny - 1):
        for i in range(1, nx - 1):
            r = idx[j, i]
            rows.append(r), cols.append(r), vals.append(aP[j, i])
            for (jj, ii, c) in ((j, i + 1, aE[j, i]), (j, i - 1, aW[j, i]), (j + 1, i, aN[j, i]), (j - 1, i, aS[j, i])):
                if idx[jj, ii] >= 0:
                    rows.append(r), cols.append(idx[jj, ii]), vals.append(c)
                else:
                    rhs[r] -= c * p0[jj, ii]
    A = sp.csr_matrix((vals, (rows, cols)))
    x = spl.spsolve(A, rhs)
    for method, iters in ((0, 20000), (1, 6000), (2, 3000)):
        po, _ = oracle.ref_ppe(xf, yf, itermax=iters, tol=-np.inf, method=method)
        assert np.abs(po[1:-1, 1:-1].ravel() - x).max() <= 1e-8 * 100, method


def test_iteration_counts_under_the_reference_stop_rule(oracle, golden_dir):
    d = os.path.join(golden_dir, "inputs")
    xf, yf = grid_read(os.path.join(d, "xgrid.dat2"), 51), grid_read(os.path.join(d, "ygrid.dat2"), 51)
    _, jac = oracle.ref_ppe(xf, yf)
    _, gs = oracle.ref_ppe(xf, yf, method=1)
    _, sor = oracle.ref_ppe(xf, yf, method=1, w=1.8)
    _, line = oracle.ref_ppe(xf, yf, method=2)
    _, lsor = oracle.ref_ppe(xf, yf, method=2, w=1.6)
    assert jac > 14000  # the Jacobi solve of p.dat takes about 1.5e4 sweeps
    assert sor < gs < jac
    assert line < gs and lsor < line


def test_unit_ad_relaxation_is_identity(oracle, golden, golden_dir):
    d = os.path.join(golden_dir, "inputs")
    xf, yf = grid_read(os.path.join(d, "xgrid.dat2"), 51), grid_read(os.path.join(d, "ygrid.dat2"), 51)
    u1, v1, _, _, _ = oracle.ref_ad(xf, yf, 1e-3, 150.0, 25, 20)
    u8, v8, it8, _, _ = oracle.ref_ad(xf, yf, 1e-3, 150.0, 25, 20, w_ad=0.8)
    assert np.abs(u1 - golden["uc"]).max() <= 5e-7 + 1e-12
    assert not np.array_equal(u1, u8) and np.all(np.isfinite(u8))
