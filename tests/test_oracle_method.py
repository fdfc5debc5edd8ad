"""Method-level properties of the oracle's METHOD part (projection, ghost-cell
IBM, multigrid-preconditioned pressure solve), which has no reference
implementation to pin it: mirror symmetry of a symmetric flow, a
divergence-free projection, and second-order convergence under refinement."""
import numpy as np

from immerseflow_gb300 import _capi as capi
from immerseflow_gb300 import cases


def test_symmetric_cylinder_flow(oracle):
    """A circle on the centreline of a grid stretched symmetrically about it,
    uniform inflow: u and p stay mirror-symmetric and v antisymmetric to
    round-off, and the lift vanishes (the force samples and their probe
    distances are mirror-invariant)."""
    cfg, xf, yf = cases.external(96, 64, 12.0, 8.0, 4.0, 4.0, 0.5, 0.5, 0.0, 100.0, 1e-2, capi.PREC_FP64,
                                 ratio=4.0, width=1.0)
    assert np.abs((yf - 4.0) + (yf[::-1] - 4.0)).max() < 1e-12
    s = oracle.method(cfg, xf, yf)
    s.step(10)
    u, v, p = s.get(capi.FIELD_U), s.get(capi.FIELD_V), s.get(capi.FIELD_P)
    assert np.abs(u - u[::-1, :]).max() <= 1e-10 * np.abs(u).max()
    assert np.abs(v + v[::-1, :]).max() <= 1e-10 * np.abs(v).max()
    assert np.abs(p - p[::-1, :]).max() <= 1e-10 * np.abs(p).max()
    st = s.stats()
    assert st.cd > 1.0 and abs(st.cl) <= 1e-10 * st.cd
    assert st.max_div < 1e-6


def test_cavity_second_order_under_refinement(oracle):
    """Lid-driven cavity, Re 100, t = 0.5 with the same time step on 32^2,
    64^2 and 128^2 cells: u on the vertical centreline changes by about four
    times less from 64 to 128 than from 32 to 64 (3.65 measured; 4.4 from 128
    to 256)."""
    T, dt = 0.5, 2e-3
    yq = np.linspace(0.1, 0.9, 17)
    prof = {}
    for n in (32, 64, 128):
        cfg, xf, yf = cases.cavity(n=n, dt=dt)
        s = oracle.method(cfg, xf, yf, nthreads=8)
        s.step(int(round(T / dt)))
        assert s.stats().max_div < 1e-6
        u = s.get(capi.FIELD_U)
        yc = s.get(capi.FIELD_YC)
        uc = 0.5 * (u[:, n // 2] + u[:, n // 2 + 1])  # x = 0.5
        prof[n] = np.interp(yq, yc[1:-1], uc[1:-1])
    d1 = np.abs(prof[32] - prof[64]).max()
    d2 = np.abs(prof[64] - prof[128]).max()
    assert d2 < 2e-3
    assert 3.0 <= d1 / d2 <= 5.5, d1 / d2


def test_predictor_initial_guess(oracle):
    """The predictor starts from q^n plus the step before's increment q* - q^n:
    after the first steps it needs fewer Jacobi sweeps than on the first step
    (from q^n alone), and the solution is unchanged within the predictor's own
    tolerance (the stop rule is the same)."""
    cfg, xf, yf = cases.cylinder(nx=192, ny=128, precision=capi.PREC_FP64)
    s = oracle.method(cfg, xf, yf, nthreads=8)
    its = []
    for _ in range(12):
        s.step(1)
        its.append(s.stats().last_ad_iters)
    # the first step has no increment; from the fourth step on the guess is O(dt^2) away
    assert max(its[4:]) < its[0], its
    assert s.stats().max_div < 1e-6
