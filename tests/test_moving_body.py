"""Prescribed body motion on the CPU: the oracle's pose arithmetic, its
per-step geometry, and the configuration checks of the library."""
import numpy as np
import pytest

import immerseflow_gb300 as ifx
from immerseflow_gb300 import _capi as capi
from immerseflow_gb300 import cases


def small(prec=capi.PREC_FP64, b=0.5, angle=0.0):
    return cases.external(96, 64, 12.0, 8.0, 4.0, 4.0, 0.5, b, angle, 100.0, 1e-2, prec, ratio=4.0, width=1.0)


def test_sincos_turns_accuracy(oracle):
    """Against 40-digit sin and cos of 2 pi x: within 6e-16 (a few units in
    the last place; the reduction to [0, 1/8] turn is exact)."""
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.dps = 40
    rng = np.random.default_rng(0)
    xs = np.concatenate([rng.uniform(-3.0, 3.0, 400), np.arange(-16, 17) / 8.0, [0.0, 1e-12, 0.5 - 1e-15, 0.1249999]])
    for x in xs:
        s, c = oracle.sincos_turns(x)
        a = 2 * mpmath.pi * mpmath.mpf(float(x))
        assert abs(s - float(mpmath.sin(a))) <= 6e-16 and abs(c - float(mpmath.cos(a))) <= 6e-16, x
    # exact at the quarter turns
    assert oracle.sincos_turns(0.0) == (0.0, 1.0)
    assert oracle.sincos_turns(0.25) == (1.0, 0.0)


def test_zero_motion_equals_static(oracle):
    """A body 'moving' with zero velocity and amplitude is rebuilt every step
    with the same geometry: the same results bit for bit."""
    cfg, xf, yf = small()
    a = oracle.method(cfg, xf, yf)
    cfgm, _, _ = small()
    cases.set_motion(cfgm, freq=0.7, phase_y=30.0)
    b = oracle.method(cfgm, xf, yf)
    a.step(3)
    b.step(3)
    for f in (capi.FIELD_U, capi.FIELD_V, capi.FIELD_P, capi.FIELD_IBLANK):
        assert np.array_equal(a.get(f), b.get(f)), f
    assert a.stats().cd == b.stats().cd


def test_heaving_cylinder_geometry_follows_the_pose(oracle):
    cfg, xf, yf = small()
    cases.set_motion(cfg, amp_y=0.3, freq=1.0)
    o = oracle.method(cfg, xf, yf)
    ib0 = o.get(capi.FIELD_IBLANK).copy()
    n = 10
    o.step(n)
    t = n * cfg.dt
    x, y, c, s, u, v, w = o.body()
    assert x == cfg.body_cx and abs(y - (cfg.body_cy + 0.3 * np.sin(2 * np.pi * t))) < 1e-14
    assert abs(v - 0.3 * 2 * np.pi * np.cos(2 * np.pi * t)) < 1e-13 and u == 0.0 and w == 0.0
    ib = o.get(capi.FIELD_IBLANK)
    assert (ib != ib0).sum() > 20  # cells covered and uncovered
    # the tagging is the body predicate at the new pose
    xc, yc = o.get(capi.FIELD_XC), o.get(capi.FIELD_YC)
    X, Y = np.meshgrid(xc, yc)
    inside = ((X - x) ** 2 + (Y - y) ** 2) / 0.25 < 1.0
    assert np.array_equal(ib.reshape(inside.shape)[1:-1, 1:-1] == 0.0, inside[1:-1, 1:-1])
    st = o.stats()
    # projection to the pressure tolerance (relative 1e-8 of a right-hand side
    # that now carries the wall's motion)
    assert np.isfinite(st.cd) and np.isfinite(st.cl) and st.max_div < 1e-6
    assert all(np.isfinite(o.get(f)).all() for f in (capi.FIELD_U, capi.FIELD_V, capi.FIELD_P))


def test_pitching_ellipse_moves_its_ghosts(oracle):
    cfg, xf, yf = small(b=0.2, angle=10.0)
    cases.set_motion(cfg, amp_deg=25.0, freq=1.5)
    o = oracle.method(cfg, xf, yf)
    c0 = set(o.ghosts()[0].tolist())
    o.step(6)
    x, y, c, s, u, v, w = o.body()
    t = 6 * cfg.dt
    th = np.deg2rad(10.0 + 25.0 * np.sin(2 * np.pi * 1.5 * t))
    assert abs(c - np.cos(th)) < 1e-14 and abs(s - np.sin(th)) < 1e-14
    assert abs(w - np.deg2rad(25.0) * 2 * np.pi * 1.5 * np.cos(2 * np.pi * 1.5 * t)) < 1e-12
    c1 = set(o.ghosts()[0].tolist())
    assert c0 != c1
    assert o.stats().max_div < 1e-6


def test_motion_configuration_checks():
    srv = ifx.Server(1 << 30, max_cohort=4)
    cfg, xf, yf = small()
    cases.set_motion(cfg, amp_y=0.2, freq=1.0)
    cfg.bc_type[capi.SIDE_E] = capi.BC_WALL  # closed domain: refused
    with pytest.raises(ifx.IFXError) as e:
        srv.submit(cfg, xf, yf, 2)
    assert e.value.status == capi.IFX_ERR_ARG
    cfg, xf, yf = small()
    cases.set_motion(cfg, amp_y=float("nan"), freq=1.0)
    with pytest.raises(ifx.IFXError):
        srv.submit(cfg, xf, yf, 2)
    cfg, xf, yf = small()
    cfg.body = capi.BODY_NONE
    cases.set_motion(cfg, amp_y=0.2, freq=1.0)
    with pytest.raises(ifx.IFXError):
        srv.submit(cfg, xf, yf, 2)
    srv.close()
