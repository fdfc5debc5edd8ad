"""Body intercepts of the oracle's ghost cells (CPU): the closest boundary point
of every ghost cell centre, checked against the geometry it must satisfy and
against a brute-force search over the ellipse.

  - the intercept BI lies on the ellipse to 5e-14 (body frame, after the
    test's own rotation of BI into it);
  - the ghost centre G lies on the normal through BI (cross product of G - BI
    with the unit normal below 1e-12 of |G - BI|);
  - no point of a dense parameter sweep of the ellipse, refined by golden-
    section search, is closer to G than BI by more than 1e-12;
  - the image point is IP = 2 BI - G.
"""
import math

import numpy as np
import pytest

from immerseflow_gb300 import _capi as capi
from immerseflow_gb300 import cases


def _closest_brute(a, b, px, py):
    """Distance from (px, py) (body frame) to the ellipse: a parameter sweep,
    then golden-section refinement around the best sample."""
    t = np.linspace(0.0, 2.0 * math.pi, 4097)
    d = np.hypot(a * np.cos(t) - px, b * np.sin(t) - py)
    k = int(np.argmin(d))
    lo, hi = t[k] - 2.0 * math.pi / 4096, t[k] + 2.0 * math.pi / 4096
    f = lambda s: math.hypot(a * math.cos(s) - px, b * math.sin(s) - py)
    r = (math.sqrt(5.0) - 1.0) / 2.0
    for _ in range(200):
        m1, m2 = hi - r * (hi - lo), lo + r * (hi - lo)
        if f(m1) < f(m2):
            hi = m2
        else:
            lo = m1
    return f(0.5 * (lo + hi))


@pytest.mark.parametrize("angle,b", [(0.0, 0.5), (17.0, 0.15), (-30.0, 0.3), (10.0, 0.1)])
def test_body_intercepts_are_closest_points(oracle, angle, b):
    cfg, xf, yf = cases.external(96, 64, 12.0, 8.0, 4.0, 4.0, 0.5, b, angle, 100.0, 1e-2, capi.PREC_FP64,
                                 ratio=4.0, width=1.0)
    o = oracle.method(cfg, xf, yf)
    cells, nb, wu, wp, bi, ip = o.ghosts()
    assert len(cells) > 0
    nx = cfg.nx + 2
    xc, yc, _, _ = oracle.grid(nx, cfg.ny + 2, xf, yf)
    th = math.radians(angle)
    cs, sn = math.cos(th), math.sin(th)
    worst_on, worst_cross, worst_dist = 0.0, 0.0, -1.0
    for k, cell in enumerate(cells):
        gx, gy = xc[cell % nx], yc[cell // nx]
        bx, by = bi[k]
        # body frame
        rx, ry = (bx - 4.0) * cs + (by - 4.0) * sn, -(bx - 4.0) * sn + (by - 4.0) * cs
        worst_on = max(worst_on, abs((rx / 0.5) ** 2 + (ry / b) ** 2 - 1.0))
        # unit normal at BI (world frame)
        nxb, nyb = rx / 0.25, ry / (b * b)
        nl = math.hypot(nxb, nyb)
        nxw, nyw = (nxb * cs - nyb * sn) / nl, (nxb * sn + nyb * cs) / nl
        dx, dy = gx - bx, gy - by
        dist = math.hypot(dx, dy)
        worst_cross = max(worst_cross, abs(dx * nyw - dy * nxw) / max(dist, 1e-300))
        gxr, gyr = (gx - 4.0) * cs + (gy - 4.0) * sn, -(gx - 4.0) * sn + (gy - 4.0) * cs
        worst_dist = max(worst_dist, dist - _closest_brute(0.5, b, gxr, gyr))
        assert ip[k][0] == 2.0 * bx - gx and ip[k][1] == 2.0 * by - gy
    assert worst_on <= 5e-14, worst_on
    assert worst_cross <= 1e-12, worst_cross
    assert worst_dist <= 1e-12, worst_dist
