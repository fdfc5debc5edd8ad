"""Closed-form (manufactured) solutions for the ghost-cell immersed boundary.

A cylinder of radius R = 0.5 sits near the middle of a 4 x 4 box (walls at rest,
outflow on the east side: Dirichlet p = 0 there fixes the pressure constant).
A step with dt = 1e-8 and Re = 1e8 is, up to O(dt), one discrete projection of
the initial velocity: the predictor changes nothing, and dt * p solves
L (dt p) = div u with the ghost-cell closures.

  potential:  u = grad phi, phi = g(s), s = (r - R) / (R_out - R) on [0, 1],
              g(1) = g'(1) = g''(1) = 0 and g'(0) = 0 (zero normal derivative at
              the body), phi = 0 beyond R_out.  Then dt * p = phi exactly in
              the continuum, and the projected velocity is zero.
                wendland  g = (1-s)^4 (1+4s):           g''(0) = -20
                quintic   g = 1 - 10 s^3 + 15 s^4 - 6 s^5: g''(0) = 0
  swirl:      u = (d psi/dy, -d psi/dx) with psi = g_wendland(s): a
              divergence-free swirl that vanishes on the body (psi'(R) = 0),
              exactly what the no-slip velocity ghosts must continue into the
              body; the polynomial continued to s < 0 gives the exact ghost
              values.

The pressure's image-point closure is exact for a pressure that is even about
the wall, but the bilinear interpolation at the image point errs by
O(h^2 p''), with one sign all round the body when p'' does not change sign
there.  Divided by the face distance that is an O(h) flux error per face, a
net body flux of O(h): the pressure converges at first order when phi''(R) != 0
(wendland) and at second order when phi''(R) = 0 (quintic).
"""
import numpy as np

from immerseflow_gb300 import _capi as capi
from immerseflow_gb300 import cases

L_BOX = 4.0
R = 0.5
R_OUT = 1.6
CX = CY = 2.0 + 0.013  # off the cell faces of every grid used


def g_and_dg(kind, r, clip=True):
    """g(s(r)) and d g / d r for the profiles above."""
    s = (r - R) / (R_OUT - R)
    if clip:
        s = np.clip(s, None, 1.0)
        s = np.where(s < 0, 0.0, s) if kind != "swirl" else s
    if kind in ("wendland", "swirl"):
        g = (1 - s) ** 4 * (1 + 4 * s)
        dg = -20 * s * (1 - s) ** 3
    else:
        g = 1 - 10 * s ** 3 + 15 * s ** 4 - 6 * s ** 5
        dg = -30 * s ** 2 * (1 - s) ** 2
    return g, dg / (R_OUT - R)


def config(n, precision=capi.PREC_FP64):
    c = capi.default_config()
    c.mode = capi.MODE_METHOD
    c.precision = precision
    c.nx = c.ny = n
    c.lx = c.ly = L_BOX
    c.re = 1e8
    c.dt = 1e-8
    c.init = capi.INIT_REST
    c.ad_itermax = 100
    c.ppe_itermax = 200
    c.ad_tol = 1e-14
    c.ppe_tol = 1e-10
    for s in range(4):
        c.bc_type[s] = capi.BC_WALL
        c.bc_u[s] = 0.0
        c.bc_v[s] = 0.0
    c.bc_type[capi.SIDE_E] = capi.BC_OUTFLOW
    c.outflow_uc = 1.0
    c.body = capi.BODY_ELLIPSE
    c.body_cx, c.body_cy = CX, CY
    c.body_a = c.body_b = R
    c.body_angle_deg = 0.0
    c.force_ref_u = 1.0
    c.force_ref_len = 2 * R
    xf = cases.uniform_faces(n, L_BOX)
    return c, xf, xf.copy()


def initial_field(kind, xc, yc):
    """(u, v, phi or None) at the cell centres (every cell; callers mask)."""
    X, Y = np.meshgrid(xc, yc)
    r = np.hypot(X - CX, Y - CY)
    rr = np.maximum(r, 1e-300)
    if kind == "swirl":
        # psi continued into the body (s < 0) by its polynomial: the exact ghost values
        s = (r - R) / (R_OUT - R)
        dpsi = np.where(s >= 1, 0.0, -20 * s * (1 - s) ** 3 / (R_OUT - R))
        return dpsi * (Y - CY) / rr, -dpsi * (X - CX) / rr, None
    g, dg = g_and_dg(kind, r)
    return dg * (X - CX) / rr, dg * (Y - CY) / rr, g


def run(solver, kind):
    """One projection step of a solver (GPU handle or oracle) from the
    manufactured field; returns (fluid mask, ghost mask, u, v, u_exact,
    v_exact, dt*p, phi, stats)."""
    xc, yc = solver.get(capi.FIELD_XC), solver.get(capi.FIELD_YC)
    ct = solver.get(capi.FIELD_CELLTYPE)
    fl, gh = ct == 1, ct == 2
    ue, ve, phi = initial_field(kind, xc, yc)
    solver.set(capi.FIELD_U, np.where(fl, ue, 0.0))
    solver.set(capi.FIELD_V, np.where(fl, ve, 0.0))
    solver.step(1)
    st = solver.stats()
    dt = 1e-8
    return (fl, gh, solver.get(capi.FIELD_U), solver.get(capi.FIELD_V), ue, ve, solver.get(capi.FIELD_P) * dt, phi,
            st)


def pressure_error(res):
    fl, _, _, _, _, _, p, phi, _ = res
    return float(np.abs(p - phi)[fl].max())


def ghost_error(res):
    _, gh, u, v, ue, ve, _, _, _ = res
    return float(max(np.abs(u - ue)[gh].max(), np.abs(v - ve)[gh].max()))


def fluid_velocity_error(res):
    fl, _, u, v, ue, ve, _, _, _ = res
    return float(max(np.abs(u - ue)[fl].max(), np.abs(v - ve)[fl].max()))
