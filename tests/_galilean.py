"""Galilean consistency of the moving-body path (shared by the oracle and GPU
tests): a cylinder (D = 1) towed at velocity (-1, 0) through fluid at rest
against the same cylinder fixed in a uniform stream (1, 0), on uniform grids
of a 12 x 8 domain (slip top and bottom, Dirichlet inflow on the west side,
convective outflow on the east), Re 40, dt 0.01, 40 steps from the impulsive
start.  In an unbounded domain the two are the same flow seen from two frames;
here the domain boundaries and the moving geometry (cells uncovered by the
body restart their convection history) separate them.  Drag is measured with
the velocity relative to the body in both.  The drag of the towed body
oscillates from step to step as cells are uncovered, so the time average over
steps 11..40 is compared."""
import numpy as np

from immerseflow_gb300 import _capi as capi
from immerseflow_gb300 import cases


def case(n, towed, precision=capi.PREC_FP64):
    lx, ly = 12.0, 8.0
    nx = int(n * 1.5)
    c, _, _ = cases.external(nx, n, lx, ly, 8.0, 4.0, 0.5, 0.5, 0.0, 40.0, 0.01, precision)
    xf, yf = cases.uniform_faces(nx, lx), cases.uniform_faces(n, ly)
    if towed:
        c.init = capi.INIT_REST
        c.bc_u[capi.SIDE_W] = 0.0
        cases.set_motion(c, u=-1.0)
    return c, xf, yf


def mean_drag(solver, steps=40, skip=10):
    cd = []
    for _ in range(steps):
        solver.step(1)
        cd.append(solver.stats().cd)
    return float(np.mean(cd[skip:]))
