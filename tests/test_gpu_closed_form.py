"""The GPU's ghost-cell immersed boundary against the closed-form solutions of
tests/_closed_form.py, under grid refinement 64^2, 128^2, 256^2, in plain FP64
and in mixed precision; the same convergence orders as the oracle tests
(second order for the no-slip ghosts and for a Neumann pressure whose wall
curvature vanishes, first order with an O(h) body flux otherwise).  The FP64
fields also equal the oracle's on the same grids to 1e-9 of their maximum,
the mixed ones to 1e-6."""
import numpy as np
import pytest

import _closed_form as cf
import immerseflow_gb300 as ifx
from immerseflow_gb300 import _capi as capi

pytestmark = pytest.mark.gpu
SIZES = (64, 128, 256)


def _orders(errs):
    return [np.log2(a / b) for a, b in zip(errs, errs[1:])]


def _rel(a, b, mask):
    return float(np.abs(a - b)[mask].max() / max(np.abs(b)[mask].max(), 1e-300))


@pytest.mark.parametrize("prec", [capi.PREC_FP64, capi.PREC_MIXED])
def test_closed_form_orders_and_oracle(oracle, prec):
    tol = 1e-9 if prec == capi.PREC_FP64 else 1e-6
    err = {k: [] for k in ("quintic", "wendland", "swirl")}
    flux = []
    for kind in err:
        for n in SIZES:
            c, xf, yf = cf.config(n, prec)
            g = cf.run(ifx.Solver.create(c, xf, yf), kind)
            o = cf.run(oracle.method(*cf.config(n), nthreads=8), kind)
            fl = g[0]
            assert _rel(g[2], o[2], fl) <= tol and _rel(g[3], o[3], fl) <= tol, (kind, n)
            if kind == "swirl":
                err[kind].append(cf.ghost_error(g))
            else:
                assert _rel(g[6], o[6], fl) <= tol, (kind, n)
                err[kind].append(cf.pressure_error(g))
                if kind == "wendland":
                    flux.append(abs(g[-1].mass_flux_out))
    assert all(o >= 1.9 for o in _orders(err["quintic"])), err["quintic"]
    assert all(0.85 <= o <= 1.2 for o in _orders(err["wendland"])), err["wendland"]
    assert all(1.7 <= a / b <= 2.3 for a, b in zip(flux, flux[1:])), flux
    assert all(o >= 1.9 for o in _orders(err["swirl"])), err["swirl"]
