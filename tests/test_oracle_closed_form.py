"""The oracle's ghost-cell immersed boundary against closed-form solutions
(the cases of tests/_closed_form.py), under grid refinement 64^2, 128^2, 256^2.

  - Neumann pressure, phi''(R) = 0 (quintic): max |dt p - phi| on fluid cells
    falls at second order (observed order >= 1.9 per halving).
  - Neumann pressure, phi''(R) != 0 (wendland): first order (0.85..1.2), with a
    net body flux of order h (the outflow flux halves with h): the bilinear
    image point's O(h^2) error, divided by the face distance.
  - No-slip velocity ghosts: the ghost values continue the exact swirl into the
    body at second order (>= 1.9), and the fluid velocity after the projection
    stays within O(h^2) of it (>= 1.7).
"""
import numpy as np
import pytest

import _closed_form as cf

SIZES = (64, 128, 256)


def _orders(errs):
    return [np.log2(a / b) for a, b in zip(errs, errs[1:])]


@pytest.fixture(scope="module")
def runs(oracle):
    out = {}
    for kind in ("quintic", "wendland", "swirl"):
        out[kind] = [cf.run(oracle.method(*cf.config(n), nthreads=8), kind) for n in SIZES]
    return out


def test_neumann_pressure_second_order_when_wall_curvature_vanishes(runs):
    errs = [cf.pressure_error(r) for r in runs["quintic"]]
    assert all(o >= 1.9 for o in _orders(errs)), errs
    assert errs[-1] <= 2e-3, errs
    for r in runs["quintic"]:
        assert r[-1].last_ppe_iters < 20


def test_neumann_pressure_first_order_body_flux(runs):
    errs = [cf.pressure_error(r) for r in runs["wendland"]]
    assert all(0.85 <= o <= 1.2 for o in _orders(errs)), errs
    flux = [abs(r[-1].mass_flux_out) for r in runs["wendland"]]
    assert all(1.7 <= a / b <= 2.3 for a, b in zip(flux, flux[1:])), flux


def test_noslip_velocity_ghosts_second_order(runs):
    eg = [cf.ghost_error(r) for r in runs["swirl"]]
    ef = [cf.fluid_velocity_error(r) for r in runs["swirl"]]
    assert all(o >= 1.9 for o in _orders(eg)), eg
    assert all(o >= 1.7 for o in _orders(ef)), ef
