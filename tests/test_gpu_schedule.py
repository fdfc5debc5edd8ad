"""Sweep schedules of the pressure solve on the GPU.

  - a non-default schedule set through ifx_set_schedule gives the oracle's
    fields for the same schedule (FP64, 1e-10 of the field maximum; pressure
    iterations within one);
  - the schedule autotuner leaves the state as it found it, keeps a schedule
    under which every pressure solve meets ppe_tol, and the run with the tuned
    schedule stays within the mixed-precision bounds of a plain FP64 run with
    the default schedule (relative L2 velocity <= 1e-6, drag <= 1e-3): tuning
    never moves a result beyond the solve's own tolerance.
"""
import numpy as np
import pytest

import immerseflow_gb300 as ifx
from immerseflow_gb300 import _capi as capi
from immerseflow_gb300 import cases

pytestmark = pytest.mark.gpu


def cyl(prec=capi.PREC_FP64, nx=96, ny=64):
    return cases.external(nx, ny, 12.0, 8.0, 4.0, 4.0, 0.5, 0.35, 12.0, 150.0, 1e-2, prec, ratio=4.0, width=1.0)


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("mode", [ifx.EXEC_PERSISTENT, ifx.EXEC_GRAPH])
def test_set_schedule_matches_oracle(oracle, mode):
    cfg, xf, yf = cyl()
    s = ifx.Solver.create(cfg, xf, yf)
    s.set_exec_mode(mode)
    sc = s.schedule()
    assert (sc.mg_pre, sc.mg_post, sc.coarse_sweeps, sc.mixed_inner) == (2, 2, 40, 8)
    sc.mg_pre, sc.mg_post, sc.mg_omega, sc.coarse_sweeps = 1, 3, 0.7, 12
    s.set_schedule(sc)
    got = s.schedule()
    assert (got.mg_pre, got.mg_post, got.mg_omega, got.coarse_sweeps) == (1, 3, 0.7, 12)
    ocfg = capi.Config.from_buffer_copy(cfg)
    ocfg.mg_pre, ocfg.mg_post, ocfg.mg_omega, ocfg.coarse_sweeps = 1, 3, 0.7, 12
    o = oracle.method(ocfg, xf, yf)
    for _ in range(3):
        s.step(1)
        o.step(1)
        assert abs(s.stats().last_ppe_iters - o.stats().last_ppe_iters) <= 1
    for f in (capi.FIELD_U, capi.FIELD_V, capi.FIELD_P):
        assert rel(s.get(f), o.get(f)) <= 1e-10, f


def test_invalid_schedule_refused():
    s = ifx.Solver.create(*cyl())
    sc = s.schedule()
    sc.mg_omega = 2.5
    with pytest.raises(ifx.IFXError) as e:
        s.set_schedule(sc)
    assert e.value.status == capi.IFX_ERR_ARG


@pytest.mark.parametrize("prec", [capi.PREC_FP64, capi.PREC_MIXED])
def test_autotuned_schedule_keeps_state_and_tolerance(prec):
    cfg, xf, yf = cyl(prec, 192, 128)
    s = ifx.Solver.create(cfg, xf, yf)
    s.step(2)
    before = {f: s.get(f) for f in (capi.FIELD_U, capi.FIELD_V, capi.FIELD_P)}
    s.autotune(steps=1)
    sched, ms = s.autotune_schedule(steps=2)
    assert ms > 0 and s.stats().steps == 2
    for f, a in before.items():
        assert np.array_equal(s.get(f), a), f
    assert s.schedule().as_dict() == sched.as_dict()
    ref_cfg, _, _ = cyl(capi.PREC_FP64, 192, 128)
    ref = ifx.Solver.create(ref_cfg, xf, yf)
    ref.step(2)
    for _ in range(8):
        s.step(1)
        ref.step(1)
        assert s.stats().last_ppe_residual <= cfg.ppe_tol
        assert s.stats().status == capi.IFX_OK
    a = np.concatenate([s.get(capi.FIELD_U).ravel(), s.get(capi.FIELD_V).ravel()])
    b = np.concatenate([ref.get(capi.FIELD_U).ravel(), ref.get(capi.FIELD_V).ravel()])
    assert np.linalg.norm(a - b) / np.linalg.norm(b) <= 1e-6
    assert abs(s.stats().cd - ref.stats().cd) <= 1e-3 * abs(ref.stats().cd)


def test_autotuned_schedule_of_a_batch():
    specs = cases.batch_sample(4, seed=3, precision=capi.PREC_MIXED)
    s = ifx.Solver.batch([c for c, _, _ in specs], [x for _, x, _ in specs], [y for _, _, y in specs])
    s.step(1)
    sched, _ = s.autotune_schedule(steps=1)
    for k in range(4):
        assert s.schedule(k).as_dict() == sched.as_dict()
    s.step(3)
    for k in range(4):
        assert s.stats(k).status == capi.IFX_OK and s.stats(k).last_ppe_residual <= specs[k][0].ppe_tol
