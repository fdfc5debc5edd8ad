"""Host-side bookkeeping of the solve server and the memory estimate (no GPU)."""
import pytest

import immerseflow_gb300 as ifx
from immerseflow_gb300 import _capi as capi
from immerseflow_gb300 import cases


def small(nx, ny, re=100.0):
    return cases.external(nx, ny, 12.0, 8.0, 4.0, 4.0, 0.5, 0.5, 0.0, re, 1e-2, capi.PREC_MIXED, ratio=4.0, width=1.0)


def test_estimate_grows_with_grid_and_precision():
    a = ifx.estimate_bytes(small(64, 48)[0])
    b = ifx.estimate_bytes(small(128, 96)[0])
    assert 2.0 < b / a < 4.5
    c64 = small(64, 48)[0]
    c64.precision = capi.PREC_FP64
    assert ifx.estimate_bytes(c64) > a
    # at least the 24 FP64 cell fields of one instance
    assert a > 24 * 8 * 66 * 50


def test_queue_bookkeeping_without_ticks():
    srv = ifx.Server(1 << 30, max_cohort=4)
    ids = [srv.submit(*small(48 + 8 * k, 32), nsteps=3) for k in range(3)]
    assert ids == sorted(ids) and len(set(ids)) == 3
    info = srv.info()
    assert info["waiting"] == 3 and info["running"] == 0 and info["cohorts"] == 0 and info["used_bytes"] == 0
    assert srv.poll() == []
    assert srv.state(ids[0])[0] == ifx.REQ_WAITING
    with pytest.raises(ifx.IFXError):
        srv.result(ids[0], capi.FIELD_U)
    with pytest.raises(ifx.IFXError):
        srv.release(ids[1])
    with pytest.raises(ifx.IFXError):
        srv.submit(*small(48, 32), nsteps=0)
    srv.close()


def test_reference_mode_case_is_refused():
    srv = ifx.Server(1 << 30)
    cfg, xf, yf = cases.cavity(n=32)
    cfg.mode = capi.MODE_REFERENCE
    with pytest.raises(ifx.IFXError):
        srv.submit(cfg, xf, yf, nsteps=2)
    srv.close()


@pytest.mark.parametrize("field,value", [("re", -1.0), ("dt", 0.0), ("mg_pre", 0), ("ppe_method", capi.PPE_LINE_SOR),
                                         ("nx", 1 << 28), ("closed_box_body", None), ("mixed_inner", 1)])
def test_invalid_request_refused_at_submit(field, value):
    """A configuration the solver would refuse is refused at submit, not when its
    cohort is created (which would fail the requests admitted with it)."""
    cfg, xf, yf = small(48, 32)
    if field == "closed_box_body":
        # a body with no outflow side: the pressure problem is refused (its
        # compatibility condition is not the area-weighted mean)
        cfg.bc_type[capi.SIDE_E] = capi.BC_WALL
    else:
        setattr(cfg, field, value)
    srv = ifx.Server(1 << 30, max_cohort=4)
    with pytest.raises(ifx.IFXError) as e:
        srv.submit(cfg, xf, yf, nsteps=3)
    assert e.value.status == capi.IFX_ERR_ARG
    assert srv.info()["waiting"] == 0
    srv.close()
