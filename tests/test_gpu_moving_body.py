"""Prescribed body motion on the GPU: the geometry redone on the device every
step (tagging, ghosts, weights, stencil bytes of every level, force samples)
against the oracle, which rebuilds it on the whole grid."""
import numpy as np
import pytest

import immerseflow_gb300 as ifx
from immerseflow_gb300 import _capi as capi
from immerseflow_gb300 import cases

pytestmark = pytest.mark.gpu

FIELDS = (capi.FIELD_U, capi.FIELD_V, capi.FIELD_P)
FIELD_RTOL = 1e-9  # GPU vs oracle, FP64: FMA contraction and reduction order only


def small(prec=capi.PREC_FP64, b=0.5, angle=0.0, cx=4.0, dt=1e-2):
    return cases.external(96, 64, 12.0, 8.0, cx, 4.0, 0.5, b, angle, 100.0, dt, prec, ratio=4.0, width=1.0)


def heaving(prec=capi.PREC_FP64):
    cfg, xf, yf = small(prec)
    cases.set_motion(cfg, amp_y=0.3, freq=1.0)
    return cfg, xf, yf


def pitching(prec=capi.PREC_FP64):
    cfg, xf, yf = small(prec, b=0.2, angle=10.0)
    cases.set_motion(cfg, amp_x=0.2, amp_deg=25.0, freq=1.5, phase_x=90.0)
    return cfg, xf, yf


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def run(spec, nsteps, mode=ifx.EXEC_DEFAULT):
    s = ifx.Solver.create(*spec)
    if mode != ifx.EXEC_DEFAULT:
        s.set_exec_mode(mode)
    s.step(nsteps)
    return s


@pytest.mark.parametrize("mode", [ifx.EXEC_GRAPH, ifx.EXEC_HOST])
@pytest.mark.parametrize("prec", [capi.PREC_FP64, capi.PREC_MIXED])
def test_zero_motion_bit_identical_to_static(mode, prec):
    """A body 'moving' with zero velocity and amplitude has its geometry redone
    on the device every step; it must reproduce the static set-up exactly."""
    a = run(small(prec), 4, mode)
    cfg, xf, yf = small(prec)
    cases.set_motion(cfg, freq=0.7, phase_y=30.0)
    b = run((cfg, xf, yf), 4, mode)
    for f in FIELDS + (capi.FIELD_IBLANK, capi.FIELD_UF, capi.FIELD_VF):
        assert np.array_equal(a.get(f), b.get(f)), f
    sa, sb = a.stats(), b.stats()
    assert sa.cd == sb.cd and sa.cl == sb.cl
    assert sa.n_ibm_ghost == sb.n_ibm_ghost and sa.last_ppe_iters == sb.last_ppe_iters


@pytest.mark.parametrize("make", [heaving, pitching])
def test_moving_body_vs_oracle(oracle, make):
    cfg, xf, yf = make()
    s = ifx.Solver.create(cfg, xf, yf)
    o = oracle.method(cfg, xf, yf)
    ib0 = s.get(capi.FIELD_IBLANK).copy()
    for k in range(8):
        s.step(1)
        o.step(1)
        assert np.array_equal(s.get(capi.FIELD_IBLANK), o.get(capi.FIELD_IBLANK)), k
        st, so = s.stats(), o.stats()
        assert st.n_ibm_ghost == so.n_ibm_ghost, k
        assert abs(st.last_ppe_iters - so.last_ppe_iters) <= 1
        for f in FIELDS:
            assert rel(s.get(f), o.get(f)) <= FIELD_RTOL, (k, f, rel(s.get(f), o.get(f)))
        assert abs(st.cd - so.cd) <= 1e-8 * max(abs(so.cd), abs(so.cl), 1.0)
        assert abs(st.cl - so.cl) <= 1e-8 * max(abs(so.cd), abs(so.cl), 1.0)
    assert (s.get(capi.FIELD_IBLANK) != ib0).sum() > 10  # the body moved across cells
    assert s.stats().max_div < 1e-6


def test_moving_mixed_close_to_fp64():
    a = run(heaving(capi.PREC_FP64), 20)
    b = run(heaving(capi.PREC_MIXED), 20)
    for f in (capi.FIELD_U, capi.FIELD_V):
        ua, ub = a.get(f), b.get(f)
        assert np.linalg.norm(ub - ua) / np.linalg.norm(ua) <= 1e-6, f
    sa, sb = a.stats(), b.stats()
    scale = max(abs(sa.cd), abs(sa.cl))
    assert abs(sa.cd - sb.cd) <= 1e-3 * scale and abs(sa.cl - sb.cl) <= 1e-3 * scale


def test_moving_bodies_in_a_batch_equal_alone():
    specs = [heaving(), small(b=0.3, angle=-15.0), pitching()]
    bt = ifx.Solver.batch([c for c, _, _ in specs], [x for _, x, _ in specs], [y for _, _, y in specs])
    bt.step(5)
    for k, spec in enumerate(specs):
        s = run(spec, 5)
        for f in FIELDS + (capi.FIELD_IBLANK,):
            assert np.array_equal(bt.get(f, inst=k), s.get(f)), (k, f)
        assert bt.stats(k).n_ibm_ghost == s.stats().n_ibm_ghost


def test_body_leaving_the_domain_is_retired():
    """A body towed towards the outflow side: when it comes within three cells
    of the domain edge its instance is retired with IFX_ERR_GEOMETRY; the other
    instance of the batch goes on as alone."""
    towed = small(cx=8.5, dt=4e-3)
    cases.set_motion(towed[0], u=5.0)
    other = small(b=0.3)
    specs = [towed, other]
    bt = ifx.Solver.batch([c for c, _, _ in specs], [x for _, x, _ in specs], [y for _, _, y in specs])
    failed_at = None
    for k in range(200):
        try:
            bt.step(1)
        except ifx.IFXError as e:
            assert e.status == capi.IFX_ERR_GEOMETRY
            failed_at = k + 1
            break
    assert failed_at is not None and failed_at > 20
    assert bt.stats(0).status == capi.IFX_ERR_GEOMETRY
    frozen = bt.get(capi.FIELD_U, inst=0).copy()
    bt.step(2)
    assert np.array_equal(bt.get(capi.FIELD_U, inst=0), frozen)
    s = run(other, failed_at + 2)
    for f in FIELDS:
        assert np.array_equal(bt.get(f, inst=1), s.get(f)), f


def test_autotuners_refuse_a_moving_body():
    # their trial steps would move the geometry, which the restored state lacks
    s = ifx.Solver.create(*heaving())
    s.step(1)
    with pytest.raises(ifx.IFXError) as e:
        s.autotune(steps=1)
    assert e.value.status == capi.IFX_ERR_STATE
    with pytest.raises(ifx.IFXError) as e:
        s.autotune_schedule(steps=1)
    assert e.value.status == capi.IFX_ERR_STATE


def test_set_schedule_keeps_the_device_pose():
    # the schedule fields are written into the device descriptors without
    # touching the pose the moving body keeps there: re-setting the same
    # schedule mid-run changes nothing, bit for bit
    a = ifx.Solver.create(*heaving())
    a.set_exec_mode(ifx.EXEC_GRAPH)
    b = ifx.Solver.create(*heaving())
    b.set_exec_mode(ifx.EXEC_GRAPH)
    a.step(3)
    b.step(3)
    b.set_schedule(b.schedule())
    a.step(3)
    b.step(3)
    for f in (capi.FIELD_U, capi.FIELD_V, capi.FIELD_P, capi.FIELD_CELLTYPE):
        assert np.array_equal(a.get(f), b.get(f)), f


@pytest.mark.parametrize("prec", [capi.PREC_FP64, capi.PREC_MIXED])
def test_galilean_consistency_of_the_towed_cylinder(prec):
    """The GPU's towed cylinder against its fixed cylinder in a uniform stream
    (tests/_galilean.py): the time-averaged drag difference falls under
    refinement (128 -> 192 cells across) and is below 3% on the finer grid."""
    import _galilean as gl

    diffs = []
    for n in (128, 192):
        fixed = ifx.Solver.create(*gl.case(n, False, prec))
        towed = ifx.Solver.create(*gl.case(n, True, prec))
        f, t = gl.mean_drag(fixed), gl.mean_drag(towed)
        diffs.append(abs(t - f) / abs(f))
    assert diffs[0] > diffs[1] and diffs[1] < 0.03, diffs
