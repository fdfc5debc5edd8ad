"""The benchmark configurations at their full sizes, on the GPU against the
CPU oracle, in plain FP64 and in mixed precision.

  cavity    128x128 uniform, lid u=1, Re 100, dt 1e-3, pressure to 1e-8, 50 steps
  cylinder  384x256 tanh-stretched, D=1 at (10,10) in 30x20, Re 100, dt 5e-3, 50 steps
  ellipse   1024x768 stretched, chord 1, thickness 0.2, 10 deg, Re 300, dt 2e-3, 5 steps
  batch     a 512x384 instance with the batched sweep's sampling rules, run as
            member 0 of a four-instance batch on 32x32 tiles, 20 steps
  served    a 1024x1024 request with the served stream's sampling rules, run
            through the continuous-batching server beside a smaller request, 5 steps

Tolerances (every one is stated where it is asserted):
  - cell types, iBlank, IBM ghost cells, image-point stencils and weights:
    bit-exact (the set-up kernels are built without FMA contraction, like the
    oracle);
  - plain FP64 fields: max |GPU - oracle| <= 1e-9 of the field's max (FMA
    contraction in the step kernels and another summation order perturb the
    last bits; the pressure solve stops on ||r|| <= 1e-8 ||b||, so a step
    whose iteration count differs by one moves the fields by less than that);
    per step the predictor sweeps are equal and the pressure iterations
    differ by at most one; drag and lift within 1e-7 of the drag;
  - mixed precision (FP32 multigrid and sweeps, FP64 defects): relative L2
    velocity error <= 1e-6 against the FP64 oracle, drag and lift within 1e-3
    of the drag, pressure within 1e-6 relative L2;
  - divergence after projection: max |div U| of the GPU at most 10x the
    oracle's (both are dt times the pressure residual) and below 1e-5.
"""
import math
import os

import numpy as np
import pytest

import immerseflow_gb300 as ifx
from immerseflow_gb300 import _capi as capi
from immerseflow_gb300 import cases

pytestmark = pytest.mark.gpu

NCPU = os.cpu_count() or 4
FP64_RTOL = 1e-9
FP64_FORCE = 1e-7
MIXED_L2 = 1e-6
MIXED_FORCE = 1e-3
FIELDS = (capi.FIELD_U, capi.FIELD_V, capi.FIELD_P, capi.FIELD_UF, capi.FIELD_VF)


def _with_prec(spec, prec):
    cfg, xf, yf = spec
    c = capi.Config.from_buffer_copy(cfg)
    c.precision = prec
    return c, xf, yf


def _gpu(spec, rows=1):
    s = ifx.Solver.create(*spec)
    s.set_exec_mode(ifx.EXEC_GRAPH)
    s.set_mg_tile_rows(rows)
    return s


def _max_rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _l2_rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _geometry_bit_exact(get, ghosts, o):
    assert np.array_equal(get(capi.FIELD_IBLANK), o.get(capi.FIELD_IBLANK))
    assert np.array_equal(get(capi.FIELD_CELLTYPE), o.get(capi.FIELD_CELLTYPE))
    if ghosts is None:
        return
    cells, nb, wu, wp, bip = ghosts
    oc, onb, owu, owp, obi, oip = o.ghosts()
    assert np.array_equal(cells, oc)
    assert np.array_equal(nb, onb)
    assert np.array_equal(wu, owu)
    assert np.array_equal(wp, owp)
    assert np.array_equal(bip[:, :2], obi) and np.array_equal(bip[:, 2:], oip)


def _fp64_vs_oracle(get, st, o, so, body):
    errs = {f: _max_rel(get(f), o.get(f)) for f in FIELDS}
    assert all(e <= FP64_RTOL for e in errs.values()), errs
    if body:
        scale = abs(so.cd)
        assert abs(st.cd - so.cd) <= FP64_FORCE * scale, (st.cd, so.cd)
        assert abs(st.cl - so.cl) <= FP64_FORCE * scale, (st.cl, so.cl)
    assert st.max_div <= 1e-5 and st.max_div <= 10.0 * so.max_div + 1e-14, (st.max_div, so.max_div)
    return errs


def _mixed_vs_oracle(get, st, o, so, body):
    vel = _l2_rel(np.concatenate([get(capi.FIELD_U).ravel(), get(capi.FIELD_V).ravel()]),
                  np.concatenate([o.get(capi.FIELD_U).ravel(), o.get(capi.FIELD_V).ravel()]))
    assert vel <= MIXED_L2, vel
    pe = _l2_rel(get(capi.FIELD_P), o.get(capi.FIELD_P))
    assert pe <= MIXED_L2, pe
    if body:
        scale = abs(so.cd)
        assert abs(st.cd - so.cd) <= MIXED_FORCE * scale, (st.cd, so.cd)
        assert abs(st.cl - so.cl) <= MIXED_FORCE * scale, (st.cl, so.cl)
    assert st.max_div <= 1e-5 and st.max_div <= 10.0 * so.max_div + 1e-14, (st.max_div, so.max_div)
    return vel


def _lockstep(spec, nsteps, oracle, body, rows=1):
    """Steps the FP64 and mixed GPU solvers and the oracle together; per step the
    FP64 solver takes the oracle's predictor sweeps and pressure iterations (+-1)."""
    s64 = _gpu(_with_prec(spec, capi.PREC_FP64), rows)
    smx = _gpu(_with_prec(spec, capi.PREC_MIXED), rows)
    o = oracle.method(_with_prec(spec, capi.PREC_FP64)[0], spec[1], spec[2], NCPU)
    _geometry_bit_exact(s64.get, s64.ibm_ghosts() if body else None, o)
    _geometry_bit_exact(smx.get, smx.ibm_ghosts() if body else None, o)
    for _ in range(nsteps):
        s64.step(1)
        smx.step(1)
        o.step(1)
        st, so = s64.stats(), o.stats()
        assert st.last_ad_iters == so.last_ad_iters, (st.last_ad_iters, so.last_ad_iters)
        assert abs(st.last_ppe_iters - so.last_ppe_iters) <= 1, (st.last_ppe_iters, so.last_ppe_iters)
        assert st.last_ppe_residual <= spec[0].ppe_tol
        assert smx.stats().last_ppe_residual <= spec[0].ppe_tol
    so = o.stats()
    _fp64_vs_oracle(s64.get, s64.stats(), o, so, body)
    _mixed_vs_oracle(smx.get, smx.stats(), o, so, body)


def test_cavity_128_50_steps_vs_oracle(oracle):
    spec = cases.cavity(n=128, re=100.0, dt=1e-3)
    assert spec[0].ppe_tol == 1e-8
    _lockstep(spec, 50, oracle, body=False)


def test_cylinder_384x256_50_steps_vs_oracle(oracle):
    _lockstep(cases.cylinder(), 50, oracle, body=True)


def test_ellipse_1024x768_5_steps_vs_oracle(oracle):
    _lockstep(cases.ellipse(), 5, oracle, body=True)


def _batch_rules(nx, ny, re, ar, ang, prec, lx=12.0, ly=8.0):
    """One instance by the batched sweep's rules (cases.batch_sample)."""
    hmin = min(lx / nx, ly / ny) / 2.5
    dt = float(min(5e-3, 0.4 * hmin))
    return cases.external(nx, ny, lx, ly, lx / 3.0, ly / 2.0, 0.5, 0.5 * ar, ang, re, dt, prec)


@pytest.mark.parametrize("prec", [capi.PREC_FP64, capi.PREC_MIXED])
def test_batch_member_512x384_vs_oracle(oracle, prec):
    big = _batch_rules(512, 384, 275.0, 0.35, 22.0, prec)
    others = [c for c in cases.batch_sample(3, seed=7, precision=prec)]
    specs = [big] + others
    s = ifx.Solver.batch([c for c, _, _ in specs], [x for _, x, _ in specs], [y for _, _, y in specs])
    s.set_exec_mode(ifx.EXEC_GRAPH)
    s.set_mg_tile_rows(4)
    o = oracle.method(_with_prec(big, capi.PREC_FP64)[0], big[1], big[2], NCPU)
    _geometry_bit_exact(lambda f: s.get(f, inst=0), s.ibm_ghosts(inst=0), o)
    for _ in range(20):
        s.step(1)
        o.step(1)
        if prec == capi.PREC_FP64:
            st, so = s.stats(0), o.stats()
            assert st.last_ad_iters == so.last_ad_iters
            assert abs(st.last_ppe_iters - so.last_ppe_iters) <= 1
    get = lambda f: s.get(f, inst=0)  # noqa: E731
    if prec == capi.PREC_FP64:
        _fp64_vs_oracle(get, s.stats(0), o, o.stats(), body=True)
    else:
        _mixed_vs_oracle(get, s.stats(0), o, o.stats(), body=True)


def _served_rules(n, re, ar, ang, prec, lx=12.0, ly=8.0):
    """One request by the served stream's rules (cases.served_stream)."""
    hmin = min(lx, ly) / n / 2.5
    dt = float(min(5e-3, 0.4 * hmin))
    return cases.external(n, n, lx, ly, lx / 3, ly / 2, 0.5, 0.5 * ar, ang, re, dt, prec)


@pytest.mark.parametrize("prec", [capi.PREC_MIXED, capi.PREC_FP64])
def test_served_request_1024_vs_oracle(oracle, prec):
    big = _served_rules(1024, 850.0, 0.4, -25.0, prec)
    small = _served_rules(96, 300.0, 1.0, 0.0, prec)
    srv = ifx.Server(1 << 34, max_cohort=8, steps_per_tick=1)
    rid = srv.submit(*big, nsteps=5)
    sid = srv.submit(*small, nsteps=9)
    done = []
    for _ in range(40):
        srv.tick()
        done += srv.poll()
        if len(done) == 2:
            break
    assert sorted(done) == sorted([rid, sid])
    state, steps, nx, ny = srv.state(rid)
    assert state == ifx.REQ_FINISHED and steps == 5 and (nx, ny) == (1026, 1026)
    o = oracle.method(_with_prec(big, capi.PREC_FP64)[0], big[1], big[2], NCPU)
    o.step(5)
    res = {f: srv.result(rid, f) for f in (capi.FIELD_U, capi.FIELD_V, capi.FIELD_P)}
    st, so = srv.stats(rid), o.stats()
    if prec == capi.PREC_FP64:
        for f, a in res.items():
            e = _max_rel(a, o.get(f))
            assert e <= FP64_RTOL, (f, e)
        assert abs(st.cd - so.cd) <= FP64_FORCE * abs(so.cd)
        assert abs(st.cl - so.cl) <= FP64_FORCE * abs(so.cd)
    else:
        vel = _l2_rel(np.concatenate([res[capi.FIELD_U].ravel(), res[capi.FIELD_V].ravel()]),
                      np.concatenate([o.get(capi.FIELD_U).ravel(), o.get(capi.FIELD_V).ravel()]))
        assert vel <= MIXED_L2, vel
        assert abs(st.cd - so.cd) <= MIXED_FORCE * abs(so.cd)
        assert abs(st.cl - so.cl) <= MIXED_FORCE * abs(so.cd)
    assert math.isfinite(st.max_div) and st.max_div <= 1e-5
    srv.close()
