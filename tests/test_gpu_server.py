"""Batch membership, asynchronous steps and the continuous-batching server on
the GPU.  A request's result must not depend on the cohort it ran in: every
finished request is compared bit for bit with the same case run alone."""
import numpy as np
import pytest

import immerseflow_gb300 as ifx
from immerseflow_gb300 import _capi as capi
from immerseflow_gb300 import cases

pytestmark = pytest.mark.gpu


def case(nx, ny, re=100.0, b=0.5, angle=0.0, prec=capi.PREC_MIXED):
    return cases.external(nx, ny, 12.0, 8.0, 4.0, 4.0, 0.5, b, angle, re, 1e-2, prec, ratio=4.0, width=1.0)


def alone(cfg, xf, yf, nsteps):
    s = ifx.Solver.create(cfg, xf, yf)
    s.step(nsteps)
    return {f: s.get(f) for f in (capi.FIELD_U, capi.FIELD_V, capi.FIELD_P)}


def test_async_step_equals_step():
    spec = case(64, 48)
    a = ifx.Solver.create(*spec)
    b = ifx.Solver.create(*spec)
    a.step(3)
    for _ in range(3):
        b.step_async(1)
        b.step_wait()
    for f in (capi.FIELD_U, capi.FIELD_P):
        assert np.array_equal(a.get(f), b.get(f))


def test_inactive_instance_is_left_unchanged():
    specs = [case(64, 48), case(56, 40, re=150.0, b=0.25, angle=15.0)]
    s = ifx.Solver.batch([c for c, _, _ in specs], [x for _, x, _ in specs], [y for _, _, y in specs])
    s.step(2)
    frozen = {f: s.get(f, inst=0) for f in (capi.FIELD_U, capi.FIELD_V, capi.FIELD_P, capi.FIELD_UF)}
    s.set_active(0, False)
    s.step(2)
    for f, a in frozen.items():
        assert np.array_equal(s.get(f, inst=0), a), f
    ref = alone(*specs[1], 4)
    for f, a in ref.items():
        assert np.array_equal(s.get(f, inst=1), a), f
    s.set_active(0, True)
    s.step(1)
    assert not np.array_equal(s.get(capi.FIELD_U, inst=0), frozen[capi.FIELD_U])


def test_server_results_equal_alone_runs():
    stream = [(case(64, 48), 4), (case(48, 40, re=80.0, b=0.2, angle=-20.0), 2),
              (case(72, 40, re=200.0, b=0.35, angle=10.0), 3), (case(40, 40, re=60.0), 5),
              (case(56, 48, re=120.0, b=0.5), 1)]
    srv = ifx.Server(1 << 33, max_cohort=8, steps_per_tick=3)
    ids = {}
    done = []
    # arrivals interleaved with ticks: later requests join while earlier ones run
    for t in range(40):
        if t < len(stream):
            spec, n = stream[t]
            ids[srv.submit(*spec, nsteps=n)] = (spec, n)
        srv.tick()
        done += srv.poll()
        if len(done) == len(stream):
            break
    assert sorted(done) == sorted(ids)
    assert srv.info()["cohorts"] == 0 and srv.info()["used_bytes"] == 0
    for rid, (spec, n) in ids.items():
        st, steps, _, _ = srv.state(rid)
        assert st == ifx.REQ_FINISHED and steps == n
        ref = alone(*spec, n)
        for f, a in ref.items():
            assert np.array_equal(srv.result(rid, f), a), (rid, f)
        srv.release(rid)
    srv.close()


def test_server_admits_by_memory_budget():
    stream = [(case(64, 48), 2), (case(64, 48, re=150.0), 2), (case(64, 48, re=60.0), 2)]
    one = ifx.estimate_bytes(stream[0][0][0])
    srv = ifx.Server(int(one * 1.5), max_cohort=8, steps_per_tick=1)
    ids = [srv.submit(*spec, nsteps=n) for spec, n in stream]
    srv.tick()
    info = srv.info()
    assert info["running"] == 1 and info["waiting"] == 2
    done = []
    for _ in range(20):
        srv.tick()
        done += srv.poll()
        if len(done) == 3:
            break
    assert sorted(done) == ids
    for rid, (spec, n) in zip(ids, stream):
        ref = alone(*spec, n)
        assert np.array_equal(srv.result(rid, capi.FIELD_U), ref[capi.FIELD_U])
    srv.close()


def test_autotune_keeps_results():
    spec = case(64, 48)
    a = ifx.Solver.create(*spec)
    a.step(1)
    mode, ms = a.autotune(steps=2)
    assert mode in (ifx.EXEC_PERSISTENT, ifx.EXEC_GRAPH) and ms > 0
    assert a.exec_mode() == mode
    a.step(2)
    b = ifx.Solver.create(*spec)
    b.step(3)
    for f in (capi.FIELD_U, capi.FIELD_V, capi.FIELD_P):
        assert np.array_equal(a.get(f), b.get(f)), f


def test_server_fails_only_the_diverged_request():
    """A request whose state becomes non-finite fails; the rest of its cohort
    finishes with the same results as alone.  The fault is planted on the host:
    a request whose Reynolds number (1e-300) overflows its diffusion
    coefficients."""
    good = [case(64, 48), case(56, 40, re=150.0, b=0.25, angle=15.0)]
    bad = case(48, 40, re=1e-300)
    v = ifx.Server(1 << 34, max_cohort=8, steps_per_tick=1)
    ids = [v.submit(c, x, y, 4) for c, x, y in good]
    bad_id = v.submit(*bad, 4)
    diverged = False
    for _ in range(20):
        try:
            v.tick()
        except ifx.IFXError as e:
            assert e.status == capi.IFX_ERR_DIVERGED
            diverged = True
        if all(v.state(i)[0] in (ifx.REQ_FINISHED, ifx.REQ_FAILED) for i in ids + [bad_id]):
            break
    assert diverged
    assert v.state(bad_id)[0] == ifx.REQ_FAILED
    for rid, (c, x, y) in zip(ids, good):
        assert v.state(rid)[0] == ifx.REQ_FINISHED
        ref = alone(c, x, y, 4)
        for f in (capi.FIELD_U, capi.FIELD_V, capi.FIELD_P):
            assert np.array_equal(v.result(rid, f), ref[f]), (rid, f)
    v.close()


@pytest.mark.parametrize("prec,rows", [(capi.PREC_FP64, 1), (capi.PREC_MIXED, 1), (capi.PREC_MIXED, 4)])
def test_retired_instances_leave_the_tile_lists(prec, rows):
    """Retiring three of five instances compacts the device tile lists to the two
    left (their partial sums move with them); an instance set active again is
    listed again.  Every result equals the same case run alone."""
    specs = [case(64, 48, prec=prec), case(56, 40, re=150.0, b=0.25, angle=15.0, prec=prec),
             case(72, 40, re=200.0, b=0.35, angle=10.0, prec=prec), case(40, 40, re=60.0, prec=prec),
             case(48, 48, re=120.0, prec=prec)]
    s = ifx.Solver.batch([c for c, _, _ in specs], [x for _, x, _ in specs], [y for _, _, y in specs])
    s.set_mg_tile_rows(rows)
    s.step(2)
    for k in (0, 2, 3):
        s.set_active(k, False)
    s.step(3)
    for k in (1, 4):
        ref = alone(*specs[k], 5)
        for f, a in ref.items():
            assert np.array_equal(s.get(f, inst=k), a), (k, f)
    s.set_active(2, True)
    s.step(2)
    for k, n in ((2, 4), (1, 7), (4, 7)):
        ref = alone(*specs[k], n)
        for f, a in ref.items():
            assert np.array_equal(s.get(f, inst=k), a), (k, f)
    s.set_exec_mode(ifx.EXEC_PERSISTENT)  # the persistent kernel on the compacted lists
    s.step(1)
    ref = alone(*specs[2], 5)
    for f, a in ref.items():
        assert np.array_equal(s.get(f, inst=2), a), f


def test_server_stream_of_mixed_precisions():
    """FP64 and mixed-precision requests interleaved in one queue: a cohort
    holds one precision (a batch shares it), so each cohort stops at the first
    request of the other precision; every request finishes and equals its
    alone run."""
    stream = [(case(48, 40, prec=capi.PREC_MIXED), 3), (case(56, 40, prec=capi.PREC_FP64), 2),
              (case(40, 48, prec=capi.PREC_MIXED), 2), (case(48, 48, prec=capi.PREC_FP64), 3)]
    srv = ifx.Server(1 << 33, max_cohort=8)
    ids = {srv.submit(*spec, nsteps=n): (spec, n) for spec, n in stream}
    done = []
    for _ in range(20):
        srv.tick()
        done += srv.poll()
        if len(done) == len(stream):
            break
    assert sorted(done) == sorted(ids)
    for rid, (spec, n) in ids.items():
        assert srv.state(rid)[0] == ifx.REQ_FINISHED
        ref = alone(*spec, n)
        for f, a in ref.items():
            assert np.array_equal(srv.result(rid, f), a), (rid, f)
    srv.close()
