"""Checkpoint / restart, snapshots, time history and server pre-emption on the GPU.

Bar: a run restarted from a binary checkpoint continues bit for bit (same
u, v, p and iteration counts as the uninterrupted run), in every execution
mode, for a batch member loaded into a handle of its own, and for a server
request that was pre-empted and resumed.  The ASCII snapshot reproduces the
fields it holds exactly (%.17g).  The time history holds, for every step, the
same cd, cl and probe-cell values the solver reports after that step.
"""
import os
import subprocess

import numpy as np
import pytest

import immerseflow_gb300 as ifx
from immerseflow_gb300 import _capi as capi
from immerseflow_gb300 import cases

pytestmark = pytest.mark.gpu
FIELDS = (capi.FIELD_U, capi.FIELD_V, capi.FIELD_P, capi.FIELD_UF, capi.FIELD_VF)
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def cyl(prec=capi.PREC_FP64, nx=96, ny=64, angle=0.0, b=0.5):
    return cases.external(nx, ny, 12.0, 8.0, 4.0, 4.0, 0.5, b, angle, 100.0, 1e-2, prec, ratio=4.0, width=1.0)


def same(a, b, inst_a=0, inst_b=0):
    for f in FIELDS:
        assert np.array_equal(a.get(f, inst=inst_a), b.get(f, inst=inst_b)), f


@pytest.mark.parametrize("prec", [capi.PREC_FP64, capi.PREC_MIXED])
@pytest.mark.parametrize("mode", ["persistent", "graph"])
def test_binary_checkpoint_resumes_bit_for_bit(prec, mode):
    cfg, xf, yf = cyl(prec)
    a = ifx.Solver.create(cfg, xf, yf)
    a.set_exec_mode({"persistent": ifx.EXEC_PERSISTENT, "graph": ifx.EXEC_GRAPH}[mode])
    a.step(3)
    blob = a.checkpoint()
    a.step(3)
    b = ifx.Solver.create(cfg, xf, yf)
    b.set_exec_mode(a.exec_mode())
    b.restore(blob)
    assert b.stats().steps == 3
    b.step(3)
    same(a, b)
    assert b.stats().steps == 6
    assert a.stats().last_ppe_iters == b.stats().last_ppe_iters
    assert a.stats().last_ad_iters == b.stats().last_ad_iters
    assert a.stats().cd == b.stats().cd


def test_checkpoint_file_of_a_batch_and_member_into_own_handle(tmp_path):
    specs = [cyl(), cases.cavity(n=40), cyl(nx=70, ny=90, angle=25.0, b=0.25)]
    cfgs, xfs, yfs = [c for c, _, _ in specs], [x for _, x, _ in specs], [y for _, _, y in specs]
    a = ifx.Solver.batch(cfgs, xfs, yfs)
    a.step(2)
    path = str(tmp_path / "batch.ifx")
    a.checkpoint_write(path)
    member = a.checkpoint(inst=2)
    a.step(2)
    b = ifx.Solver.batch(cfgs, xfs, yfs)
    b.checkpoint_read(path)
    b.step(2)
    for k in range(3):
        same(a, b, k, k)
    # a batch member continues alone (instances share no arithmetic)
    c = ifx.Solver.create(*specs[2])
    c.restore(member)
    c.step(2)
    same(a, c, 2, 0)


def test_checkpoint_file_with_a_corrupt_record_changes_nothing(tmp_path):
    """A checkpoint file whose second record is corrupt is refused, and the
    first instance keeps its state: every record is checked before any is
    loaded."""
    specs = [cyl(), cases.cavity(n=40)]
    cfgs, xfs, yfs = [c for c, _, _ in specs], [x for _, x, _ in specs], [y for _, _, y in specs]
    a = ifx.Solver.batch(cfgs, xfs, yfs)
    a.step(1)
    path = str(tmp_path / "batch.ifx")
    a.checkpoint_write(path)
    data = bytearray(open(path, "rb").read())
    data[-100] ^= 0xFF  # a payload byte of the last (second) record
    open(path, "wb").write(bytes(data))
    a.step(2)
    before = {f: a.get(f, inst=0) for f in FIELDS}
    with pytest.raises(ifx.IFXError) as e:
        a.checkpoint_read(path)
    assert e.value.status == capi.IFX_ERR_PARSE and "record 1" in str(e.value)
    for f, v in before.items():
        assert np.array_equal(a.get(f, inst=0), v), f


def test_checkpoint_across_precision_and_rejections():
    cfg64, xf, yf = cyl()
    cfg32, _, _ = cyl(capi.PREC_MIXED)
    a = ifx.Solver.create(cfg64, xf, yf)
    a.step(2)
    blob = a.checkpoint()
    m = ifx.Solver.create(cfg32, xf, yf)
    m.restore(blob)  # FP64 state continues on the mixed path
    for f in (capi.FIELD_U, capi.FIELD_V, capi.FIELD_P):
        assert np.array_equal(m.get(f), a.get(f))
    # another grid
    other, oxf, oyf = cyl(nx=80, ny=64)
    o = ifx.Solver.create(other, oxf, oyf)
    with pytest.raises(ifx.IFXError) as e:
        o.restore(blob)
    assert e.value.status == capi.IFX_ERR_ARG
    # another body on the same grid
    rot, rxf, ryf = cyl(angle=20.0, b=0.3)
    r = ifx.Solver.create(rot, rxf, ryf)
    with pytest.raises(ifx.IFXError) as e:
        r.restore(blob)
    assert e.value.status == capi.IFX_ERR_ARG
    # corrupted payload, truncated buffer
    bad = bytearray(blob)
    bad[len(bad) // 2] ^= 0x40
    with pytest.raises(ifx.IFXError) as e:
        m.restore(bytes(bad))
    assert e.value.status == capi.IFX_ERR_PARSE
    with pytest.raises(ifx.IFXError) as e:
        m.restore(blob[:100])
    assert e.value.status == capi.IFX_ERR_PARSE


def test_reference_mode_checkpoint(golden_dir):
    c = ifx.config_read(os.path.join(golden_dir, "inputs", "inputs.txt"))
    xf = ifx.grid_read(c.xgrid.decode(), c.nx + 1)
    yf = ifx.grid_read(c.ygrid.decode(), c.ny + 1)
    a = ifx.Solver.create(c, xf, yf)
    a.step(3)
    blob = a.checkpoint()
    a.step(2)
    b = ifx.Solver.create(c, xf, yf)
    b.restore(blob)
    b.step(2)
    for f in (capi.FIELD_U, capi.FIELD_V, capi.FIELD_P):
        assert np.array_equal(a.get(f), b.get(f)), f
    assert b.stats().steps == 5


def test_ascii_snapshot_round_trip(tmp_path):
    cfg, xf, yf = cyl()
    a = ifx.Solver.create(cfg, xf, yf)
    a.step(3)
    path = str(tmp_path / "data.0000000.dat")
    a.write_snapshot_ascii(path)
    lines = open(path).read().splitlines()
    nx, ny = a.grid_dims()
    assert len(lines) == 3 + nx * ny
    assert 'T="step 3"' in lines[2]
    assert len(lines[3].split()) == 8
    b = ifx.Solver.create(cfg, xf, yf)
    b.read_snapshot_ascii(path)
    same(a, b)
    assert b.stats().steps == 3
    # the restarted run restarts the convection history: close, not identical
    a.step(2)
    b.step(2)
    u_a, u_b = a.get(capi.FIELD_U), b.get(capi.FIELD_U)
    assert np.all(np.isfinite(u_b))
    assert np.abs(u_a - u_b).max() <= 1e-2 * np.abs(u_a).max()


@pytest.mark.parametrize("mode", ["persistent", "graph", "host"])
def test_time_history_records_every_step(mode):
    cfg, xf, yf = cyl()
    s = ifx.Solver.create(cfg, xf, yf)
    s.set_exec_mode({"persistent": ifx.EXEC_PERSISTENT, "graph": ifx.EXEC_GRAPH, "host": ifx.EXEC_HOST}[mode])
    probes = [(6.0, 4.0), (5.1, 4.6), (-1.0, 100.0)]  # wake, near the body, outside the domain (nearest ghost)
    s.set_history(3, probes)
    cells = s.probe_cells()
    xc, yc = s.get(capi.FIELD_XC), s.get(capi.FIELD_YC)
    for (x, y), (i, j) in zip(probes, cells):
        assert i == int(np.argmin(np.abs(xc - x))) and j == int(np.argmin(np.abs(yc - y)))
    recs = []
    for k in range(5):
        s.step(1)
        st = s.stats()
        u, v, p = s.get(capi.FIELD_U), s.get(capi.FIELD_V), s.get(capi.FIELD_P)
        recs.append([k + 1, st.cd, st.cl] + [q[j, i] for (i, j) in cells for q in (u, v, p)])
    h = s.history()
    assert h.shape == (3, 3 + 3 * len(probes))  # ring of three records: the last three steps
    assert np.array_equal(h, np.array(recs[-3:]))


def test_history_and_checkpoint_files(tmp_path):
    cfg, xf, yf = cyl()
    s = ifx.Solver.create(cfg, xf, yf)
    pf = tmp_path / "probe.dat"
    pf.write_text("2\nx y\n6.0 4.0\n5.1, 4.6\n")
    xy = ifx.probes_read(str(pf))
    s.set_history(100, xy)
    s.step(4)
    s.write_probe_file(str(tmp_path / "probe_output.dat"))
    s.write_force_file(str(tmp_path / "forces.dat"))
    lines = (tmp_path / "probe_output.dat").read_text().splitlines()
    assert lines[0].split()[0] == "2" and lines[1] == "" and lines[2].split() == ["Time", "U", "V", "P"]
    rows = np.array([[float(t) for t in l.split()] for l in lines[3:]])
    h = s.history()
    assert rows.shape == (4, 7)
    assert np.allclose(rows[:, 0], h[:, 0] * cfg.dt)
    assert np.array_equal(rows[:, 1:], h[:, 3:])
    f = (tmp_path / "forces.dat").read_text().splitlines()
    assert f[0].split() == ["Time", "Cd", "Cl"]
    assert np.array_equal(np.array([[float(t) for t in l.split()][1:] for l in f[1:]]), h[:, 1:3])


def test_autotune_keeps_history():
    cfg, xf, yf = cyl(capi.PREC_MIXED)
    s = ifx.Solver.create(cfg, xf, yf)
    s.set_history(4, [(6.0, 4.0)])
    s.step(6)
    before = s.history()
    s.autotune(2)
    assert np.array_equal(s.history(), before)
    s.step(1)
    assert s.history()[-1, 0] == 7


@pytest.mark.parametrize("front", [True, False])
def test_server_preempt_resume_is_bit_identical(front):
    specs = [cyl(capi.PREC_MIXED), cyl(capi.PREC_MIXED, nx=70, ny=90, angle=25.0, b=0.25)]
    v = ifx.Server(1 << 34, max_cohort=8, steps_per_tick=1)
    ids = [v.submit(c, x, y, 6) for c, x, y in specs]
    for _ in range(3):
        v.tick()
    v.preempt(ids[0], front=front)
    assert v.state(ids[0])[0] == ifx.REQ_WAITING
    for _ in range(40):
        v.tick()
        if all(v.state(i)[0] == ifx.REQ_FINISHED for i in ids):
            break
    for rid, (c, x, y) in zip(ids, specs):
        assert v.state(rid)[0] == ifx.REQ_FINISHED
        alone = ifx.Solver.create(c, x, y)
        alone.step(6)
        for f in (capi.FIELD_U, capi.FIELD_V, capi.FIELD_P):
            assert np.array_equal(v.result(rid, f), alone.get(f)), (rid, f)
    v.close()


def test_cli_restart_continues_the_run(golden_dir, tmp_path):
    """The command-line driver writes snapshots every Write Interval steps and
    restarts from one (Restart = 1): 4 steps + restart + 2 steps equals 6 steps."""
    exe = os.path.join(ROOT, "immerseflow_gb300", "bin", "immerseflow_gb300")
    src = open(os.path.join(golden_dir, "inputs", "inputs.txt")).read()

    def inputs(dirname, restart, tmax, interval):
        d = tmp_path / dirname
        d.mkdir(exist_ok=True)
        (d / "results").mkdir(exist_ok=True)
        for g in ("xgrid.dat2", "ygrid.dat2"):
            (d / g).write_text(open(os.path.join(golden_dir, "inputs", g)).read())
        text = src.replace("0           9", f"{restart}           0")
        text = text.replace("100       0.001", f"{tmax}       0.001").replace("\n1000", f"\n{interval}")
        (d / "inputs.txt").write_text(text)
        return str(d / "inputs.txt"), str(d / "results")

    i6, r6 = inputs("straight", 0, 6, 0)
    subprocess.run([exe, i6, r6], check=True, capture_output=True)
    i4, r4 = inputs("restarted", 0, 4, 4)
    subprocess.run([exe, i4, r4], check=True, capture_output=True)
    assert os.path.exists(os.path.join(r4, "Data", "data.0000000.ifx"))
    assert os.path.exists(os.path.join(r4, "Data", "data.0000000.dat"))
    i4b, _ = inputs("restarted", 1, 6, 0)
    subprocess.run([exe, i4b, r4], check=True, capture_output=True)
    for name in ("uc.dat", "vc.dat", "p.dat"):
        assert open(os.path.join(r4, name)).read() == open(os.path.join(r6, name)).read(), name
