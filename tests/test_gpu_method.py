"""METHOD mode (fractional step + ghost-cell IBM) on the GPU against the oracle.

Tolerances:
  - iBlank, cell types, ghost cells, image-point stencils and weights: bit-exact
    (the set-up kernels are built without FMA contraction, like the oracle);
  - FP64 fields after several steps: 1e-10 relative to the field's max
    (FMA contraction in the step kernels, sums reduced in another order);
  - a batched instance equals the same instance run alone, bit for bit;
  - persistent, graph and host-loop execution agree bit for bit.
"""
import os

import numpy as np
import pytest

import immerseflow_gb300 as ifx
from immerseflow_gb300 import _capi as capi
from immerseflow_gb300 import cases

pytestmark = pytest.mark.gpu
FIELD_RTOL = 1e-10


def small_cylinder(prec=capi.PREC_FP64, nx=96, ny=64, angle=0.0, b=0.5):
    return cases.external(nx, ny, 12.0, 8.0, 4.0, 4.0, 0.5, b, angle, 100.0, 1e-2, prec, ratio=4.0, width=1.0)


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("angle,b", [(0.0, 0.5), (17.0, 0.15), (-30.0, 0.3)])
def test_tagging_and_ghost_table_bit_exact(oracle, angle, b):
    cfg, xf, yf = small_cylinder(angle=angle, b=b)
    s = ifx.Solver.create(cfg, xf, yf)
    o = oracle.method(cfg, xf, yf)
    assert np.array_equal(s.get(capi.FIELD_IBLANK), o.get(capi.FIELD_IBLANK))
    assert np.array_equal(s.get(capi.FIELD_CELLTYPE), o.get(capi.FIELD_CELLTYPE))
    cells, nb, wu, wp, bip = s.ibm_ghosts()
    oc, onb, owu, owp, obi, oip = o.ghosts()
    assert len(cells) > 0
    assert np.array_equal(cells, oc)
    assert np.array_equal(nb, onb)
    assert np.array_equal(wu, owu)
    assert np.array_equal(wp, owp)
    assert np.array_equal(bip[:, :2], obi) and np.array_equal(bip[:, 2:], oip)


def _compare(s, o, fields=(capi.FIELD_U, capi.FIELD_V, capi.FIELD_P, capi.FIELD_UF, capi.FIELD_VF), tol=FIELD_RTOL):
    for f in fields:
        a, b = s.get(f), o.get(f)
        assert rel(a, b) <= tol, (f, rel(a, b))


def test_cavity_vs_oracle(oracle):
    cfg, xf, yf = cases.cavity(n=64)
    s = ifx.Solver.create(cfg, xf, yf)
    o = oracle.method(cfg, xf, yf)
    for k in range(4):
        s.step(1)
        o.step(1)
        st, so = s.stats(), o.stats()
        assert st.last_ad_iters == so.last_ad_iters
        assert st.last_ppe_iters == so.last_ppe_iters
        assert st.last_ppe_residual <= cfg.ppe_tol
    _compare(s, o)
    assert s.stats().max_div < 1e-5


def test_cylinder_vs_oracle(oracle):
    cfg, xf, yf = small_cylinder()
    s = ifx.Solver.create(cfg, xf, yf)
    o = oracle.method(cfg, xf, yf)
    for k in range(3):
        s.step(1)
        o.step(1)
        st, so = s.stats(), o.stats()
        assert st.last_ad_iters == so.last_ad_iters
        assert abs(st.last_ppe_iters - so.last_ppe_iters) <= 1
    _compare(s, o, tol=1e-9)
    st, so = s.stats(), o.stats()
    assert abs(st.cd - so.cd) <= 1e-8 * abs(so.cd)
    assert abs(st.cl - so.cl) <= 1e-8 * max(abs(so.cd), 1.0)


def test_rotated_ellipse_stretched_vs_oracle(oracle):
    cfg, xf, yf = small_cylinder(nx=80, ny=72, angle=20.0, b=0.2)
    s = ifx.Solver.create(cfg, xf, yf)
    o = oracle.method(cfg, xf, yf)
    s.step(3)
    o.step(3)
    _compare(s, o, tol=1e-9)


def _run_mode(mode, specs, nsteps, rows=1):
    os.environ["IFX_EXEC"] = mode
    try:
        if len(specs) == 1:
            s = ifx.Solver.create(*specs[0])
        else:
            s = ifx.Solver.batch([c for c, _, _ in specs], [x for _, x, _ in specs], [y for _, _, y in specs])
        s.set_mg_tile_rows(rows)
        s.step(nsteps)
        return s
    finally:
        del os.environ["IFX_EXEC"]


@pytest.mark.parametrize("prec", [capi.PREC_FP64, capi.PREC_MIXED])
def test_execution_modes_bit_identical(prec):
    """Persistent per-step kernel, CUDA graph and host-driven loop run the same
    device bodies: the results must agree bit for bit."""
    specs = [small_cylinder(prec=prec)]
    runs = {m: _run_mode(m, specs, 3) for m in ("persistent", "graph", "host")}
    runs["graph_wide"] = _run_mode("graph", specs, 3, rows=4)
    for f in (capi.FIELD_U, capi.FIELD_V, capi.FIELD_P, capi.FIELD_UF):
        a = runs["persistent"].get(f)
        assert np.array_equal(a, runs["graph"].get(f)), f
        assert np.array_equal(a, runs["host"].get(f)), f
        assert np.array_equal(a, runs["graph_wide"].get(f)), f
    assert runs["persistent"].stats().last_ppe_iters == runs["graph"].stats().last_ppe_iters


@pytest.mark.parametrize("prec", [capi.PREC_FP64, capi.PREC_MIXED])
def test_execution_modes_bit_identical_many_waves(prec):
    """A 400x400 grid: every multigrid tile phase runs in several waves of
    blocks, so a phase that read values another block of the same phase writes
    would give results that depend on scheduling and differ between modes."""
    specs = [cases.external(400, 400, 12.0, 8.0, 4.0, 4.0, 0.5, 0.5, 0.0, 535.0, 3.2e-3, prec)]
    runs = {m: _run_mode(m, specs, 4) for m in ("persistent", "graph", "host")}
    runs["graph_wide"] = _run_mode("graph", specs, 4, rows=4)
    for f in (capi.FIELD_U, capi.FIELD_V, capi.FIELD_P):
        a = runs["persistent"].get(f)
        assert np.all(np.isfinite(a))
        for m in ("graph", "host", "graph_wide"):
            assert np.array_equal(a, runs[m].get(f)), (m, f)


def test_persistent_batch_equals_graph_batch():
    specs = [small_cylinder(nx=96, ny=64), cases.cavity(n=40), small_cylinder(nx=70, ny=90, angle=25.0, b=0.25)]
    a = _run_mode("persistent", specs, 2)
    b = _run_mode("graph", specs, 2)
    c = _run_mode("graph", specs, 2, rows=4)
    for k in range(3):
        for f in (capi.FIELD_U, capi.FIELD_V, capi.FIELD_P):
            assert np.array_equal(a.get(f, inst=k), b.get(f, inst=k)), (k, f)
            assert np.array_equal(a.get(f, inst=k), c.get(f, inst=k)), (k, f)


@pytest.mark.parametrize("prec", [capi.PREC_FP64, capi.PREC_MIXED])
def test_persistent_grid_does_not_change_results(prec):
    """The persistent kernel's phases stride over their tiles, so a launch of a
    few blocks gives the graph mode's results bit for bit; with fewer blocks
    than instances the small levels' geometry is staged in every V-cycle."""
    specs = [small_cylinder(prec=prec, nx=96, ny=64), cases.cavity(n=40, precision=prec),
             small_cylinder(prec=prec, nx=70, ny=90, angle=25.0, b=0.25)]
    ref = _run_mode("graph", specs, 3)
    for grid in (2, 38):
        os.environ["IFX_EXEC"] = "persistent"
        try:
            s = ifx.Solver.batch([c for c, _, _ in specs], [x for _, x, _ in specs], [y for _, _, y in specs])
            s.set_persistent_grid(grid)
            assert s.persistent_grid() == grid
            s.step(3)
        finally:
            del os.environ["IFX_EXEC"]
        for k in range(3):
            for f in (capi.FIELD_U, capi.FIELD_V, capi.FIELD_P):
                assert np.array_equal(s.get(f, inst=k), ref.get(f, inst=k)), (grid, k, f)
            assert s.stats(k).last_ppe_iters == ref.stats(k).last_ppe_iters
    with pytest.raises(ifx.IFXError):
        s.set_persistent_grid(1 << 20)  # more blocks than can be co-resident
    s.set_persistent_grid(0)
    assert s.persistent_grid() >= 38


def test_batch_member_equals_alone():
    specs = [small_cylinder(nx=96, ny=64), cases.cavity(n=40), small_cylinder(nx=70, ny=90, angle=25.0, b=0.25)]
    batch = ifx.Solver.batch([c for c, _, _ in specs], [x for _, x, _ in specs], [y for _, _, y in specs])
    assert batch.n_instances == 3
    batch.step(3)
    for k, (c, x, y) in enumerate(specs):
        alone = ifx.Solver.create(c, x, y)
        alone.step(3)
        for f in (capi.FIELD_U, capi.FIELD_V, capi.FIELD_P):
            assert np.array_equal(batch.get(f, inst=k), alone.get(f)), (k, f)
        assert batch.stats(k).last_ppe_iters == alone.stats().last_ppe_iters


def test_mixed_precision_close_to_fp64():
    cfg64, xf, yf = small_cylinder()
    cfg32, _, _ = small_cylinder(prec=capi.PREC_MIXED)
    a = ifx.Solver.create(cfg64, xf, yf)
    b = ifx.Solver.create(cfg32, xf, yf)
    a.step(5)
    b.step(5)
    for f in (capi.FIELD_U, capi.FIELD_V):
        ua, ub = a.get(f), b.get(f)
        assert np.linalg.norm(ub - ua) / np.linalg.norm(ua) <= 1e-6, f
    cda, cdb = a.stats().cd, b.stats().cd
    assert abs(cda - cdb) <= 1e-3 * abs(cda)


def test_mixed_precision_long_run_forces():
    """Over 300 steps from the impulsive start, every step's drag and lift
    (device-side force history) stay within 1e-3 of plain FP64 and the velocity
    within 1e-6 relative L2: the FP32 sweeps' error does not accumulate."""
    hist, vel = {}, {}
    for prec in (capi.PREC_FP64, capi.PREC_MIXED):
        cfg, xf, yf = small_cylinder(prec=prec)
        s = ifx.Solver.create(cfg, xf, yf)
        s.set_history(300)
        s.step(300)
        hist[prec] = s.history(cap=300)
        vel[prec] = np.concatenate([s.get(capi.FIELD_U).ravel(), s.get(capi.FIELD_V).ravel()])
    h6, hm = hist[capi.PREC_FP64], hist[capi.PREC_MIXED]
    assert h6.shape[0] == 300 and np.array_equal(h6[:, 0], hm[:, 0])
    scale = np.max(np.abs(h6[:, 1]))
    assert np.max(np.abs(hm[:, 1] - h6[:, 1]) / np.abs(h6[:, 1])) <= 1e-3
    assert np.max(np.abs(hm[:, 2] - h6[:, 2])) <= 1e-3 * scale
    v6, vm = vel[capi.PREC_FP64], vel[capi.PREC_MIXED]
    assert np.linalg.norm(vm - v6) / np.linalg.norm(v6) <= 1e-6


@pytest.mark.parametrize("nx,ny", [(48, 200), (240, 40)])
def test_anisotropic_grid_semicoarsening_vs_oracle(oracle, nx, ny):
    """Cells up to ~6:1 use semi-coarsened multigrid levels; same hierarchy,
    iterations and fields as the oracle."""
    cfg, xf, yf = cases.external(nx, ny, 12.0, 8.0, 4.0, 4.0, 0.5, 0.3, 10.0, 120.0, 5e-3, capi.PREC_FP64,
                                 ratio=4.0, width=1.0)
    s = ifx.Solver.create(cfg, xf, yf)
    o = oracle.method(cfg, xf, yf)
    for _ in range(2):
        s.step(1)
        o.step(1)
        assert abs(s.stats().last_ppe_iters - o.stats().last_ppe_iters) <= 1
        assert s.stats().last_ppe_iters <= 16
    _compare(s, o, tol=1e-9)


@pytest.mark.parametrize("prec", [capi.PREC_FP64, capi.PREC_MIXED])
@pytest.mark.parametrize("nx,ny", [(96, 64), (256, 160)])
def test_cluster_vcycle_bit_identical(prec, nx, ny):
    """The V-cycle on one thread-block cluster (levels in distributed shared
    memory) gives the tile path's result bit for bit."""
    spec = small_cylinder(prec=prec, nx=nx, ny=ny)
    a = _run_mode("graph", [spec], 3)
    os.environ["IFX_EXEC"] = "graph"
    try:
        b = ifx.Solver.create(*spec)
        available, _ = b.cluster_vcycle()
        if not available:
            pytest.skip("cluster V-cycle does not fit this case on this device")
        b.set_cluster_vcycle(True)
        assert b.cluster_vcycle() == (True, True)
        b.step(3)
    finally:
        del os.environ["IFX_EXEC"]
    for f in (capi.FIELD_U, capi.FIELD_V, capi.FIELD_P, capi.FIELD_UF):
        assert np.array_equal(a.get(f), b.get(f)), f
    assert a.stats().last_ppe_iters == b.stats().last_ppe_iters


def test_nan_in_one_batch_slot_leaves_the_others_unaffected():
    """Fault injection on the host side: a NaN planted in one instance's state.
    That instance is reported diverged and retired; the others continue and
    equal the same instances run alone, bit for bit."""
    specs = [small_cylinder(nx=96, ny=64), cases.cavity(n=40), small_cylinder(nx=70, ny=90, angle=25.0, b=0.25)]
    batch = ifx.Solver.batch([c for c, _, _ in specs], [x for _, x, _ in specs], [y for _, _, y in specs])
    batch.step(1)
    u = batch.get(capi.FIELD_U, inst=1)
    u[5, 7] = np.nan
    batch.set(capi.FIELD_U, u, inst=1)
    with pytest.raises(ifx.IFXError) as e:
        batch.step(1)
    assert e.value.status == capi.IFX_ERR_DIVERGED
    assert batch.stats(1).status == capi.IFX_ERR_DIVERGED
    assert batch.stats(0).status == capi.IFX_OK and batch.stats(2).status == capi.IFX_OK
    batch.step(2)  # the retired instance no longer stops the batch
    for k in (0, 2):
        alone = ifx.Solver.create(*specs[k])
        alone.step(4)
        for f in (capi.FIELD_U, capi.FIELD_V, capi.FIELD_P):
            assert np.array_equal(batch.get(f, inst=k), alone.get(f)), (k, f)


def test_pressure_iteration_cap_is_reported():
    cfg, xf, yf = small_cylinder()
    cfg.ppe_itermax = 1
    s = ifx.Solver.create(cfg, xf, yf)
    s.step(1)
    assert s.stats().status == capi.IFX_ERR_NOT_CONVERGED
    assert s.stats().last_ppe_iters == 1
    s.step(1)  # a warning: the steps go on
    assert np.all(np.isfinite(s.get(capi.FIELD_U)))


@pytest.mark.parametrize("nx,ny", [(17, 13), (12, 20), (33, 9)])
@pytest.mark.parametrize("prec", [capi.PREC_FP64, capi.PREC_MIXED])
def test_small_uneven_grids_vs_oracle(oracle, nx, ny, prec):
    """Small uneven grids (partial tiles, two- and three-level hierarchies, the
    coarsest level straight after the finest): every tile edge and the
    sub-cycle bounds are exercised.  FP64 against the oracle to 1e-10; the mixed
    path against the oracle to the mixed tolerance."""
    cfg, xf, yf = cases.cavity(n=nx)
    cfg.ny = ny
    cfg.ly = 1.0 * ny / nx
    yf = cases.uniform_faces(ny, cfg.ly)
    cfg.precision = prec
    s = ifx.Solver.create(cfg, xf, yf)
    ocfg, _, _ = cases.cavity(n=nx)
    ocfg.ny, ocfg.ly = cfg.ny, cfg.ly
    o = oracle.method(ocfg, xf, yf)
    s.step(4)
    o.step(4)
    assert np.all(np.isfinite(s.get(capi.FIELD_U)))
    tol = FIELD_RTOL if prec == capi.PREC_FP64 else 1e-6
    _compare(s, o, tol=tol)
    if prec == capi.PREC_FP64:
        assert s.stats().last_ppe_iters == o.stats().last_ppe_iters


@pytest.mark.gpu
def test_state_transfer_matches_field_calls(golden_dir):
    """ifx_set_state / ifx_get_state move u, v, p like the per-field calls."""
    specs = [cases.cylinder(nx=96, ny=64, precision=capi.PREC_MIXED),
             cases.cylinder(nx=64, ny=48, precision=capi.PREC_MIXED)]
    s = ifx.Solver.batch([c for c, _, _ in specs], [x for _, x, _ in specs], [y for _, _, y in specs])
    s.step(3)
    for inst in (0, 1):
        ref = [s.get(f, inst) for f in (capi.FIELD_U, capi.FIELD_V, capi.FIELD_P)]
        for a, b in zip(ref, s.get_state(inst)):
            assert np.array_equal(a, b)
        rng = np.random.default_rng(inst)
        new = [rng.standard_normal(a.shape) for a in ref]
        s.set_state(new[0], None, new[2], inst)  # v kept
        assert np.array_equal(s.get(capi.FIELD_U, inst), new[0])
        assert np.array_equal(s.get(capi.FIELD_V, inst), ref[1])
        assert np.array_equal(s.get(capi.FIELD_P, inst), new[2])
    # REFERENCE mode (dense device arrays): the reference's own inputs
    c = ifx.config_read(os.path.join(golden_dir, "inputs", "inputs.txt"))
    xf = ifx.grid_read(c.xgrid.decode(), c.nx + 1)
    yf = ifx.grid_read(c.ygrid.decode(), c.ny + 1)
    r = ifx.Solver.create(c, xf, yf)
    r.step(2)
    ref = [r.get(f) for f in (capi.FIELD_U, capi.FIELD_V, capi.FIELD_P)]
    for a, b in zip(ref, r.get_state()):
        assert np.array_equal(a, b)
    r.set_state(None, None, ref[2] + 1.0)
    assert np.array_equal(r.get(capi.FIELD_P), ref[2] + 1.0)


@pytest.mark.parametrize("mode", ["persistent", "graph", "host"])
def test_step_state_equals_separate_calls(mode):
    """ifx_step_state (state in, steps, state out, one wait) gives what
    ifx_set_state + ifx_step + ifx_get_state give, in every execution mode,
    also with the same buffers for input and output."""
    c, x, y = small_cylinder(prec=capi.PREC_MIXED)
    os.environ["IFX_EXEC"] = mode
    try:
        a, b = ifx.Solver.create(c, x, y), ifx.Solver.create(c, x, y)
    finally:
        del os.environ["IFX_EXEC"]
    a.step(2)
    b.step(2)
    nx, ny = a.grid_dims()
    state = [f.ravel().copy() for f in a.get_state()]
    state[0] += 1e-3 * np.sin(np.arange(nx * ny))  # a perturbed velocity passed in
    for _ in range(3):
        a.set_state(*state)
        a.step(2)
        ra = [f.ravel().copy() for f in a.get_state()]
        buf = tuple(s.copy() for s in state)
        rb = b.step_state(*buf, n=2, out=buf)  # in place
        for u, w in zip(ra, rb):
            assert np.array_equal(u, w.ravel())
        assert a.stats().last_ppe_iters == b.stats().last_ppe_iters
        state = ra
    # u, v, p back to back in one allocation (one copy each way), against the separate calls
    big = np.concatenate(state)
    views = tuple(big[k * nx * ny:(k + 1) * nx * ny] for k in range(3))
    a.set_state(*state)
    a.step(1)
    ra = [f.ravel().copy() for f in a.get_state()]
    b.step_state(*views, n=1, out=views)
    for u, w in zip(ra, views):
        assert np.array_equal(u, w)
    got = tuple(np.zeros(nx * ny) for _ in range(3))
    b.set_state(*views)  # contiguous in, separate out
    b.get_state(out=got)
    assert all(np.array_equal(u, w) for u, w in zip(views, got))
    state = ra
    # outputs only, and inputs only
    out = tuple(np.zeros(nx * ny) for _ in range(3))
    assert b.step_state(None, None, None, n=0, out=out) is not None
    assert all(np.array_equal(u, w) for u, w in zip(state, out))
    assert b.step_state(*state, n=1) is None
