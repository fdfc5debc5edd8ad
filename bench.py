#!/usr/bin/env python3
"""Benchmark: Mcell-updates/s of the fractional step on one GB300.

Workload (one "step" = one full time step: predictor, pressure solve to
||r|| <= 1e-8 ||b||, projection, ghost refresh, drag/lift):
  flow past a circular cylinder, D=1 at (10,10) in a 30x20 domain,
  tanh-stretched 384x256 grid, uniform inflow u=1, convective outflow,
  slip top/bottom, Re=100, dt=5e-3, ghost-cell immersed boundary.
Synthetic: the grid and the impulsively started flow are generated here.

value     : interior cells x steps / device time of the timed steps (CUDA
            events on the solver's stream), mixed precision (FP32 multigrid
            inside FP64 BiCGSTAB), L2 flushed before every step;
e2e       : same metric through the C ABI with the state copied from pinned
            host buffers and the result copied back every step, wall clock;
plain_fp64: the same steps with every kernel in FP64;
roofline  : the step's kernels as the autotuner runs them (one CUDA-graph
            launch per step, or the persistent per-step kernel); achieved =
            algorithmic bytes of the step / its event time; traffic = the DRAM
            bytes of one warm-cache step from the committed ncu launch list.
            Algorithmic bytes per interior cell (s = 4 B FP32 multigrid
            word, state words 8 B, stencil byte 1 B):
              convection+AB2 rhs 81, predictor sweep 49 (x sweeps),
              faces+source 41, BiCGSTAB start 49, projection 81,
              per BiCGSTAB iteration 2 V-cycles x (15.25 s + 6) x 4/3
              (coarse levels) + 2 applies x (s + 25) + updates 33 + s + 25 +
              s + 65;
            phase_roofline times the finest-level smoothing sweep alone;
cpu_baseline: the CPU oracle (same scheme, FP64, all host threads);
batched   : the batched sweep (256 seeded instances of uneven grid, Re and
            ellipse, one batched solver each for mixed and plain FP64,
            execution mode picked by the autotuner), Mcell-updates/s, solves/s
            of 500-step runs, error of mixed vs FP64 per instance;
ellipse   : the large single-instance configuration (1024x768 ellipse,
            Re 300), autotuned, mixed and plain FP64;
long_run_accuracy: the cylinder over 1000 steps in both precisions: largest
            drag and lift deviation of any step, velocity error at the end;
moving_body: the cylinder heaving (prescribed motion, geometry redone on the
            device every step), mixed and plain FP64, beside the cylinder at rest;
reference_path: the REFERENCE-mode step (the reference's own scheme) at 52^2,
            130^2 and 514^2 cells, GPU and one CPU thread;
served    : a seeded Poisson request stream through the continuous-batching
            server (real-time arrivals, cohorts admitted by device memory),
            solves/s, Mcell-updates/s and p50/p99 latency, the two smallest
            requests re-run alone in FP64 for the error; the same stream
            served in plain FP64 (served.fp64), and both precisions with every
            request arriving at t = 0 (served.capacity: the server's
            throughput, mixed over FP64).

--impl reference times the CPU restatement of the reference scheme (the
reference's pressure solver does not compile and it has no projection or
immersed boundary) on the same workload.
Under torchrun with N>1 every rank advances its own replica (weak scaling,
no collective on the data path).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mcell-updates/s"
WORKLOAD = "cylinder D=1, 30x20 domain, 384x256 tanh-stretched, Re=100, dt=5e-3, ghost-cell IBM"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--batch", type=int, default=256, help="instances of the batched sweep (0: skip)")
    ap.add_argument("--batch-steps", type=int, default=5)
    ap.add_argument("--serve", type=int, default=48, help="requests of the served stream (0: skip)")
    ap.add_argument("--rate", type=float, default=16.0, help="served stream arrival rate [1/s]")
    ap.add_argument("--profile", default=None, choices=["mixed", "fp64"],
                    help="profiler driver: warm-up steps, then --steps steps inside the NVTX range 'step', no output")
    ap.add_argument("--profile-workload", default="cylinder", choices=["cylinder", "batch", "moving"],
                    help="workload of --profile: the cylinder, the cylinder heaving (moving), or the batched sweep of --batch instances")
    ap.add_argument("--profile-rows", type=int, default=1, choices=[1, 4],
                    help="rows per thread of the multigrid tile phases under --profile")
    return ap.parse_args()


def dist_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def max_over_ranks(x, world, device="cuda"):
    """Largest x over the ranks: each rank times its own replica and the job
    ends with the slowest one.  With one rank, x itself."""
    if world == 1:
        return float(x)
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.path = tempfile.mktemp(suffix=".csv")
        self.p = None

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait()
        self.f.close()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            t = [x.strip() for x in line.split(",")]
            if len(t) < 9:
                continue
            try:
                sm.append(float(t[1]))
                smax = float(t[2])
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if t[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def committed_traffic(persistent):
    """DRAM bytes per step of the cylinder step from the committed ncu summary:
    the persistent kernel's launch, or the sum over the step's kernels."""
    name = "persist_step_cylinder_384x256.md" if persistent else "launch_list_cylinder_384x256_host.md"
    key = "traffic_bytes_per_launch:" if persistent else "traffic_bytes_per_step:"
    try:
        for line in open(os.path.join(ROOT, "profiles", name)):
            if line.startswith(key):
                return float(line.split(":")[1])
    except Exception:
        pass
    return None


def cell_step_bytes(ad_iters, ppe_iters, mixed):
    """Algorithmic bytes per interior cell of one time step (stencil byte 1 B).

    s: multigrid word, k: Krylov vector word (4/4 mixed, 8/8 plain FP64); the
    state (u, v, U, V, p, b, history) is FP64.  Convection + AB2 rhs 81,
    faces + source 41, BiCGSTAB start 16 + 4k + 1, projection 81; predictor
    sweep 49 (FP64) or 25 + 89/8 (FP32 sweep on the correction plus the FP64
    refresh every 8 sweeps); per BiCGSTAB iteration 2 V-cycles x
    (15.25 s + 6) x 4/3 (coarse levels), 2 applies x (s + 3k + 1), direction
    4k + s + 1, s-update 3k + s + 1, iterate update 16 + 6k + 1; the mixed
    path adds about two FP64 restarts (16 + 4k + 1 each) per step.
    """
    s = k = 4 if mixed else 8
    v = 15.25 * s + 6.0
    per_it = 2 * v * 4.0 / 3.0 + 2 * (s + 3 * k + 1) + (4 * k + s + 1) + (3 * k + s + 1) + (16 + 6 * k + 1)
    pred = 25 + 89 / 8 if mixed else 49
    start = 16 + 4 * k + 1
    restarts = 2 * start if mixed else 0
    return 81 + pred * ad_iters + 41 + start + restarts + 81 + per_it * ppe_iters


def exec_name(s):
    mode = {0: "persistent", 1: "graph", 2: "host"}.get(s.exec_mode(), "?")
    rows = s.mg_tile_rows()
    cmg = s.cluster_vcycle()[1]
    return f"{mode}, multigrid tiles 32x{8 * rows}" + (", cluster V-cycle" if cmg else "") + " (autotuned)"


def rel_l2(a, b):
    return float(np.sqrt(np.sum((a - b) ** 2) / max(np.sum(b ** 2), 1e-300)))


def copy_cfg(cfg, precision):
    c = type(cfg).from_buffer_copy(cfg)
    c.precision = precision
    return c


def batched_sweep(ifx, capi, cases, n_inst, steps, warm, peak):
    """Batched sweep: n_inst uneven instances (seeded), mixed vs plain FP64, each
    advanced in one batch; execution mode chosen by the autotuner."""
    res, fields = {}, {}
    for name, prec in (("mixed", capi.PREC_MIXED), ("fp64", capi.PREC_FP64)):
        specs = cases.batch_sample(count=n_inst, seed=0, precision=prec)
        ncell = sum(c.nx * c.ny for c, _, _ in specs)
        s = ifx.Solver.batch([c for c, _, _ in specs], [x for _, x, _ in specs], [y for _, _, y in specs])
        s.step(max(1, warm - 2))
        mode, _ = s.autotune(steps=1)
        s.step(2)
        l0 = s.stats().kernel_launches
        s.step(steps)
        ms = s.last_step_ms()
        launches = s.stats().kernel_launches - l0
        its = [s.stats(k).last_ppe_iters for k in range(n_inst)]
        ads = [s.stats(k).last_ad_iters for k in range(n_inst)]
        # algorithmic bytes of the last timed step, per instance with its own iteration counts
        nbytes = sum(c.nx * c.ny * cell_step_bytes(a, p, prec == capi.PREC_MIXED)
                     for (c, _, _), a, p in zip(specs, ads, its))
        fields[name] = [(s.get(capi.FIELD_U, inst=k), s.get(capi.FIELD_V, inst=k), s.stats(k).cd) for k in range(n_inst)]
        res[name] = {"value": ncell * steps / (ms * 1e-3) / 1e6, "unit": METRIC, "ms_per_step": ms / steps,
                     "exec": {0: "persistent", 1: "graph"}.get(mode, str(mode)), "mg_tile_rows": s.mg_tile_rows(),
                     "gpu_launches": launches,
                     "ppe_iters_mean": float(np.mean(its)), "ppe_iters_max": int(max(its)),
                     "predictor_iters_max": int(max(ads)), "device_bytes": s.device_bytes(),
                     "roofline": {"bound": "hbm", "achieved": nbytes / (ms / steps * 1e-3) / 1e9, "unit": "GB/s",
                                  "bytes_per_step": nbytes, "peak": peak, "frac": nbytes / (ms / steps * 1e-3) / 1e9 / peak}}
        res["cells"] = ncell
        s.close()
    errs = [rel_l2(np.concatenate([um.ravel(), vm.ravel()]), np.concatenate([u6.ravel(), v6.ravel()]))
            for (um, vm, _), (u6, v6, _) in zip(fields["mixed"], fields["fp64"])]
    cds = [abs(cm - c6) / max(abs(c6), 1e-12) for (_, _, cm), (_, _, c6) in zip(fields["mixed"], fields["fp64"])]
    res.update({"workload": f"batched sweep: {n_inst} instances (seed 0), grids log-uniform 64x64..512x384, "
                            "Re U[50,300], ellipse aspect U[0.1,1], angle U[-30,30] deg",
                "instances": n_inst, "timed_steps": steps,
                "speedup_mixed_over_fp64": res["mixed"]["value"] / res["fp64"]["value"],
                "solves_per_s_500_steps": n_inst / (res["mixed"]["ms_per_step"] * 1e-3 * 500),
                "accuracy_vs_fp64": {"rel_l2_velocity_max": max(errs), "rel_l2_velocity_median": float(np.median(errs)),
                                     "cd_rel_err_max": max(cds)},
                "l2": "inputs larger than L2 (device_bytes)"})
    return res


def served_stream(ifx, capi, cases, nreq, rate, budget, prec, check=True, max_cohort=32):
    """Served stream through the continuous-batching server: seeded arrivals
    (Poisson at `rate` per second in real time, or all at t = 0 when rate is
    None: the server's capacity); latency = completion - arrival."""
    stream = cases.served_stream(nreq, rate or 1.0, seed=0, precision=prec, nmin=64, nmax=512, smin=20, smax=200)
    if rate is None:
        stream = [(0.0,) + tuple(r[1:]) for r in stream]
    srv = ifx.Server(budget, max_cohort=max_cohort)
    arr, done, work, spec_of = {}, {}, 0, {}
    t0 = time.perf_counter()
    i = 0
    ticks = 0
    peak_cohorts = 0
    while len(done) < nreq:
        now = time.perf_counter() - t0
        while i < nreq and stream[i][0] <= now:
            t_arr, cfg, xf, yf, n = stream[i]
            rid = srv.submit(cfg, xf, yf, n)
            arr[rid] = t_arr
            spec_of[rid] = (cfg, xf, yf, n)
            work += cfg.nx * cfg.ny * n
            i += 1
        info = srv.info()
        if info["running"] == 0 and info["waiting"] == 0:
            if i < nreq:
                time.sleep(max(0.0, stream[i][0] - (time.perf_counter() - t0)))
            continue
        srv.tick()
        ticks += 1
        peak_cohorts = max(peak_cohorts, srv.info()["cohorts"])
        tnow = time.perf_counter() - t0
        for rid in srv.poll():
            done[rid] = tnow
    lat = np.array([done[r] - arr[r] for r in arr]) * 1e3
    span = max(done.values()) - stream[0][0]
    out = {"workload": f"served stream: {nreq} requests (seed 0), "
                       + (f"Poisson arrivals at {rate}/s" if rate else "all arriving at t = 0 (capacity)")
                       + ", cylinder or ellipse, grids log-uniform 64^2..512^2, Re U[50,1000], 20..200 steps each",
           "requests": nreq, "solves_per_s": nreq / span, "value": work / span / 1e6, "unit": METRIC,
           "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                          "max": float(lat.max())},
           "ticks": ticks, "peak_cohorts": peak_cohorts, "hbm_budget_bytes": budget,
           "precision": "mixed" if prec == capi.PREC_MIXED else "fp64"}
    if check:
        # accuracy: the two smallest requests re-run alone in plain FP64
        small = sorted(arr, key=lambda r: spec_of[r][0].nx * spec_of[r][0].ny)[:2]
        errs = []
        for r in small:
            cfg, xf, yf, n = spec_of[r]
            s = ifx.Solver.create(copy_cfg(cfg, capi.PREC_FP64), xf, yf)
            s.step(n)
            a = np.concatenate([srv.result(r, capi.FIELD_U).ravel(), srv.result(r, capi.FIELD_V).ravel()])
            b = np.concatenate([s.get(capi.FIELD_U).ravel(), s.get(capi.FIELD_V).ravel()])
            errs.append(rel_l2(a, b))
            s.close()
        out["accuracy_vs_fp64"] = {"rel_l2_velocity_max": max(errs), "requests_checked": len(errs)}
    srv.close()
    return out


def served_lines(ifx, capi, cases, nreq, rate, budget):
    """The Poisson stream (latency) and the all-at-once stream (capacity), each
    served in mixed precision and in plain FP64."""
    res = served_stream(ifx, capi, cases, nreq, rate, budget, capi.PREC_MIXED)
    res["fp64"] = served_stream(ifx, capi, cases, nreq, rate, budget, capi.PREC_FP64, check=False)
    cap = {"mixed": served_stream(ifx, capi, cases, nreq, None, budget, capi.PREC_MIXED, check=False),
           "fp64": served_stream(ifx, capi, cases, nreq, None, budget, capi.PREC_FP64, check=False)}
    cap["speedup_mixed_over_fp64"] = cap["mixed"]["value"] / cap["fp64"]["value"]
    res["capacity"] = cap
    return res


def long_run_accuracy(ifx, capi, cases, steps=1000):
    """Mixed against plain FP64 over a long run of the cylinder (1000 steps, t = 5,
    the impulsive start and the growth of the wake): the drag and lift of every
    step from the device-side force history, and the velocity at the end."""
    hist, fields = {}, {}
    for name, prec in (("mixed", capi.PREC_MIXED), ("fp64", capi.PREC_FP64)):
        cfg, xf, yf = cases.cylinder(precision=prec)
        s = ifx.Solver.create(cfg, xf, yf)
        s.set_history(steps)
        s.step(steps)
        hist[name] = s.history(cap=steps)
        fields[name] = np.concatenate([s.get(capi.FIELD_U).ravel(), s.get(capi.FIELD_V).ravel()])
        s.close()
    hm, h6 = hist["mixed"], hist["fp64"]
    cd_err = float(np.max(np.abs(hm[:, 1] - h6[:, 1]) / np.maximum(np.abs(h6[:, 1]), 1e-12)))
    cl_err = float(np.max(np.abs(hm[:, 2] - h6[:, 2])) / max(float(np.max(np.abs(h6[:, 1]))), 1e-12))
    return {"workload": f"cylinder 384x256, Re 100, {steps} steps from the impulsive start, mixed vs plain FP64",
            "steps": steps, "rel_l2_velocity_final": rel_l2(fields["mixed"], fields["fp64"]),
            "cd_rel_err_max": cd_err, "cl_err_max_rel_to_cd": cl_err,
            "cd_final": float(h6[-1, 1]), "cl_final": float(h6[-1, 2])}


def ellipse_line(ifx, capi, cases, steps=10):
    """The large single-instance configuration: ellipse of aspect 0.2 and chord
    1 at 10 deg, 1024x768 cells on a 20x12 domain, Re 300, dt 2e-3; autotuned,
    mixed and plain FP64 (device time, CUDA events)."""
    out = {"workload": "ellipse aspect 0.2, chord 1, 10 deg, 20x12 domain, 1024x768 tanh-stretched, Re 300, dt 2e-3",
           "unit": METRIC, "steps": steps}
    fields = {}
    for name, prec in (("mixed", capi.PREC_MIXED), ("fp64", capi.PREC_FP64)):
        cfg, xf, yf = cases.ellipse(precision=prec)
        s = ifx.Solver.create(cfg, xf, yf)
        s.step(1)
        s.autotune(steps=1)
        s.step(2)
        s.step(steps)
        ms = s.last_step_ms()
        st = s.stats()
        out[name] = {"value": cfg.nx * cfg.ny * steps / (ms * 1e-3) / 1e6, "ms_per_step": ms / steps,
                     "execution": exec_name(s), "ppe_iters_last": st.last_ppe_iters,
                     "predictor_iters_last": st.last_ad_iters, "cd": st.cd}
        fields[name] = np.concatenate([s.get(capi.FIELD_U).ravel(), s.get(capi.FIELD_V).ravel()])
        s.close()
    out["speedup_mixed_over_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    out["rel_l2_velocity_vs_fp64"] = rel_l2(fields["mixed"], fields["fp64"])
    return out


def moving_line(ifx, capi, cases, steps=50):
    """A body in prescribed motion: the cylinder configuration (384x256, Re 100,
    dt 5e-3) heaving with amplitude 0.25 D at frequency 0.2, its geometry redone
    on the device every step; mixed and plain FP64, and the same cylinder at
    rest for the cost of the per-step geometry (device time, CUDA events)."""
    out = {"workload": "cylinder D=1, 30x20 domain, 384x256 tanh-stretched, Re 100, dt 5e-3, "
                       "heaving y = 0.25 sin(2 pi 0.2 t)", "unit": METRIC, "steps": steps}
    fields = {}
    for name, prec, moving in (("mixed", capi.PREC_MIXED, True), ("fp64", capi.PREC_FP64, True),
                               ("mixed_at_rest", capi.PREC_MIXED, False)):
        cfg, xf, yf = cases.cylinder(precision=prec)
        if moving:
            cases.set_motion(cfg, amp_y=0.25, freq=0.2)
        s = ifx.Solver.create(cfg, xf, yf)
        s.step(1)
        s.autotune(steps=1)
        s.step(2)
        s.step(steps)
        ms = s.last_step_ms()
        st = s.stats()
        out[name] = {"value": cfg.nx * cfg.ny * steps / (ms * 1e-3) / 1e6, "ms_per_step": ms / steps,
                     "execution": exec_name(s), "ppe_iters_last": st.last_ppe_iters, "cd": st.cd, "cl": st.cl,
                     "ibm_ghosts": st.n_ibm_ghost}
        if moving:
            fields[name] = np.concatenate([s.get(capi.FIELD_U).ravel(), s.get(capi.FIELD_V).ravel()])
        s.close()
    out["speedup_mixed_over_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    out["rel_l2_velocity_vs_fp64"] = rel_l2(fields["mixed"], fields["fp64"])
    out["motion_overhead_ms_per_step"] = out["mixed"]["ms_per_step"] - out["mixed_at_rest"]["ms_per_step"]
    return out


def reference_path(ifx, capi, cases, steps=20, cpu=True):
    """The REFERENCE-mode time step (the reference's ADsolver: vortex IC,
    explicit convection, backward-Euler diffusion by Jacobi to the L1 stop rule,
    src/include/ADSolver.cu:268-395) on uniform unit-square grids of 52^2, 130^2
    and 514^2 cells (ghosts included), Re 150, dt 1e-3, AD_itermax 25: GPU time
    (CUDA events) beside the CPU restatement of the same scheme (one thread)."""
    lines = []
    for n in (50, 128, 512):
        c = ifx.default_config()
        c.nx = c.ny = n
        c.lx = c.ly = 1.0
        xf = cases.uniform_faces(n, 1.0)
        s = ifx.Solver.create(c, xf, xf)
        s.step(2)
        s.step(steps)
        ms = s.last_step_ms()
        st = s.stats()
        line = {"grid": [n + 2, n + 2], "steps": steps, "gpu_value": n * n * steps / (ms * 1e-3) / 1e6,
                "gpu_ms_per_step": ms / steps, "jacobi_iterations_last_step": st.last_ad_iters}
        if cpu:
            sys.path.insert(0, os.path.join(ROOT, "tests"))
            import _oracle

            o = _oracle.Oracle()
            k = steps if n <= 128 else 4
            t0 = time.perf_counter()
            o.ref_ad(xf, xf, 1e-3, 150.0, 25, k)
            dt = time.perf_counter() - t0
            line.update({"cpu_value": n * n * k / dt / 1e6, "cpu_steps": k, "cpu_cores": 1})
        lines.append(line)
        s.close()
    return {"workload": "REFERENCE mode (the reference's ADsolver step), uniform grids on [0,1]^2, "
                        "vortex IC, Re 150, dt 1e-3, AD_itermax 25",
            "unit": METRIC, "lines": lines,
            "note": "the reference's own CUDA executable builds from its sources, which are not present on "
                    "the GPU host; this is the drop-in REFERENCE mode on the same scheme"}


def cpu_oracle_run(cfg, xf, yf, seconds, min_steps=3, warm=1, nthreads=None):
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import _oracle

    nthreads = nthreads or os.cpu_count() or 1
    o = _oracle.Oracle().method(cfg, xf, yf, nthreads)
    o.step(warm)
    n = 0
    t0 = time.perf_counter()
    while n < min_steps or time.perf_counter() - t0 < seconds:
        o.step(1)
        n += 1
    dt = time.perf_counter() - t0
    return n, dt, nthreads


def main():
    args = parse()
    rank, world, local = dist_info()
    import numpy as np

    from immerseflow_gb300 import _capi as capi
    from immerseflow_gb300 import cases

    cfg_m, xf, yf = cases.cylinder(precision=capi.PREC_MIXED)
    cells = cfg_m.nx * cfg_m.ny

    if args.impl == "reference":
        if rank != 0:
            return 0
        cfg64, _, _ = cases.cylinder(precision=capi.PREC_FP64)
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        import _oracle

        nth = os.cpu_count() or 1
        o = _oracle.Oracle().method(cfg64, xf, yf, nth)
        o.step(args.warmup)
        t0 = time.perf_counter()
        o.step(args.steps)
        dt = time.perf_counter() - t0
        val = cells * args.steps / dt / 1e6
        line = {"metric": METRIC, "value": val, "unit": METRIC, "impl": "reference", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": WORKLOAD, "grid": [384, 256], "solver": "CPU restatement (oracle), FP64"},
                "cpu_baseline": {"value": val, "unit": METRIC, "cores": nth, "kind": "port",
                                 "sample": f"{args.steps} time steps after {args.warmup} warm-up steps"},
                "e2e": {"value": val, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return 0

    import torch

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group(backend="nccl", device_id=torch.device("cuda", local))

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    import immerseflow_gb300 as ifx

    if args.profile:
        prec = capi.PREC_MIXED if args.profile == "mixed" else capi.PREC_FP64
        if args.profile_workload == "batch":
            specs = cases.batch_sample(count=args.batch, seed=0, precision=prec)
            s = ifx.Solver.batch([c for c, _, _ in specs], [x for _, x, _ in specs], [y for _, _, y in specs])
        else:
            cfg, _, _ = cases.cylinder(precision=prec)
            if args.profile_workload == "moving":  # heaving as in the moving_body line
                cases.set_motion(cfg, amp_y=0.25, freq=0.2)
            s = ifx.Solver.create(cfg, xf, yf)
        s.set_mg_tile_rows(args.profile_rows)
        s.step(args.warmup)
        s.synchronize()
        torch.cuda.nvtx.range_push("step")
        s.step(args.steps)
        s.synchronize()
        torch.cuda.nvtx.range_pop()
        return 0

    flush_buf = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")

    def flush():
        flush_buf.zero_()
        torch.cuda.synchronize()

    def step_bytes(st, sword):
        return cells * cell_step_bytes(st.last_ad_iters, st.last_ppe_iters, sword == 4)

    def timed(prec):
        cfg, _, _ = cases.cylinder(precision=prec)
        s = ifx.Solver.create(cfg, xf, yf)
        s.step(1)
        s.autotune(steps=2)  # execution mode and tile shape; the state is restored afterwards
        for _ in range(args.warmup):
            flush()
            s.step(1)
        l0 = s.stats().kernel_launches
        barrier()
        clk = Clocks(local)
        clk.start()
        ms, nbytes, pits, adits = [], 0.0, [], []
        sword = 4 if prec == capi.PREC_MIXED else 8
        for _ in range(args.steps):
            flush()
            s.step(1)
            ms.append(s.last_step_ms())
            st = s.stats()
            nbytes += step_bytes(st, sword)
            pits.append(st.last_ppe_iters)
            adits.append(st.last_ad_iters)
        clocks = clk.stop()
        barrier()
        total = sum(ms)
        launches = s.stats().kernel_launches - l0
        return s, total, launches, clocks, nbytes, pits, adits

    s, total_ms, launches, clocks, step_bytes_total, pits, adits = timed(capi.PREC_MIXED)
    st = s.stats()
    u_m, v_m = s.get(capi.FIELD_U), s.get(capi.FIELD_V)
    cd_m, cl_m = st.cd, st.cl
    total_ms = max_over_ranks(total_ms, world)
    value = world * cells * args.steps / (total_ms * 1e-3) / 1e6

    # plain FP64 path on the same steps
    s64, total64, launches64, _, _, pits64, _ = timed(capi.PREC_FP64)
    total64 = max_over_ranks(total64, world)
    st64 = s64.stats()
    u64, v64 = s64.get(capi.FIELD_U), s64.get(capi.FIELD_V)
    err_u = float(np.sqrt(np.sum((u_m - u64) ** 2 + (v_m - v64) ** 2) / np.sum(u64 ** 2 + v64 ** 2)))
    err_cd = abs(cd_m - st64.cd) / abs(st64.cd)
    value64 = world * cells * args.steps / (total64 * 1e-3) / 1e6

    # end to end through the C ABI: pinned host state in, result out, every step
    nx, ny = s.grid_dims()
    host = {f: torch.empty(nx * ny, dtype=torch.float64, pin_memory=True).numpy() for f in (capi.FIELD_U, capi.FIELD_V, capi.FIELD_P)}
    for f, a in host.items():
        a[:] = s.get(f).ravel()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for f, a in host.items():
            s.set(f, a)
        s.step(1)
        for f, a in host.items():
            lib_out = s.get(f).ravel()
            a[:] = lib_out
    barrier()
    e2e_s = max_over_ranks(time.perf_counter() - t0, world)
    e2e = world * cells * args.steps / e2e_s / 1e6
    nbytes = 3 * nx * ny * 8

    # roofline of the dominant kernel: the per-step kernel (persistent mode)
    peak, peak_kind = measured_peak()
    persistent = s.exec_mode() == 0
    traffic = committed_traffic(persistent)
    achieved = step_bytes_total / (total_ms * 1e-3) / 1e9
    # one phase alone: the finest-level smoothing sweep, FP32 in the mixed path
    k_ms, k_cells = s.profile_kernel(0, reps=200)
    k_bw = k_cells * (3 * 4 + 1) / (k_ms * 1e-3) / 1e9
    try:
        bar_us = s.profile_kernel(4, reps=5)[0] * 1e3
    except Exception:
        bar_us = None

    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 multigrid + f64 BiCGSTAB/state", "data": "synthetic",
        "config": {"workload": WORKLOAD, "grid": [384, 256], "cells": cells, "parallelism": f"replicas x{world}",
                   "precision": "mixed", "ppe_tol": cfg_m.ppe_tol, "l2": "flushed before every timed step (256 MB write)",
                   "execution": exec_name(s)},
        "plain_fp64": {"value": value64, "ms_per_step": total64 / args.steps, "gpu_launches": launches64,
                       "execution": exec_name(s64),
                       "speedup_mixed_over_fp64": value / value64},
        "accuracy_vs_fp64": {"rel_l2_velocity": err_u, "cd_rel_err": err_cd, "cd": cd_m, "cd_fp64": st64.cd},
        "e2e": {"value": e2e, "unit": METRIC, "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "kernel": ("k_persist_step<float> (one launch per time step)" if persistent else
                                                "the step's kernels (one CUDA graph launch per time step)"),
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind, "traffic": traffic,
                     "bytes_per_launch": step_bytes_total / args.steps, "ms_per_launch": total_ms / args.steps,
                     "note": "working set ~30 MB is L2-resident; launch/barrier latency bound at this size"},
        "phase_roofline": {"kernel": "finest-level smoothing sweep as the step launches it (k_smooth_grid_tma<float>), launched alone", "bytes_per_cell": 13,
                           "cells_per_launch": k_cells, "ms_per_launch": k_ms, "achieved_gbs": k_bw,
                           "frac": k_bw / peak, "grid_barrier_us": bar_us},
        "iterations": {"ppe_mean": sum(pits) / len(pits), "predictor_mean": sum(adits) / len(adits),
                       "ppe_mean_fp64": sum(pits64) / len(pits64)},
        "clocks": clocks,
    }
    if args.batch > 0:
        line["batched"] = batched_sweep(ifx, capi, cases, args.batch, args.batch_steps, args.warmup, peak)
    if args.serve > 0:
        line["served"] = served_lines(ifx, capi, cases, args.serve, args.rate, 64 << 30)
    if rank == 0 and world == 1:
        line["ellipse"] = ellipse_line(ifx, capi, cases)
        line["long_run_accuracy"] = long_run_accuracy(ifx, capi, cases)
        line["moving_body"] = moving_line(ifx, capi, cases)
        line["reference_path"] = reference_path(ifx, capi, cases, cpu=not args.no_cpu)
    if rank == 0 and world == 1 and not args.no_cpu:
        cfg64, _, _ = cases.cylinder(precision=capi.PREC_FP64)
        n, dt, nth = cpu_oracle_run(cfg64, xf, yf, args.cpu_seconds)
        line["cpu_baseline"] = {"value": cells * n / dt / 1e6, "unit": METRIC, "cores": nth, "kind": "port",
                                "sample": f"{n} time steps of the same workload after 1 warm-up step ({dt:.1f} s)"}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
