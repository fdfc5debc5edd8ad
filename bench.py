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
            inside FP64 BiCGSTAB), L2 flushed before every step.  The timed
            steps are steps S+1..S+K of the run (--window-start S, default
            200): the configuration runs 5000 steps, and after the impulsive
            start's first ~100 steps (5-8 Krylov iterations a step) a step takes
            2; both arms time the same steps (transient: the first steps);
e2e       : same metric through the C ABI with the state copied from pinned
            host buffers and the result copied back every step, wall clock
            (ifx_step_state: copies in, the step and copies out in one call
            that waits once; three_calls_value: the same steps again, from
            a checkpoint, through ifx_set_state, ifx_step and ifx_get_state);
plain_fp64: the same steps with every kernel in FP64;
roofline  : the step's kernels as the autotuner runs them (one CUDA-graph
            launch per step, or the persistent per-step kernel); achieved =
            algorithmic bytes of the step / its event time; traffic = the DRAM
            bytes of one step (L2 flushed before it) summed over the committed
            ncu launch list of the step's kernels.
            Algorithmic bytes per interior cell (s = 4 B FP32 multigrid
            word, state words 8 B, stencil byte 1 B):
              convection+AB2 rhs 81, predictor guess 65, predictor sweep 49
              (x sweeps), faces+source+pressure extrapolation 121, BiCGSTAB
              start 49, projection 81,
              per BiCGSTAB iteration 2 V-cycles x (15.25 s + 6) x 4/3
              (coarse levels) + 2 applies x (s + 25) + updates 33 + s + 25 +
              s + 65;
            phase_roofline times the finest-level smoothing sweep alone;
cpu_baseline: the CPU oracle (same scheme, FP64, all host threads);
batched   : the batched sweep (256 seeded instances of uneven grid, Re and
            ellipse, one batched solver each for mixed and plain FP64,
            execution mode picked by the autotuner): Mcell-updates/s and
            roofline over the same window of steps in both precisions, error
            of mixed vs FP64 per instance, and solves/s measured over a full
            500-step mixed run (batched.solve);
ellipse   : the large single-instance configuration (1024x768 ellipse,
            Re 300), autotuned, mixed and plain FP64, timed over steps
            201-210 and over the transient steps 4-13, both against the CPU
            oracle after 13 steps (Linf velocity and divergence errors);
cavity    : the lid-driven cavity (128x128, Re 100, dt 1e-3, pressure to
            1e-8) over 2000 steps from rest, mixed and plain FP64, both against
            the CPU oracle after the same 2000 steps;
whole_run : the cylinder configuration's whole 5000-step run in both
            precisions, Mcell-updates/s over it, and mixed vs FP64: largest
            drag and lift deviation of any step, velocity error at the end;
transient : the same line over the impulsive start's steps 2+W..1+W+K;
moving_body: the cylinder heaving (prescribed motion, geometry redone on the
            device every step), mixed and plain FP64, beside the cylinder at rest;
reference_path: the REFERENCE-mode step (the reference's own scheme) at 52^2,
            130^2 and 514^2 cells, GPU and one CPU thread;
reference_cuda: the reference's own AD-only CUDA executable (oracle/_ref,
            built on this machine from the staged reference sources) on the
            same three grids, per-step wall time with its printing to a file
            and to /dev/null;
served    : the first 16 requests of the seeded served stream (cylinder or
            ellipse, grids log-uniform 64^2..1024^2, Re U[50,1000], 200..2000
            steps) through the continuous-batching server, Poisson arrivals at
            1/s in real time, cohorts admitted by device memory: solves/s,
            Mcell-updates/s and p50/p99 latency in mixed precision and in plain
            FP64 (served.fp64), every request's mixed velocity against its FP64
            result, and both precisions with every request arriving at t = 0
            (served.capacity: the server's throughput, mixed over FP64);
summary   : the headline figures of all blocks in a few hundred bytes, the
            last key of the line.

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
    ap.add_argument("--batch-solve-steps", type=int, default=500,
                    help="steps of the mixed batched run that solves/s is measured over")
    ap.add_argument("--serve", type=int, default=16, help="requests of the served stream (0: skip)")
    ap.add_argument("--rate", type=float, default=1.0, help="served stream arrival rate [1/s]")
    ap.add_argument("--cavity-steps", type=int, default=2000, help="steps of the cavity line (0: skip)")
    ap.add_argument("--window-start", type=int, default=200,
                    help="the timed steps of both arms are steps S+1..S+K of the run: S-W steps are advanced "
                         "untimed, then W warm-up steps (0: from the impulsive start, as the transient block)")
    ap.add_argument("--whole-run-steps", type=int, default=5000,
                    help="steps of the whole-run block (the cylinder configuration's 5000 steps; 0: skip)")
    ap.add_argument("--no-reference-build", action="store_true",
                    help="skip the timing of the reference's own CUDA executable")
    ap.add_argument("--profile", default=None, choices=["mixed", "fp64"],
                    help="profiler driver: warm-up steps, then --steps steps inside the NVTX range 'step', no output")
    ap.add_argument("--profile-workload", default="cylinder", choices=["cylinder", "batch", "moving", "ellipse"],
                    help="workload of --profile: the cylinder, the cylinder heaving (moving), the 1024x768 "
                         "ellipse, or the batched sweep of --batch instances")
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


def committed_traffic():
    """DRAM bytes of one cylinder step past the impulsive start (step 201, L2
    flushed before it, as before every timed step) from the committed ncu launch
    list of the step's kernels: the sum of dram__bytes_read.sum +
    dram__bytes_write.sum over its launches."""
    try:
        for line in open(os.path.join(ROOT, "profiles", "launch_list_cylinder_384x256_step201.md")):
            if line.startswith("traffic_bytes_per_step:"):
                return float(line.split(":")[1])
    except Exception:
        pass
    return None


def cell_step_bytes(ad_iters, ppe_iters, mixed):
    """Algorithmic bytes per interior cell of one time step (stencil byte 1 B).

    s: multigrid word, k: Krylov vector word (4/4 mixed, 8/8 plain FP64); the
    state (u, v, U, V, p, b, history) is FP64.  Convection + AB2 rhs 81,
    predictor initial guess 65 (u, v and their increments read and written),
    faces + source 121 (u, v in; U*, V*, b out; the pressure extrapolation's
    p, pold, pold2 and the predictor increments read and written), BiCGSTAB
    start 16 + 4k + 1, projection 81 (p, U*, V*, u, v in; U, V, u, v, div
    out); predictor
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
    return 81 + 65 + pred * ad_iters + 121 + start + restarts + 81 + per_it * ppe_iters


def exec_name(s, tuned=True):
    mode = {0: "persistent", 1: "graph", 2: "host"}.get(s.exec_mode(), "?")
    rows = s.mg_tile_rows()
    cmg = s.cluster_vcycle()[1]
    return f"{mode}, multigrid tiles 32x{8 * rows}" + (", cluster V-cycle" if cmg else "") + (" (autotuned)" if tuned else "")


def rel_l2(a, b):
    return float(np.sqrt(np.sum((a - b) ** 2) / max(np.sum(b ** 2), 1e-300)))


def copy_cfg(cfg, precision):
    c = type(cfg).from_buffer_copy(cfg)
    c.precision = precision
    return c


def batched_sweep(ifx, capi, cases, n_inst, steps, solve_steps, peak):
    """Batched sweep: n_inst uneven instances (seeded), mixed vs plain FP64, each
    advanced in one batch; execution mode chosen by the autotuner (which restores
    the state).  Both precisions time the same window (steps 11 .. 10 + steps
    from the impulsive start, past its first transient) for the rate and the
    roofline; the mixed batch then runs on to `solve_steps` steps, and solves/s
    is measured over that whole run (from step 1)."""
    res, fields = {}, {}
    for name, prec in (("mixed", capi.PREC_MIXED), ("fp64", capi.PREC_FP64)):
        specs = cases.batch_sample(count=n_inst, seed=0, precision=prec)
        ncell = sum(c.nx * c.ny for c, _, _ in specs)
        s = ifx.Solver.batch([c for c, _, _ in specs], [x for _, x, _ in specs], [y for _, _, y in specs])
        mode, _ = s.autotune(steps=1)
        sched, _ = s.autotune_schedule(steps=1)
        s.synchronize()
        w0 = time.perf_counter()
        s.step(10)
        ms_head = s.last_step_ms()
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
                     "schedule": sched.as_dict(),
                     "gpu_launches": launches,
                     "ppe_iters_mean": float(np.mean(its)), "ppe_iters_max": int(max(its)),
                     "predictor_iters_max": int(max(ads)), "device_bytes": s.device_bytes(),
                     "roofline": {"bound": "hbm", "achieved": nbytes / (ms / steps * 1e-3) / 1e9, "unit": "GB/s",
                                  "bytes_per_step": nbytes, "peak": peak, "frac": nbytes / (ms / steps * 1e-3) / 1e9 / peak}}
        if name == "mixed" and solve_steps > 10 + steps:
            s.step(solve_steps - 10 - steps)
            dev_ms = ms_head + ms + s.last_step_ms()
            s.synchronize()
            wall = time.perf_counter() - w0
            res["solve"] = {"steps": solve_steps, "device_s": dev_ms * 1e-3, "wall_s": wall,
                            "solves_per_s": n_inst / wall, "value": ncell * solve_steps / wall / 1e6,
                            "unit": METRIC, "all_finite": bool(all(np.isfinite(s.stats(k).cd) for k in range(n_inst)))}
        res["cells"] = ncell
        s.close()
    errs = [rel_l2(np.concatenate([um.ravel(), vm.ravel()]), np.concatenate([u6.ravel(), v6.ravel()]))
            for (um, vm, _), (u6, v6, _) in zip(fields["mixed"], fields["fp64"])]
    cds = [abs(cm - c6) / max(abs(c6), 1e-12) for (_, _, cm), (_, _, c6) in zip(fields["mixed"], fields["fp64"])]
    res.update({"workload": f"batched sweep: {n_inst} instances (seed 0), grids log-uniform 64x64..512x384, "
                            "Re U[50,300], ellipse aspect U[0.1,1], angle U[-30,30] deg",
                "instances": n_inst, "timed_steps": steps,
                "speedup_mixed_over_fp64": res["mixed"]["value"] / res["fp64"]["value"],
                "accuracy_vs_fp64": {"rel_l2_velocity_max": max(errs), "rel_l2_velocity_median": float(np.median(errs)),
                                     "cd_rel_err_max": max(cds), "after_steps": 10 + steps},
                "l2": "inputs larger than L2 (device_bytes)"})
    return res


def served_stream(ifx, capi, cases, nreq, rate, budget, prec, max_cohort=32, keep=False):
    """Served stream through the continuous-batching server: the first `nreq`
    requests of the seeded C5 stream (cylinder or ellipse, grids log-uniform
    64^2..1024^2, Re U[50,1000], 200..2000 steps), arriving in real time as a
    Poisson process at `rate` per second, or all at t = 0 when rate is None
    (the server's capacity); latency = completion - arrival.  With `keep`, the
    velocity and drag of every finished request are returned for the accuracy
    comparison."""
    stream = cases.served_stream(nreq, rate or 1.0, seed=0, precision=prec)
    if rate is None:
        stream = [(0.0,) + tuple(r[1:]) for r in stream]
    srv = ifx.Server(budget, max_cohort=max_cohort)
    arr, done, work, index = {}, {}, 0, {}
    kept = {}
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
            index[rid] = i
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
            if keep:
                st = srv.stats(rid)
                kept[index[rid]] = (np.concatenate([srv.result(rid, capi.FIELD_U).ravel(),
                                                    srv.result(rid, capi.FIELD_V).ravel()]), st.cd, st.cl)
            srv.release(rid)
    lat = np.array([done[r] - arr[r] for r in arr]) * 1e3
    span = max(done.values()) - stream[0][0]
    sizes = [c.nx for _, c, _, _, _ in stream]
    nsteps = [n for _, _, _, _, n in stream]
    out = {"workload": f"served stream: the first {nreq} requests of the seeded stream (seed 0) with grids "
                       "log-uniform 64^2..1024^2, Re U[50,1000], 200..2000 steps, cylinder or ellipse; "
                       + (f"Poisson arrivals at {rate}/s" if rate else "all arriving at t = 0 (capacity)"),
           "requests": nreq, "grid_range": [min(sizes), max(sizes)], "steps_range": [min(nsteps), max(nsteps)],
           "cell_steps": work, "solves_per_s": nreq / span, "value": work / span / 1e6, "unit": METRIC,
           "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                          "max": float(lat.max())},
           "ticks": ticks, "peak_cohorts": peak_cohorts, "hbm_budget_bytes": budget,
           "precision": "mixed" if prec == capi.PREC_MIXED else "fp64"}
    srv.close()
    return (out, kept) if keep else out


def served_lines(ifx, capi, cases, nreq, rate, budget):
    """The Poisson stream (latency) and the all-at-once stream (capacity), each
    served in mixed precision and in plain FP64.  Every request's mixed result
    is compared with its plain FP64 result (a request's result does not depend
    on its cohort, so the FP64 stream gives the FP64 answer of each request)."""
    res, km = served_stream(ifx, capi, cases, nreq, rate, budget, capi.PREC_MIXED, keep=True)
    res["fp64"], k6 = served_stream(ifx, capi, cases, nreq, rate, budget, capi.PREC_FP64, keep=True)
    errs = {k: rel_l2(km[k][0], k6[k][0]) for k in km}
    cds = {k: abs(km[k][1] - k6[k][1]) / max(abs(k6[k][1]), 1e-12) for k in km}
    big = max(km, key=lambda k: km[k][0].size)
    res["accuracy_vs_fp64"] = {"requests_checked": len(errs), "rel_l2_velocity_max": max(errs.values()),
                               "rel_l2_velocity_median": float(np.median(list(errs.values()))),
                               "cd_rel_err_max": max(cds.values()),
                               "largest_request": {"cells": km[big][0].size // 2, "rel_l2_velocity": errs[big]}}
    cap = {"mixed": served_stream(ifx, capi, cases, nreq, None, budget, capi.PREC_MIXED),
           "fp64": served_stream(ifx, capi, cases, nreq, None, budget, capi.PREC_FP64)}
    cap["speedup_mixed_over_fp64"] = cap["mixed"]["value"] / cap["fp64"]["value"]
    res["capacity"] = cap
    return res


def whole_run(ifx, capi, cases, steps=5000):
    """The cylinder configuration's whole run (5000 steps from the impulsive
    start, t = 25, the wake shedding) in both precisions, as a user runs it: the
    execution mode tuned after the first step, the default sweep schedule (the
    same in both precisions), then the remaining steps in one call, L2 not
    flushed between steps.  Mcell-updates/s over those steps (device time of
    the call), and mixed against plain FP64: the drag and lift of every step
    from the device-side force history, and the velocity at the end."""
    hist, fields, out = {}, {}, {}
    for name, prec in (("mixed", capi.PREC_MIXED), ("fp64", capi.PREC_FP64)):
        cfg, xf, yf = cases.cylinder(precision=prec)
        s = ifx.Solver.create(cfg, xf, yf)
        s.step(1)
        s.autotune(steps=2)  # execution mode and tile shape; the state is restored afterwards
        s.set_history(steps - 1)
        s.step(steps - 1)
        ms = s.last_step_ms()
        out[name] = {"value": cfg.nx * cfg.ny * (steps - 1) / (ms * 1e-3) / 1e6, "unit": METRIC,
                     "ms_per_step": ms / (steps - 1), "execution": exec_name(s)}
        hist[name] = s.history(cap=steps - 1)
        fields[name] = np.concatenate([s.get(capi.FIELD_U).ravel(), s.get(capi.FIELD_V).ravel()])
        s.close()
    hm, h6 = hist["mixed"], hist["fp64"]
    cd_err = float(np.max(np.abs(hm[:, 1] - h6[:, 1]) / np.maximum(np.abs(h6[:, 1]), 1e-12)))
    cl_err = float(np.max(np.abs(hm[:, 2] - h6[:, 2])) / max(float(np.max(np.abs(h6[:, 1]))), 1e-12))
    out.update({"workload": f"cylinder 384x256, Re 100, dt 5e-3, {steps} steps from the impulsive start "
                            f"(steps 2..{steps} timed), mixed vs plain FP64, default schedule",
                "steps": steps, "l2": "not flushed between steps (the run as a user runs it)",
                "speedup_mixed_over_fp64": out["mixed"]["value"] / out["fp64"]["value"],
                "rel_l2_velocity_final": rel_l2(fields["mixed"], fields["fp64"]),
                "cd_rel_err_max": cd_err, "cl_err_max_rel_to_cd": cl_err,
                "cd_final": float(h6[-1, 1]), "cl_final": float(h6[-1, 2]),
                "cd_mean_last_1000": float(np.mean(h6[-1000:, 1])), "cl_amplitude_last_1000":
                    float((np.max(h6[-1000:, 2]) - np.min(h6[-1000:, 2])) / 2)})
    return out


def _oracle_solver(cfg, xf, yf, schedule=None):
    """The CPU oracle (FP64 restatement of the same scheme) on all host threads:
    the checker of the accuracy lines; `schedule` (a tuned capi.Schedule) sets
    its sweep schedule, which the oracle follows like the GPU."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import _oracle

    if schedule is not None:
        cfg = type(cfg).from_buffer_copy(cfg)
        for k, v in schedule.as_dict().items():
            setattr(cfg, k, v)
    return _oracle.Oracle().method(cfg, xf, yf, os.cpu_count() or 1)


def vs_oracle(capi, get, stats, o):
    """Errors of a GPU result against the oracle after the same steps: Linf of
    u and v relative to the oracle's largest |velocity|, relative L2 of the
    velocity, Linf of the per-cell divergence field (absolute), both max |div|,
    and drag / lift relative to the oracle's drag."""
    ug, vg = get(capi.FIELD_U), get(capi.FIELD_V)
    uo, vo = o.get(capi.FIELD_U), o.get(capi.FIELD_V)
    vmax = max(float(np.abs(uo).max()), float(np.abs(vo).max()), 1e-300)
    so = o.stats()
    out = {"linf_velocity": float(max(np.abs(ug - uo).max(), np.abs(vg - vo).max()) / vmax),
           "rel_l2_velocity": rel_l2(np.concatenate([ug.ravel(), vg.ravel()]), np.concatenate([uo.ravel(), vo.ravel()])),
           "linf_divergence": float(np.abs(get(capi.FIELD_DIV) - o.get(capi.FIELD_DIV)).max()),
           "max_div": stats.max_div, "max_div_oracle": so.max_div}
    if abs(so.cd) > 0:
        out["cd_rel_err"] = abs(stats.cd - so.cd) / abs(so.cd)
        out["cl_err_rel_to_cd"] = abs(stats.cl - so.cl) / abs(so.cd)
    return out


def ellipse_line(ifx, capi, cases, steps=10, oracle=True, settled_start=200):
    """The large single-instance configuration: ellipse of aspect 0.2 and chord
    1 at 10 deg, 1024x768 cells on a 20x12 domain, Re 300, dt 2e-3; autotuned,
    mixed and plain FP64 (device time, CUDA events).  Timed twice: steps
    4..3+`steps` from the impulsive start (transient), and `steps` steps from
    step settled_start+1 on (the run past its start, as most of the
    configuration's 10000 steps are; `value`).  Both results are compared with
    the CPU oracle after the first 3 + `steps` steps (Linf velocity and
    divergence errors); the oracle follows the FP64 run's tuned schedule, so the
    mixed run's errors include its own schedule's difference (within the
    pressure tolerance)."""
    out = {"workload": "ellipse aspect 0.2, chord 1, 10 deg, 20x12 domain, 1024x768 tanh-stretched, Re 300, dt 2e-3",
           "unit": METRIC, "steps": steps,
           "timed_steps": f"steps {settled_start + 1}..{settled_start + steps} (value); "
                          f"4..{3 + steps} (transient)"}
    fields = {}
    snaps = {}
    fp64_schedule = None
    for name, prec in (("mixed", capi.PREC_MIXED), ("fp64", capi.PREC_FP64)):
        cfg, xf, yf = cases.ellipse(precision=prec)
        s = ifx.Solver.create(cfg, xf, yf)
        s.step(1)
        s.autotune(steps=1)
        sched, _ = s.autotune_schedule(steps=1)
        s.step(2)
        s.step(steps)
        ms_t = s.last_step_ms()
        st = s.stats()
        fields[name] = np.concatenate([s.get(capi.FIELD_U).ravel(), s.get(capi.FIELD_V).ravel()])
        snap = {f: s.get(f) for f in (capi.FIELD_U, capi.FIELD_V, capi.FIELD_DIV)}
        snaps[name] = (snap, st)
        if name == "fp64":
            fp64_schedule = s.schedule()
        s.step(max(0, settled_start - 3 - steps))  # untimed, to the settled window
        s.step(steps)
        ms = s.last_step_ms()
        st2 = s.stats()
        out[name] = {"value": cfg.nx * cfg.ny * steps / (ms * 1e-3) / 1e6, "ms_per_step": ms / steps,
                     "execution": exec_name(s), "schedule": sched.as_dict(), "ppe_iters_last": st2.last_ppe_iters,
                     "predictor_iters_last": st2.last_ad_iters, "cd": st2.cd,
                     "transient": {"value": cfg.nx * cfg.ny * steps / (ms_t * 1e-3) / 1e6, "ms_per_step": ms_t / steps,
                                   "ppe_iters_last": st.last_ppe_iters}}
        s.close()
    out["speedup_mixed_over_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    out["speedup_mixed_over_fp64_transient"] = out["mixed"]["transient"]["value"] / out["fp64"]["transient"]["value"]
    out["rel_l2_velocity_vs_fp64"] = rel_l2(fields["mixed"], fields["fp64"])
    if oracle:
        cfg, xf, yf = cases.ellipse(precision=capi.PREC_FP64)
        o = _oracle_solver(cfg, xf, yf, fp64_schedule)
        o.step(3 + steps)
        out["vs_oracle"] = {name: vs_oracle(capi, snap.__getitem__, st, o) for name, (snap, st) in snaps.items()}
        out["vs_oracle"]["steps"] = 3 + steps
    return out


def cavity_line(ifx, capi, cases, steps=2000, oracle=True):
    """Lid-driven cavity: unit square, uniform 128x128, lid u = 1, no-slip
    walls, Re 100, dt 1e-3, pressure to 1e-8, `steps` steps from rest (device
    time of the last steps - 1, CUDA events), mixed and plain FP64; both against
    the CPU oracle after the same steps (with the FP64 run's tuned schedule)."""
    out = {"workload": "lid-driven cavity, unit square, uniform 128x128, lid u=1, Re 100, dt 1e-3, "
                       f"pressure to 1e-8, {steps} steps", "unit": METRIC, "steps": steps}
    solvers = {}
    for name, prec in (("mixed", capi.PREC_MIXED), ("fp64", capi.PREC_FP64)):
        cfg, xf, yf = cases.cavity(precision=prec)
        s = ifx.Solver.create(cfg, xf, yf)
        s.step(1)
        s.autotune(steps=1)
        sched, _ = s.autotune_schedule(steps=2)
        s.step(steps - 1)
        ms = s.last_step_ms()
        st = s.stats()
        out[name] = {"value": cfg.nx * cfg.ny * (steps - 1) / (ms * 1e-3) / 1e6, "ms_per_step": ms / (steps - 1),
                     "execution": exec_name(s), "schedule": sched.as_dict(), "ppe_iters_last": st.last_ppe_iters,
                     "predictor_iters_last": st.last_ad_iters, "max_div": st.max_div}
        solvers[name] = s
    out["speedup_mixed_over_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    gm, g6 = solvers["mixed"], solvers["fp64"]
    out["rel_l2_velocity_mixed_vs_fp64"] = rel_l2(
        np.concatenate([gm.get(capi.FIELD_U).ravel(), gm.get(capi.FIELD_V).ravel()]),
        np.concatenate([g6.get(capi.FIELD_U).ravel(), g6.get(capi.FIELD_V).ravel()]))
    if oracle:
        cfg, xf, yf = cases.cavity(precision=capi.PREC_FP64)
        o = _oracle_solver(cfg, xf, yf, solvers["fp64"].schedule())
        t0 = time.perf_counter()
        o.step(steps)
        dt = time.perf_counter() - t0
        out["vs_oracle"] = {name: vs_oracle(capi, s.get, s.stats(), o) for name, s in solvers.items()}
        out["cpu_oracle"] = {"value": cfg.nx * cfg.ny * steps / dt / 1e6, "cores": os.cpu_count() or 1}
    for s in solvers.values():
        s.close()
    return out


def reference_cuda(steps=(50, 20, 6)):
    """The reference's own AD-only CUDA executable (oracle/_ref, built from the
    staged, unmodified sources) on the REFERENCE-mode workload at 52^2, 130^2
    and 514^2 cells (ghosts included): seconds per ADsolver step as the
    difference of two runs of k and 2k steps over k, with its per-iteration
    printing sent to a file (as shipped) and to /dev/null.  Each of its steps
    also writes uc.dat and vc.dat (src/include/ADSolver.cu:374-375)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ref_run

    if not ref_run.available():
        return {"unavailable": "reference executable not built (its sources were not staged)"}
    lines = []
    with tempfile.TemporaryDirectory() as d:
        for n, k in zip((50, 128, 512), steps):
            row = {"grid": [n + 2, n + 2], "steps": k}
            for name, dest in (("stdout_file", os.path.join(d, "stdout.txt")), ("stdout_devnull", os.devnull)):
                sec, t1, t2 = ref_run.time_per_step(os.path.join(d, f"c{n}"), n, k, stdout_path=dest)
                row[name] = {"value": n * n / sec / 1e6, "ms_per_step": sec * 1e3, "run_s": [t1, t2]}
            lines.append(row)
    return {"workload": "the reference's ADsolver (src/include/ADSolver.cu:268-395), uniform grids on [0,1]^2, "
                        "vortex IC, Re 150, dt 1e-3, AD_itermax 25", "unit": METRIC, "lines": lines,
            "build": "oracle/ref.mk: nvcc -gencode arch=compute_103a,code=sm_103a, cudaMalloc padded (oracle/ref_guard.h)"}


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
        # the autotuners refuse moving bodies (their trial steps would move
        # the geometry); graph mode with 32x8 tiles, the cylinder's choice
        s.set_exec_mode(ifx.EXEC_GRAPH)
        s.set_mg_tile_rows(1)
        s.step(1)
        s.step(2)
        s.step(steps)
        ms = s.last_step_ms()
        st = s.stats()
        out[name] = {"value": cfg.nx * cfg.ny * steps / (ms * 1e-3) / 1e6, "ms_per_step": ms / steps,
                     "execution": exec_name(s, tuned=False), "ppe_iters_last": st.last_ppe_iters, "cd": st.cd, "cl": st.cl,
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
            "unit": METRIC, "lines": lines}


def window_pre(args):
    """Untimed steps before the warm-up, so that the timed steps are steps
    window_start+1 .. window_start+K of the run (at least one)."""
    return max(1, args.window_start - args.warmup)


def bench_config(cells, world, args):
    """The workload's config, identical in both arms of the bench."""
    first = window_pre(args) + args.warmup + 1
    return {"workload": WORKLOAD, "grid": [384, 256], "cells": cells, "parallelism": f"replicas x{world}",
            "ppe_tol": 1e-8, "l2": "flushed before every timed GPU step (256 MB write)",
            "timed_steps": f"steps {first}..{first + args.steps - 1} of the 5000-step run "
                           f"({window_pre(args)} steps advanced untimed, then {args.warmup} warm-up steps)"}


def _r(x, d=3):
    return None if x is None else float(f"{x:.{d}g}")


def summary(line):
    """The figures of the long blocks in a few hundred bytes, as the last key of
    the line: Mcell-updates/s (M), mixed/FP64 ratios (x), errors, fractions."""
    out = {"cyl": {"M": _r(line["value"]), "fp64_M": _r(line["plain_fp64"]["value"]),
                   "x": _r(line["plain_fp64"]["speedup_mixed_over_fp64"]), "e2e_M": _r(line["e2e"]["value"]),
                   "frac": _r(line["roofline"]["frac"]), "err": _r(line["accuracy_vs_fp64"]["rel_l2_velocity"], 2)},
           "sweep_frac": _r(line["phase_roofline"]["frac"])}
    if "transient" in line:
        t = line["transient"]
        out["cyl_transient"] = {"M": _r(t["mixed"]["value"]), "fp64_M": _r(t["fp64"]["value"]),
                                "x": _r(t["speedup_mixed_over_fp64"])}
    if "whole_run" in line:
        w = line["whole_run"]
        out["cyl_whole_run"] = {"M": _r(w["mixed"]["value"]), "fp64_M": _r(w["fp64"]["value"]),
                                "x": _r(w["speedup_mixed_over_fp64"]), "err": _r(w["rel_l2_velocity_final"], 2),
                                "cd_err": _r(w["cd_rel_err_max"], 2)}
    if "cavity" in line:
        c = line["cavity"]
        out["cavity"] = {"M": _r(c["mixed"]["value"]), "fp64_M": _r(c["fp64"]["value"]),
                         "x": _r(c["speedup_mixed_over_fp64"])}
        if "vs_oracle" in c:
            out["cavity"]["linf_vs_oracle"] = [_r(c["vs_oracle"]["fp64"]["linf_velocity"], 2),
                                               _r(c["vs_oracle"]["mixed"]["linf_velocity"], 2)]
    if "ellipse" in line:
        e = line["ellipse"]
        out["ellipse"] = {"M": _r(e["mixed"]["value"]), "fp64_M": _r(e["fp64"]["value"]),
                          "x": _r(e["speedup_mixed_over_fp64"])}
        if "vs_oracle" in e:
            out["ellipse"]["linf_vs_oracle"] = [_r(e["vs_oracle"]["fp64"]["linf_velocity"], 2),
                                                _r(e["vs_oracle"]["mixed"]["linf_velocity"], 2)]
            out["ellipse"]["linf_div"] = [_r(e["vs_oracle"]["fp64"]["linf_divergence"], 2),
                                          _r(e["vs_oracle"]["mixed"]["linf_divergence"], 2)]
    if "batched" in line:
        b = line["batched"]
        out["batch"] = {"M": _r(b["mixed"]["value"]), "fp64_M": _r(b["fp64"]["value"]),
                        "x": _r(b["speedup_mixed_over_fp64"]), "frac": _r(b["mixed"]["roofline"]["frac"]),
                        "err": _r(b["accuracy_vs_fp64"]["rel_l2_velocity_max"], 2)}
        if "solve" in b:
            out["batch"]["solves_s"] = _r(b["solve"]["solves_per_s"])
    if "served" in line:
        v = line["served"]
        out["served"] = {"n": v["requests"], "solves_s": _r(v["solves_per_s"]),
                         "p50_ms": _r(v["latency_ms"]["p50"]), "p99_ms": _r(v["latency_ms"]["p99"]),
                         "fp64_p50_ms": _r(v["fp64"]["latency_ms"]["p50"]),
                         "fp64_p99_ms": _r(v["fp64"]["latency_ms"]["p99"]),
                         "cap_x": _r(v["capacity"]["speedup_mixed_over_fp64"]),
                         "err": _r(v["accuracy_vs_fp64"]["rel_l2_velocity_max"], 2)}
    if "reference_cuda" in line and "lines" in line["reference_cuda"]:
        out["ref_cuda_M"] = [_r(r["stdout_devnull"]["value"]) for r in line["reference_cuda"]["lines"]]
        out["ref_mode_M"] = [_r(r["gpu_value"]) for r in line["reference_path"]["lines"]]
    return out


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
        o.step(window_pre(args))  # the same steps as the GPU arm: advanced untimed, then the warm-up
        o.step(args.warmup)
        t0 = time.perf_counter()
        o.step(args.steps)
        dt = time.perf_counter() - t0
        val = cells * args.steps / dt / 1e6
        line = {"metric": METRIC, "value": val, "unit": METRIC, "impl": "reference", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": bench_config(cells, world, args),
                "solver": "CPU restatement (oracle), FP64, all host threads",
                "cpu_baseline": {"value": val, "unit": METRIC, "cores": nth, "kind": "port",
                                 "sample": f"{args.steps} time steps after {window_pre(args)} untimed and "
                                           f"{args.warmup} warm-up steps"},
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
        elif args.profile_workload == "ellipse":
            s = ifx.Solver.create(*cases.ellipse(precision=prec))
        else:
            cfg, _, _ = cases.cylinder(precision=prec)
            if args.profile_workload == "moving":  # heaving as in the moving_body line
                cases.set_motion(cfg, amp_y=0.25, freq=0.2)
            s = ifx.Solver.create(cfg, xf, yf)
        s.set_mg_tile_rows(args.profile_rows)
        s.step(args.warmup)
        s.synchronize()
        # L2 flushed before the profiled steps, as before every timed step
        torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda").zero_()
        torch.cuda.synchronize()
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

    def timed(prec, pre):
        cfg, _, _ = cases.cylinder(precision=prec)
        s = ifx.Solver.create(cfg, xf, yf)
        s.step(pre)  # untimed: the run up to the warm-up of the timed window
        s.autotune(steps=2)  # execution mode and tile shape; the state is restored afterwards
        s.autotune_schedule(steps=2)  # sweep schedule, the same way
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

    s, total_ms, launches, clocks, step_bytes_total, pits, adits = timed(capi.PREC_MIXED, window_pre(args))
    st = s.stats()
    u_m, v_m = s.get(capi.FIELD_U), s.get(capi.FIELD_V)
    cd_m, cl_m = st.cd, st.cl
    total_ms = max_over_ranks(total_ms, world)
    value = world * cells * args.steps / (total_ms * 1e-3) / 1e6

    # plain FP64 path on the same steps
    s64, total64, launches64, _, _, pits64, _ = timed(capi.PREC_FP64, window_pre(args))
    total64 = max_over_ranks(total64, world)
    st64 = s64.stats()
    u64, v64 = s64.get(capi.FIELD_U), s64.get(capi.FIELD_V)
    err_u = float(np.sqrt(np.sum((u_m - u64) ** 2 + (v_m - v64) ** 2) / np.sum(u64 ** 2 + v64 ** 2)))
    err_cd = abs(cd_m - st64.cd) / abs(st64.cd)
    value64 = world * cells * args.steps / (total64 * 1e-3) / 1e6

    # end to end through the C ABI: pinned host state in, result out, every step
    nx, ny = s.grid_dims()
    # u, v, p back to back in one pinned allocation: one copy each way per step
    pinned = torch.empty(3 * nx * ny, dtype=torch.float64, pin_memory=True).numpy()
    host = tuple(pinned[k * nx * ny:(k + 1) * nx * ny] for k in range(3))
    s.get_state(out=host)
    snap = s.checkpoint()  # the three-call timing below repeats the same steps
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        # u, v, p in, one step, u, v, p out into the same pinned buffers: one call, one wait (ifx_step_state)
        s.step_state(*host, n=1, out=host)
    barrier()
    e2e_s = max_over_ranks(time.perf_counter() - t0, world)
    e2e = world * cells * args.steps / e2e_s / 1e6
    nbytes = 3 * nx * ny * 8
    # the same steps through three calls, each waiting (ifx_set_state, ifx_step, ifx_get_state)
    s.restore(snap)
    s.get_state(out=host)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        s.set_state(*host)
        s.step(1)
        s.get_state(out=host)
    barrier()
    e2e3 = world * cells * args.steps / max_over_ranks(time.perf_counter() - t0, world) / 1e6

    # roofline of the dominant kernel: the per-step kernel (persistent mode)
    peak, peak_kind = measured_peak()
    persistent = s.exec_mode() == 0
    traffic = committed_traffic()
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
        "config": bench_config(cells, world, args),
        "precision": "mixed", "execution": exec_name(s), "schedule": s.schedule().as_dict(),
        "e2e": {"value": e2e, "unit": METRIC, "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                "call": "ifx_step_state (state in, one step, state out, one wait) from pinned host buffers",
                "three_calls_value": e2e3},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "kernel": ("k_persist_step<float> (one launch per time step)" if persistent else
                                                "the step's kernels (one CUDA graph launch per time step)"),
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind, "traffic": traffic,
                     "bytes_per_launch": step_bytes_total / args.steps, "ms_per_launch": total_ms / args.steps,
                     "note": "working set ~30 MB is L2-resident; launch/barrier latency bound at this size"},
        "clocks": clocks,
    }
    # long detail blocks first; the short summary is the last key of the line
    if rank == 0 and world == 1:
        line["reference_path"] = reference_path(ifx, capi, cases, cpu=not args.no_cpu)
        if not args.no_reference_build:
            line["reference_cuda"] = reference_cuda()
        line["moving_body"] = moving_line(ifx, capi, cases)
        if args.whole_run_steps > 1:
            line["whole_run"] = whole_run(ifx, capi, cases, steps=args.whole_run_steps)
        if window_pre(args) > 1:
            # the impulsive start's transient: steps 2+W .. 1+W+K, the timed
            # window of this line before it moved past the transient
            tr = {}
            for name, prec in (("mixed", capi.PREC_MIXED), ("fp64", capi.PREC_FP64)):
                s_t, ms_t, _, _, _, it_t, _ = timed(prec, 1)
                s_t.close()
                tr[name] = {"value": cells * args.steps / (ms_t * 1e-3) / 1e6, "unit": METRIC,
                            "ms_per_step": ms_t / args.steps, "ppe_iters_mean": sum(it_t) / len(it_t)}
            tr["steps"] = f"steps {2 + args.warmup}..{1 + args.warmup + args.steps} of the run, L2 flushed before each"
            tr["speedup_mixed_over_fp64"] = tr["mixed"]["value"] / tr["fp64"]["value"]
            line["transient"] = tr
        line["ellipse"] = ellipse_line(ifx, capi, cases, oracle=not args.no_cpu)
        if args.cavity_steps > 1:
            line["cavity"] = cavity_line(ifx, capi, cases, steps=args.cavity_steps, oracle=not args.no_cpu)
    if args.batch > 0:
        line["batched"] = batched_sweep(ifx, capi, cases, args.batch, args.batch_steps, args.batch_solve_steps, peak)
    if args.serve > 0:
        line["served"] = served_lines(ifx, capi, cases, args.serve, args.rate, 64 << 30)
    line["phase_roofline"] = {"kernel": "finest-level smoothing sweep as the step launches it (k_smooth_grid_tma<float>), "
                                        "launched alone", "bytes_per_cell": 13,
                              "cells_per_launch": k_cells, "ms_per_launch": k_ms, "achieved_gbs": k_bw,
                              "frac": k_bw / peak, "grid_barrier_us": bar_us}
    line["iterations"] = {"ppe_mean": sum(pits) / len(pits), "predictor_mean": sum(adits) / len(adits),
                          "ppe_mean_fp64": sum(pits64) / len(pits64)}
    line["accuracy_vs_fp64"] = {"rel_l2_velocity": err_u, "cd_rel_err": err_cd, "cd": cd_m, "cd_fp64": st64.cd}
    line["plain_fp64"] = {"value": value64, "ms_per_step": total64 / args.steps, "gpu_launches": launches64,
                          "execution": exec_name(s64), "schedule": s64.schedule().as_dict(),
                          "speedup_mixed_over_fp64": value / value64}
    if rank == 0 and world == 1 and not args.no_cpu:
        cfg64, _, _ = cases.cylinder(precision=capi.PREC_FP64)
        warm = window_pre(args) + args.warmup
        n, dt, nth = cpu_oracle_run(cfg64, xf, yf, args.cpu_seconds, warm=warm)
        line["cpu_baseline"] = {"value": cells * n / dt / 1e6, "unit": METRIC, "cores": nth, "kind": "port",
                                "sample": f"{n} time steps of the same workload after {warm} untimed steps "
                                          f"(the GPU arm's window) ({dt:.1f} s)"}
    line["summary"] = summary(line)
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
