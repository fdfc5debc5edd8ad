"""Runs the reference's own AD-only CUDA executable (oracle/_ref/immerseflow_ref,
built by oracle/ref.mk from the staged, unmodified reference sources).

Test and baseline infrastructure only: the GPU parity test of the REFERENCE
mode and bench.py's reference-build timing call it; the product never does.

The executable (src/main.cu:75-102 of the reference) reads
../inputs/inputs.txt with the keyword grammar of src/main.cu:10-59 and the face
files ../inputs/xgrid.dat2 / ygrid.dat2 (src/include/preSim.cu:268,281),
runs `tmax` ADsolver steps (src/include/ADSolver.cu:268-395; each step writes
../results/uc.dat and vc.dat, src/include/ADSolver.cu:374-375) and prints a
line per Jacobi iteration.  `case_dir` lays out that tree for an n x n uniform
grid on the unit square (inputs/uniformGrid.py's layout).
"""
import os
import subprocess
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
EXE = os.path.join(HERE, "_ref", "immerseflow_ref")

INPUTS = """===============================| INPUT FILE |====================================
Restart     Restart_Time
0           0

___________________________| Domain Information |________________________________
nx      ny
{n}      {n}

Lx      Ly
1      1


________________________| Iterative Solver Settings |____________________________
w-AD    w-PPE   AD-itermax  PPE-itermax  AD_Solver PPE_Solver(1. Point GS, 2. Line SOR)
1       1       {itermax}          100000          1         1


___________________________| Simulation Settings |_______________________________
ErrorMax    tmax    dt       Re      mu
1E-6        {steps}       {dt}    {re}    0.01

___________________________| Data Write |_______________________________
Write Interval(t/dt)
1000
"""


def available():
    return os.access(EXE, os.X_OK)


def _grid_file(path, n):
    with open(path, "w") as f:
        for i, v in enumerate(np.linspace(0.0, 1.0, n + 1)):
            f.write(f"{i + 1:>10} {v:.7E}\n")


def case_dir(root, n, steps, dt=1e-3, re=150.0, itermax=25):
    """root/inputs/{inputs.txt, xgrid.dat2, ygrid.dat2}, root/results/, root/run/."""
    for d in ("inputs", "results", "run"):
        os.makedirs(os.path.join(root, d), exist_ok=True)
    with open(os.path.join(root, "inputs", "inputs.txt"), "w") as f:
        f.write(INPUTS.format(n=n, steps=steps, dt=dt, re=re, itermax=itermax))
    _grid_file(os.path.join(root, "inputs", "xgrid.dat2"), n)
    _grid_file(os.path.join(root, "inputs", "ygrid.dat2"), n)
    return os.path.join(root, "inputs", "inputs.txt")


def run(root, stdout_path=os.devnull, timeout=600):
    """Runs the executable in root/run; returns its wall-clock seconds."""
    with open(stdout_path, "w") as out:
        t0 = time.perf_counter()
        r = subprocess.run([EXE], cwd=os.path.join(root, "run"), stdout=out, stderr=subprocess.STDOUT,
                           stdin=subprocess.DEVNULL, timeout=timeout)
        t1 = time.perf_counter()
    if r.returncode != 0:
        raise RuntimeError(f"reference executable exited with {r.returncode}")
    return t1 - t0


def read_tecplot(path, n):
    """A Tecplot POINT file of write_results_to_file (src/include/postSim.cu:41-66)
    as an (n+2, n+2) array of its third column."""
    a = np.loadtxt(path, delimiter=",", skiprows=3)
    return a[:, 2].reshape(n + 2, n + 2)


def time_per_step(root, n, steps, stdout_path=os.devnull, dt=1e-3, re=150.0):
    """Seconds per ADsolver step: two runs of `steps` and 2*`steps` steps, the
    difference of their wall times divided by `steps` (the process start, CUDA
    context creation and set-up cancel)."""
    case_dir(root, n, steps, dt=dt, re=re)
    t1 = run(root, stdout_path)
    case_dir(root, n, 2 * steps, dt=dt, re=re)
    t2 = run(root, stdout_path)
    return (t2 - t1) / steps, t1, t2
