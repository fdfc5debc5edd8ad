"""Synthetic workloads: grids (xgrid/ygrid face coordinates) and configs.

No dataset is involved: every case is generated from a few parameters (and a
seed for the batched / served sampling), at the sizes of the benchmark
configurations:

  cavity     unit square, uniform 128x128, lid u=1, Re=100, dt=1e-3
  cylinder   D=1 at (10,10) in 30x20, tanh-stretched 384x256, Re=100, dt=5e-3
  ellipse    chord 1, thickness 0.2, 10 deg incidence, 20x12, 1024x768,
             Re=300, dt=2e-3
  batch      seeded sample: grids log-uniform 64x64..512x384, Re U[50,300],
             ellipse aspect U[0.1,1], angle U[-30,30] deg, body 1/3 downstream
  served     seeded Poisson arrivals of cylinder/ellipse requests, grids
             log-uniform 64^2..1024^2, Re U[50,1000], 200-2000 steps
"""
import math

import numpy as np

from . import _capi as capi
from ._capi import default_config


def uniform_faces(n, length, x0=0.0):
    """n cells on [x0, x0+length]: n+1 faces (inputs/uniformGrid.py layout)."""
    return np.linspace(x0, x0 + length, n + 1)


def tanh_faces(n, length, centre, ratio=4.0, width=3.0):
    """n cells on [0, length], finest at `centre`.  The cell size grows with
    the distance d from the centre as 1 + (ratio-1) tanh(d/width); faces are
    placed at equal increments of the integrated cell density."""
    xs = np.linspace(0.0, length, 200001)
    h = 1.0 + (ratio - 1.0) * np.tanh(np.abs(xs - centre) / width)
    cum = np.concatenate([[0.0], np.cumsum(0.5 * (1.0 / h[1:] + 1.0 / h[:-1]) * np.diff(xs))])
    cum *= n / cum[-1]
    faces = np.interp(np.arange(n + 1, dtype=np.float64), cum, xs)
    faces[0], faces[-1] = 0.0, length
    return faces


def write_grid(path, faces):
    """Grid file in the reference layout: '<index> <coordinate>' per line."""
    with open(path, "w") as f:
        for i, v in enumerate(faces):
            f.write(f"{i + 1:>10} {v:.7E}\n")


def _method_cfg(precision):
    c = default_config()
    c.mode = capi.MODE_METHOD
    c.precision = precision
    c.ad_itermax = 100
    c.ppe_itermax = 200
    c.ad_tol = 1e-12
    c.ppe_tol = 1e-8
    return c


def cavity(n=128, re=100.0, dt=1e-3, precision=capi.PREC_FP64):
    c = _method_cfg(precision)
    c.nx = c.ny = n
    c.lx = c.ly = 1.0
    c.re = re
    c.dt = dt
    c.init = capi.INIT_REST
    for s in range(4):
        c.bc_type[s] = capi.BC_WALL
        c.bc_u[s] = 0.0
        c.bc_v[s] = 0.0
    c.bc_u[capi.SIDE_N] = 1.0
    return c, uniform_faces(n, 1.0), uniform_faces(n, 1.0)


def external(nx, ny, lx, ly, cx, cy, a, b, angle_deg, re, dt, precision=capi.PREC_FP64, ratio=4.0, width=3.0):
    c = _method_cfg(precision)
    c.nx, c.ny = nx, ny
    c.lx, c.ly = lx, ly
    c.re = re
    c.dt = dt
    c.init = capi.INIT_UNIFORM
    c.bc_type[capi.SIDE_W] = capi.BC_INFLOW
    c.bc_u[capi.SIDE_W] = 1.0
    c.bc_v[capi.SIDE_W] = 0.0
    c.bc_type[capi.SIDE_E] = capi.BC_OUTFLOW
    c.bc_type[capi.SIDE_S] = capi.BC_SLIP
    c.bc_type[capi.SIDE_N] = capi.BC_SLIP
    c.outflow_uc = 1.0
    c.body = capi.BODY_ELLIPSE
    c.body_cx, c.body_cy = cx, cy
    c.body_a, c.body_b = a, b
    c.body_angle_deg = angle_deg
    c.force_ref_u = 1.0
    c.force_ref_len = 2.0 * max(a, b)
    return c, tanh_faces(nx, lx, cx, ratio, width), tanh_faces(ny, ly, cy, ratio, width)


def set_motion(c, u=0.0, v=0.0, amp_x=0.0, amp_y=0.0, amp_deg=0.0, freq=0.0, phase_x=0.0, phase_y=0.0,
               phase_deg=0.0):
    """Prescribed rigid motion of the configuration's body: centre
    (body_cx + u t + amp_x (sin(2 pi (freq t + phase_x/360)) - sin(2 pi phase_x/360)),
    likewise y), angle likewise with amp_deg and phase_deg."""
    c.motion = capi.MOTION_PRESCRIBED
    c.motion_u, c.motion_v = u, v
    c.motion_amp_x, c.motion_amp_y, c.motion_amp_deg = amp_x, amp_y, amp_deg
    c.motion_freq = freq
    c.motion_phase_x, c.motion_phase_y, c.motion_phase_deg = phase_x, phase_y, phase_deg
    return c


def cylinder(nx=384, ny=256, re=100.0, dt=5e-3, precision=capi.PREC_FP64):
    return external(nx, ny, 30.0, 20.0, 10.0, 10.0, 0.5, 0.5, 0.0, re, dt, precision)


def ellipse(nx=1024, ny=768, re=300.0, dt=2e-3, precision=capi.PREC_FP64):
    # chord 1 (semi-axes 0.5 and 0.1), 10 deg nose-up incidence in a uniform stream
    return external(nx, ny, 20.0, 12.0, 6.0, 6.0, 0.5, 0.1, -10.0, re, dt, precision)


def batch_sample(count=256, seed=0, precision=capi.PREC_MIXED, lx=12.0, ly=8.0):
    """Instances of the batched sweep: uneven grids, Re and body shapes."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        nx = int(round(math.exp(rng.uniform(math.log(64), math.log(512)))))
        ny = int(round(math.exp(rng.uniform(math.log(64), math.log(384)))))
        re = float(rng.uniform(50.0, 300.0))
        ar = float(rng.uniform(0.1, 1.0))
        ang = float(rng.uniform(-30.0, 30.0))
        hmin = min(lx / nx, ly / ny) / 2.5
        dt = float(min(5e-3, 0.4 * hmin))
        out.append(external(nx, ny, lx, ly, lx / 3.0, ly / 2.0, 0.5, 0.5 * ar, ang, re, dt, precision))
    return out


def served_stream(count, rate, seed=0, precision=capi.PREC_MIXED, nmin=64, nmax=1024, smin=200, smax=2000):
    """Seeded request stream: (arrival time [s], cfg, xf, yf, nsteps)."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for _ in range(count):
        t += float(rng.exponential(1.0 / rate))
        n = int(round(math.exp(rng.uniform(math.log(nmin), math.log(nmax)))))
        re = float(rng.uniform(50.0, 1000.0))
        steps = int(rng.integers(smin, smax + 1))
        lx, ly = 12.0, 8.0
        hmin = min(lx, ly) / n / 2.5
        dt = float(min(5e-3, 0.4 * hmin))
        if rng.uniform() < 0.5:
            cfg, xf, yf = external(n, n, lx, ly, lx / 3, ly / 2, 0.5, 0.5, 0.0, re, dt, precision)
        else:
            ar = float(rng.uniform(0.1, 1.0))
            ang = float(rng.uniform(-30.0, 30.0))
            cfg, xf, yf = external(n, n, lx, ly, lx / 3, ly / 2, 0.5, 0.5 * ar, ang, re, dt, precision)
        out.append((t, cfg, xf, yf, steps))
    return out
