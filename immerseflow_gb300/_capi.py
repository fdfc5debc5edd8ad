"""ctypes declarations of the C ABI in include/immerseflow_gb300.h.

The structures below mirror the header field for field; tests/test_abi.py
checks their sizes against the compiled library.
"""
import ctypes as C

IFX_OK = 0
IFX_ERR_ARG = 1
IFX_ERR_IO = 2
IFX_ERR_PARSE = 3
IFX_ERR_CUDA = 4
IFX_ERR_NOMEM = 5
IFX_ERR_NOT_CONVERGED = 6
IFX_ERR_DIVERGED = 7
IFX_ERR_BUDGET = 8
IFX_ERR_STATE = 9
IFX_ERR_NODEVICE = 10
IFX_ERR_GEOMETRY = 11
MOTION_NONE, MOTION_PRESCRIBED = 0, 1
PPE_JACOBI, PPE_POINT_GS, PPE_LINE_SOR = 0, 1, 2

MODE_REFERENCE = 0
MODE_METHOD = 1
PREC_FP64 = 0
PREC_MIXED = 1
INIT_VORTEX = 0
INIT_UNIFORM = 1
INIT_REST = 2
SIDE_W, SIDE_E, SIDE_S, SIDE_N = 0, 1, 2, 3
BC_WALL, BC_INFLOW, BC_OUTFLOW, BC_SLIP = 0, 1, 2, 3
BODY_NONE, BODY_ELLIPSE = 0, 1

FIELD_U = 0
FIELD_V = 1
FIELD_P = 2
FIELD_IBLANK = 3
FIELD_UF = 4
FIELD_VF = 5
FIELD_CELLTYPE = 6
FIELD_DIV = 7
FIELD_XC = 8
FIELD_YC = 9

PATH_MAX = 512
MAX_CELLS = 1 << 28  # IFX_MAX_CELLS: largest instance, cells including the ghost ring


class Config(C.Structure):
    _fields_ = [
        ("restart", C.c_int), ("restart_time", C.c_int),
        ("nx", C.c_int), ("ny", C.c_int),
        ("lx", C.c_double), ("ly", C.c_double),
        ("w_ad", C.c_int), ("w_ppe", C.c_int), ("ad_itermax", C.c_int),
        ("ppe_itermax", C.c_int), ("ad_solver", C.c_int), ("ppe_solver", C.c_int),
        ("error_max", C.c_double), ("tmax", C.c_double), ("dt", C.c_double),
        ("re", C.c_double), ("mu", C.c_double),
        ("write_interval", C.c_int),
        ("mode", C.c_int), ("precision", C.c_int), ("init", C.c_int),
        ("bc_type", C.c_int * 4),
        ("bc_u", C.c_double * 4), ("bc_v", C.c_double * 4),
        ("outflow_uc", C.c_double),
        ("body", C.c_int),
        ("body_cx", C.c_double), ("body_cy", C.c_double), ("body_a", C.c_double),
        ("body_b", C.c_double), ("body_angle_deg", C.c_double),
        ("ppe_tol", C.c_double), ("ad_tol", C.c_double),
        ("mg_pre", C.c_int), ("mg_post", C.c_int),
        ("mg_omega", C.c_double),
        ("mixed_inner", C.c_int),
        ("force_ref_u", C.c_double), ("force_ref_len", C.c_double),
        ("ppe_method", C.c_int), ("relax_ad", C.c_double), ("relax_ppe", C.c_double),
        ("motion", C.c_int), ("motion_u", C.c_double), ("motion_v", C.c_double),
        ("motion_amp_x", C.c_double), ("motion_amp_y", C.c_double), ("motion_amp_deg", C.c_double),
        ("motion_freq", C.c_double),
        ("motion_phase_x", C.c_double), ("motion_phase_y", C.c_double), ("motion_phase_deg", C.c_double),
        ("coarse_sweeps", C.c_int), ("restart_drop", C.c_double), ("restart_every", C.c_int),
        ("xgrid", C.c_char * PATH_MAX), ("ygrid", C.c_char * PATH_MAX),
    ]


class Schedule(C.Structure):
    _fields_ = [
        ("mg_pre", C.c_int), ("mg_post", C.c_int), ("mg_omega", C.c_double),
        ("coarse_sweeps", C.c_int), ("mixed_inner", C.c_int),
        ("restart_drop", C.c_double), ("restart_every", C.c_int),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Stats(C.Structure):
    _fields_ = [
        ("steps", C.c_longlong),
        ("last_ad_iters", C.c_int), ("last_ppe_iters", C.c_int),
        ("last_ad_metric", C.c_double), ("last_ppe_residual", C.c_double),
        ("max_div", C.c_double), ("cd", C.c_double), ("cl", C.c_double),
        ("mass_flux_in", C.c_double), ("mass_flux_out", C.c_double),
        ("ad_iters_total", C.c_longlong), ("ppe_iters_total", C.c_longlong),
        ("kernel_launches", C.c_longlong),
        ("n_fluid", C.c_int), ("n_ibm_ghost", C.c_int), ("mg_levels", C.c_int),
        ("status", C.c_int),
    ]


def default_config():
    """The reference's inputs/inputs.txt values (mode REFERENCE), same as
    ifx_config_default in the library."""
    c = Config()
    c.restart, c.restart_time = 0, 9
    c.nx, c.ny = 50, 50
    c.lx, c.ly = 10.0, 5.0
    c.w_ad, c.w_ppe, c.ad_itermax, c.ppe_itermax, c.ad_solver, c.ppe_solver = 1, 1, 25, 100000, 1, 1
    c.error_max, c.tmax, c.dt, c.re, c.mu = 1e-6, 100.0, 0.001, 150.0, 0.01
    c.write_interval = 1000
    c.mode, c.precision, c.init = MODE_REFERENCE, PREC_FP64, INIT_VORTEX
    for s in range(4):
        c.bc_type[s] = BC_WALL
        c.bc_u[s] = 1.0
        c.bc_v[s] = 0.0
    c.outflow_uc = 1.0
    c.body = BODY_NONE
    c.body_cx, c.body_cy, c.body_a, c.body_b, c.body_angle_deg = 0.0, 0.0, 0.5, 0.5, 0.0
    c.ppe_tol = 1e-8
    c.ad_tol = 1e-12
    c.mg_pre, c.mg_post = 2, 2
    c.mg_omega = 0.8
    c.mixed_inner = 8
    c.coarse_sweeps, c.restart_drop, c.restart_every = 40, 1e-4, 25
    c.force_ref_u, c.force_ref_len = 1.0, 1.0
    c.ppe_method, c.relax_ad, c.relax_ppe = PPE_JACOBI, 1.0, 1.0
    c.xgrid = b"xgrid.dat2"
    c.ygrid = b"ygrid.dat2"
    return c
