"""ctypes binding of libmpxg.so (include/mpxg.h).

The library is built in-tree by mpx_gb300/build.py.  There is no CPU
fallback: if the library is missing or CUDA is unavailable, load() raises.
"""
import ctypes
import os

from . import build as _build

c_int_p = ctypes.POINTER(ctypes.c_int)
c_float_p = ctypes.POINTER(ctypes.c_float)

MPXG_OK = 0
STATUS_NAMES = {0: "ok", 1: "invalid argument", 2: "out of device memory", 3: "device-memory budget exhausted",
                4: "CUDA error", 5: "timeout", 6: "numerical failure", 7: "not ready", 8: "unsupported"}

# per-instance status bits
INST_NAN = 1
INST_NON_PD = 2
INST_LS_FAIL = 4


class ProblemDesc(ctypes.Structure):
    _fields_ = [("model", ctypes.c_int), ("n", ctypes.c_int), ("m", ctypes.c_int), ("n_contact", ctypes.c_int),
                ("n_max", ctypes.c_int), ("batch_max", ctypes.c_int),
                ("dt", ctypes.c_float), ("mass", ctypes.c_float), ("gravity", ctypes.c_float), ("mu", ctypes.c_float),
                ("barrier_alpha", ctypes.c_float), ("barrier_sigma", ctypes.c_float),
                ("foot_length", ctypes.c_float), ("foot_width", ctypes.c_float),
                ("barrier_kind", ctypes.c_int), ("barrier_masked", ctypes.c_int),
                ("barrier_hess_scale", ctypes.c_float),
                ("inertia", ctypes.c_float * 9), ("inertia_inv", ctypes.c_float * 9), ("cone_eps2", ctypes.c_float)]


class SolverOpts(ctypes.Structure):
    _fields_ = [("sqp_iters", ctypes.c_int), ("ls_max_trials", ctypes.c_int), ("ls_beta", ctypes.c_float),
                ("ls_eta", ctypes.c_float), ("reg", ctypes.c_float), ("rho0", ctypes.c_float),
                ("ls_skip_tol", ctypes.c_float), ("compute_kkt", ctypes.c_int),
                ("warps_per_block", ctypes.c_int), ("blocks_per_sm", ctypes.c_int),
                ("team_warps", ctypes.c_int), ("team_min_horizon", ctypes.c_int), ("team_exact_last", ctypes.c_int)]


class XlaOpaque(ctypes.Structure):
    _fields_ = [("desc", ProblemDesc), ("opts", SolverOpts), ("batch", ctypes.c_int), ("reserved", ctypes.c_int)]


class ServedModel(ctypes.Structure):
    _fields_ = [("desc", ProblemDesc), ("duty_factor", ctypes.c_float), ("step_freq", ctypes.c_float),
                ("height", ctypes.c_float), ("offsets", ctypes.c_float * 12), ("phase0", ctypes.c_float * 4),
                ("w", ctypes.c_float * 24)]


class ServerDesc(ctypes.Structure):
    _fields_ = [("n_models", ctypes.c_int), ("models", ctypes.POINTER(ServedModel)), ("n_max", ctypes.c_int),
                ("budget_bytes", ctypes.c_size_t), ("max_slots", ctypes.c_int), ("streams", ctypes.c_int),
                ("drift_std", ctypes.c_float), ("seed", ctypes.c_uint), ("opts", SolverOpts),
                ("mixed_launch", ctypes.c_int)]


class Result(ctypes.Structure):
    _fields_ = [("ticket", ctypes.c_longlong), ("episode", ctypes.c_int), ("status", ctypes.c_int),
                ("u0", ctypes.c_float * 12), ("kkt", ctypes.c_float * 3)]


class LqEqIO(ctypes.Structure):
    _fields_ = [("batch", ctypes.c_int), ("N", ctypes.c_int), ("n", ctypes.c_int), ("m", ctypes.c_int),
                ("n_eq", ctypes.c_int)] + [(k, ctypes.c_void_p) for k in (
                    "A", "Bm", "c", "Q", "R", "M", "q", "r", "C", "D", "e", "x0",
                    "K", "k", "Knu", "knu", "X", "U", "lam", "nu", "workspace")]


class LqEqSqpIO(ctypes.Structure):
    _fields_ = [("lq", LqEqIO), ("iters", ctypes.c_int), ("method", ctypes.c_int), ("kkt", ctypes.c_void_p),
                ("step", ctypes.c_void_p)]


class BatchIO(ctypes.Structure):
    _fields_ = [("batch", ctypes.c_int), ("slot", ctypes.c_void_p), ("horizon", ctypes.c_void_p),
                ("x0", ctypes.c_void_p), ("X_in", ctypes.c_void_p), ("U_in", ctypes.c_void_p),
                ("V_in", ctypes.c_void_p), ("reference", ctypes.c_void_p), ("parameter", ctypes.c_void_p),
                ("w", ctypes.c_void_p), ("X", ctypes.c_void_p), ("U", ctypes.c_void_p), ("V", ctypes.c_void_p),
                ("K", ctypes.c_void_p), ("k", ctypes.c_void_p), ("kkt", ctypes.c_void_p),
                ("status", ctypes.c_void_p), ("first", ctypes.c_void_p)]


class VjpIO(ctypes.Structure):
    _fields_ = [("io", BatchIO)] + [(k, ctypes.c_void_p) for k in ("gX", "gU", "wX", "wU", "wL", "gx0", "gref")]


class GaitArgs(ctypes.Structure):
    _fields_ = [("model", ctypes.c_int), ("batch", ctypes.c_int), ("n_max", ctypes.c_int), ("mode", ctypes.c_int),
                ("slot", ctypes.c_void_p), ("horizon", ctypes.c_void_p),
                ("dt", ctypes.c_float), ("duty_factor", ctypes.c_float), ("step_freq", ctypes.c_float),
                ("height", ctypes.c_float), ("weight", ctypes.c_float), ("drift_std", ctypes.c_float),
                ("seed", ctypes.c_uint), ("offsets", ctypes.c_float * 12),
                ("x0", ctypes.c_void_p), ("X", ctypes.c_void_p), ("U", ctypes.c_void_p), ("V", ctypes.c_void_p),
                ("v_ref", ctypes.c_void_p), ("leg_time", ctypes.c_void_p),
                ("reference", ctypes.c_void_p), ("parameter", ctypes.c_void_p)]


class LqIO(ctypes.Structure):
    _fields_ = [("batch", ctypes.c_int), ("N", ctypes.c_int), ("n", ctypes.c_int), ("m", ctypes.c_int)] + \
               [(k, ctypes.c_void_p) for k in ("A", "Bm", "c", "Q", "R", "M", "q", "r", "x0",
                                                "K", "k", "X", "U", "lam", "workspace")]


WB_MAX_BODY, WB_MAX_DOF, WB_MAX_CONTACT = 32, 32, 8


class WbModel(ctypes.Structure):
    """mpxg_wb_model (include/mpxg.h)."""
    _B, _C = WB_MAX_BODY, WB_MAX_CONTACT
    _fields_ = [("nbody", ctypes.c_int), ("nq", ctypes.c_int), ("nv", ctypes.c_int), ("n_contact", ctypes.c_int),
                ("parent", ctypes.c_int * _B), ("jnt_type", ctypes.c_int * _B), ("qpos_adr", ctypes.c_int * _B),
                ("dof_adr", ctypes.c_int * _B),
                ("body_pos", (ctypes.c_float * 3) * _B), ("body_quat", (ctypes.c_float * 4) * _B),
                ("jnt_pos", (ctypes.c_float * 3) * _B), ("jnt_axis", (ctypes.c_float * 3) * _B),
                ("mass", ctypes.c_float * _B), ("com", (ctypes.c_float * 3) * _B),
                ("inertia", (ctypes.c_float * 9) * _B), ("armature", ctypes.c_float * WB_MAX_DOF),
                ("gravity", ctypes.c_float * 3),
                ("contact_point_body", ctypes.c_int * _C), ("contact_jac_body", ctypes.c_int * _C),
                ("contact_point_pos", (ctypes.c_float * 3) * _C)]


class WbSqpIO(ctypes.Structure):
    """mpxg_wb_sqp_io (include/mpxg.h)."""
    _fields_ = [("model", ctypes.POINTER(WbModel)), ("batch", ctypes.c_int), ("N", ctypes.c_int),
                ("iters", ctypes.c_int), ("dt", ctypes.c_float), ("alpha", ctypes.c_float),
                ("swing_tracking", ctypes.c_int), ("reg", ctypes.c_float), ("rho0", ctypes.c_float),
                ("ls_beta", ctypes.c_float), ("ls_eta", ctypes.c_float), ("ls_skip_tol", ctypes.c_float),
                ("ls_max_trials", ctypes.c_int)] + \
               [(k, ctypes.c_void_p) for k in ("x0", "X", "U", "V", "reference", "contact", "W", "kkt", "status",
                                                "workspace")]


# Exported symbols (every entry point declared in include/mpxg.h).
EXPORTS = ["mpxg_create", "mpxg_destroy", "mpxg_query_geometry", "mpxg_workspace_bytes", "mpxg_solve",
           "mpxg_solve_plain", "mpxg_shift_warm_start", "mpxg_timer_run", "mpxg_refgen_srbd", "mpxg_gait_tables",
           "mpxg_lqr_workspace_bytes", "mpxg_lqr_solve", "mpxg_solve_noalloc", "mpxg_evaluate", "mpxg_xla_solve", "mpxg_xla_solve_vjp", "mpxg_xla_prepare", "mpxg_lqr_eq_workspace_bytes", "mpxg_lqr_eq_solve", "mpxg_lqr_eq_solve_method", "mpxg_lqr_eq_sqp_workspace_bytes", "mpxg_lqr_eq_sqp", "mpxg_mixed_create", "mpxg_mixed_destroy", "mpxg_solve_mixed", "mpxg_queue_start", "mpxg_queue_push", "mpxg_queue_result", "mpxg_queue_finish", "mpxg_solve_vjp",
           "mpxg_server_create", "mpxg_server_destroy", "mpxg_server_capacity", "mpxg_server_admit",
           "mpxg_server_reset", "mpxg_server_release", "mpxg_submit", "mpxg_submit_many", "mpxg_server_step", "mpxg_poll",
           "mpxg_server_completed", "mpxg_server_stats", "mpxg_server_last_error", "mpxg_last_error", "mpxg_status_string", "mpxg_version",
           "mpxg_wb_terms", "mpxg_wb_interface", "mpxg_wb_step", "mpxg_wb_sqp_workspace_bytes", "mpxg_wb_sqp",
           "mpxg_refgen_wb"]

_lib = None


class MpxgError(RuntimeError):
    pass


def lib_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load libmpxg.so (building it first if its sources are newer)."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_missing:
        _build.build()
    path = _build.LIB
    if not os.path.exists(path):
        raise MpxgError("libmpxg.so is not built (%s); run mpx_gb300.build.build()" % path)
    L = ctypes.CDLL(path)
    vp = ctypes.c_void_p
    L.mpxg_create.argtypes = [ctypes.POINTER(ProblemDesc), ctypes.POINTER(SolverOpts), ctypes.POINTER(vp)]
    L.mpxg_create.restype = ctypes.c_int
    ci, cll, cf = ctypes.c_int, ctypes.c_longlong, ctypes.c_float
    L.mpxg_server_create.argtypes = [ctypes.POINTER(ServerDesc), ctypes.POINTER(vp)]
    L.mpxg_server_destroy.argtypes = [vp]
    L.mpxg_server_destroy.restype = None
    L.mpxg_server_capacity.argtypes = [vp, ci]
    L.mpxg_server_admit.argtypes = [vp, ci, vp, ci, cf, cf, ctypes.POINTER(ci)]
    L.mpxg_server_reset.argtypes = [vp, ci, vp]
    L.mpxg_server_release.argtypes = [vp, ci]
    L.mpxg_submit.argtypes = [vp, ci, ctypes.POINTER(cll)]
    L.mpxg_submit_many.argtypes = [vp, vp, ci, vp]
    L.mpxg_server_step.argtypes = [vp, ci, ctypes.POINTER(ci), ctypes.POINTER(ci)]
    L.mpxg_poll.argtypes = [vp, cll, ctypes.POINTER(Result)]
    L.mpxg_server_completed.argtypes = [vp, ctypes.POINTER(Result), ci, ctypes.POINTER(ci)]
    L.mpxg_server_stats.argtypes = [vp, ctypes.POINTER(ci), ctypes.POINTER(ci), ctypes.POINTER(cll)]
    L.mpxg_server_last_error.argtypes = [vp]
    L.mpxg_server_last_error.restype = ctypes.c_char_p
    for fn in ("mpxg_server_create", "mpxg_server_capacity", "mpxg_server_admit", "mpxg_server_reset",
               "mpxg_server_release", "mpxg_submit", "mpxg_submit_many", "mpxg_server_step", "mpxg_poll", "mpxg_server_completed",
               "mpxg_server_stats"):
        getattr(L, fn).restype = ctypes.c_int
    L.mpxg_solve_vjp.argtypes = [vp, vp, ctypes.POINTER(VjpIO)]
    L.mpxg_solve_vjp.restype = ctypes.c_int
    L.mpxg_lqr_eq_workspace_bytes.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int]
    L.mpxg_lqr_eq_workspace_bytes.restype = ctypes.c_size_t
    L.mpxg_lqr_eq_solve.argtypes = [vp, ctypes.POINTER(LqEqIO)]
    L.mpxg_lqr_eq_solve.restype = ctypes.c_int
    L.mpxg_lqr_eq_solve_method.argtypes = [vp, ctypes.POINTER(LqEqIO), ctypes.c_int]
    L.mpxg_lqr_eq_solve_method.restype = ctypes.c_int
    L.mpxg_lqr_eq_sqp_workspace_bytes.argtypes = [ctypes.c_int] * 5
    L.mpxg_lqr_eq_sqp_workspace_bytes.restype = ctypes.c_size_t
    L.mpxg_lqr_eq_sqp.argtypes = [vp, ctypes.POINTER(LqEqSqpIO)]
    L.mpxg_lqr_eq_sqp.restype = ctypes.c_int
    L.mpxg_mixed_create.argtypes = [vp, vp, ctypes.POINTER(vp)]
    L.mpxg_mixed_create.restype = ctypes.c_int
    L.mpxg_mixed_destroy.argtypes = [vp]
    L.mpxg_mixed_destroy.restype = None
    L.mpxg_solve_mixed.argtypes = [vp, vp, ctypes.POINTER(BatchIO), ctypes.POINTER(BatchIO)]
    L.mpxg_solve_mixed.restype = ctypes.c_int
    L.mpxg_queue_start.argtypes = [vp, vp, ctypes.POINTER(BatchIO), ctypes.c_int, ctypes.c_longlong, ctypes.POINTER(vp)]
    L.mpxg_queue_start.restype = ctypes.c_int
    L.mpxg_queue_push.argtypes = [vp, ctypes.c_int, ctypes.POINTER(ctypes.c_longlong)]
    L.mpxg_queue_push.restype = ctypes.c_int
    L.mpxg_queue_result.argtypes = [vp, ctypes.c_longlong, ctypes.POINTER(ctypes.c_float)]
    L.mpxg_queue_result.restype = ctypes.c_int
    L.mpxg_queue_finish.argtypes = [vp]
    L.mpxg_queue_finish.restype = ctypes.c_int
    L.mpxg_wb_terms.argtypes = [vp, ctypes.POINTER(WbModel), ctypes.c_int] + [vp] * 7
    L.mpxg_wb_terms.restype = ctypes.c_int
    L.mpxg_wb_interface.argtypes = [vp, ctypes.POINTER(WbModel), ctypes.c_int] + [vp] * 10
    L.mpxg_wb_interface.restype = ctypes.c_int
    L.mpxg_wb_step.argtypes = [vp, ctypes.POINTER(WbModel), ctypes.c_int, ctypes.c_float, ctypes.c_float] + [vp] * 4
    L.mpxg_wb_step.restype = ctypes.c_int
    L.mpxg_wb_sqp_workspace_bytes.argtypes = [ctypes.POINTER(WbModel), ctypes.c_int, ctypes.c_int]
    L.mpxg_wb_sqp_workspace_bytes.restype = ctypes.c_size_t
    L.mpxg_wb_sqp.argtypes = [vp, ctypes.POINTER(WbSqpIO)]
    L.mpxg_wb_sqp.restype = ctypes.c_int
    L.mpxg_refgen_wb.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_float, vp, vp,
                                 ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_int] + \
        [vp] * 8
    L.mpxg_refgen_wb.restype = ctypes.c_int
    L.mpxg_xla_solve.argtypes = [vp, ctypes.POINTER(vp), ctypes.c_char_p, ctypes.c_size_t, vp]
    L.mpxg_xla_solve.restype = None
    L.mpxg_xla_solve_vjp.argtypes = [vp, ctypes.POINTER(vp), ctypes.c_char_p, ctypes.c_size_t, vp]
    L.mpxg_xla_solve_vjp.restype = None
    L.mpxg_xla_prepare.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
    L.mpxg_xla_prepare.restype = ctypes.c_int
    L.mpxg_evaluate.argtypes = [vp, vp, ctypes.c_int] + [vp] * 9
    L.mpxg_evaluate.restype = ctypes.c_int
    L.mpxg_destroy.argtypes = [vp]
    L.mpxg_destroy.restype = None
    L.mpxg_query_geometry.argtypes = [vp, c_int_p, c_int_p, c_int_p]
    L.mpxg_query_geometry.restype = ctypes.c_int
    L.mpxg_workspace_bytes.argtypes = [ctypes.POINTER(ProblemDesc), ctypes.POINTER(SolverOpts)]
    L.mpxg_workspace_bytes.restype = ctypes.c_size_t
    for name in ("mpxg_solve", "mpxg_solve_plain"):
        f = getattr(L, name)
        f.argtypes = [vp, vp, ctypes.POINTER(BatchIO)]
        f.restype = ctypes.c_int
    L.mpxg_shift_warm_start.argtypes = [vp, vp, ctypes.c_int, vp, vp, ctypes.c_int, vp, vp, vp, vp, vp, vp]
    L.mpxg_shift_warm_start.restype = ctypes.c_int
    L.mpxg_timer_run.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                 vp, vp]
    L.mpxg_timer_run.restype = ctypes.c_int
    L.mpxg_refgen_srbd.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float, c_float_p,
                                   ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                   vp, vp, vp, vp, vp, vp, vp, vp, vp]
    L.mpxg_refgen_srbd.restype = ctypes.c_int
    L.mpxg_gait_tables.argtypes = [vp, ctypes.POINTER(GaitArgs)]
    L.mpxg_gait_tables.restype = ctypes.c_int
    L.mpxg_lqr_workspace_bytes.argtypes = [ctypes.c_int] * 5
    L.mpxg_lqr_workspace_bytes.restype = ctypes.c_size_t
    L.mpxg_lqr_solve.argtypes = [vp, ctypes.POINTER(LqIO), ctypes.c_int]
    L.mpxg_lqr_solve.restype = ctypes.c_int
    L.mpxg_solve_noalloc.argtypes = [ctypes.POINTER(ProblemDesc), ctypes.POINTER(SolverOpts), vp,
                                     ctypes.POINTER(BatchIO)]
    L.mpxg_solve_noalloc.restype = ctypes.c_int
    L.mpxg_last_error.argtypes = [vp]
    L.mpxg_last_error.restype = ctypes.c_char_p
    L.mpxg_status_string.argtypes = [ctypes.c_int]
    L.mpxg_status_string.restype = ctypes.c_char_p
    L.mpxg_version.restype = ctypes.c_int
    _lib = L
    return L


def check(status, handle=None, what="mpxg call"):
    if status != MPXG_OK:
        L = load()
        msg = L.mpxg_last_error(handle).decode() if L is not None else ""
        raise MpxgError("%s failed: %s (%s)" % (what, STATUS_NAMES.get(status, status), msg))
