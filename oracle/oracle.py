"""ctypes bindings of the CPU oracle (test infrastructure, not the product).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
arm import this module.  It loads oracle/_build/liboracle.so (built by
oracle/build_oracle.py) and exposes numpy-level helpers:

  * sqp_solve(...)      full primal-dual SQP of a batch, FP32 or FP64
  * kkt_residual(...)   FP64 KKT residual of given trajectories
  * lqr_solve(...)      sequential-Riccati LQR in absolute coordinates
  * dense_lqr(...)      the same LQR by one dense KKT solve (numpy), the
                        ground truth the Riccati recursion is checked against
  * dynamics/cost/linearize/penalty, timer_run, refgen_srbd, refgen_wb

See oracle.hpp for what each restates (reference file:line) and the parity
status ("parity unpinned" for the SQP/KKT solver).
"""
import ctypes
import os

import numpy as np

from . import build_oracle

_lib = None

c_int_p = ctypes.POINTER(ctypes.c_int)
c_double_p = ctypes.POINTER(ctypes.c_double)
c_float_p = ctypes.POINTER(ctypes.c_float)


class OrcModel(ctypes.Structure):
    _fields_ = [("model", ctypes.c_int), ("n", ctypes.c_int), ("m", ctypes.c_int), ("n_contact", ctypes.c_int),
                ("dt", ctypes.c_double), ("mass", ctypes.c_double), ("gravity", ctypes.c_double),
                ("mu", ctypes.c_double), ("barrier_alpha", ctypes.c_double), ("barrier_sigma", ctypes.c_double),
                ("foot_length", ctypes.c_double), ("foot_width", ctypes.c_double),
                ("barrier_kind", ctypes.c_int), ("barrier_masked", ctypes.c_int), ("barrier_hess_scale", ctypes.c_double),
                ("inertia", ctypes.c_double * 9), ("inertia_inv", ctypes.c_double * 9), ("cone_eps2", ctypes.c_double)]


class OrcOpts(ctypes.Structure):
    _fields_ = [("sqp_iters", ctypes.c_int), ("ls_max_trials", ctypes.c_int), ("ls_beta", ctypes.c_double),
                ("ls_eta", ctypes.c_double), ("reg", ctypes.c_double), ("rho0", ctypes.c_double),
                ("ls_skip_tol", ctypes.c_double)]


class OrcLQ(ctypes.Structure):
    _fields_ = [(k, c_double_p) for k in ("A", "B", "c", "Q", "R", "M", "q", "r")]


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = ctypes.CDLL(path)
        L.orc_sqp_solve.restype = ctypes.c_int
        L.orc_kkt_residual.restype = ctypes.c_int
        L.orc_cost.restype = ctypes.c_double
        L.orc_cost_f32.restype = ctypes.c_float
        L.orc_penalty.restype = ctypes.c_double
        L.orc_penalty.argtypes = [ctypes.POINTER(OrcModel), ctypes.c_double]
        L.orc_penalty_dd.restype = ctypes.c_double
        L.orc_penalty_dd.argtypes = [ctypes.POINTER(OrcModel), ctypes.c_double]
        L.orc_timer_run.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_int, c_float_p, c_int_p]
        L.orc_num_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _dp(a):
    return None if a is None else a.ctypes.data_as(c_double_p)


def _fp(a):
    return None if a is None else a.ctypes.data_as(c_float_p)


def _ip(a):
    return None if a is None else a.ctypes.data_as(c_int_p)


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


def _f32(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float32)


def make_model(desc):
    """OrcModel from any object with the model-description attributes."""
    md = OrcModel()
    md.model = int(desc.model)
    md.n = int(desc.n)
    md.m = int(desc.m)
    md.n_contact = int(getattr(desc, "n_contact", 0))
    md.dt = float(getattr(desc, "dt", 0.0))
    md.mass = float(getattr(desc, "mass", 1.0))
    md.gravity = float(getattr(desc, "gravity", 9.81))
    md.mu = float(getattr(desc, "mu", 0.7))
    md.barrier_alpha = float(getattr(desc, "barrier_alpha", 0.1))
    md.barrier_sigma = float(getattr(desc, "barrier_sigma", 5.0))
    md.foot_length = float(getattr(desc, "foot_length", 0.0))
    md.foot_width = float(getattr(desc, "foot_width", 0.0))
    md.barrier_kind = int(getattr(desc, "barrier_kind", 0))
    md.barrier_masked = int(getattr(desc, "barrier_masked", 0))
    md.barrier_hess_scale = float(getattr(desc, "barrier_hess_scale", 1.0))
    md.cone_eps2 = float(getattr(desc, "cone_eps2", 1e-2))
    I = np.asarray(getattr(desc, "inertia", np.eye(3)), dtype=np.float64).reshape(9)
    Ii = np.asarray(getattr(desc, "inertia_inv", np.linalg.inv(I.reshape(3, 3))), dtype=np.float64).reshape(9)
    for i in range(9):
        md.inertia[i] = I[i]
        md.inertia_inv[i] = Ii[i]
    return md


def make_opts(opts):
    od = OrcOpts()
    od.sqp_iters = int(opts.sqp_iters)
    od.ls_max_trials = int(opts.ls_max_trials)
    od.ls_beta = float(opts.ls_beta)
    od.ls_eta = float(opts.ls_eta)
    od.reg = float(opts.reg)
    od.rho0 = float(opts.rho0)
    od.ls_skip_tol = float(opts.ls_skip_tol)
    return od


def _lq_struct(lq):
    if lq is None:
        return None, []
    keep = [_f64(lq[k]) for k in ("A", "B", "c", "Q", "R", "M", "q", "r")]
    s = OrcLQ(*[_dp(a) for a in keep])
    return s, keep


def sqp_solve(desc, opts, x0, X0, U0, V0, reference=None, parameter=None, W=None, horizon=None, lq=None,
              precision=64, n_threads=0, want_kkt=True):
    """Batched SQP solve on the CPU.  Returns dict of numpy float64 arrays."""
    L = lib()
    md, od = make_model(desc), make_opts(opts)
    x0, X0, U0, V0 = _f64(x0), _f64(X0), _f64(U0), _f64(V0)
    B, Np1, n = X0.shape
    Nmax = Np1 - 1
    m = U0.shape[2]
    reference, parameter, W = _f64(reference), _f64(parameter), _f64(W)
    hz = None if horizon is None else np.ascontiguousarray(horizon, dtype=np.int32)
    X, U, V = X0.copy(), U0.copy(), V0.copy()
    K = np.zeros((B, Nmax, m, n))
    k = np.zeros((B, Nmax, m))
    kkt = np.zeros((B, 3)) if want_kkt else None
    status = np.zeros(B, dtype=np.int32)
    lqs, keep = _lq_struct(lq)
    rc = L.orc_sqp_solve(ctypes.byref(md), ctypes.byref(od), int(precision), B, Nmax, _ip(hz), _dp(x0), _dp(X0),
                         _dp(U0), _dp(V0), _dp(reference), _dp(parameter), _dp(W),
                         ctypes.byref(lqs) if lqs is not None else None, _dp(X), _dp(U), _dp(V), _dp(K), _dp(k),
                         _dp(kkt), _ip(status), int(n_threads))
    assert rc == 0
    return dict(X=X, U=U, V=V, K=K, k=k, kkt=kkt, status=status)


def kkt_residual(desc, x0, X, U, V, reference=None, parameter=None, W=None, horizon=None, lq=None):
    """FP64 KKT residual [B, 3] = (r_prim, r_dual, max) of given trajectories."""
    L = lib()
    md = make_model(desc)
    X, U, V, x0 = _f64(X), _f64(U), _f64(V), _f64(x0)
    B, Np1, n = X.shape
    hz = None if horizon is None else np.ascontiguousarray(horizon, dtype=np.int32)
    out = np.zeros((B, 3))
    lqs, keep = _lq_struct(lq)
    L.orc_kkt_residual(ctypes.byref(md), B, Np1 - 1, _ip(hz), _dp(x0), _dp(X), _dp(U), _dp(V), _dp(_f64(reference)),
                       _dp(_f64(parameter)), _dp(_f64(W)), ctypes.byref(lqs) if lqs is not None else None, _dp(out))
    return out


def dynamics(desc, x, u, par, precision=64):
    L = lib()
    md = make_model(desc)
    if precision == 32:
        x, u, par = _f32(x), _f32(u), _f32(par)
        out = np.zeros(md.n, dtype=np.float32)
        L.orc_dynamics_f32(ctypes.byref(md), _fp(x), _fp(u), _fp(par), _fp(out))
        return out
    x, u, par = _f64(x), _f64(u), _f64(par)
    out = np.zeros(md.n)
    L.orc_dynamics(ctypes.byref(md), _dp(x), _dp(u), _dp(par), _dp(out))
    return out


def cost(desc, x, u, ref, W, terminal=False, precision=64):
    L = lib()
    md = make_model(desc)
    if precision == 32:
        return float(L.orc_cost_f32(ctypes.byref(md), _fp(_f32(x)), _fp(_f32(u)), _fp(_f32(ref)), _fp(_f32(W)),
                                    int(terminal)))
    return float(L.orc_cost(ctypes.byref(md), _dp(_f64(x)), _dp(_f64(u)), _dp(_f64(ref)), _dp(_f64(W)), int(terminal)))


def linearize(desc, x, u, ref, par, W, terminal=False):
    """(A, B, fx, g, H, l) of one SRBD stage in FP64."""
    L = lib()
    md = make_model(desc)
    n, m = md.n, md.m
    A = np.zeros((n, n)); Bm = np.zeros((n, m)); fx = np.zeros(n); g = np.zeros(n + m)
    H = np.zeros((n + m, n + m)); l = np.zeros(1)
    L.orc_linearize(ctypes.byref(md), _dp(_f64(x)), _dp(_f64(u)), _dp(_f64(ref)), _dp(_f64(par)), _dp(_f64(W)),
                    int(terminal), _dp(A), _dp(Bm), _dp(fx), _dp(g), _dp(H), _dp(l))
    return A, Bm, fx, g, H, float(l[0])


def stage_flops(desc, x, u, ref, par, W):
    """Model FLOPs of one non-terminal stage at (x, u), counted on the
    oracle's model functions with the counting scalar of flops.hpp: dict of
    dyn_value, dyn_jacobian, cost_value, linearisation and trial."""
    out = np.zeros(5)
    lib().orc_stage_flops(ctypes.byref(make_model(desc)), _dp(_f64(x)), _dp(_f64(u)), _dp(_f64(ref)),
                          _dp(_f64(par)), _dp(_f64(W)), _dp(out))
    return dict(zip(("dyn_value", "dyn_jacobian", "cost_value", "linearisation", "trial"), out.tolist()))


def penalty(desc, c):
    return lib().orc_penalty(ctypes.byref(make_model(desc)), float(c))


def penalty_dd(desc, c):
    return lib().orc_penalty_dd(ctypes.byref(make_model(desc)), float(c))


def timer_run(duty, step_freq, dt, leg_time):
    lt = _f32(leg_time).copy()
    cont = np.zeros(lt.shape[0], dtype=np.int32)
    lib().orc_timer_run(float(duty), float(step_freq), float(dt), lt.shape[0], _fp(lt), _ip(cont))
    return cont, lt


def refgen_srbd(N, dt, mass, foot0, duty_factor, step_freq, step_height, clearence_speed, t_timer, x, foot, input,
                contact, liftoff):
    """One instance of the SRBD reference generator (FP32).  Returns
    (reference[N+1,17], parameter[N+1,16], liftoff[12], foot_ref_dot[N+1,12])."""
    L = lib()
    lo = _f32(liftoff).copy()
    ref = np.zeros((N + 1, 17), dtype=np.float32)
    par = np.zeros((N + 1, 16), dtype=np.float32)
    frd = np.zeros((N + 1, 12), dtype=np.float32)
    f = ctypes.c_float
    L.orc_refgen_srbd(int(N), f(dt), f(mass), _fp(_f32(foot0)), f(duty_factor), f(step_freq), f(step_height),
                      f(clearence_speed), _fp(_f32(t_timer)), _fp(_f32(x)), _fp(_f32(foot)), _fp(_f32(input)),
                      _fp(_f32(contact)), _fp(lo), _fp(ref), _fp(par), _fp(frd))
    return ref, par, lo, frd


def refgen_wb(N, nj, dt, mass, foot0, q0, duty_factor, step_freq, step_height, clearence_speed, terrain, t_timer, x,
              foot, input, contact, liftoff):
    """One instance of the whole-body reference generator (FP32; terrain:
    use_terrain_estimation).  Returns (reference[N+1,13+nj+28],
    parameter[N+1,4], liftoff[12])."""
    L = lib()
    lo = _f32(liftoff).copy()
    ref = np.zeros((N + 1, 13 + nj + 28), dtype=np.float32)
    par = np.zeros((N + 1, 4), dtype=np.float32)
    f = ctypes.c_float
    L.orc_refgen_wb(int(N), int(nj), f(dt), f(mass), _fp(_f32(foot0)), _fp(_f32(q0)), f(duty_factor), f(step_freq),
                    f(step_height), f(clearence_speed), int(terrain), _fp(_f32(t_timer)), _fp(_f32(x)),
                    _fp(_f32(foot)), _fp(_f32(input)), _fp(_f32(contact)), _fp(lo), _fp(ref), _fp(par))
    return ref, par, lo


def lqr_solve(A, Bm, c, Q, R, M, q, r, x0, precision=64, n_threads=0):
    """Sequential-Riccati LQR in absolute coordinates for a batch.

    A [B,N,n,n], Bm [B,N,n,m], c [B,N,n], Q [B,N+1,n,n] (row N terminal),
    R [B,N,m,m], M [B,N,n,m], q [B,N+1,n], r [B,N,m], x0 [B,n].
    Returns dict K [B,N,m,n], k [B,N,m], X [B,N+1,n], U [B,N,m], lam [B,N+1,n]."""
    L = lib()
    A = _f64(A)
    B_, N, n, _ = A.shape
    m = Bm.shape[-1]
    args = [_f64(a) for a in (A, Bm, c, Q, R, M, q, r, x0)]
    K = np.zeros((B_, N, m, n)); k = np.zeros((B_, N, m))
    X = np.zeros((B_, N + 1, n)); U = np.zeros((B_, N, m)); lam = np.zeros((B_, N + 1, n))
    L.orc_lqr_solve(int(precision), B_, N, n, m, *[_dp(a) for a in args], _dp(K), _dp(k), _dp(X), _dp(U), _dp(lam),
                    int(n_threads))
    return dict(K=K, k=k, X=X, U=U, lam=lam)


def dense_lqr(A, Bm, c, Q, R, M, q, r, x0):
    """One instance of the LQR solved as a single dense KKT system (FP64).

    Variables z = [x_0, u_0, x_1, u_1, ..., x_N]; constraints x_0 = x0 and
    x_{t+1} = A_t x_t + B_t u_t + c_t.  Returns (X, U, lam) with lam the
    multipliers in the convention lam_t = dV_t/dx_t (the costates)."""
    N, n, _ = A.shape
    m = Bm.shape[-1]
    nv = (N + 1) * n + N * m
    ne = (N + 1) * n

    def xi(t):
        return t * (n + m)

    def ui(t):
        return t * (n + m) + n

    H = np.zeros((nv, nv)); g = np.zeros(nv)
    C = np.zeros((ne, nv)); d = np.zeros(ne)
    for t in range(N):
        H[xi(t):xi(t) + n, xi(t):xi(t) + n] = Q[t]
        H[xi(t):xi(t) + n, ui(t):ui(t) + m] = M[t]
        H[ui(t):ui(t) + m, xi(t):xi(t) + n] = M[t].T
        H[ui(t):ui(t) + m, ui(t):ui(t) + m] = R[t]
        g[xi(t):xi(t) + n] = q[t]
        g[ui(t):ui(t) + m] = r[t]
    H[xi(N):xi(N) + n, xi(N):xi(N) + n] = Q[N]
    g[xi(N):xi(N) + n] = q[N]
    # x_0 - x0 = 0 ; x_{t+1} - A x_t - B u_t - c_t = 0
    C[0:n, xi(0):xi(0) + n] = np.eye(n)
    d[0:n] = x0
    for t in range(N):
        rows = slice((t + 1) * n, (t + 2) * n)
        C[rows, xi(t + 1):xi(t + 1) + n] = np.eye(n)
        C[rows, xi(t):xi(t) + n] = -A[t]
        C[rows, ui(t):ui(t) + m] = -Bm[t]
        d[rows] = c[t]
    K = np.block([[H, C.T], [C, np.zeros((ne, ne))]])
    rhs = np.concatenate([-g, d])
    sol = np.linalg.solve(K, rhs)
    z, nu = sol[:nv], sol[nv:]
    X = np.stack([z[xi(t):xi(t) + n] for t in range(N + 1)])
    U = np.stack([z[ui(t):ui(t) + m] for t in range(N)])
    # stationarity: H z + g + C^T nu = 0; with L = J + lam_0.(x0 - x_0) + sum lam_{t+1}.(f - x_{t+1})
    # the costates are lam = -nu.
    lam = -nu.reshape(N + 1, n)
    return X, U, lam


def num_threads():
    return int(lib().orc_num_threads())
