"""Host-side solver object: owns one libmpxg handle and runs batched solves
on torch CUDA tensors (torch provides device memory and streams only).

    solver = Solver(desc, opts, n_max=100, batch_max=4096)
    out = solver.solve(x0, X0, U0, V0, reference, parameter, W, horizon)

mirrors `optimizers.mpc(cost, dynamics, hessian_approx, limited_memory,
reference, parameter, W, x0, X0, U0, V0) -> (X, U, V)` under jax.vmap
(mpx/utils/mpc_wrapper_srbd.py:68,77,124-132), with the model fixed at
construction instead of passed as callables.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .problem import NW, ModelDesc, SolverOptions

_F32 = torch.float32


def _ptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _stream_handle(stream):
    if stream is None:
        return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    return ctypes.c_void_p(stream.cuda_stream)


def problem_desc(desc, n_max, batch_max):
    d = _lib.ProblemDesc()
    d.model = int(desc.model); d.n = int(desc.n); d.m = int(desc.m); d.n_contact = int(desc.n_contact)
    d.n_max = int(n_max); d.batch_max = int(batch_max)
    d.dt = float(desc.dt); d.mass = float(desc.mass); d.gravity = float(desc.gravity); d.mu = float(desc.mu)
    d.barrier_alpha = float(desc.barrier_alpha); d.barrier_sigma = float(desc.barrier_sigma)
    d.foot_length = float(desc.foot_length); d.foot_width = float(desc.foot_width)
    d.barrier_kind = int(desc.barrier_kind); d.barrier_masked = int(desc.barrier_masked)
    d.barrier_hess_scale = float(desc.barrier_hess_scale)
    d.cone_eps2 = float(desc.cone_eps2)
    I = np.asarray(desc.inertia, dtype=np.float64).reshape(9)
    Ii = np.asarray(desc.inertia_inv, dtype=np.float64).reshape(9)
    for i in range(9):
        d.inertia[i] = float(I[i])
        d.inertia_inv[i] = float(Ii[i])
    return d


def solver_opts(opts, warps_per_block=0, blocks_per_sm=0):
    o = _lib.SolverOpts()
    o.sqp_iters = int(opts.sqp_iters); o.ls_max_trials = int(opts.ls_max_trials); o.ls_beta = float(opts.ls_beta)
    o.ls_eta = float(opts.ls_eta); o.reg = float(opts.reg); o.rho0 = float(opts.rho0)
    o.ls_skip_tol = float(opts.ls_skip_tol); o.compute_kkt = int(bool(opts.compute_kkt))
    o.warps_per_block = int(warps_per_block); o.blocks_per_sm = int(blocks_per_sm)
    o.team_warps = int(getattr(opts, "team_warps", 0))
    o.team_min_horizon = int(getattr(opts, "team_min_horizon", 64))
    o.team_exact_last = int(bool(getattr(opts, "team_exact_last", False)))
    return o


def weights_diagonal(W, batch=None):
    """The solver takes the diagonal of the reference's W [B, 24, 24]
    (mpc_wrapper_srbd.py:127 tiles one W per instance).  Off-diagonal entries
    are rejected: the compiled models use diagonal weights."""
    W = torch.as_tensor(W)
    if W.dim() == 1:
        w = W.reshape(1, NW)
    elif W.dim() == 2 and W.shape == (NW, NW):
        off = W - torch.diag_embed(torch.diagonal(W))
        if torch.count_nonzero(off).item() != 0:
            raise ValueError("W must be diagonal for the compiled SRBD models")
        w = torch.diagonal(W).reshape(1, NW)
    elif W.dim() == 2 and W.shape[1] == NW:
        w = W
    elif W.dim() == 3:
        d = torch.diagonal(W, dim1=-2, dim2=-1)
        off = W - torch.diag_embed(d)
        if torch.count_nonzero(off).item() != 0:
            raise ValueError("W must be diagonal for the compiled SRBD models")
        w = d
    else:
        raise ValueError("W must be [24,24], [B,24,24], [24] or [B,24]")
    if batch is not None and w.shape[0] == 1 and batch > 1:
        w = w.expand(batch, NW)
    return w


def check_shapes(desc, n_max, batch, **arrays):
    """Raise ValueError unless every given array has the shape the kernels
    index it with ([batch, ...], padded to n_max): the device reads these
    buffers without bounds of its own, so a short one would be read past its
    end.  (A check that python -O cannot strip.)"""
    N, n, m = n_max, desc.n, desc.m
    want = dict(x0=(batch, n), X0=(batch, N + 1, n), U0=(batch, N, m), V0=(batch, N + 1, n),
                reference=(batch, N + 1, desc.ref_cols), parameter=(batch, N + 1, desc.par_cols), w=(batch, NW),
                horizon=(batch,))
    for name, a in arrays.items():
        if a is not None and tuple(a.shape) != want[name]:
            raise ValueError("%s has shape %s; the solve needs %s (batch %d, padded to n_max = %d)"
                             % (name, tuple(a.shape), want[name], batch, N))


class Solver:
    """One libmpxg handle (fixed model, n_max and batch_max)."""

    def __init__(self, desc: ModelDesc, opts: SolverOptions = None, n_max=50, batch_max=1, device=None,
                 warps_per_block=0, blocks_per_sm=0):
        if not torch.cuda.is_available():
            raise _lib.MpxgError("CUDA is not available: the mpx_gb300 solver has no CPU path")
        self.L = _lib.load()
        self.desc = desc
        self.opts = opts or SolverOptions()
        self.n_max = int(n_max)
        self.batch_max = int(batch_max)
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self._pd = problem_desc(desc, self.n_max, self.batch_max)
        self._po = solver_opts(self.opts, warps_per_block, blocks_per_sm)
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            st = self.L.mpxg_create(ctypes.byref(self._pd), ctypes.byref(self._po), ctypes.byref(h))
        _lib.check(st, None, "mpxg_create")
        self.handle = h

    def close(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            self.L.mpxg_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def total_warps(self):
        """Warps of one persistent launch; mpxg_solve orders batches larger
        than this longest-horizon-first with one extra launch."""
        if getattr(self, "_total_warps", None) is None:
            g = self.geometry()
            self._total_warps = g["warps_per_block"] * g["blocks_per_sm"] * g["num_sms"]
        return self._total_warps

    def launches_per_solve(self, batch, horizon=True):
        """Kernel launches of one mpxg_solve: the solve, the longest-first
        ordering when needed, and the time-parallel team kernel beside the
        one-warp kernel when the team path is on."""
        tw = int(getattr(self.opts, "team_warps", 0))
        team = tw in (4, 8) and max(tw, int(self.opts.team_min_horizon)) <= self.n_max
        n = 1
        if horizon and (batch > self.total_warps or team):
            n += 1
        if team and horizon:
            n += 1
        return n

    def geometry(self):
        a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _lib.check(self.L.mpxg_query_geometry(self.handle, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)),
                   self.handle, "mpxg_query_geometry")
        return dict(warps_per_block=a.value, blocks_per_sm=b.value, num_sms=c.value)

    # ------------------------------------------------------------ tensors
    def _dev(self, a, dtype=_F32):
        if a is None:
            return None
        t = torch.as_tensor(a)
        if t.device != self.device or t.dtype != dtype:
            t = t.to(device=self.device, dtype=dtype)
        return t.contiguous()

    def empty_outputs(self, batch, want_gains=False):
        n, m, N = self.desc.n, self.desc.m, self.n_max
        dev = self.device
        out = dict(X=torch.empty(batch, N + 1, n, device=dev), U=torch.empty(batch, N, m, device=dev),
                   V=torch.empty(batch, N + 1, n, device=dev), kkt=torch.empty(batch, 3, device=dev),
                   status=torch.empty(batch, dtype=torch.int32, device=dev))
        if want_gains:
            out["K"] = torch.empty(batch, N, m, n, device=dev)
            out["k"] = torch.empty(batch, N, m, device=dev)
        return out

    def io(self, x0, X0, U0, V0, reference, parameter, w, horizon, out, slot=None):
        """Batch descriptor.  With `slot` (int32 device tensor [B]) the arrays
        are pools indexed by slot[b]; otherwise batch entry b is row b."""
        io = _lib.BatchIO()
        io.batch = int(slot.shape[0]) if slot is not None else int(x0.shape[0])
        io.slot = _ptr(slot)
        io.horizon = _ptr(horizon)
        io.x0, io.X_in, io.U_in, io.V_in = _ptr(x0), _ptr(X0), _ptr(U0), _ptr(V0)
        io.reference, io.parameter, io.w = _ptr(reference), _ptr(parameter), _ptr(w)
        io.X, io.U, io.V = _ptr(out["X"]), _ptr(out["U"]), _ptr(out["V"])
        io.K, io.k = _ptr(out.get("K")), _ptr(out.get("k"))
        io.kkt, io.status = _ptr(out.get("kkt")), _ptr(out.get("status"))
        io.first = _ptr(out.get("first"))
        return io

    def prepare(self, x0, X0, U0, V0, reference, parameter, W, horizon=None):
        """Move/convert inputs to contiguous float32 device tensors."""
        B = int(torch.as_tensor(x0).shape[0])
        x0, X0, U0, V0 = self._dev(x0), self._dev(X0), self._dev(U0), self._dev(V0)
        reference, parameter = self._dev(reference), self._dev(parameter)
        w = self._dev(weights_diagonal(torch.as_tensor(W), B)).contiguous()
        if horizon is not None:
            horizon = self._dev(horizon, torch.int32)
        check_shapes(self.desc, self.n_max, B, x0=x0, X0=X0, U0=U0, V0=V0, reference=reference, parameter=parameter,
                     w=w, horizon=horizon)
        return x0, X0, U0, V0, reference, parameter, w, horizon

    def solve(self, x0, X0, U0, V0, reference, parameter, W, horizon=None, stream=None, plain=False, out=None,
              want_gains=False):
        """Batched (or, with plain=True, one-launch-per-instance) SQP solve.
        Returns dict with X, U, V, kkt [B,3], status [B] (and K, k)."""
        x0, X0, U0, V0, reference, parameter, w, horizon = self.prepare(x0, X0, U0, V0, reference, parameter, W,
                                                                        horizon)
        B = x0.shape[0]
        if out is None:
            out = self.empty_outputs(B, want_gains)
        io = self.io(x0, X0, U0, V0, reference, parameter, w, horizon, out)
        fn = self.L.mpxg_solve_plain if plain else self.L.mpxg_solve
        with torch.cuda.device(self.device):
            st = fn(self.handle, _stream_handle(stream), ctypes.byref(io))
        _lib.check(st, self.handle, "mpxg_solve_plain" if plain else "mpxg_solve")
        out["_keep"] = (x0, X0, U0, V0, reference, parameter, w, horizon)
        return out

    def vjp(self, x0, X, U, V, reference, parameter, W, gX, gU, horizon=None, stream=None):
        """Vector-Jacobian product of a converged solve (mpxg_solve_vjp):
        cotangents gX [B,n_max+1,n], gU [B,n_max,m] of a scalar loss of the
        solution -> dict gx0 [B,n] (dLoss/dx0), gref [B,n_max+1,12]
        (dLoss/dreference, tracked state columns), and the adjoint solution
        wX, wU, wL."""
        x0, X, U, V, reference, parameter, w, horizon = self.prepare(x0, X, U, V, reference, parameter, W, horizon)
        gX, gU = self._dev(gX), self._dev(gU)
        B = x0.shape[0]
        N, n, m = self.n_max, self.desc.n, self.desc.m
        dev = self.device
        out = dict(gx0=torch.empty(B, n, device=dev), gref=torch.zeros(B, N + 1, 12, device=dev),
                   wX=torch.empty(B, N + 1, n, device=dev), wU=torch.empty(B, N, m, device=dev),
                   wL=torch.empty(B, N + 1, n, device=dev))
        v = _lib.VjpIO()
        v.io = self.io(x0, X, U, V, reference, parameter, w, horizon, dict(X=X, U=U, V=V))
        v.gX, v.gU = _ptr(gX), _ptr(gU)
        for k in ("wX", "wU", "wL", "gx0", "gref"):
            setattr(v, k, _ptr(out[k]))
        with torch.cuda.device(self.device):
            st = self.L.mpxg_solve_vjp(self.handle, _stream_handle(stream), ctypes.byref(v))
        _lib.check(st, self.handle, "mpxg_solve_vjp")
        out["_keep"] = (x0, X, U, V, reference, parameter, w, horizon, gX, gU)
        return out

    def evaluate(self, x0, X, U, reference, parameter, W, horizon=None, stream=None):
        """(g, c) of trajectories X, U (the reference's model_evaluator_helper,
        mpc_wrapper.py:419-423,452-465): g [B, n_max+1] the stage costs (sum =
        the objective), c [B, n_max+1, n] the initial-state and dynamics
        defects."""
        x0, X, U, _, reference, parameter, w, horizon = self.prepare(x0, X, U, X, reference, parameter, W, horizon)
        B = x0.shape[0]
        g = torch.empty(B, self.n_max + 1, device=self.device)
        c = torch.empty(B, self.n_max + 1, self.desc.n, device=self.device)
        st = self.L.mpxg_evaluate(self.handle, _stream_handle(stream), B, _ptr(horizon), _ptr(x0), _ptr(X), _ptr(U),
                                  _ptr(reference), _ptr(parameter), _ptr(w), _ptr(g), _ptr(c))
        _lib.check(st, self.handle, "mpxg_evaluate")
        return g, c

    def shift(self, X, U, V, horizon=None, shift=1, stream=None, out=None, slot=None):
        """Warm-start shift (mpc_wrapper_srbd.py:135-137) on the device; in
        place when out is None; only the pool rows in `slot` when given."""
        Xo, Uo, Vo = (X, U, V) if out is None else out
        batch = int(slot.shape[0]) if slot is not None else int(X.shape[0])
        st = self.L.mpxg_shift_warm_start(self.handle, _stream_handle(stream), batch, _ptr(slot), _ptr(horizon),
                                          int(shift), _ptr(X), _ptr(U), _ptr(V), _ptr(Xo), _ptr(Uo), _ptr(Vo))
        _lib.check(st, self.handle, "mpxg_shift_warm_start")
        return Xo, Uo, Vo


class MixedSolver:
    """One persistent launch over the batches of two solvers of different
    models (mpxg_solve_mixed): e.g. quadrupeds on `a` and bipeds on `b`.
    Each instance gives the bits its own solver's one-warp solve gives."""

    def __init__(self, a: Solver, b: Solver):
        self.a, self.b, self.L = a, b, _lib.load()
        h = ctypes.c_void_p()
        with torch.cuda.device(a.device):
            st = self.L.mpxg_mixed_create(a.handle, b.handle, ctypes.byref(h))
        _lib.check(st, None, "mpxg_mixed_create")
        self.handle = h

    def close(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            self.L.mpxg_mixed_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def solve(self, batch_a, batch_b, stream=None, want_gains=False):
        """batch_a / batch_b: tuples (x0, X0, U0, V0, reference, parameter, W,
        horizon) for solver a / b.  Returns (out_a, out_b) as Solver.solve."""
        outs, ios, keep = [], [], []
        for s, args in ((self.a, batch_a), (self.b, batch_b)):
            p = s.prepare(*args)
            out = s.empty_outputs(p[0].shape[0], want_gains)
            ios.append(s.io(*p, out))
            outs.append(out)
            keep.append(p)
        with torch.cuda.device(self.a.device):
            st = self.L.mpxg_solve_mixed(self.handle, _stream_handle(stream), ctypes.byref(ios[0]), ctypes.byref(ios[1]))
        _lib.check(st, None, "mpxg_solve_mixed")
        for out, p in zip(outs, keep):
            out["_keep"] = p
        return outs[0], outs[1]


MPXG_ERR_TIMEOUT, MPXG_ERR_NOT_READY = 5, 7


class SolveQueue:
    """Device work queue (mpxg_queue_*): one persistent kernel on `stream`
    solves the rows of `pool` (x0, X0, U0, V0, reference, parameter, W,
    horizon -- as Solver.solve takes them) as the host pushes them, while it
    runs.  `inputs` holds the device copies of the pool (update a row there
    before pushing it again), `out` the X, U, V, kkt, status outputs.  Every
    wait of the kernel is bounded by `idle_timeout_s`: a warp that waits
    longer for work stops, and push / result / finish then raise with
    "timeout" instead of blocking."""

    def __init__(self, solver: Solver, pool, capacity=1024, idle_timeout_s=1.0, stream=None):
        x0, X0, U0, V0, reference, parameter, w, horizon = solver.prepare(*pool)
        self.inputs = dict(x0=x0, X=X0, U=U0, V=V0, reference=reference, parameter=parameter, w=w, horizon=horizon)
        self.out = solver.empty_outputs(x0.shape[0])
        self._io = solver.io(x0, X0, U0, V0, reference, parameter, w, horizon, self.out)
        self.solver, self.L, self.m = solver, solver.L, solver.desc.m
        h = ctypes.c_void_p()
        with torch.cuda.device(solver.device):
            st = self.L.mpxg_queue_start(solver.handle, _stream_handle(stream), ctypes.byref(self._io), int(capacity),
                                         int(idle_timeout_s * 1e9), ctypes.byref(h))
        _lib.check(st, solver.handle, "mpxg_queue_start")
        self.handle = h

    def push(self, row):
        """Publish pool row `row`; returns its ticket, or None while the ring
        entry it needs still holds an unfinished ticket."""
        t = ctypes.c_longlong()
        st = self.L.mpxg_queue_push(self.handle, int(row), ctypes.byref(t))
        if st == MPXG_ERR_NOT_READY:
            return None
        _lib.check(st, self.solver.handle, "mpxg_queue_push")
        return t.value

    def result(self, ticket):
        """The ticket's result row [m controls, KKT triple, status] once
        solved, else None."""
        row = (ctypes.c_float * (self.m + 4))()
        st = self.L.mpxg_queue_result(self.handle, int(ticket), row)
        if st == MPXG_ERR_NOT_READY:
            return None
        _lib.check(st, self.solver.handle, "mpxg_queue_result")
        return np.frombuffer(row, dtype=np.float32).copy()

    def finish(self):
        """Let the kernel drain what was pushed, wait for it and free the queue."""
        if self.handle is None:
            return
        h, self.handle = self.handle, None
        _lib.check(self.L.mpxg_queue_finish(h), self.solver.handle, "mpxg_queue_finish")

    def __del__(self):
        try:
            self.finish()
        except Exception:
            pass


def lqr_solve(A, B, c, Q, R, M, q, r, x0, method=0, stream=None):
    """Batched time-varying LQR (absolute coordinates) on the device.
    Shapes as in include/mpxg.h mpxg_lqr_solve.  Returns dict K, k, X, U, lam."""
    L = _lib.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    t = [torch.as_tensor(a).to(device=dev, dtype=_F32).contiguous() for a in (A, B, c, Q, R, M, q, r, x0)]
    Bsz, N, n, _ = t[0].shape
    m = t[1].shape[-1]
    out = dict(K=torch.empty(Bsz, N, m, n, device=dev), k=torch.empty(Bsz, N, m, device=dev),
               X=torch.empty(Bsz, N + 1, n, device=dev), U=torch.empty(Bsz, N, m, device=dev),
               lam=torch.empty(Bsz, N + 1, n, device=dev))
    ws_bytes = int(L.mpxg_lqr_workspace_bytes(Bsz, N, n, m, method))
    ws = torch.empty(max(ws_bytes // 4, 1), device=dev)
    io = _lib.LqIO()
    io.batch, io.N, io.n, io.m = Bsz, N, n, m
    for name, ten in zip(("A", "Bm", "c", "Q", "R", "M", "q", "r", "x0"), t):
        setattr(io, name, _ptr(ten))
    for name in ("K", "k", "X", "U", "lam"):
        setattr(io, name, _ptr(out[name]))
    io.workspace = _ptr(ws)
    st = L.mpxg_lqr_solve(_stream_handle(stream), ctypes.byref(io), int(method))
    _lib.check(st, None, "mpxg_lqr_solve")
    out["_keep"] = (t, ws)
    return out


def lqr_eq_solve(A, B, c, Q, R, M, q, r, C, D, e, x0, stream=None, method=0):
    """Batched equality-constrained LQR on the device (mpxg_lqr_eq_solve_method:
    method 0 = stage products on the tensor cores, 1 = CUDA cores).  Shapes as
    in include/mpxg.h.  Returns dict K, k, Knu, knu, X, U, lam, nu."""
    L = _lib.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    names = ("A", "Bm", "c", "Q", "R", "M", "q", "r", "C", "D", "e", "x0")
    t = [torch.as_tensor(a).to(device=dev, dtype=_F32).contiguous() for a in (A, B, c, Q, R, M, q, r, C, D, e, x0)]
    Bsz, N, n, _ = t[0].shape
    m, ne = t[1].shape[-1], t[8].shape[-2]
    out = dict(K=torch.empty(Bsz, N, m, n, device=dev), k=torch.empty(Bsz, N, m, device=dev),
               Knu=torch.empty(Bsz, N, ne, n, device=dev), knu=torch.empty(Bsz, N, ne, device=dev),
               X=torch.empty(Bsz, N + 1, n, device=dev), U=torch.empty(Bsz, N, m, device=dev),
               lam=torch.empty(Bsz, N + 1, n, device=dev), nu=torch.empty(Bsz, N, ne, device=dev))
    ws = torch.empty(max(int(L.mpxg_lqr_eq_workspace_bytes(Bsz, N, n)) // 4, 1), device=dev)
    io = _lib.LqEqIO()
    io.batch, io.N, io.n, io.m, io.n_eq = Bsz, N, n, m, ne
    for name, ten in zip(names, t):
        setattr(io, name, _ptr(ten))
    for name in ("K", "k", "Knu", "knu", "X", "U", "lam", "nu"):
        setattr(io, name, _ptr(out[name]))
    io.workspace = _ptr(ws)
    _lib.check(L.mpxg_lqr_eq_solve_method(_stream_handle(stream), ctypes.byref(io), int(method)), None,
               "mpxg_lqr_eq_solve")
    out["_keep"] = (t, ws)
    return out


def lqr_eq_sqp(A, B, c, Q, R, M, q, r, C, D, e, x0, X, U, iters=2, stream=None, method=0, lam=None, nu=None):
    """SQP iterations on the batched equality-constrained LQ problem
    (mpxg_lqr_eq_sqp) from the iterate X [B,N+1,n], U [B,N,m]: each iteration
    solves the step problem at the iterate with the constrained Riccati
    (method 0 tensor cores, 1 CUDA cores) and takes the full step.  Returns
    dict X, U (the result), lam, nu (its multipliers), K, k, Knu, knu (the
    last step's gains), kkt [B,3] (primal residual, relative dual residual,
    their maximum).  iters=0 evaluates kkt at X, U and the given lam, nu."""
    L = _lib.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    names = ("A", "Bm", "c", "Q", "R", "M", "q", "r", "C", "D", "e", "x0")
    t = [torch.as_tensor(a).to(device=dev, dtype=_F32).contiguous() for a in (A, B, c, Q, R, M, q, r, C, D, e, x0)]
    Bsz, N, n, _ = t[0].shape
    m, ne = t[1].shape[-1], t[8].shape[-2]
    out = dict(K=torch.empty(Bsz, N, m, n, device=dev), k=torch.empty(Bsz, N, m, device=dev),
               Knu=torch.empty(Bsz, N, ne, n, device=dev), knu=torch.empty(Bsz, N, ne, device=dev),
               X=torch.as_tensor(X).to(device=dev, dtype=_F32).contiguous().clone(),
               U=torch.as_tensor(U).to(device=dev, dtype=_F32).contiguous().clone(),
               lam=torch.empty(Bsz, N + 1, n, device=dev), nu=torch.empty(Bsz, N, ne, device=dev),
               kkt=torch.empty(Bsz, 3, device=dev))
    if lam is not None:
        out["lam"].copy_(torch.as_tensor(lam, dtype=_F32))
    if nu is not None:
        out["nu"].copy_(torch.as_tensor(nu, dtype=_F32))
    ws = torch.empty(max(int(L.mpxg_lqr_eq_workspace_bytes(Bsz, N, n)) // 4, 1), device=dev)
    step = torch.empty(max(int(L.mpxg_lqr_eq_sqp_workspace_bytes(Bsz, N, n, m, ne)) // 4, 1), device=dev)
    io = _lib.LqEqSqpIO()
    io.lq.batch, io.lq.N, io.lq.n, io.lq.m, io.lq.n_eq = Bsz, N, n, m, ne
    for name, ten in zip(names, t):
        setattr(io.lq, name, _ptr(ten))
    for name in ("K", "k", "Knu", "knu", "X", "U", "lam", "nu"):
        setattr(io.lq, name, _ptr(out[name]))
    io.lq.workspace = _ptr(ws)
    io.iters, io.method, io.kkt, io.step = int(iters), int(method), _ptr(out["kkt"]), _ptr(step)
    _lib.check(L.mpxg_lqr_eq_sqp(_stream_handle(stream), ctypes.byref(io)), None, "mpxg_lqr_eq_sqp")
    out["_keep"] = (t, ws, step)
    return out


def gait_tables(stream, desc, batch, n_max, x0, X, U, V, v_ref, leg_time, reference, parameter, gait, mode,
                slot=None, horizon=None, drift_std=0.0, seed=0):
    """mpxg_gait_tables for `batch` entries (pool rows `slot`); `gait` =
    dict(duty, step_freq, height, offsets).  mode 0: first tick (cold start of
    X, U, V); mode 1: next tick (x0 from the shifted warm start + drift)."""
    L = _lib.load()
    a = _lib.GaitArgs()
    a.model, a.batch, a.n_max, a.mode = int(desc.model), int(batch), int(n_max), int(mode)
    a.slot, a.horizon = _ptr(slot), _ptr(horizon)
    a.dt, a.duty_factor, a.step_freq = float(desc.dt), float(gait["duty"]), float(gait["step_freq"])
    a.height, a.weight = float(gait["height"]), float(desc.mass * desc.gravity)
    a.drift_std, a.seed = float(drift_std), int(seed) & 0xFFFFFFFF
    off = np.zeros(12, dtype=np.float32)
    o = np.asarray(gait["offsets"], dtype=np.float32).reshape(-1)
    off[:o.size] = o
    for i in range(12):
        a.offsets[i] = float(off[i])
    a.x0, a.X, a.U, a.V = _ptr(x0), _ptr(X), _ptr(U), _ptr(V)
    a.v_ref, a.leg_time, a.reference, a.parameter = _ptr(v_ref), _ptr(leg_time), _ptr(reference), _ptr(parameter)
    _lib.check(L.mpxg_gait_tables(_stream_handle(stream), ctypes.byref(a)), None, "mpxg_gait_tables")
