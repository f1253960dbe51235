"""Generate golden vectors by executing the reference's own Python source.

JAX and MuJoCo are not installable here, so this script runs the reference
files (mpx/utils/mpc_utils.py, models.py, objectives.py and
mpx/config/config_srbd.py, read from a reference checkout) under a small
stand-in for the parts of `jax`, `jax.numpy` and `mujoco.mjx` they use:

  * jax.numpy   -> numpy with JAX's default dtype rules (float32, int32, Python
                   scalars weakly typed, integer powers by square-and-multiply,
                   `.at[...].set(...)`);
  * jax.lax.fori_loop, jax.jit, jax.vmap -> plain Python equivalents;
  * jax.jacobian / jax.grad -> central finite differences (only used in the
                   float64 mode, to evaluate the Gauss-Newton Hessian of
                   objectives.py:39-75);
  * mujoco.mjx math (quat_to_mat, quat_integrate, quat_sub, norm, normalize)
                -> restated from their mathematical definition (third-party
                   code, not present in the reference tree);
  * jax.scipy.linalg.cho_factor / cho_solve -> scipy's.

With --wb it runs the whole-body MPC models instead.  These are the
quadruped of config_aliengo.py (quadruped_wb_dynamics, models.py:39-117;
quadruped_wb_obj and quadruped_wb_hessian_gn, objectives.py:77-203) and the
humanoid models of config_h1.py and config_talos.py (h1_wb_dynamics and
talos_wb_dynamics, models.py:119-216; their costs and Gauss-Newton Hessians,
objectives.py:204-450).  The humanoids run on the models of
tests/golden/{h1,talos}_wb.npz, written by make_wb_fixture.py.  mjx.make_data,
fwd_position, fwd_velocity and jac are then stood in for by the float64
rigid-body oracle (oracle/wholebody.py) on the aliengo MJCF.  Those vectors
therefore pin the model's own formulas (the contact-force solve, the masking,
the integration, the cost and its Hessian) to the reference's source.  The
rigid-body terms themselves are pinned separately
(tests/test_oracle_wholebody.py).

Usage:  python tests/golden/make_golden.py /path/to/reference [--wb] [out.npz]
Output: tests/golden/srbd_golden.npz, or tests/golden/wb_golden.npz with --wb
(committed).  The tests never run this script; they only read the .npz.
"""
import functools
import importlib.util
import os
import sys
import types

import numpy as np
import scipy.linalg as scipy_linalg

HERE = os.path.dirname(os.path.abspath(__file__))
DT = {"f": np.float32, "i": np.int32}


# ----------------------------------------------------------------- array type
def _canon(a):
    if isinstance(a, np.ndarray) and not isinstance(a, JArr):
        if a.dtype == np.float64 and DT["f"] == np.float32:
            return a.astype(np.float32)
        if a.dtype.kind in "iu" and a.dtype != DT["i"]:
            return a.astype(DT["i"])
    return a


def _is_float(a):
    if isinstance(a, float):
        return True
    return isinstance(a, np.ndarray) and a.dtype.kind == "f"


def _wrap(x):
    if isinstance(x, tuple):
        return tuple(_wrap(v) for v in x)
    if isinstance(x, np.ndarray):
        x = _canon(np.asarray(x))
        return x.view(JArr)
    if isinstance(x, (np.floating, np.integer, np.bool_)):
        return _wrap(np.asarray(x))
    return x


def _prep(args, float_op=True):
    args = [np.asarray(a) if isinstance(a, JArr) else a for a in args]
    args = [_canon(a) if isinstance(a, np.ndarray) else a for a in args]
    if float_op and any(_is_float(a) for a in args):
        args = [a.astype(DT["f"]) if isinstance(a, np.ndarray) and a.dtype.kind in "iub" else a for a in args]
    return args


class _At:
    def __init__(self, arr):
        self.arr = arr

    def __getitem__(self, idx):
        arr = self.arr

        class _Setter:
            def set(self_inner, v):
                out = np.array(arr, copy=True)
                out[idx] = np.asarray(v)
                return _wrap(out)
        return _Setter()


class JArr(np.ndarray):
    @property
    def at(self):
        return _At(self)

    @property
    def T(self):
        return _wrap(np.asarray(self).T)

    def __array_ufunc__(self, ufunc, method, *inputs, **kwargs):
        logical = ufunc in (np.logical_and, np.logical_or, np.logical_not, np.greater, np.less, np.equal,
                            np.not_equal, np.greater_equal, np.less_equal)
        args = _prep(inputs, float_op=not logical)
        out = kwargs.pop("out", None)
        if ufunc is np.power and isinstance(args[1], (int, np.integer)) and not isinstance(args[1], bool):
            res = _ipow(args[0], int(args[1]))
        else:
            res = getattr(ufunc, method)(*args, **kwargs)
        if out is not None:  # in-place operators (a += b): write through the plain view
            np.asarray(out[0])[...] = res
            return out[0]
        return _wrap(res)

    def __matmul__(self, other):
        return _matmul(self, other)

    def __rmatmul__(self, other):
        return _matmul(other, self)

    def __pow__(self, p):
        if isinstance(p, (int, np.integer)):
            return _wrap(_ipow(np.asarray(self), int(p)))
        return _wrap(np.power(*_prep([self, p])))


def _ipow(x, y):
    """jax.lax.integer_pow: square-and-multiply."""
    if y == 0:
        return np.ones_like(x)
    acc = None
    while y > 0:
        if y & 1:
            acc = x if acc is None else (acc * x).astype(x.dtype)
        y >>= 1
        if y > 0:
            x = (x * x).astype(x.dtype)
    return acc


def _matmul(a, b):
    a, b = _prep([a, b])
    a = np.asarray(a); b = np.asarray(b)
    vec_a, vec_b = a.ndim == 1, b.ndim == 1
    A = a[None, :] if vec_a else a
    Bm = b[:, None] if vec_b else b
    out = np.zeros((A.shape[0], Bm.shape[1]), dtype=np.result_type(A, Bm))
    for k in range(A.shape[1]):  # sequential accumulation, one rounding per multiply and add
        out = (out + (A[:, k:k + 1] * Bm[k:k + 1, :]).astype(out.dtype)).astype(out.dtype)
    if vec_a:
        out = out[0]
    if vec_b:
        out = out[..., 0]
    return _wrap(out)


# ----------------------------------------------------------------- jax.numpy
def _np_fn(name, float_op=True):
    f = getattr(np, name)

    @functools.wraps(f)
    def g(*args, **kw):
        return _wrap(f(*_prep(args, float_op), **kw))
    return g


def _array(x, dtype=None):
    if isinstance(x, (list, tuple)):
        elems = [np.asarray(e) for e in x]
        kinds = {e.dtype.kind for e in elems}
        pyfloat = any(isinstance(e, float) for e in x)
        if dtype is None:
            dtype = DT["f"] if ("f" in kinds or pyfloat) else (DT["i"] if kinds <= {"i", "u"} else None)
        return _wrap(np.array([np.asarray(e) for e in x], dtype=dtype))
    a = np.asarray(x)
    if dtype is None:
        dtype = DT["f"] if a.dtype.kind == "f" else (DT["i"] if a.dtype.kind in "iu" else a.dtype)
    return _wrap(a.astype(dtype))


def _where(c, a, b):
    a2, b2 = _prep([a, b])
    if isinstance(a2, (int, np.integer)) and isinstance(b2, (int, np.integer)):
        return _wrap(np.where(np.asarray(c), np.int32(a2), np.int32(b2)))
    return _wrap(np.where(np.asarray(c), a2, b2))


def _sum(x, axis=None):
    x = np.asarray(_prep([x])[0])
    if axis is None:
        x = x.reshape(-1)
        acc = np.zeros((), dtype=x.dtype)
        for v in x:
            acc = (acc + v).astype(x.dtype)
        return _wrap(acc)
    return _wrap(np.sum(x, axis=axis))


def _norm(x, axis=None):
    x = np.asarray(_prep([x])[0])
    return _wrap(np.sqrt(_sum(x * x)))


def _zeros(shape, dtype=None):
    return _wrap(np.zeros(shape, dtype=dtype or DT["f"]))


def _ones(shape, dtype=None):
    return _wrap(np.ones(shape, dtype=dtype or DT["f"]))


def _arange(*a):
    return _wrap(np.arange(*a, dtype=DT["i"]))


def _tile(x, reps):
    return _wrap(np.tile(np.asarray(_prep([x])[0]), reps))


def _concatenate(xs, axis=0):
    xs = _prep(xs)
    return _wrap(np.concatenate([np.atleast_1d(np.asarray(v)) for v in xs], axis=axis))


def _stack(xs, axis=0):
    return _wrap(np.stack(_prep(xs), axis=axis))


def _block_diag(*ms):
    ms = [np.atleast_2d(np.asarray(_prep([m])[0])) for m in ms]
    r = sum(m.shape[0] for m in ms)
    c = sum(m.shape[1] for m in ms)
    out = np.zeros((r, c), dtype=np.result_type(*ms))
    i = j = 0
    for m in ms:
        out[i:i + m.shape[0], j:j + m.shape[1]] = m
        i += m.shape[0]; j += m.shape[1]
    return _wrap(out)


def _fori_loop(lo, hi, body, init):
    carry = init
    for i in range(lo, hi):
        carry = body(i, carry)
    return carry


def _jit(f=None, **kw):
    if f is None:
        return lambda g: g
    return f


def _vmap(f, in_axes=0):
    def g(*args):
        n = np.asarray(args[0]).shape[0]
        outs = [f(*[np.asarray(a)[i] for a in args]) for i in range(n)]
        return _wrap(np.stack([np.asarray(o) for o in outs]))
    return g


def _fd_jacobian(f, argnums=0, h=1e-6):
    """Central-difference Jacobian (float64 mode only)."""
    def jac(*args):
        args = list(args)
        x = np.asarray(args[argnums], dtype=np.float64)
        f0 = np.asarray(f(*args))
        J = np.zeros(f0.shape + x.shape)
        for idx in np.ndindex(x.shape):
            e = np.zeros_like(x); e[idx] = h
            ap = list(args); ap[argnums] = _wrap(x + e)
            am = list(args); am[argnums] = _wrap(x - e)
            J[(...,) + idx] = (np.asarray(f(*ap)) - np.asarray(f(*am))) / (2 * h)
        return _wrap(J)
    return jac


def _fd_grad(f, argnums=0, h=1e-3):
    """Derivative of a scalar function by the 4th-order five-point stencil
    (nested for grad(grad(.)), so its error must stay small)."""
    def d(*args, **kw):
        args = list(args)
        x = np.asarray(args[argnums], dtype=np.float64)

        def at(s):
            a = list(args)
            a[argnums] = _wrap(x + s)
            return np.asarray(f(*a, **kw), dtype=np.float64)
        return _wrap((-at(2 * h) + 8 * at(h) - 8 * at(-h) + at(-2 * h)) / (12 * h))
    return d


# ----------------------------------------------------------------- mjx math
def _mjx_norm(x, axis=None):
    x = np.asarray(x)
    return _wrap(np.sqrt(np.sum(x * x, axis=axis)))


def _normalize_with_norm(x):
    n = _mjx_norm(x)
    return _wrap(np.asarray(x) / (n + 1e-6 * (n == 0.0))), n


def _quat_mul(u, v):
    u = np.asarray(u); v = np.asarray(v)
    return _array([u[0] * v[0] - u[1] * v[1] - u[2] * v[2] - u[3] * v[3],
                   u[0] * v[1] + u[1] * v[0] + u[2] * v[3] - u[3] * v[2],
                   u[0] * v[2] - u[1] * v[3] + u[2] * v[0] + u[3] * v[1],
                   u[0] * v[3] + u[1] * v[2] - u[2] * v[1] + u[3] * v[0]])


def _quat_to_mat(q):
    q = np.asarray(q)
    o = np.outer(q, q)
    return _array([[o[0, 0] + o[1, 1] - o[2, 2] - o[3, 3], 2 * (o[1, 2] - o[0, 3]), 2 * (o[1, 3] + o[0, 2])],
                   [2 * (o[1, 2] + o[0, 3]), o[0, 0] - o[1, 1] + o[2, 2] - o[3, 3], 2 * (o[2, 3] - o[0, 1])],
                   [2 * (o[1, 3] - o[0, 2]), 2 * (o[2, 3] + o[0, 1]), o[0, 0] - o[1, 1] - o[2, 2] + o[3, 3]]])


def _quat_integrate(q, v, dt):
    v, nrm = _normalize_with_norm(v)
    angle = np.asarray(nrm) * dt
    s, c = np.sin(angle / 2), np.cos(angle / 2)
    qr = _concatenate([_array([c]), _wrap(np.asarray(v) * s)])
    qn = _quat_mul(q, qr)
    n, _ = _normalize_with_norm(qn)
    return n


def _quat_sub(u, v):
    vc = _wrap(np.asarray(v) * np.array([1, -1, -1, -1], dtype=np.asarray(v).dtype))
    q = _quat_mul(vc, u)
    axis, sin_a_2 = _normalize_with_norm(np.asarray(q)[1:])
    angle = 2 * np.arctan2(np.asarray(sin_a_2), np.asarray(q)[0])
    angle = np.where(angle > np.pi, angle - 2 * np.pi, angle)
    return _wrap(np.asarray(axis) * angle)


# ----------------------------------------------------------------- install
class _Rotation:
    """jax.scipy.spatial.transform.Rotation.from_matrix(m).as_quat() (x, y, z,
    w) in the active float type, by the published algorithm jax's Rotation
    follows (scipy's before it orthogonalised its input): pick the largest of
    the diagonal and the trace, form the quaternion from that pivot, and
    normalise it; no orthogonalisation of a matrix whose columns are not
    orthogonal (scipy >= 1.11 projects such a matrix first, so it cannot
    stand in)."""

    def __init__(self, q):
        self.q = q

    @classmethod
    def from_matrix(cls, m):
        m = np.asarray(m, dtype=DT["f"])
        f = DT["f"]
        tr = f(f(m[0, 0] + m[1, 1]) + m[2, 2])
        dec = [m[0, 0], m[1, 1], m[2, 2], tr]
        c = int(np.argmax(dec))
        q = np.zeros(4, dtype=f)
        if c != 3:
            i, j, k = c, (c + 1) % 3, (c + 2) % 3
            q[i] = f(f(1.0 - tr) + f(2.0 * m[i, i]))
            q[j] = f(m[j, i] + m[i, j])
            q[k] = f(m[k, i] + m[i, k])
            q[3] = f(m[k, j] - m[j, k])
        else:
            q[0] = f(m[2, 1] - m[1, 2])
            q[1] = f(m[0, 2] - m[2, 0])
            q[2] = f(m[1, 0] - m[0, 1])
            q[3] = f(1.0 + tr)
        n = f(np.sqrt(f(f(f(q[0] * q[0] + q[1] * q[1]) + q[2] * q[2]) + q[3] * q[3])))
        return cls(q / n)

    def as_quat(self):
        return _wrap(np.asarray(self.q, dtype=DT["f"]))


def install_shim():
    jnp = types.ModuleType("jax.numpy")
    for name in ("sqrt", "square", "cos", "sin", "arctan2", "arcsin", "log", "clip", "cross", "logical_and",
                 "logical_or", "logical_not", "ones_like", "diag", "abs", "maximum", "minimum"):
        setattr(jnp, name, _np_fn(name, float_op=name not in ("logical_and", "logical_or", "logical_not")))
    jnp.array = _array
    jnp.where = _where
    jnp.sum = _sum
    jnp.zeros = _zeros
    jnp.ones = _ones
    jnp.arange = _arange
    jnp.tile = _tile
    jnp.concatenate = _concatenate
    jnp.stack = _stack
    jnp.pi = np.pi
    jnp.float32 = np.float32
    jnp.kron = lambda a, b: _wrap(np.kron(*_prep([a, b])))
    jnp.roll = lambda a, k: _wrap(np.roll(np.asarray(a), k))
    jnp.eye = lambda n, dtype=None: _wrap(np.eye(n, dtype=DT["f"]))
    linalg = types.ModuleType("jax.numpy.linalg")
    linalg.norm = _norm
    linalg.inv = lambda a: _wrap(np.linalg.inv(np.asarray(a)))
    jnp.linalg = linalg
    jax = types.ModuleType("jax")
    jax.numpy = jnp
    jax.jit = _jit
    jax.vmap = _vmap
    jax.jacobian = _fd_jacobian
    jax.grad = _fd_grad
    jax.config = types.SimpleNamespace(update=lambda *a, **k: None)
    lax = types.ModuleType("jax.lax")
    lax.fori_loop = _fori_loop
    jax.lax = lax
    scipy = types.ModuleType("jax.scipy")
    sl = types.ModuleType("jax.scipy.linalg")
    sl.block_diag = _block_diag
    sl.cho_factor = lambda a, lower=False: (_wrap(np.asarray(scipy_linalg.cho_factor(np.asarray(a), lower=lower)[0])),
                                            lower)
    sl.cho_solve = lambda cl, b: _wrap(scipy_linalg.cho_solve((np.asarray(cl[0]), cl[1]), np.asarray(b)))
    scipy.linalg = sl
    st = types.ModuleType("jax.scipy.spatial")
    stt = types.ModuleType("jax.scipy.spatial.transform")
    stt.Rotation = _Rotation
    st.transform = stt
    scipy.spatial = st
    jax.scipy = scipy
    mj = types.ModuleType("mujoco")
    mjx = types.ModuleType("mujoco.mjx")
    src = types.ModuleType("mujoco.mjx._src")
    mth = types.ModuleType("mujoco.mjx._src.math")
    mth.quat_to_mat = _quat_to_mat
    mth.quat_integrate = _quat_integrate
    mth.quat_sub = _quat_sub
    mth.norm = _mjx_norm
    mth.normalize_with_norm = _normalize_with_norm
    src.math = mth
    mjx._src = src
    mj.mjx = mjx
    for name, mod in (("jax", jax), ("jax.numpy", jnp), ("jax.numpy.linalg", linalg), ("jax.lax", lax),
                      ("jax.scipy", scipy), ("jax.scipy.linalg", sl), ("jax.scipy.spatial", st),
                      ("jax.scipy.spatial.transform", stt), ("mujoco", mj), ("mujoco.mjx", mjx),
                      ("mujoco.mjx._src", src), ("mujoco.mjx._src.math", mth)):
        sys.modules[name] = mod


def load(ref_root, rel, name):
    path = os.path.join(ref_root, rel)
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


# ----------------------------------------------------------------- generation
def main(ref_root, out):
    install_shim()
    cfg = load(ref_root, "mpx/config/config_srbd.py", "ref_config_srbd")
    mu = load(ref_root, "mpx/utils/mpc_utils.py", "ref_mpc_utils")
    mo = load(ref_root, "mpx/utils/models.py", "ref_models")
    ob = load(ref_root, "mpx/utils/objectives.py", "ref_objectives")
    rng = np.random.default_rng(2024)
    g = {}

    # --- gait timer (mpc_utils.py:7-14), config_srbd gait and the trot of the benchmark
    for tag, duty, freq in (("srbd", float(cfg.duty_factor), float(cfg.step_freq)), ("trot", 0.6, 2.0)):
        lt = rng.uniform(0, 1, (32, 4)).astype(np.float32)
        g["timer_%s_init" % tag] = lt.copy()
        cs, ts = [], []
        cur = _wrap(lt)
        for _ in range(60):
            c, cur = mu.timer_run(np.float32(duty), np.float32(freq), cur, np.float32(cfg.dt))
            cs.append(np.asarray(c)); ts.append(np.asarray(cur))
        g["timer_%s_contact" % tag] = np.stack(cs).astype(np.int32)
        g["timer_%s_time" % tag] = np.stack(ts).astype(np.float32)
        g["timer_%s_params" % tag] = np.array([duty, freq, cfg.dt], dtype=np.float32)

    # --- reference generator (mpc_utils.py:146-270) with config_srbd constants
    foot0 = np.asarray(cfg.p_legs0, dtype=np.float32)
    R = 12
    ins = dict(t_timer=rng.uniform(0, 1, (R, 4)), x=np.zeros((R, 13)), foot=np.zeros((R, 12)),
               input=np.zeros((R, 7)), contact=rng.integers(0, 2, (R, 4)).astype(np.float64),
               liftoff=np.zeros((R, 12)))
    for r in range(R):
        q = rng.normal(0, 0.1, 4); q[0] += 1; q /= np.linalg.norm(q)
        ins["x"][r] = np.concatenate([rng.normal(0, 0.1, 3) + [0, 0, 0.33], q, rng.normal(0, 0.3, 6)])
        ins["foot"][r] = foot0 + rng.normal(0, 0.02, 12)
        ins["input"][r] = np.concatenate([rng.uniform(-1, 1, 3), rng.uniform(-0.5, 0.5, 3), [cfg.robot_height]])
        ins["liftoff"][r] = ins["foot"][r] + rng.normal(0, 0.01, 12)
    for k in ins:
        ins[k] = ins[k].astype(np.float32)
        g["refgen_in_" + k] = ins[k]
    outs = {"reference": [], "parameter": [], "liftoff": [], "foot_ref_dot": []}
    for r in range(R):
        ref, par, lo, frd = mu.reference_generator_srbd(
            cfg.use_terrain_estimator, cfg.N, cfg.dt, cfg.n_contact, float(cfg.mass), _wrap(foot0),
            _wrap(ins["t_timer"][r]), _wrap(ins["x"][r]), _wrap(ins["foot"][r]), _wrap(ins["input"][r]),
            np.float32(cfg.duty_factor), np.float32(cfg.step_freq), np.float32(cfg.step_height),
            _wrap(ins["liftoff"][r]), _wrap(ins["contact"][r]), np.float32(cfg.clearence_speed))
        outs["reference"].append(np.asarray(ref)); outs["parameter"].append(np.asarray(par))
        outs["liftoff"].append(np.asarray(lo)); outs["foot_ref_dot"].append(np.asarray(frd))
    for k, v in outs.items():
        g["refgen_out_" + k] = np.stack(v).astype(np.float32)
    g["refgen_cfg"] = np.array([cfg.N, cfg.dt, cfg.mass, cfg.duty_factor, cfg.step_freq, cfg.step_height,
                                cfg.clearence_speed], dtype=np.float64)
    g["refgen_foot0"] = foot0

    # --- dynamics (models.py:6-37), float32, config_srbd body
    mass = float(cfg.mass)
    inertia = np.asarray(cfg.inertia, dtype=np.float32)
    inertia_inv = np.linalg.inv(np.asarray(cfg.inertia, dtype=np.float64)).astype(np.float32)
    D = 40
    xs, us, pars, xn = [], [], [], []
    for _ in range(D):
        q = rng.normal(0, 0.2, 4); q[0] += 1; q /= np.linalg.norm(q)
        x = np.concatenate([rng.normal(0, 0.1, 3) + [0, 0, 0.33], q, rng.normal(0, 0.5, 6)]).astype(np.float32)
        u = rng.normal(0, 20, 12).astype(np.float32); u[2::3] += 60
        par = np.concatenate([rng.integers(0, 2, 4), foot0 + rng.normal(0, 0.05, 12)]).astype(np.float32)
        parameter = np.stack([par, par])
        xnext = mo.quadruped_srbd_dynamics(mass, _wrap(inertia), _wrap(inertia_inv), float(cfg.dt), _wrap(x),
                                           _wrap(u), 0, _wrap(parameter))
        xs.append(x); us.append(u); pars.append(par); xn.append(np.asarray(xnext))
    g["dyn_x"], g["dyn_u"], g["dyn_par"], g["dyn_xnext"] = [np.stack(a).astype(np.float32) for a in (xs, us, pars, xn)]
    g["dyn_const"] = np.array([mass, cfg.dt], dtype=np.float64)
    g["dyn_inertia"] = np.asarray(cfg.inertia, dtype=np.float64)

    # --- stage cost (objectives.py:15-37), float32, config_srbd W
    W = np.asarray(cfg.W, dtype=np.float32)
    C = 40
    cx, cu, cref, cval, cterm = [], [], [], [], []
    for i in range(C):
        q = rng.normal(0, 0.2, 4); q[0] += 1; q /= np.linalg.norm(q)
        x = np.concatenate([rng.normal(0, 0.1, 3) + [0, 0, 0.33], q, rng.normal(0, 0.5, 6)]).astype(np.float32)
        u = rng.normal(0, 10, 12).astype(np.float32); u[2::3] = np.abs(u[2::3]) * rng.uniform(0, 6)
        qr = rng.normal(0, 0.1, 4); qr[0] += 1; qr /= np.linalg.norm(qr)
        refrow = np.concatenate([rng.normal(0, 0.1, 3) + [0, 0, 0.33], qr, rng.normal(0, 0.5, 6),
                                 rng.integers(0, 2, 4)]).astype(np.float32)
        reference = np.stack([refrow, refrow])
        term = (i % 4 == 3)
        t = 1 if term else 0
        val = ob.quadruped_srbd_obj(cfg.n_contact, 1, _wrap(W), _wrap(reference), _wrap(x), _wrap(u), t)
        cx.append(x); cu.append(u); cref.append(refrow); cval.append(float(np.asarray(val))); cterm.append(term)
    g["cost_x"], g["cost_u"], g["cost_ref"] = [np.stack(a).astype(np.float32) for a in (cx, cu, cref)]
    g["cost_val"] = np.array(cval, dtype=np.float32)
    g["cost_terminal"] = np.array(cterm, dtype=np.int32)
    g["cost_W"] = W

    # --- Gauss-Newton Hessian (objectives.py:39-75), float64 mode with finite-difference autodiff
    DT["f"] = np.float64
    H = 20
    hx, hu, href, hQ, hR, hM = [], [], [], [], [], []
    for i in range(H):
        q = rng.normal(0, 0.2, 4); q[0] += 1; q /= np.linalg.norm(q)
        x = np.concatenate([rng.normal(0, 0.1, 3) + [0, 0, 0.33], q, rng.normal(0, 0.5, 6)])
        u = rng.normal(0, 10, 12); u[2::3] = np.abs(u[2::3]) * rng.uniform(0.05, 2.0)
        qr = rng.normal(0, 0.1, 4); qr[0] += 1; qr /= np.linalg.norm(qr)
        refrow = np.concatenate([rng.normal(0, 0.1, 3) + [0, 0, 0.33], qr, rng.normal(0, 0.5, 6),
                                 rng.integers(0, 2, 4)])
        reference = np.stack([refrow, refrow])
        Q, Rm, M = ob.quadruped_srbd_hessian_gn(cfg.n_contact, _wrap(W.astype(np.float64)), _wrap(reference),
                                                _wrap(x), _wrap(u), 0)
        hx.append(x); hu.append(u); href.append(refrow)
        hQ.append(np.asarray(Q)); hR.append(np.asarray(Rm)); hM.append(np.asarray(M))
    DT["f"] = np.float32
    g["hess_x"], g["hess_u"], g["hess_ref"] = [np.stack(a) for a in (hx, hu, href)]
    g["hess_Q"], g["hess_R"], g["hess_M"] = [np.stack(a) for a in (hQ, hR, hM)]
    np.savez_compressed(out, **g)
    print("wrote", out, {k: v.shape for k, v in g.items()})


# ----------------------------------------------------------------- whole-body model
class _FakeMjxData:
    """The fields of an mjx Data that models.py:39-117 reads, computed by the
    float64 rigid-body oracle (oracle/wholebody.py) for the parsed model."""

    def __init__(self, model, qpos=None, qvel=None):
        self.model, self.qpos, self.qvel = model, qpos, qvel

    def replace(self, qpos=None, qvel=None):
        return _FakeMjxData(self.model, self.qpos if qpos is None else qpos, self.qvel if qvel is None else qvel)


def _install_fake_mjx():
    """mjx.make_data / fwd_position / fwd_velocity / jac over the oracle:
    qLD is the upper Cholesky factor U of qM (qM = U'U), which is what the
    reference's cho_solve((qLD, False), .) needs; geom_xpos rows are the
    contact points in the model's contact order."""
    sys.path.insert(0, os.path.join(HERE, "..", ".."))
    from oracle import wholebody as Wb
    mjx = sys.modules["mujoco.mjx"]

    def fwd_position(m, d):
        t = Wb.terms(m, np.asarray(d.qpos, dtype=np.float64), np.zeros(m.nv))
        d.qM = _wrap(t["M"])
        d.qLD = _wrap(np.linalg.cholesky(t["M"]).T)
        d.geom_xpos = _wrap(t["cpos"].reshape(-1, 3))
        d.T = Wb.kinematics(m, np.asarray(d.qpos, dtype=np.float64))
        return d

    def fwd_velocity(m, d):
        t = Wb.terms(m, np.asarray(d.qpos, dtype=np.float64), np.asarray(d.qvel, dtype=np.float64))
        d.qfrc_bias = _wrap(t["bias"])
        return d

    def jac(m, d, point, body_id):
        Jp, Jr = Wb.point_jacobian(m, d.T, int(body_id), np.asarray(point, dtype=np.float64))
        return _wrap(Jp.T), _wrap(Jr.T)

    mjx.make_data = lambda model: _FakeMjxData(model)
    mjx.fwd_position = fwd_position
    mjx.fwd_velocity = fwd_velocity
    mjx.jac = jac


def main_wb(ref_root, out):
    """Golden vectors of the whole-body MPC model: quadruped_wb_dynamics
    (models.py:39-117, float64, over the oracle's rigid-body terms for the
    aliengo model), quadruped_wb_obj (objectives.py:77-144, float32) and
    quadruped_wb_hessian_gn (objectives.py:146-203, float64 with
    finite-difference autodiff), with config_aliengo's W."""
    install_shim()
    _install_fake_mjx()
    sys.path.insert(0, os.path.join(HERE, "..", ".."))
    from mpx_gb300 import mjcf
    mo = load(ref_root, "mpx/utils/models.py", "ref_models")
    ob = load(ref_root, "mpx/utils/objectives.py", "ref_objectives")
    pkg, utils = types.ModuleType("mpx"), types.ModuleType("mpx.utils")
    utils.models, utils.objectives, pkg.utils = mo, ob, utils
    sys.modules.update({"mpx": pkg, "mpx.utils": utils, "mpx.utils.models": mo, "mpx.utils.objectives": ob})
    cfg = load(ref_root, "mpx/config/config_aliengo.py", "ref_config_aliengo")
    model = mjcf.parse(os.path.join(ref_root, "mpx", "data", "aliengo", "aliengo.xml"), list(cfg.contact_frame),
                       list(cfg.body_name))
    nj, nc = int(cfg.n_joints), int(cfg.n_contact)
    rng = np.random.default_rng(77)
    q0 = np.asarray(cfg.q0, dtype=np.float64) if hasattr(cfg, "q0") else np.tile([0.0, 0.8, -1.6], 4)
    g = {"wb_dt": np.float64(cfg.dt), "wb_W": np.asarray(cfg.W, dtype=np.float64)}

    def rand_state():
        quat = rng.normal(0, 0.2, 4); quat[0] += 1; quat /= np.linalg.norm(quat)
        qpos = np.concatenate([rng.normal(0, 0.05, 3) + [0, 0, 0.33], quat, q0 + rng.normal(0, 0.2, nj)])
        qvel = rng.normal(0, 0.5, nj + 6)
        return np.concatenate([qpos, qvel, rng.normal(0, 0.1, 3 * nc), rng.normal(0, 20, 3 * nc)])

    # dynamics, float64
    DT["f"] = np.float64
    xs, us, cs, xn = [], [], [], []
    for _ in range(12):
        x = rand_state()
        u = rng.normal(0, 10, nj)
        c = rng.integers(0, 2, nc).astype(np.float64)
        par = np.stack([np.concatenate([c, np.zeros(12)])] * 2)
        x1 = mo.quadruped_wb_dynamics(model, model, list(range(nc)), [int(b) for b in model.contact_jac_body], nj,
                                      float(cfg.dt), _wrap(x), _wrap(u), 0, _wrap(par))
        xs.append(x); us.append(u); cs.append(c); xn.append(np.asarray(x1))
    g["wbdyn_x"], g["wbdyn_u"], g["wbdyn_contact"], g["wbdyn_xnext"] = [np.stack(a) for a in (xs, us, cs, xn)]

    def rand_ref():
        quat = rng.normal(0, 0.2, 4); quat[0] += 1; quat /= np.linalg.norm(quat)
        return np.concatenate([rng.normal(0, 0.05, 3) + [0, 0, 0.33], quat, q0 + rng.normal(0, 0.1, nj),
                               rng.normal(0, 0.3, 6), rng.normal(0, 0.1, 3 * nc), rng.integers(0, 2, nc),
                               rng.normal(0, 20, 3 * nc)])

    # cost, float32 (the reference's dtype), both swing-tracking settings
    DT["f"] = np.float32
    W32 = np.asarray(cfg.W, dtype=np.float32)
    cx, cu, cr, cv, ct, cst = [], [], [], [], [], []
    for i in range(24):
        x = rand_state().astype(np.float32)
        x[13 + 2 * nj + 3 * nc + 2::3] = np.abs(x[13 + 2 * nj + 3 * nc + 2::3]) + 5.0   # vertical forces
        u = rng.normal(0, 15, nj).astype(np.float32)
        ref = rand_ref().astype(np.float32)
        term, swing = (i % 4 == 3), bool(i % 2)
        val = ob.quadruped_wb_obj(swing, nj, nc, 1, _wrap(W32), _wrap(np.stack([ref, ref])), _wrap(x), _wrap(u),
                                  1 if term else 0)
        cx.append(x); cu.append(u); cr.append(ref); cv.append(float(np.asarray(val))); ct.append(term)
        cst.append(swing)
    g["wbcost_x"], g["wbcost_u"], g["wbcost_ref"] = [np.stack(a) for a in (cx, cu, cr)]
    g["wbcost_val"] = np.array(cv, dtype=np.float32)
    g["wbcost_terminal"] = np.array(ct, dtype=np.int32)
    g["wbcost_swing"] = np.array(cst, dtype=np.int32)

    # Gauss-Newton Hessian, float64
    DT["f"] = np.float64
    hx, hu, hr, hs, hQ, hR, hM = [], [], [], [], [], [], []
    for i in range(8):
        x = rand_state()
        x[13 + 2 * nj + 3 * nc + 2::3] = np.abs(x[13 + 2 * nj + 3 * nc + 2::3]) * 0.1 + 0.5  # cone near its edge
        x[13 + nj:13 + 2 * nj] = rng.uniform(-9.0, 9.0, nj)                                   # speeds near limits
        u = rng.uniform(-43.0, 43.0, nj)
        ref = rand_ref()
        swing = bool(i % 2)
        Q, Rm, M = ob.quadruped_wb_hessian_gn(swing, nj, nc, _wrap(np.asarray(cfg.W, dtype=np.float64)),
                                              _wrap(np.stack([ref, ref])), _wrap(x), _wrap(u), 0)
        hx.append(x); hu.append(u); hr.append(ref); hs.append(swing)
        hQ.append(np.asarray(Q)); hR.append(np.asarray(Rm)); hM.append(np.asarray(M))
    # the humanoid dynamics (h1_wb_dynamics, models.py:119-168; talos_wb_dynamics,
    # models.py:170-216) on the fixtures' models, float64
    rng2 = np.random.default_rng(78)
    for name, fn, forces_in_u in (("h1", mo.h1_wb_dynamics, False), ("talos", mo.talos_wb_dynamics, True)):
        fx = np.load(os.path.join(HERE, "%s_wb.npz" % name))
        hm = mjcf.load_npz(os.path.join(HERE, "%s_wb.npz" % name))
        nvh, nch = hm.nv, len(hm.contact_point_body)
        njh = nvh - 6
        bodies = [int(hm.contact_jac_body[0]), int(hm.contact_jac_body[-1])]
        xs, us, cs, xn = [], [], [], []
        for _ in range(8):
            quat = rng2.normal(0, 0.1, 4); quat[0] += 1; quat /= np.linalg.norm(quat)
            qpos = np.concatenate([fx["p0"] + rng2.normal(0, 0.02, 3), quat, fx["q0"] + rng2.normal(0, 0.1, njh)])
            x = np.concatenate([qpos, rng2.normal(0, 0.3, nvh), np.zeros(3 * nch if forces_in_u else 6 * nch)])
            u = rng2.normal(0, 10, njh)
            if forces_in_u:
                f = rng2.normal(0, 20, 3 * nch); f[2::3] = np.abs(f[2::3]) + 50
                u = np.concatenate([u, f])
            c = rng2.integers(0, 2, nch).astype(np.float64)
            par = np.stack([np.concatenate([c, np.zeros(8)])] * 2)
            x1 = fn(hm, hm, list(range(nch)), bodies, njh, float(cfg.dt), _wrap(x), _wrap(u), 0, _wrap(par))
            xs.append(x); us.append(u); cs.append(c); xn.append(np.asarray(x1))
        g[name + "dyn_x"], g[name + "dyn_u"], g[name + "dyn_contact"], g[name + "dyn_xnext"] = \
            [np.stack(a) for a in (xs, us, cs, xn)]
    # the humanoid costs (h1_wb_obj / talos_wb_obj, float32) and Gauss-Newton
    # Hessians (h1_wb_hessian_gn / talos_wb_hessian_gn, float64), with the
    # configs' W
    rng3 = np.random.default_rng(79)
    for name, obj, hes, forces_in_u in (("h1", ob.h1_wb_obj, ob.h1_wb_hessian_gn, False),
                                        ("talos", ob.talos_wb_obj, ob.talos_wb_hessian_gn, True)):
        hc = load(ref_root, "mpx/config/config_%s.py" % name, "ref_config_" + name)
        fx = np.load(os.path.join(HERE, "%s_wb.npz" % name))
        njh, nch = int(hc.n_joints), int(hc.n_contact)
        Wh = np.asarray(hc.W, dtype=np.float64)
        g[name + "_W"] = Wh
        ex, eu, er, ev, et, eQ, eR, eM = [], [], [], [], [], [], [], []
        for i in range(10):
            quat = rng3.normal(0, 0.1, 4); quat[0] += 1; quat /= np.linalg.norm(quat)
            qpos = np.concatenate([fx["p0"] + rng3.normal(0, 0.02, 3), quat, fx["q0"] + rng3.normal(0, 0.1, njh)])
            x = np.concatenate([qpos, rng3.normal(0, 0.3, njh + 6), rng3.normal(0, 0.1, 3 * nch)] +
                               ([] if forces_in_u else [rng3.normal(0, 50, 3 * nch)]))
            u = np.concatenate([rng3.normal(0, 20, njh)] + ([rng3.normal(0, 50, 3 * nch)] if forces_in_u else []))
            qr = rng3.normal(0, 0.1, 4); qr[0] += 1; qr /= np.linalg.norm(qr)
            ref = np.concatenate([fx["p0"] + rng3.normal(0, 0.02, 3), qr, fx["q0"] + rng3.normal(0, 0.1, njh),
                                  rng3.normal(0, 0.3, 6), rng3.normal(0, 0.1, 3 * nch), rng3.integers(0, 2, nch),
                                  rng3.normal(0, 50, 3 * nch)])
            term = (i % 3 == 2)
            DT["f"] = np.float32
            val = obj(njh, nch, 1, _wrap(Wh.astype(np.float32)), _wrap(np.stack([ref, ref]).astype(np.float32)),
                      _wrap(x.astype(np.float32)), _wrap(u.astype(np.float32)), 1 if term else 0)
            DT["f"] = np.float64
            Q, Rm, M = hes(njh, nch, _wrap(Wh), _wrap(np.stack([ref, ref])), _wrap(x), _wrap(u), 0)
            ex.append(x); eu.append(u); er.append(ref); ev.append(float(np.asarray(val))); et.append(term)
            eQ.append(np.asarray(Q)); eR.append(np.asarray(Rm)); eM.append(np.asarray(M))
        g[name + "cost_x"], g[name + "cost_u"], g[name + "cost_ref"] = [np.stack(a) for a in (ex, eu, er)]
        g[name + "cost_val"] = np.array(ev, dtype=np.float32)
        g[name + "cost_terminal"] = np.array(et, dtype=np.int32)
        g[name + "hess_Q"], g[name + "hess_R"], g[name + "hess_M"] = [np.stack(a) for a in (eQ, eR, eM)]
    DT["f"] = np.float32
    g["wbhess_x"], g["wbhess_u"], g["wbhess_ref"] = [np.stack(a) for a in (hx, hu, hr)]
    g["wbhess_swing"] = np.array(hs, dtype=np.int32)
    g["wbhess_Q"], g["wbhess_R"], g["wbhess_M"] = [np.stack(a) for a in (hQ, hR, hM)]
    np.savez_compressed(out, **g)
    print("wrote", out)


def main_wbref(ref_root, out):
    """The whole-body reference generator (mpc_utils.py:15-145,
    reference_generator with terrain_orientation) with config_aliengo
    constants, on seeded states, both terrain settings."""
    install_shim()
    _install_fake_mjx()
    mo = load(ref_root, "mpx/utils/models.py", "ref_models")
    ob = load(ref_root, "mpx/utils/objectives.py", "ref_objectives")
    pkg, utils = types.ModuleType("mpx"), types.ModuleType("mpx.utils")
    utils.models, utils.objectives, pkg.utils = mo, ob, utils
    sys.modules.update({"mpx": pkg, "mpx.utils": utils, "mpx.utils.models": mo, "mpx.utils.objectives": ob})
    cfg = load(ref_root, "mpx/config/config_aliengo.py", "ref_config_aliengo")
    mu = load(ref_root, "mpx/utils/mpc_utils.py", "ref_mpc_utils")
    rng = np.random.default_rng(77)
    nj, nc = int(cfg.n_joints), int(cfg.n_contact)
    foot0 = np.asarray(cfg.p_legs0, dtype=np.float32)
    q0 = np.asarray(cfg.q0, dtype=np.float32)
    mass = np.float32(42.0)
    R = 12
    ins = dict(t_timer=rng.uniform(0, 1, (R, 4)), x=np.zeros((R, 13 + 2 * nj + 6 * nc)), foot=np.zeros((R, 12)),
               input=np.zeros((R, 7)), contact=rng.integers(0, 2, (R, 4)).astype(np.float64),
               liftoff=np.zeros((R, 12)))
    for r in range(R):
        q = rng.normal(0, 0.1, 4); q[0] += 1; q /= np.linalg.norm(q)
        ins["x"][r] = np.concatenate([rng.normal(0, 0.1, 3) + [0, 0, 0.33], q, q0 + rng.normal(0, 0.1, nj),
                                      rng.normal(0, 0.3, 6 + nj), foot0 + rng.normal(0, 0.02, 12),
                                      rng.normal(0, 30, 12)])
        ins["foot"][r] = foot0 + rng.normal(0, 0.02, 12)
        ins["input"][r] = np.concatenate([rng.uniform(-1, 1, 3), rng.uniform(-0.5, 0.5, 3), [cfg.initial_height]])
        ins["liftoff"][r] = ins["foot"][r] + rng.normal(0, 0.01 if r % 2 else 0.05, 12)
    g = {}
    for k in ins:
        ins[k] = ins[k].astype(np.float32)
        g["wbref_in_" + k] = ins[k]
    for terrain in (False, True):
        outs = {"reference": [], "parameter": [], "liftoff": []}
        for r in range(R):
            ref, par, lo = mu.reference_generator(
                terrain, cfg.N, cfg.dt, nj, nc, float(mass), _wrap(foot0), _wrap(q0),
                _wrap(ins["t_timer"][r]), _wrap(ins["x"][r]), _wrap(ins["foot"][r]), _wrap(ins["input"][r]),
                np.float32(cfg.duty_factor), np.float32(cfg.step_freq), np.float32(cfg.step_height),
                _wrap(ins["liftoff"][r]), _wrap(ins["contact"][r]), np.float32(0.4))
            outs["reference"].append(np.asarray(ref)); outs["parameter"].append(np.asarray(par))
            outs["liftoff"].append(np.asarray(lo))
        for k, v in outs.items():
            g["wbref_%s_%s" % ("terrain" if terrain else "flat", k)] = np.stack(v).astype(np.float32)
    g["wbref_cfg"] = np.array([cfg.N, cfg.dt, mass, cfg.duty_factor, cfg.step_freq, cfg.step_height, 0.4],
                              dtype=np.float64)
    g["wbref_foot0"] = foot0
    g["wbref_q0"] = q0
    np.savez_compressed(out, **g)
    print("wrote", out)


def reference_root():
    """The reference checkout named by MPX_REFERENCE ("" when unset)."""
    return os.environ.get("MPX_REFERENCE", "")


if __name__ == "__main__":
    wb, wbref = "--wb" in sys.argv, "--wbref" in sys.argv
    argv = [a for a in sys.argv[1:] if a not in ("--wb", "--wbref")]
    ref_root = argv[0] if argv else reference_root()
    default = "wb_golden.npz" if wb else ("wb_refgen.npz" if wbref else "srbd_golden.npz")
    out = argv[1] if len(argv) > 1 else os.path.join(HERE, default)
    if not ref_root or not os.path.isdir(os.path.join(ref_root, "mpx")):
        sys.exit("usage: make_golden.py <reference checkout containing mpx/> [--wb | --wbref] [out.npz]")
    (main_wb if wb else (main_wbref if wbref else main))(ref_root, out)
