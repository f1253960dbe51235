"""JAX binding of the batched solve: libmpxg's `mpxg_xla_solve` as an XLA
custom call, so a JAX program keeps the solve inside `jax.jit` as the
reference does with `jax.jit(jax.vmap(optimizers.mpc ...))`
(mpx/utils/mpc_wrapper_srbd.py:68,77; mpx/utils/mpc_wrapper.py:74).

Registered only when `jax` imports; nothing here runs otherwise.  Usage:

    from mpx_gb300 import jax_ffi
    solve = jax_ffi.make_mpc(desc, opts, n_max=N, batch=B)   # jit-compatible
    X, U, V = solve(reference, parameter, W, x0, X0, U0, V0)  # [B, ...] arrays

The call is batched natively ([B, ...] operands, one persistent launch), so
it replaces the vmapped solve as a whole rather than being vmapped itself.
It is differentiable (jax.custom_vjp over mpxg_xla_solve_vjp).
W is reduced to its diagonal in the program (the SRBD weights are diagonal,
mpx/config/config_srbd.py:90).  The custom call uses XLA's status-returning
legacy signature (api_version 2); the target is registered for the CUDA
platform through `jax.ffi.register_ffi_target(..., api_version=0)`.
"""
import ctypes

from . import _lib
from .solver import problem_desc, solver_opts

try:  # optional dependency
    import jax
    import jax.numpy as jnp
    from jax.interpreters import mlir
    from jax.interpreters.mlir import ir
    try:
        from jax.extend.core import Primitive
    except ImportError:  # older jax
        from jax.core import Primitive
    HAVE_JAX = True
except ImportError:
    HAVE_JAX = False

TARGET = "mpxg_xla_solve"
TARGET_VJP = "mpxg_xla_solve_vjp"
_registered = False
_prim = None
_prim_vjp = None


def available():
    return HAVE_JAX


def register():
    """Register the custom-call target with XLA (once)."""
    global _registered
    if not HAVE_JAX:
        raise RuntimeError("jax is not installed; the XLA custom call is unavailable")
    if _registered:
        return
    L = _lib.load()
    fn = ctypes.cast(L.mpxg_xla_solve, ctypes.c_void_p).value
    capsule_new = ctypes.pythonapi.PyCapsule_New
    capsule_new.restype = ctypes.py_object
    capsule_new.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p]
    capsule = capsule_new(fn, b"xla._CUSTOM_CALL_TARGET", None)
    jax.ffi.register_ffi_target(TARGET, capsule, platform="CUDA", api_version=0)
    fn_vjp = ctypes.cast(L.mpxg_xla_solve_vjp, ctypes.c_void_p).value
    jax.ffi.register_ffi_target(TARGET_VJP, capsule_new(fn_vjp, b"xla._CUSTOM_CALL_TARGET", None), platform="CUDA",
                                api_version=0)
    _registered = True


def opaque_bytes(desc, opts, n_max, batch):
    op = _lib.XlaOpaque()
    op.desc = problem_desc(desc, n_max, batch)
    op.opts = solver_opts(opts)
    op.batch = int(batch)
    return bytes(op)


def prepare(opaque, devices=(None,)):
    """Create the device workspace of an opaque on each CUDA device (None:
    the current one) now, so that the custom call allocates nothing when the
    jitted program runs."""
    import torch
    L = _lib.load()
    for d in devices:
        if d is None:
            _lib.check(L.mpxg_xla_prepare(opaque, len(opaque)), None, "mpxg_xla_prepare")
        else:
            with torch.cuda.device(d):
                _lib.check(L.mpxg_xla_prepare(opaque, len(opaque)), None, "mpxg_xla_prepare")


def _primitive():
    global _prim
    if _prim is not None:
        return _prim
    p = Primitive("mpxg_mpc")
    p.multiple_results = True

    def abstract(reference, parameter, w, x0, X0, U0, V0, *, opaque):
        return (jax.core.ShapedArray(X0.shape, jnp.float32), jax.core.ShapedArray(U0.shape, jnp.float32),
                jax.core.ShapedArray(V0.shape, jnp.float32))

    def lowering(ctx, reference, parameter, w, x0, X0, U0, V0, *, opaque):
        outs = [mlir.aval_to_ir_type(a) for a in ctx.avals_out]
        call = mlir.custom_call(TARGET, result_types=outs, operands=[reference, parameter, w, x0, X0, U0, V0],
                                backend_config=opaque, api_version=2, has_side_effect=False)
        return call.results

    p.def_abstract_eval(abstract)
    mlir.register_lowering(p, lowering, platform="cuda")
    _prim = p
    return p


def _primitive_vjp():
    global _prim_vjp
    if _prim_vjp is not None:
        return _prim_vjp
    p = Primitive("mpxg_mpc_vjp")
    p.multiple_results = True

    def abstract(reference, parameter, w, x0, X, U, V, gX, gU, *, opaque):
        B, N1 = X.shape[0], X.shape[1]
        return (jax.core.ShapedArray(x0.shape, jnp.float32), jax.core.ShapedArray((B, N1, 12), jnp.float32))

    def lowering(ctx, *operands, opaque):
        outs = [mlir.aval_to_ir_type(a) for a in ctx.avals_out]
        call = mlir.custom_call(TARGET_VJP, result_types=outs, operands=list(operands), backend_config=opaque,
                                api_version=2, has_side_effect=False)
        return call.results

    p.def_abstract_eval(abstract)
    mlir.register_lowering(p, lowering, platform="cuda")
    _prim_vjp = p
    return p


def make_mpc(desc, opts, n_max, batch, devices=(None,)):
    """A jit-compatible batched solve (reference, parameter, W, x0, X0, U0, V0)
    -> (X, U, V) for `batch` instances of horizon n_max, differentiable with
    jax.grad / jax.vjp: the backward pass is mpxg_xla_solve_vjp (implicit
    differentiation of the converged solution), giving gradients with respect
    to x0 and to the 12 tracked columns of the reference; the warm start,
    parameter table and weights get zero gradients.  The device workspace is
    created here, on each of `devices` (CUDA indices; None: the current
    device), so the custom calls allocate nothing when the program runs."""
    register()
    opaque = opaque_bytes(desc, opts, n_max, batch)
    prepare(opaque, devices)
    prim, prim_vjp = _primitive(), _primitive_vjp()
    f32 = lambda a: jnp.asarray(a, jnp.float32)

    def diag(W):
        return jnp.diagonal(f32(W), axis1=-2, axis2=-1) if jnp.ndim(W) == 3 else f32(W)

    @jax.custom_vjp
    def solve(reference, parameter, W, x0, X0, U0, V0):
        return tuple(prim.bind(f32(reference), f32(parameter), diag(W), f32(x0), f32(X0), f32(U0), f32(V0),
                               opaque=opaque))

    def fwd(reference, parameter, W, x0, X0, U0, V0):
        out = solve(reference, parameter, W, x0, X0, U0, V0)
        return out, (f32(reference), f32(parameter), diag(W), f32(x0), out, W, X0, U0, V0)

    def bwd(res, cot):
        reference, parameter, w, x0, (X, U, V), W, X0, U0, V0 = res
        gX, gU, _ = cot
        gx0, gref = prim_vjp.bind(reference, parameter, w, x0, X, U, V, f32(gX), f32(gU), opaque=opaque)
        g_reference = jnp.zeros_like(reference).at[..., :12].set(gref)
        return (g_reference, jnp.zeros_like(parameter), jnp.zeros_like(f32(W)), gx0, jnp.zeros_like(f32(X0)),
                jnp.zeros_like(f32(U0)), jnp.zeros_like(f32(V0)))

    solve.defvjp(fwd, bwd)
    return solve
