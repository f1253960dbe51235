"""The XLA custom-call target mpxg_xla_solve: opaque packing (CPU) and, on
the GPU, the same results as mpxg_solve on the same operands."""
import ctypes

import numpy as np
import pytest

from mpx_gb300 import _lib, jax_ffi
from mpx_gb300 import problem as P


def test_opaque_packs_desc_opts_and_batch():
    wl = P.quadruped_workload(3, horizons=(20,), seed=1, model=P.MODEL_SRBD_RPY12)
    b = jax_ffi.opaque_bytes(wl.desc, P.SolverOptions(sqp_iters=4), 20, 3)
    assert len(b) == ctypes.sizeof(_lib.XlaOpaque)
    op = _lib.XlaOpaque.from_buffer_copy(b)
    assert (op.batch, op.desc.n_max, op.desc.batch_max, op.opts.sqp_iters, op.desc.model) == (3, 20, 3, 4,
                                                                                                P.MODEL_SRBD_RPY12)


def test_prepare_rejects_a_malformed_opaque():
    L = _lib.load()
    assert L.mpxg_xla_prepare(b"short", 5) == 1
    assert b"mpxg_xla_opaque" in L.mpxg_last_error(None)


def test_jax_binding_is_optional():
    if not jax_ffi.available():
        with pytest.raises(RuntimeError):
            jax_ffi.register()


@pytest.mark.gpu
def test_xla_target_matches_mpxg_solve(cuda):
    import torch
    from mpx_gb300.solver import Solver, weights_diagonal
    wl = P.quadruped_workload(6, horizons=(30,), seed=5, model=P.MODEL_SRBD_RPY12, v_range=(-1, 1),
                              random_phase=True)
    opts = P.SolverOptions(sqp_iters=3)
    s = Solver(wl.desc, opts, n_max=30, batch_max=6)
    ref = s.solve(wl.x0, wl.X0, wl.U0, wl.V0, wl.reference, wl.parameter, wl.W)
    torch.cuda.synchronize()
    d = lambda a: torch.as_tensor(np.ascontiguousarray(a)).to("cuda", torch.float32).contiguous()
    ins = [d(wl.reference), d(wl.parameter), weights_diagonal(torch.as_tensor(wl.W), 6).to("cuda", torch.float32).contiguous(),
           d(wl.x0), d(wl.X0), d(wl.U0), d(wl.V0)]
    outs = [torch.empty_like(ins[4]), torch.empty_like(ins[5]), torch.empty_like(ins[6])]
    bufs = (ctypes.c_void_p * 10)(*[t.data_ptr() for t in ins + outs])
    op = jax_ffi.opaque_bytes(wl.desc, opts, 30, 6)
    L = _lib.load()
    # without a prepared handle the custom call fails and allocates nothing
    for o in outs:
        o.fill_(7.0)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    L.mpxg_xla_solve(None, bufs, op, len(op), None)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert b"mpxg_xla_prepare" in L.mpxg_last_error(None)
    assert all(bool((o == 7.0).all()) for o in outs)
    # prepared when the program is built; the custom call then allocates nothing
    assert L.mpxg_xla_prepare(op, len(op)) == 0, L.mpxg_last_error(None)
    assert L.mpxg_xla_prepare(op, len(op)) == 0  # once per (device, opaque)
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    L.mpxg_xla_solve(None, bufs, op, len(op), None)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free1
    for got, key in zip(outs, ("X", "U", "V")):
        assert np.array_equal(got.cpu().numpy(), ref[key].cpu().numpy()), key
    s.close()


@pytest.mark.gpu
def test_xla_vjp_target_matches_solver_vjp(cuda):
    import torch
    from mpx_gb300.solver import Solver, weights_diagonal
    wl = P.quadruped_workload(5, horizons=(20,), seed=6, model=P.MODEL_SRBD_RPY12, v_range=(-1, 1),
                              random_phase=True)
    opts = P.SolverOptions(sqp_iters=6)
    s = Solver(wl.desc, opts, n_max=20, batch_max=5)
    sol = s.solve(wl.x0, wl.X0, wl.U0, wl.V0, wl.reference, wl.parameter, wl.W)
    torch.cuda.synchronize()
    X, U, V = sol["X"].clone(), sol["U"].clone(), sol["V"].clone()
    rng = np.random.default_rng(2)
    gX = torch.tensor(rng.normal(size=X.shape), dtype=torch.float32, device="cuda")
    gU = torch.tensor(rng.normal(size=U.shape), dtype=torch.float32, device="cuda")
    ref = s.vjp(wl.x0, X, U, V, wl.reference, wl.parameter, wl.W, gX, gU)
    torch.cuda.synchronize()
    d = lambda a: torch.as_tensor(np.ascontiguousarray(a)).to("cuda", torch.float32).contiguous()
    ins = [d(wl.reference), d(wl.parameter), weights_diagonal(torch.as_tensor(wl.W), 5).to("cuda", torch.float32)
           .contiguous(), d(wl.x0), X, U, V, gX, gU]
    gx0 = torch.empty(5, 12, device="cuda")
    gref = torch.empty(5, 21, 12, device="cuda")
    bufs = (ctypes.c_void_p * 11)(*[t.data_ptr() for t in ins + [gx0, gref]])
    op = jax_ffi.opaque_bytes(wl.desc, opts, 20, 5)
    jax_ffi.prepare(op)
    _lib.load().mpxg_xla_solve_vjp(None, bufs, op, len(op), None)
    torch.cuda.synchronize()
    assert np.array_equal(gx0.cpu().numpy(), ref["gx0"].cpu().numpy())
    assert np.array_equal(gref.cpu().numpy(), ref["gref"].cpu().numpy())
    s.close()


def test_register_hands_xla_the_library_entry_points(monkeypatch):
    """register() with a stand-in for jax.ffi: each target is registered once,
    for the CUDA platform with the legacy custom-call API, as a capsule named
    as XLA expects that carries the address of libmpxg's own entry point."""
    import types
    calls = []
    fake = types.SimpleNamespace(ffi=types.SimpleNamespace(
        register_ffi_target=lambda name, cap, platform, api_version: calls.append((name, cap, platform, api_version))))
    monkeypatch.setattr(jax_ffi, "HAVE_JAX", True)
    monkeypatch.setattr(jax_ffi, "jax", fake, raising=False)
    monkeypatch.setattr(jax_ffi, "_registered", False)
    jax_ffi.register()
    jax_ffi.register()  # idempotent
    L = _lib.load()
    get = ctypes.pythonapi.PyCapsule_GetPointer
    get.restype, get.argtypes = ctypes.c_void_p, [ctypes.py_object, ctypes.c_char_p]
    want = {jax_ffi.TARGET: ctypes.cast(L.mpxg_xla_solve, ctypes.c_void_p).value,
            jax_ffi.TARGET_VJP: ctypes.cast(L.mpxg_xla_solve_vjp, ctypes.c_void_p).value}
    assert [c[0] for c in calls] == [jax_ffi.TARGET, jax_ffi.TARGET_VJP]
    for name, cap, platform, api_version in calls:
        assert (platform, api_version) == ("CUDA", 0)
        assert get(cap, b"xla._CUSTOM_CALL_TARGET") == want[name]
