"""The C ABI library builds, loads and exports every entry point that
include/mpxg.h declares (no GPU needed: nothing is called)."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "mpxg.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = set(re.findall(r"\b(mpxg_[a-z_0-9]+)\s*\(", text))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    from mpx_gb300 import build
    path = build.build()
    lib = ctypes.CDLL(path)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    assert len(declared_functions()) >= 10


def test_python_binding_lists_every_export():
    from mpx_gb300 import _lib
    assert set(declared_functions()) <= set(_lib.EXPORTS), set(declared_functions()) - set(_lib.EXPORTS)


def test_version_and_status_strings():
    from mpx_gb300 import _lib
    L = _lib.load()
    assert L.mpxg_version() >= 100
    assert L.mpxg_status_string(0) == b"ok"
    assert L.mpxg_status_string(3) == b"device-memory budget exhausted"


def test_struct_layouts_match_header():
    """ctypes mirrors of the ABI structs have the sizes a C compiler gives them."""
    from mpx_gb300 import _lib
    import subprocess, tempfile
    src = r'''
#include <stddef.h>
#include <stdio.h>
#include "mpxg.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(mpxg_problem_desc), sizeof(mpxg_solver_opts),
         sizeof(mpxg_batch_io), sizeof(mpxg_lq_io), sizeof(mpxg_xla_opaque), sizeof(mpxg_served_model),
         sizeof(mpxg_server_desc), sizeof(mpxg_result));
  printf("%zu %zu\n", sizeof(mpxg_lq_eq_io), sizeof(mpxg_vjp_io));
  printf("%zu %zu %zu\n", sizeof(mpxg_wb_model), offsetof(mpxg_wb_model, gravity),
         offsetof(mpxg_wb_model, contact_point_pos));
  printf("%zu %zu\n", sizeof(mpxg_wb_sqp_io), offsetof(mpxg_wb_sqp_io, x0));
  return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "s.c")
        exe = os.path.join(d, "s")
        open(c, "w").write(src)
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), "-o", exe, c], check=True)
        sizes = [int(v) for v in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()]
    assert sizes == [ctypes.sizeof(_lib.ProblemDesc), ctypes.sizeof(_lib.SolverOpts), ctypes.sizeof(_lib.BatchIO),
                     ctypes.sizeof(_lib.LqIO), ctypes.sizeof(_lib.XlaOpaque), ctypes.sizeof(_lib.ServedModel),
                     ctypes.sizeof(_lib.ServerDesc), ctypes.sizeof(_lib.Result), ctypes.sizeof(_lib.LqEqIO),
                     ctypes.sizeof(_lib.VjpIO), ctypes.sizeof(_lib.WbModel), _lib.WbModel.gravity.offset,
                     _lib.WbModel.contact_point_pos.offset, ctypes.sizeof(_lib.WbSqpIO), _lib.WbSqpIO.x0.offset]


def test_xla_target_rejects_a_malformed_opaque():
    """The XLA custom-call target checks its opaque operand before touching
    the GPU and reports through mpxg_last_error(NULL) (no XLA status setter
    in this process)."""
    from mpx_gb300 import _lib
    L = _lib.load()
    bufs = (ctypes.c_void_p * 10)()
    L.mpxg_xla_solve(None, bufs, b"short", 5, None)
    assert b"mpxg_xla_opaque" in L.mpxg_last_error(None)


def test_lqr_eq_rejects_bad_method_and_unaligned_workspace():
    """mpxg_lqr_eq_solve_method validates before touching the GPU: the method
    is 0 or 1, and the tensor-core kernel (method 0), which writes the
    workspace in 16-byte vectors, needs a 16-byte aligned workspace."""
    from mpx_gb300 import _lib
    L = _lib.load()
    io = _lib.LqEqIO()
    io.batch, io.N, io.n, io.m, io.n_eq = 1, 4, 72, 30, 12
    fake = 1 << 20  # never dereferenced: the checks fail first
    for name in ("A", "Bm", "c", "Q", "R", "M", "q", "r", "C", "D", "e", "x0", "K", "k", "Knu", "knu", "X", "U",
                 "lam", "nu"):
        setattr(io, name, ctypes.c_void_p(fake))
    io.workspace = ctypes.c_void_p(fake + 4)
    assert L.mpxg_lqr_eq_solve_method(None, ctypes.byref(io), 2) == 1
    assert b"method" in L.mpxg_last_error(None)
    assert L.mpxg_lqr_eq_solve_method(None, ctypes.byref(io), 0) == 1
    assert b"16-byte aligned" in L.mpxg_last_error(None)
    assert L.mpxg_lqr_eq_solve(None, ctypes.byref(io)) == 1


def test_wb_calls_reject_malformed_models():
    """mpxg_wb_terms / mpxg_wb_interface check the model before any launch
    (the kernel indexes its shared arrays by these fields)."""
    from mpx_gb300 import _lib, mjcf
    L = _lib.load()
    model = mjcf.load_npz(os.path.join(ROOT, "tests", "golden", "aliengo_wb.npz"))
    fake = ctypes.c_void_p(1 << 20)  # never dereferenced: the checks fail first

    def terms(S):
        return L.mpxg_wb_terms(None, ctypes.byref(S), 4, fake, fake, fake, fake, fake, fake, fake)

    def iface(S):
        return L.mpxg_wb_interface(None, ctypes.byref(S), 4, *([fake] * 10))

    S = model.to_struct()
    S.parent[3] = 5                      # a child listed before its parent
    assert terms(S) == 1 and b"parents first" in L.mpxg_last_error(None)
    S = model.to_struct()
    S.nv = 17
    assert terms(S) == 1 and b"nv / nq" in L.mpxg_last_error(None)
    S = model.to_struct()
    S.dof_adr[2] = 8
    assert terms(S) == 1 and b"dense" in L.mpxg_last_error(None)
    S = model.to_struct()
    S.contact_jac_body[1] = 13
    assert terms(S) == 1 and b"contact body" in L.mpxg_last_error(None)
    S = model.to_struct()
    S.jnt_type[4] = 1                    # a second free joint
    assert terms(S) == 1 and b"free joint" in L.mpxg_last_error(None)
    S = model.to_struct()
    S.n_contact = 3                      # nv != 6 + 3 x contacts
    assert iface(S) == 1 and b"free root" in L.mpxg_last_error(None)
    S = model.to_struct()
    assert L.mpxg_wb_interface(None, ctypes.byref(S), 4, *([fake] * 8), None, fake) == 1  # tau NULL
    assert b"null pointer" in L.mpxg_last_error(None)
    assert L.mpxg_wb_terms(None, ctypes.byref(S), 0, None, None, None, None, None, None, None) == 0


def test_wb_step_rejects_what_it_cannot_hold():
    """mpxg_wb_step needs nv + 3 x contacts + 1 <= 32 (one lane per column of
    [M | J | tau - bias]) and a positive dt; it checks before any launch."""
    from mpx_gb300 import _lib, mjcf
    L = _lib.load()
    model = mjcf.load_npz(os.path.join(ROOT, "tests", "golden", "aliengo_wb.npz"))
    fake = ctypes.c_void_p(1 << 20)  # never dereferenced: the checks fail first
    S = model.to_struct()
    assert L.mpxg_wb_step(None, ctypes.byref(S), 4, 0.0, 25.0, fake, fake, fake, fake) == 1
    assert b"dt" in L.mpxg_last_error(None)
    S.n_contact = 5                      # 18 + 15 + 1 > 32
    S.contact_point_body[4] = S.contact_jac_body[4] = 3
    assert L.mpxg_wb_step(None, ctypes.byref(S), 4, 0.02, 25.0, fake, fake, fake, fake) == 1
    assert b"<= 32" in L.mpxg_last_error(None)
    S = model.to_struct()
    assert L.mpxg_wb_step(None, ctypes.byref(S), 0, 0.02, 25.0, None, None, None, None) == 0


def test_wb_sqp_rejects_before_any_launch():
    """mpxg_wb_sqp checks the model (the built size nv = 18 with 4 contacts,
    the step's lane limits), the sizes and the options before it launches;
    a batch of 0 returns at once."""
    from mpx_gb300 import _lib, mjcf
    L = _lib.load()
    model = mjcf.load_npz(os.path.join(ROOT, "tests", "golden", "aliengo_wb.npz"))
    S = model.to_struct()
    fake = 1 << 20  # never dereferenced: the checks fail first

    def io(**kw):
        o = _lib.WbSqpIO(model=ctypes.pointer(S), batch=0, N=25, iters=5, dt=0.02, alpha=25.0, swing_tracking=1,
                         reg=1e-6, rho0=1.0, ls_beta=0.5, ls_eta=1e-4, ls_skip_tol=1e-7, ls_max_trials=8)
        for k in ("x0", "X", "U", "V", "reference", "contact", "W", "workspace"):
            setattr(o, k, fake)
        for k, v in kw.items():
            setattr(o, k, v)
        return o

    assert L.mpxg_wb_sqp(None, ctypes.byref(io())) == 0
    assert L.mpxg_wb_sqp(None, ctypes.byref(io(ls_max_trials=9))) == 1
    assert b"ls_max_trials" in L.mpxg_last_error(None)
    assert L.mpxg_wb_sqp(None, ctypes.byref(io(N=0))) == 1
    assert L.mpxg_wb_sqp(None, ctypes.byref(io(batch=1 << 20, N=100))) == 1  # grids past 2^31 blocks
    assert b"launch grids" in L.mpxg_last_error(None)
    assert L.mpxg_wb_sqp_workspace_bytes(ctypes.byref(S), 1 << 20, 100) == 0
    assert L.mpxg_wb_sqp(None, ctypes.byref(io(batch=2, workspace=fake + 16))) == 1
    assert b"256-byte" in L.mpxg_last_error(None)
    assert L.mpxg_wb_sqp(None, ctypes.byref(io(batch=2, W=None))) == 1
    assert b"null" in L.mpxg_last_error(None)
    assert L.mpxg_wb_sqp_workspace_bytes(ctypes.byref(S), 4, 25) > 4 * 25 * 61 * 61 * 4
    S2 = model.to_struct()
    S2.n_contact = 3
    assert L.mpxg_wb_sqp(None, ctypes.byref(io(model=ctypes.pointer(S2)))) == 1
    assert b"nv = 18" in L.mpxg_last_error(None)
    assert L.mpxg_wb_sqp_workspace_bytes(ctypes.byref(S2), 4, 25) == 0


def _declarations():
    """(return type, name, [parameter types]) of every function in mpxg.h."""
    text = open(os.path.join(ROOT, "include", "mpxg.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    out = []
    for ret, name, params in re.findall(r"([A-Za-z_][\w\s\*]*?)\b(mpxg_[a-z_0-9]+)\s*\(([^;{]*?)\)\s*;", text, re.S):
        types = []
        for p in params.split(","):
            p = " ".join(p.replace("*", " * ").split())
            if p in ("", "void"):
                continue
            words = p.split()
            if words[-1] != "*":
                words = words[:-1]  # the parameter's name
            types.append(" ".join(words))
        ret = " ".join(ret.replace("*", " * ").split()[-3:])
        out.append((ret, name, types))
    return out


def _c_kind(t):
    if t.endswith("*"):
        return "pointer"
    return {"int": "int", "mpxg_status": "int", "float": "float", "double": "double", "long long": "int64",
            "size_t": "size_t"}[t.replace("const ", "")]


def _ctypes_kind(ct):
    if ct in (ctypes.c_void_p, ctypes.c_char_p) or hasattr(ct, "_type_") and isinstance(ct._type_, type):
        return "pointer"
    if ct is None:
        return "void"
    return {ctypes.c_int: "int", ctypes.c_float: "float", ctypes.c_double: "double", ctypes.c_longlong: "int64",
            ctypes.c_size_t: "size_t"}[ct]


def test_python_binding_matches_every_declared_signature():
    """Each entry point that the Python layer binds passes its arguments as
    mpxg.h declares them (count and C kind: pointer, int, float, 64-bit
    integer, size_t) and reads a size_t result as size_t, so no argument is
    truncated or passed in the wrong register class."""
    from mpx_gb300 import _lib
    L = _lib.load()
    decls = _declarations()
    assert len(decls) == len(declared_functions())
    for ret, name, params in decls:
        f = getattr(L, name)
        assert f.argtypes is not None or not params, name
        assert [_ctypes_kind(a) for a in f.argtypes or []] == [_c_kind(t) for t in params], name
        if ret.endswith("size_t"):
            assert f.restype is ctypes.c_size_t, name
        if ret.endswith("*") and "char" in ret:
            assert f.restype is ctypes.c_char_p, name


def test_no_cpu_fallback():
    """Without a GPU the product path refuses to run rather than computing
    on the CPU: the Python solver raises, and the C ABI returns a CUDA error
    status from mpxg_create (no handle); a missing library raises on load."""
    import pytest
    import torch
    from mpx_gb300 import _lib, problem as P
    from mpx_gb300.solver import Solver, problem_desc, solver_opts
    if torch.cuda.is_available():
        pytest.skip("this machine has a GPU")
    desc = P.quadruped_rpy12()
    with pytest.raises(_lib.MpxgError, match="no CPU path"):
        Solver(desc, P.SolverOptions(), n_max=10, batch_max=2)
    L = _lib.load()
    h = ctypes.c_void_p()
    pd, po = problem_desc(desc, 10, 2), solver_opts(P.SolverOptions())
    st = L.mpxg_create(ctypes.byref(pd), ctypes.byref(po), ctypes.byref(h))
    assert st == 4 and not h.value  # MPXG_ERR_CUDA
    assert b"cuda" in L.mpxg_last_error(None).lower()


def test_missing_library_raises(monkeypatch, tmp_path):
    import pytest
    from mpx_gb300 import _lib
    monkeypatch.setattr(_lib, "_lib", None)
    monkeypatch.setattr(_lib._build, "LIB", str(tmp_path / "libmpxg.so"))
    with pytest.raises(_lib.MpxgError, match="not built"):
        _lib.load(build_if_missing=False)


def test_queue_and_mixed_reject_null_arguments():
    """The device work queue and the mixed-model launch refuse null handles
    and arguments before touching a device."""
    from mpx_gb300 import _lib
    L = _lib.load()
    q = ctypes.c_void_p()
    assert L.mpxg_queue_start(None, None, None, 4, 10 ** 9, ctypes.byref(q)) == 1
    t = ctypes.c_longlong()
    assert L.mpxg_queue_push(None, 0, ctypes.byref(t)) == 1
    assert L.mpxg_queue_result(None, 0, None) == 1
    assert L.mpxg_queue_finish(None) == 1
    mx = ctypes.c_void_p()
    assert L.mpxg_mixed_create(None, None, ctypes.byref(mx)) == 1
    assert L.mpxg_solve_mixed(None, None, None, None) == 1
    L.mpxg_mixed_destroy(None)
