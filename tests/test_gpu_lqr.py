"""CUDA LQR kernel vs the oracle's Riccati (isolated KKT/LQR workload shape)."""
import numpy as np
import pytest
import torch

from mpx_gb300 import problem as P
from mpx_gb300.solver import lqr_solve

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("method", [0, 1])
@pytest.mark.parametrize("n,m,N", [(24, 12, 32), (4, 2, 9), (12, 12, 17), (24, 12, 128), (8, 4, 5), (12, 12, 1)])
def test_lqr_matches_oracle(oracle, cuda, n, m, N, method):
    """Method 0 (sequential Riccati) and method 1 (associative scan over 8
    chunks; N < 8 leaves chunks empty) against the oracle's FP64 Riccati."""
    d = P.random_lq(6, n, m, N, seed=n + N)
    if n == 8:  # a cross term exercises the elimination of M
        d["M"] = 0.05 * np.random.default_rng(3).normal(size=d["M"].shape)
    o = oracle.lqr_solve(d["A"], d["B"], d["c"], d["Q"], d["R"], d["M"], d["q"], d["r"], d["x0"])
    g = lqr_solve(d["A"], d["B"], d["c"], d["Q"], d["R"], d["M"], d["q"], d["r"], d["x0"], method=method)
    torch.cuda.synchronize()
    for k in ("K", "k", "X", "U", "lam"):
        a = g[k].cpu().numpy()
        e = np.abs(a - o[k]).max() / np.abs(o[k]).max()
        assert e < 2e-4, (k, e)


@pytest.mark.parametrize("method", [0, 1])
@pytest.mark.parametrize("n,m,ne,N,B", [(8, 5, 2, 6, 3), (16, 8, 4, 20, 3), (16, 8, 4, 1, 2), (72, 30, 12, 100, 2)])
def test_lqr_eq_matches_oracle(cuda, n, m, ne, N, B, method):
    """Equality-constrained LQR on the GPU against the FP64 stagewise Riccati
    (itself checked against a dense KKT solve on the CPU): method 0 with the
    stage products on the tensor cores (split TF32), method 1 on the CUDA
    cores.  Bound: 2e-4 relative, or 8x the error of the oracle's own float32
    run where the problem's conditioning puts float32 itself near that (the
    N = 1 case: ~3e-5)."""
    from mpx_gb300.solver import lqr_eq_solve
    from oracle.lqr_eq import riccati_eq
    d = P.random_lq_eq(B, n=n, m=m, n_eq=ne, N=N, seed=n + N)
    if n == 8:  # a cross term and a control-linear cost exercise the elimination (small
        # enough that Q - M R^-1 M' stays positive definite with R = 1e-3 I)
        d["M"] = 0.002 * np.random.default_rng(3).normal(size=d["M"].shape)
        d["r"] = np.random.default_rng(4).normal(size=d["r"].shape)
    keys = ("A", "B", "c", "Q", "R", "M", "q", "r", "C", "D", "e", "x0")
    g = lqr_eq_solve(*[d[k] for k in keys], method=method)
    torch.cuda.synchronize()
    for b in range(B):
        o = riccati_eq(*[d[k][b] for k in keys])
        o32 = riccati_eq(*[d[k][b] for k in keys], dtype=np.float32)
        for k in ("K", "k", "Knu", "knu", "X", "U", "lam", "nu"):
            a = g[k][b].cpu().numpy()
            e = np.abs(a - o[k]).max() / np.abs(o[k]).max()
            e32 = np.abs(o32[k] - o[k]).max() / np.abs(o[k]).max()
            assert e < max(2e-4, 8.0 * e32), (k, b, e, e32)
        # constraint residual of the GPU trajectory, relative to the size of
        # the terms it balances (sum |C x| + sum |D u| + |e| per row)
        X, U = g["X"][b].cpu().double().numpy(), g["U"][b].cpu().double().numpy()
        res = np.einsum("tij,tj->ti", d["C"][b], X[:N]) + np.einsum("tij,tj->ti", d["D"][b], U) - d["e"][b]
        mag = (np.einsum("tij,tj->ti", np.abs(d["C"][b]), np.abs(X[:N])) +
               np.einsum("tij,tj->ti", np.abs(d["D"][b]), np.abs(U)) + np.abs(d["e"][b]))
        assert np.abs(res).max() < 2e-4 * mag.max(), (np.abs(res).max(), mag.max())


def test_lqr_eq_tensor_cores_unaligned_inputs(cuda):
    """Inputs at addresses that are not 16-byte aligned take the 4-byte copy
    path of the tensor-core kernel (no 16-byte asynchronous copies, no L2
    prefetch) and give the same result bit for bit."""
    import ctypes
    from mpx_gb300 import _lib
    from mpx_gb300.solver import _ptr, lqr_eq_solve
    n, m, ne, N, B = 16, 8, 4, 12, 3
    d = P.random_lq_eq(B, n=n, m=m, n_eq=ne, N=N, seed=77)
    keys = ("A", "B", "c", "Q", "R", "M", "q", "r", "C", "D", "e", "x0")
    ref = lqr_eq_solve(*[d[k] for k in keys], method=0)
    torch.cuda.synchronize()
    # the same inputs one float past an aligned base
    dev = torch.device("cuda")
    shifted = {}
    for k in keys:
        a = torch.as_tensor(d[k], dtype=torch.float32).reshape(-1)
        buf = torch.zeros(a.numel() + 1, device=dev)
        buf[1:] = a.to(dev)
        shifted[k] = buf
    L = _lib.load()
    out = {k: torch.empty_like(v) for k, v in ref.items() if not k.startswith("_")}
    ws = torch.empty(int(L.mpxg_lqr_eq_workspace_bytes(B, N, n)) // 4, device=dev)
    io = _lib.LqEqIO()
    io.batch, io.N, io.n, io.m, io.n_eq = B, N, n, m, ne
    for name, k in zip(("A", "Bm", "c", "Q", "R", "M", "q", "r", "C", "D", "e", "x0"), keys):
        setattr(io, name, ctypes.c_void_p(shifted[k].data_ptr() + 4))
    for k in out:
        setattr(io, k, _ptr(out[k]))
    io.workspace = _ptr(ws)
    assert L.mpxg_lqr_eq_solve_method(None, ctypes.byref(io), 0) == 0
    torch.cuda.synchronize()
    for k in out:
        assert torch.equal(out[k], ref[k]), k


@pytest.mark.parametrize("method", [0, 1])
def test_lqr_eq_two_waves(cuda, method):
    """300 problems (two waves of one block per SM): sampled problems from
    both waves match the FP64 oracle within 2e-4, or within 8x the error of
    the oracle's own float32 run where a problem's conditioning puts float32
    itself near that bound."""
    from mpx_gb300.solver import lqr_eq_solve
    from oracle.lqr_eq import riccati_eq
    n, m, ne, N, B = 16, 8, 4, 10, 300
    d = P.random_lq_eq(B, n=n, m=m, n_eq=ne, N=N, seed=5)
    keys = ("A", "B", "c", "Q", "R", "M", "q", "r", "C", "D", "e", "x0")
    g = lqr_eq_solve(*[d[k] for k in keys], method=method)
    torch.cuda.synchronize()
    for b in (0, 151, 152, 299):
        o = riccati_eq(*[d[k][b] for k in keys])
        o32 = riccati_eq(*[d[k][b] for k in keys], dtype=np.float32)
        for k in ("K", "k", "X", "U", "lam", "nu"):
            a = g[k][b].cpu().numpy()
            e = np.abs(a - o[k]).max() / np.abs(o[k]).max()
            e32 = np.abs(o32[k] - o[k]).max() / np.abs(o[k]).max()
            assert e < max(2e-4, 8.0 * e32), (k, b, e, e32)


KEYS_EQ = ("A", "B", "c", "Q", "R", "M", "q", "r", "C", "D", "e", "x0")


def _eq_case(B, n, m, ne, N, seed):
    d = P.random_lq_eq(B, n=n, m=m, n_eq=ne, N=N, seed=seed)
    if n == 8:
        d["M"] = 0.002 * np.random.default_rng(3).normal(size=d["M"].shape)
        d["r"] = np.random.default_rng(4).normal(size=d["r"].shape)
    rng = np.random.default_rng(seed + 1)
    X0, U0 = rng.normal(size=(B, N + 1, n)), rng.normal(size=(B, N, m))
    return d, X0, U0


@pytest.mark.parametrize("method", [0, 1])
@pytest.mark.parametrize("n,m,ne,N,B", [(8, 5, 2, 6, 3), (16, 8, 4, 20, 3), (72, 30, 12, 100, 2)])
def test_lqr_eq_sqp_matches_oracle(cuda, n, m, ne, N, B, method):
    """Two SQP iterations from a random iterate on the GPU against the FP64
    oracle's solution (one SQP iteration of an LQ problem is its direct
    solution): 2e-4 relative, or 8x the error of the oracle's own float32
    SQP where conditioning puts float32 near that.  The KKT residual the GPU
    reports is at the float32 level of the oracle's own float32 run."""
    from mpx_gb300.solver import lqr_eq_sqp
    from oracle.lqr_eq import kkt_eq, riccati_eq, sqp_eq
    d, X0, U0 = _eq_case(B, n, m, ne, N, seed=n + N)
    g = lqr_eq_sqp(*[d[k] for k in KEYS_EQ], X0, U0, iters=2, method=method)
    torch.cuda.synchronize()
    kkt = g["kkt"].cpu().numpy()
    for b in range(B):
        args = [d[k][b] for k in KEYS_EQ]
        o = riccati_eq(*args)
        o32 = sqp_eq(*args, X0[b], U0[b], iters=2, dtype=np.float32)
        for k in ("X", "U", "lam", "nu"):
            a = g[k][b].cpu().numpy()
            e = np.abs(a - o[k]).max() / np.abs(o[k]).max()
            e32 = np.abs(o32[k] - o[k]).max() / np.abs(o[k]).max()
            assert e < max(2e-4, 8.0 * e32), (k, b, e, e32)
        k32 = kkt_eq(*args, *[o32[k].astype(np.float64) for k in ("X", "U", "lam", "nu")])
        assert np.isfinite(kkt[b]).all() and kkt[b, 2] < max(1e-4, 8.0 * k32[2]), (b, kkt[b], k32)


@pytest.mark.parametrize("n,m,ne,N", [(8, 5, 2, 6), (72, 30, 12, 40)])
def test_lqr_eq_kkt_evaluation(cuda, n, m, ne, N):
    """iters = 0 evaluates the KKT residual of the caller's point: at points
    off the solution (a random iterate, a perturbed costate or multiplier)
    the GPU's float32 residual matches the FP64 oracle's within 1e-3
    relative; a component left on the solution sits at float32 rounding
    (absolute 2e-5)."""
    from mpx_gb300.solver import lqr_eq_sqp
    from oracle.lqr_eq import kkt_eq, riccati_eq
    B = 3
    d, X0, U0 = _eq_case(B, n, m, ne, N, seed=11)
    sol = [riccati_eq(*[d[k][b] for k in KEYS_EQ]) for b in range(B)]
    X = np.stack([s["X"] for s in sol]); U = np.stack([s["U"] for s in sol])
    lam = np.stack([s["lam"] for s in sol]); nu = np.stack([s["nu"] for s in sol])
    X[0] = X0[0]                  # instance 0: a random iterate (primal and dual off)
    lam[1, N // 2, 1] += 0.5      # instance 1: one costate off
    nu[2, N // 3, 0] += 0.5       # instance 2: one multiplier off
    g = lqr_eq_sqp(*[d[k] for k in KEYS_EQ], X, U, iters=0, lam=lam, nu=nu)
    torch.cuda.synchronize()
    kkt = g["kkt"].cpu().numpy()
    for b in range(B):
        f32 = lambda a: a.astype(np.float32).astype(np.float64)
        o = kkt_eq(*[f32(d[k][b]) for k in KEYS_EQ], f32(X[b]), f32(U[b]), f32(lam[b]), f32(nu[b]))
        assert o[2] > 1e-3, (b, o)
        assert np.allclose(kkt[b], o, rtol=1e-3, atol=2e-5), (b, kkt[b], o)
        assert abs(kkt[b, 2] - o[2]) <= 1e-3 * o[2], (b, kkt[b], o)
    assert np.array_equal(g["X"].cpu().numpy(), X.astype(np.float32))  # iters = 0 leaves the point


def test_lqr_eq_sqp_rejects_bad_arguments(cuda):
    from mpx_gb300._lib import MpxgError
    from mpx_gb300.solver import lqr_eq_sqp
    d, X0, U0 = _eq_case(1, 8, 5, 2, 4, seed=2)
    with pytest.raises(MpxgError):
        lqr_eq_sqp(*[d[k] for k in KEYS_EQ], X0, U0, iters=101)
    with pytest.raises(MpxgError):
        lqr_eq_sqp(*[d[k] for k in KEYS_EQ], X0, U0, iters=1, method=2)
