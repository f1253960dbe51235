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
