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
