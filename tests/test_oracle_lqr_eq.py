"""The equality-constrained LQR oracle against a dense KKT solve (CPU)."""
import numpy as np

from mpx_gb300 import problem as P
from oracle.lqr_eq import dense_lqr_eq, riccati_eq


def test_riccati_eq_equals_dense_kkt():
    d = P.random_lq_eq(2, n=8, m=5, n_eq=2, N=6, seed=3)
    d["M"] = 0.1 * np.random.default_rng(4).normal(size=d["M"].shape)
    d["r"] = np.random.default_rng(5).normal(size=d["r"].shape)
    for b in range(2):
        a = [d[k][b] for k in ("A", "B", "c", "Q", "R", "M", "q", "r", "C", "D", "e", "x0")]
        o = riccati_eq(*a)
        X, U, lam, nu = dense_lqr_eq(*a)
        for got, ref in ((o["X"], X), (o["U"], U), (o["lam"], lam), (o["nu"], nu)):
            assert np.abs(got - ref).max() <= 1e-8 * max(1.0, np.abs(ref).max())
        # the constraints hold on the returned trajectory
        for t in range(6):
            res = d["C"][b, t] @ o["X"][t] + d["D"][b, t] @ o["U"][t] - d["e"][b, t]
            assert np.abs(res).max() < 1e-9


def test_workload_shape_and_spectral_cap():
    d = P.random_lq_eq(2, n=72, m=30, n_eq=12, N=3, seed=1)
    assert d["A"].shape == (2, 3, 72, 72) and d["C"].shape == (2, 3, 12, 72) and d["D"].shape == (2, 3, 12, 30)
    assert np.abs(np.linalg.eigvals(d["A"])).max() <= 1.01 + 1e-9
