"""The oracle's SQP on the constrained LQ problem (CPU): one iteration from
any iterate lands on the direct constrained Riccati solution, and the KKT
residual vanishes there and not at a perturbed point."""
import numpy as np

from mpx_gb300 import problem as P
from oracle.lqr_eq import dense_lqr_eq, kkt_eq, riccati_eq, sqp_eq

KEYS = ("A", "B", "c", "Q", "R", "M", "q", "r", "C", "D", "e", "x0")


def _case(seed, n=8, m=5, ne=2, N=7):
    d = P.random_lq_eq(1, n=n, m=m, n_eq=ne, N=N, seed=seed)
    d = {k: v[0] for k, v in d.items()}
    rng = np.random.default_rng(seed + 100)
    d["M"] = 0.002 * rng.normal(size=d["M"].shape)
    d["r"] = rng.normal(size=d["r"].shape)
    X0, U0 = rng.normal(size=(N + 1, n)), rng.normal(size=(N, m))
    return d, X0, U0


def test_one_iteration_is_the_direct_solution():
    for seed in range(3):
        d, X0, U0 = _case(seed)
        args = [d[k] for k in KEYS]
        o = riccati_eq(*args)
        s = sqp_eq(*args, X0, U0, iters=1)
        for k in ("X", "U", "lam", "nu", "K", "Knu"):
            assert np.abs(s[k] - o[k]).max() < 1e-8 * (1 + np.abs(o[k]).max()), (seed, k)
        Xd, Ud, lamd, nud = dense_lqr_eq(*args)
        assert np.abs(s["X"] - Xd).max() < 1e-8 * (1 + np.abs(Xd).max())
        assert np.abs(s["nu"] - nud).max() < 1e-8 * (1 + np.abs(nud).max())


def test_kkt_vanishes_at_the_solution_only():
    d, X0, U0 = _case(7)
    args = [d[k] for k in KEYS]
    s = sqp_eq(*args, X0, U0, iters=2)
    kk = kkt_eq(*args, s["X"], s["U"], s["lam"], s["nu"])
    assert kk[2] < 1e-9, kk
    X = s["X"].copy()
    X[3, 1] += 1e-3  # a state off the solution: the defects of stages 2 and 3 see it
    assert kkt_eq(*args, X, s["U"], s["lam"], s["nu"])[0] > 5e-4
    lam = s["lam"].copy()
    lam[4, 0] += 1e-2  # a costate off the solution: the dual rows see it
    assert kkt_eq(*args, s["X"], s["U"], lam, s["nu"])[1] > 1e-4
    nu = s["nu"].copy()
    nu[2, 1] += 1e-2
    assert kkt_eq(*args, s["X"], s["U"], s["lam"], nu)[1] > 1e-4
