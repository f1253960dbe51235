"""Known-answer checks of the oracle's LQR / KKT solve (CPU)."""
import numpy as np

from mpx_gb300 import problem as P


def _lq(seed, B=3, N=7, n=5, m=3):
    d = P.random_lq(B, n, m, N, seed=seed)
    rng = np.random.default_rng(seed + 100)
    d["M"] = 0.05 * rng.standard_normal(d["M"].shape)  # exercise the cross term too
    return d


def test_riccati_equals_dense_kkt(oracle):
    d = _lq(0)
    out = oracle.lqr_solve(d["A"], d["B"], d["c"], d["Q"], d["R"], d["M"], d["q"], d["r"], d["x0"])
    for b in range(d["A"].shape[0]):
        X, U, lam = oracle.dense_lqr(d["A"][b], d["B"][b], d["c"][b], d["Q"][b], d["R"][b], d["M"][b], d["q"][b],
                                     d["r"][b], d["x0"][b])
        np.testing.assert_allclose(out["X"][b], X, atol=1e-10, rtol=1e-10)
        np.testing.assert_allclose(out["U"][b], U, atol=1e-10, rtol=1e-10)
        np.testing.assert_allclose(out["lam"][b], lam, atol=1e-10, rtol=1e-10)


def test_riccati_fp32_close_to_fp64(oracle):
    d = P.random_lq(4, 24, 12, 32, seed=1)
    o64 = oracle.lqr_solve(d["A"], d["B"], d["c"], d["Q"], d["R"], d["M"], d["q"], d["r"], d["x0"])
    o32 = oracle.lqr_solve(d["A"], d["B"], d["c"], d["Q"], d["R"], d["M"], d["q"], d["r"], d["x0"], precision=32)
    for k in ("X", "U", "lam", "K", "k"):
        scale = np.abs(o64[k]).max()
        assert np.abs(o32[k] - o64[k]).max() <= 1e-4 * scale, k


def test_lq_sqp_one_step_is_exact(oracle):
    """On a linear-quadratic problem one SQP step from any point is the optimum:
    the KKT residual after one iteration is at rounding level."""
    d = _lq(2, B=2, N=6, n=4, m=2)
    desc = P.generic_lq(4, 2)
    B, N, n, m = 2, 6, 4, 2
    rng = np.random.default_rng(5)
    X0 = rng.standard_normal((B, N + 1, n))
    U0 = rng.standard_normal((B, N, m))
    V0 = rng.standard_normal((B, N + 1, n))
    lq = dict(A=d["A"], B=d["B"], c=d["c"], Q=d["Q"], R=d["R"], M=d["M"], q=d["q"], r=d["r"])
    opts = P.SolverOptions(sqp_iters=1, reg=0.0)
    out = oracle.sqp_solve(desc, opts, d["x0"], X0, U0, V0, lq=lq)
    assert out["kkt"][:, 2].max() < 1e-9
    ref = oracle.lqr_solve(d["A"], d["B"], d["c"], d["Q"], d["R"], d["M"], d["q"], d["r"], d["x0"])
    np.testing.assert_allclose(out["X"], ref["X"], atol=1e-9)
    np.testing.assert_allclose(out["V"], ref["lam"], atol=1e-9)
