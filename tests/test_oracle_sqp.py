"""Convergence properties of the oracle's primal-dual SQP (CPU)."""
import numpy as np

from mpx_gb300 import problem as P


def test_srbd_without_barrier_converges_quadratically(oracle):
    wl = P.quadruped_workload(4, horizons=(20,), seed=1, model=P.MODEL_SRBD_RPY12)
    wl.desc.barrier_alpha = 0.0
    k = []
    for it in (3, 5, 8):
        out = oracle.sqp_solve(wl.desc, P.SolverOptions(sqp_iters=it), wl.x0, wl.X0, wl.U0, wl.V0, wl.reference,
                               wl.parameter, wl.W, wl.horizon)
        k.append(out["kkt"][:, 2].max())
    assert k[-1] < 1e-10 and k[1] < 1e-4


def test_receding_horizon_steady_state_reaches_tolerance(oracle):
    """Warm-started control ticks (shifted previous solution) reach KKT <= 1e-5
    within 5 SQP iterations for the trot workload."""
    wl = P.quadruped_workload(16, horizons=(25, 50), seed=3, model=P.MODEL_SRBD_RPY12, v_range=(-1, 1),
                              random_phase=True)
    d = wl.desc
    X, U, V, x0, lt = wl.X0, wl.U0, wl.V0, wl.x0, wl.leg_time.copy()
    ref, par = wl.reference, wl.parameter
    for tick in range(14):
        out = oracle.sqp_solve(d, P.SolverOptions(sqp_iters=5), x0, X, U, V, ref, par, wl.W, wl.horizon)
        X, U, V = P.shift_warm_start(out["X"], out["U"], out["V"], wl.horizon)
        x0 = out["X"][:, 1, :].astype(np.float32)
        X[:, 0, :] = x0
        _, lt = P.timer_run_np(wl.duty, wl.step_freq, lt, d.dt)
        ref, par = P.quadruped_tables(d, x0, lt, wl.v_ref, wl.horizon, wl.n_max)
    k = out["kkt"][:, 2]
    assert np.median(k) < 1e-6
    assert (k <= 1e-5).mean() >= 0.75


def test_fp32_solve_tracks_fp64(oracle):
    wl = P.quadruped_workload(4, horizons=(25,), seed=2, model=P.MODEL_SRBD_QUAT13)
    o64 = oracle.sqp_solve(wl.desc, P.SolverOptions(sqp_iters=3), wl.x0, wl.X0, wl.U0, wl.V0, wl.reference,
                           wl.parameter, wl.W, wl.horizon, precision=64)
    o32 = oracle.sqp_solve(wl.desc, P.SolverOptions(sqp_iters=3), wl.x0, wl.X0, wl.U0, wl.V0, wl.reference,
                           wl.parameter, wl.W, wl.horizon, precision=32)
    assert np.abs(o32["X"] - o64["X"]).max() < 1e-3
