"""CUDA solve vs the FP64 oracle at the benchmarked configurations.

* the batched tick of 4096 roll-pitch-yaw quadrupeds with horizons drawn
  from {25, 50, 100}: more instances than resident warps, so the solve runs
  the throughput variant over the longest-horizon-first queue; warm-started
  steady-state ticks; 64 sampled instances checked against the oracle;
* the single-instance recipe (N = 50, v_ref = 0.5 m/s, trot from phase 0,
  x0 perturbed by N(0, 0.05^2)) for seeds 0..99, cold start, 5 iterations;
* the quaternion model with the reference's own barrier (the drop-in model of
  mpx/utils/mpc_wrapper_srbd.py) over warm-started ticks.

Tolerances: a warm tick is near convergence, so X, U, V, K, k must agree with
the FP64 oracle to 1e-4 relative, or, where float32 cannot resolve a quantity
that well, to within 3x the oracle's own float32 error; a cold 5-iteration
solve to within 2x the oracle-FP32 error + 1e-4 (as tests/test_gpu_sqp.py).
"""
import numpy as np
import pytest
import torch

from mpx_gb300 import problem as P
from mpx_gb300.solver import Solver
from mpx_gb300.tick import TickRunner

pytestmark = pytest.mark.gpu


def _rel(a, b, horizon, rows_of):
    err = max(float(np.abs(a[i, :rows_of(N)] - b[i, :rows_of(N)]).max()) for i, N in enumerate(horizon))
    scale = max(float(np.abs(b[i, :rows_of(N)]).max()) for i, N in enumerate(horizon))
    return err / max(scale, 1e-12)


def _errors(g, o, horizon, U_scale_from=None):
    """Relative errors of X, U, V, K, k (k on the scale of the controls U,
    since it tends to 0 at convergence)."""
    xr, ur = (lambda N: N + 1), (lambda N: N)
    e = {k: _rel(g[k], o[k], horizon, xr if k in ("X", "V") else ur) for k in ("X", "U", "V", "K")}
    ek = max(float(np.abs(g["k"][i, :N] - o["k"][i, :N]).max()) for i, N in enumerate(horizon))
    us = max(float(np.abs(o["U"][i, :N]).max()) for i, N in enumerate(horizon))
    e["k"] = ek / max(us, 1e-12)
    return e


def _project_quat_gains(res, X, horizon):
    """Gain components along the quaternion's norm direction are undetermined
    (neither penalised nor controllable): compare on the tangent space."""
    for i, N in enumerate(horizon):
        for t in range(N):
            q = X[i, t, 3:7] / np.linalg.norm(X[i, t, 3:7])
            res["K"][i, t][:, 3:7] -= np.outer(res["K"][i, t][:, 3:7] @ q, q)


def _warm_tick_snapshot(wl, opts, ticks, idx):
    """Run `ticks` warm control ticks of the whole batch on the GPU, then
    shift and rebuild the tables of the next tick; solve it with gains and
    return the sampled inputs (host arrays) and outputs."""
    tr = TickRunner(wl, opts)
    tr.first_tick()
    for _ in range(ticks):
        tr.tick()
    tr.shift()
    tr.tables()
    torch.cuda.synchronize()
    ins = {k: getattr(tr, k).cpu().numpy() for k in ("x0", "X", "U", "V", "ref", "par", "w", "horizon")}
    out = tr.solver.solve(tr.x0, tr.X, tr.U, tr.V, tr.ref, tr.par, tr.w, tr.horizon, want_gains=True)
    torch.cuda.synchronize()
    g = {k: v.cpu().numpy()[idx] for k, v in out.items() if not k.startswith("_")}
    s = {k: v[idx] for k, v in ins.items()}
    tr.solver.close()
    return s, g


def test_batched_tick_4096_matches_oracle(oracle, cuda):
    wl = P.quadruped_workload(4096, horizons=(25, 50, 100), seed=7, model=P.MODEL_SRBD_RPY12, v_range=(-1, 1),
                              random_phase=True)
    opts = P.SolverOptions(sqp_iters=5)
    idx = np.random.default_rng(3).choice(wl.batch, size=64, replace=False)
    s, g = _warm_tick_snapshot(wl, opts, 4, idx)
    assert set(np.unique(s["horizon"])) == {25, 50, 100}
    W = np.stack([np.diag(w) for w in s["w"]])
    args = (wl.desc, opts, s["x0"], s["X"], s["U"], s["V"], s["ref"], s["par"], W, s["horizon"])
    o = oracle.sqp_solve(*args)
    o32 = oracle.sqp_solve(*args, precision=32)
    eg, e32 = _errors(g, o, s["horizon"]), _errors(o32, o, s["horizon"])
    for key in ("X", "U", "V", "K", "k"):
        assert eg[key] < max(1e-4, 3.0 * e32[key]), (key, eg[key], e32[key])
    # the GPU result is as good a KKT point as the oracle's (FP64 evaluation):
    # within 2x the FP64 run's residual, or 3x the oracle's own float32 run's
    # (near the 1e-5 gate float32 rounding sets the residual)
    kg = oracle.kkt_residual(wl.desc, s["x0"], g["X"], g["U"], g["V"], s["ref"], s["par"], W, s["horizon"])
    k32 = oracle.kkt_residual(wl.desc, s["x0"], o32["X"], o32["U"], o32["V"], s["ref"], s["par"], W, s["horizon"])
    bound = np.maximum(np.maximum(2.0 * o["kkt"][:, 2], 3.0 * k32[:, 2]), 1e-5)
    assert np.all(kg[:, 2] <= bound), (kg[:, 2].max(), o["kkt"][:, 2].max(), k32[:, 2].max())
    assert np.all(g["status"] == 0), g["status"]


def test_single_instance_recipe_seeds_0_to_99(oracle, cuda):
    parts = [P.quadruped_workload(1, horizons=(50,), seed=s, model=P.MODEL_SRBD_RPY12, v_range=(0.5, 0.5),
                                  random_phase=False, noise=0.05) for s in range(100)]
    cat = lambda k: np.concatenate([getattr(p, k) for p in parts])
    wl = P.Workload(parts[0].desc, cat("x0"), cat("X0"), cat("U0"), cat("V0"), cat("reference"), cat("parameter"),
                    cat("W"), cat("horizon"))
    opts = P.SolverOptions(sqp_iters=5)
    s = Solver(wl.desc, opts, n_max=50, batch_max=wl.batch)
    out = s.solve(wl.x0, wl.X0, wl.U0, wl.V0, wl.reference, wl.parameter, wl.W, wl.horizon, want_gains=True)
    torch.cuda.synchronize()
    g = {k: v.cpu().numpy() for k, v in out.items() if not k.startswith("_")}
    # the plain path (one launch per instance) gives the same bits
    p = s.solve(wl.x0[:4], wl.X0[:4], wl.U0[:4], wl.V0[:4], wl.reference[:4], wl.parameter[:4], wl.W[:4],
                wl.horizon[:4], plain=True)
    torch.cuda.synchronize()
    for k in ("X", "U", "V"):
        assert np.array_equal(p[k].cpu().numpy(), g[k][:4]), k
    s.close()
    args = (wl.desc, opts, wl.x0, wl.X0, wl.U0, wl.V0, wl.reference, wl.parameter, wl.W, wl.horizon)
    o = oracle.sqp_solve(*args)
    o32 = oracle.sqp_solve(*args, precision=32)
    for key in ("X", "U", "V"):
        rows = (lambda N: N + 1) if key != "U" else (lambda N: N)
        eg, e32 = _rel(g[key], o[key], wl.horizon, rows), _rel(o32[key], o[key], wl.horizon, rows)
        assert eg <= 2.0 * e32 + 1e-4, (key, eg, e32)
    kg = oracle.kkt_residual(wl.desc, wl.x0, g["X"], g["U"], g["V"], wl.reference, wl.parameter, wl.W, wl.horizon)
    assert np.all(kg[:, 2] <= np.maximum(2.0 * o["kkt"][:, 2], 1e-4)), (kg[:, 2].max(), o["kkt"][:, 2].max())
    assert np.all(g["status"] & 1 == 0)


def test_reference_model_warm_ticks_match_oracle(oracle, cuda):
    """The quaternion model with the reference's barrier (barrier_kind 0,
    unmasked cost, clipped) over warm ticks."""
    wl = P.quadruped_workload(256, horizons=(25, 50), seed=21, model=P.MODEL_SRBD_QUAT13, v_range=(-0.5, 0.5),
                              random_phase=True)
    assert wl.desc.barrier_kind == 0 and wl.desc.cone_eps2 == 1e-2
    opts = P.SolverOptions(sqp_iters=5)
    idx = np.arange(0, 256, 8)
    s, g = _warm_tick_snapshot(wl, opts, 4, idx)
    W = np.stack([np.diag(w) for w in s["w"]])
    args = (wl.desc, opts, s["x0"], s["X"], s["U"], s["V"], s["ref"], s["par"], W, s["horizon"])
    o = oracle.sqp_solve(*args)
    o32 = oracle.sqp_solve(*args, precision=32)
    for res in (g, o, o32):
        _project_quat_gains(res, o["X"], s["horizon"])
    eg, e32 = _errors(g, o, s["horizon"]), _errors(o32, o, s["horizon"])
    for key in ("X", "U", "V", "K", "k"):
        assert eg[key] < max(1e-4, 3.0 * e32[key]), (key, eg[key], e32[key])
    assert np.all(g["status"] & 1 == 0)
