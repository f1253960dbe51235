"""The whole-body SQP (mpxg_wb_sqp, mpx_gb300.wholebody.WholeBodySQP) against
the float64 oracle (oracle/wb_sqp.py) on the aliengo model of the reference's
whole-body configuration (tests/golden/aliengo_wb.npz, config_aliengo.py's
weights), seeded synthetic instances (mpx_gb300.problem.wb_workload).

Tolerances: the GPU takes the same float64 model step and merit terms as the
oracle; its Jacobians are exact derivatives of the step evaluated in float32
(the oracle's: float64 central differences, accurate to ~1e-9) and it solves
each step's LQ problem in float32.  The step (and so the iterate after one
iteration) then differs from the oracle's by float32 rounding of the
derivatives and of 61-state Riccati products, ~1e-5 of each quantity's scale,
and the bounds below are 2e-4 of it.  The line search must pick the same step
length."""
import os

import numpy as np
import pytest
import torch

from mpx_gb300 import configs, mjcf, problem
from mpx_gb300.wholebody import WholeBodyModel, WholeBodySQP
from oracle.wb_sqp import WbProblem, wb_kkt, wb_sqp_iteration

pytestmark = pytest.mark.gpu

FIX = os.path.join(os.path.dirname(__file__), "golden", "aliengo_wb.npz")


def setup(B, N, seed):
    model = mjcf.load_npz(FIX)
    d = np.load(FIX)
    wl = problem.wb_workload(B, N, d["q0"], d["p_legs0"], float(np.sum(model.mass)), seed=seed)
    return model, configs.aliengo_wb(), wl


def rel_err(got, ref):
    got = np.asarray(got, dtype=np.float64)
    return np.abs(got - ref).max() / (1.0 + np.abs(ref).max())


def oracle_iters(model, cfg, wl, b, iters):
    pb = WbProblem(model, cfg.dt, cfg.W, wl["reference"][b], wl["contact"][b])
    X, U, V = [wl[k][b].astype(np.float64) for k in ("X0", "U0", "V0")]
    x0 = wl["x0"][b].astype(np.float64)
    rho, out = 1.0, []
    for _ in range(iters):
        r = wb_sqp_iteration(pb, x0, X, U, V, rho)
        X, U, V, rho = r["X"], r["U"], r["V"], r["rho"]
        out.append(r)
    return pb, x0, out


def test_one_and_two_iterations_match_oracle(cuda):
    B, N = 2, 6
    model, cfg, wl = setup(B, N, seed=0)
    sqp = WholeBodySQP(WholeBodyModel(model, device=cuda), N=N, batch_max=B)
    args = [wl[k] for k in ("x0", "X0", "U0", "V0", "reference", "contact")]
    one = {k: v.cpu().numpy() for k, v in sqp.solve(*args, cfg.W_diag, iters=1).items()}
    two = {k: v.cpu().numpy() for k, v in sqp.solve(*args, cfg.W_diag, iters=2).items()}
    for b in range(B):
        pb, x0, res = oracle_iters(model, cfg, wl, b, 2)
        for got, r in ((one, res[0]), (two, res[1])):
            assert got["status"][b] == r["status"], b
            assert rel_err(got["X"][b], r["X"]) < 2e-4, (b, rel_err(got["X"][b], r["X"]))
            assert rel_err(got["U"][b], r["U"]) < 2e-4, (b, rel_err(got["U"][b], r["U"]))
            assert rel_err(got["V"][b], r["V"]) < 2e-4, (b, rel_err(got["V"][b], r["V"]))
        # the KKT residual of the result, as the oracle evaluates it
        ref_kkt = wb_kkt(pb, x0, two["X"][b].astype(np.float64), two["U"][b].astype(np.float64),
                         two["V"][b].astype(np.float64))
        assert abs(two["kkt"][b][0] - ref_kkt[0]) <= 1e-3 * (1 + ref_kkt[0]), (two["kkt"][b], ref_kkt)
        assert abs(two["kkt"][b][1] - ref_kkt[1]) <= 1e-3 * (1 + ref_kkt[1]) + 1e-6, (two["kkt"][b], ref_kkt)


def test_iterations_converge_and_batch_entries_are_independent(cuda):
    """Twelve iterations from the cold start cut every instance's KKT
    residual by more than 100x and bring most to 1e-5 (the oracle's float64
    runs of the same instances stall at the same level where these do: one of
    them near 5e-3, with failing line searches, in both); an instance's result
    does not depend on the others in its batch (bitwise)."""
    B, N = 6, 10
    model, cfg, wl = setup(B, N, seed=3)
    sqp = WholeBodySQP(WholeBodyModel(model, device=cuda), N=N, batch_max=B)
    args = [wl[k] for k in ("x0", "X0", "U0", "V0", "reference", "contact")]
    out = {k: v.cpu().numpy() for k, v in sqp.solve(*args, cfg.W_diag, iters=12).items()}
    assert np.all(np.isfinite(out["X"])) and np.all(out["status"] & 1 == 0)
    k0 = {k: v.cpu().numpy() for k, v in sqp.solve(*args, cfg.W_diag, iters=0).items()}
    assert np.all(k0["kkt"][:, 2] > 100 * out["kkt"][:, 2]), (k0["kkt"], out["kkt"])
    assert np.sum(out["kkt"][:, 2] <= 1e-5) >= 4, out["kkt"]
    # the same instance alone and in a batch of 6
    sub = [a[2:3] for a in args]
    alone = {k: v.cpu().numpy() for k, v in sqp.solve(*sub, cfg.W_diag, iters=12).items()}
    for k in ("X", "U", "V", "kkt", "status"):
        assert np.array_equal(alone[k][0], out[k][2]), k


def test_warm_tick_iteration_matches_oracle(cuda):
    """A control tick's iteration: from a GPU iterate after four iterations,
    shifted by one stage with x0 = X[1] (the wrappers' warm start, duals
    included), one GPU iteration against the oracle's from the same point."""
    B, N = 2, 6
    model, cfg, wl = setup(B, N, seed=5)
    sqp = WholeBodySQP(WholeBodyModel(model, device=cuda), N=N, batch_max=B)
    args = [wl[k] for k in ("x0", "X0", "U0", "V0", "reference", "contact")]
    four = {k: v.cpu().numpy() for k, v in sqp.solve(*args, cfg.W_diag, iters=4).items()}
    sh = lambda a: np.concatenate([a[:, 1:], a[:, -1:]], 1)
    x0 = np.ascontiguousarray(four["X"][:, 1])
    X, U, V = sh(four["X"]), sh(four["U"]), sh(four["V"])
    ref, cont = sh(wl["reference"]), sh(wl["contact"])
    got = {k: v.cpu().numpy() for k, v in sqp.solve(x0, X, U, V, ref, cont, cfg.W_diag, iters=1).items()}
    for b in range(B):
        pb = WbProblem(model, cfg.dt, cfg.W, ref[b], cont[b])
        r = wb_sqp_iteration(pb, x0[b].astype(np.float64), X[b].astype(np.float64), U[b].astype(np.float64),
                             V[b].astype(np.float64), 1.0)
        assert got["status"][b] == r["status"], b
        for k in ("X", "U", "V"):
            assert rel_err(got[k][b], r[k]) < 2e-4, (b, k, rel_err(got[k][b], r[k]))


def test_benchmarked_size_iteration_matches_oracle(cuda):
    """The benchmarked size (aliengo, N = 25, config_aliengo's horizon): one
    iteration from the cold start against the oracle's."""
    B, N = 1, 25
    model, cfg, wl = setup(B, N, seed=11)
    sqp = WholeBodySQP(WholeBodyModel(model, device=cuda), N=N, batch_max=B)
    args = [wl[k] for k in ("x0", "X0", "U0", "V0", "reference", "contact")]
    got = {k: v.cpu().numpy() for k, v in sqp.solve(*args, cfg.W_diag, iters=1).items()}
    _, _, res = oracle_iters(model, cfg, wl, 0, 1)
    assert got["status"][0] == res[0]["status"]
    for k in ("X", "U", "V"):
        assert rel_err(got[k][0], res[0][k]) < 2e-4, (k, rel_err(got[k][0], res[0][k]))
