"""Mixed-model launch: one persistent solve over a quadruped batch and a
biped batch gives every instance the bits its own model's one-warp solve
gives, and the server's mixed mode serves both models' ticks with one solve
launch per step."""
import numpy as np
import pytest
import torch

from mpx_gb300 import problem as P
from mpx_gb300.server import MPCServer, default_models
from mpx_gb300.solver import MixedSolver, Solver

pytestmark = pytest.mark.gpu


def _args(wl):
    return (wl.x0, wl.X0, wl.U0, wl.V0, wl.reference, wl.parameter, wl.W, wl.horizon)


def _same(wl, alone, mixed):
    for i, N in enumerate(wl.horizon):
        for key, rows in (("X", N + 1), ("V", N + 1), ("U", N), ("K", N), ("k", N)):
            a, b = alone[key][i, :rows].cpu().numpy(), mixed[key][i, :rows].cpu().numpy()
            assert np.array_equal(a, b), (key, i)
    assert torch.equal(alone["kkt"], mixed["kkt"]) and torch.equal(alone["status"], mixed["status"])


@pytest.mark.parametrize("quad_model", [P.MODEL_SRBD_RPY12, P.MODEL_SRBD_QUAT13])
def test_mixed_launch_matches_each_model_alone(cuda, quad_model):
    q = P.quadruped_workload(40, horizons=(20, 60), seed=3, model=quad_model, v_range=(-0.5, 0.5), random_phase=True)
    b = P.biped_workload(30, horizons=(25, 60), seed=4)
    assert q.n_max == b.n_max == 60
    opts = P.SolverOptions(sqp_iters=3)
    sa = Solver(q.desc, opts, n_max=60, batch_max=q.batch)
    sb = Solver(b.desc, opts, n_max=60, batch_max=b.batch)
    alone_a = sa.solve(*_args(q), want_gains=True)
    alone_b = sb.solve(*_args(b), want_gains=True)
    mx = MixedSolver(sa, sb)
    mixed_a, mixed_b = mx.solve(_args(q), _args(b), want_gains=True)
    torch.cuda.synchronize()
    _same(q, alone_a, mixed_a)
    _same(b, alone_b, mixed_b)
    # either batch may be empty
    q2 = P.quadruped_workload(8, horizons=(60,), seed=6, model=quad_model)
    only_a, _ = mx.solve(_args(q2), tuple(a[:0] for a in _args(b)), want_gains=True)
    ref = sa.solve(*_args(q2), want_gains=True)
    torch.cuda.synchronize()
    _same(q2, ref, only_a)
    mx.close()
    sa.close()
    sb.close()


def test_mixed_rejects_unbuilt_pairs_and_unequal_horizons(cuda):
    from mpx_gb300._lib import MpxgError
    rpy = Solver(P.quadruped_rpy12(), P.SolverOptions(), n_max=30, batch_max=4)
    rpy2 = Solver(P.quadruped_rpy12(), P.SolverOptions(), n_max=30, batch_max=4)
    biped = Solver(P.biped_wrench12(), P.SolverOptions(), n_max=31, batch_max=4)
    with pytest.raises(MpxgError):  # two quadrupeds: not a built pair
        MixedSolver(rpy, rpy2)
    with pytest.raises(MpxgError):  # n_max differs
        MixedSolver(rpy, biped)


def _server(mixed, streams=32):
    return MPCServer(default_models(), n_max=60, budget_bytes=3 << 30, opts=P.SolverOptions(sqp_iters=3),
                     drift_std=0.0, streams=streams, mixed_launch=mixed)


def _x0(server, name, seed):
    pool = server.pools[name]
    x0 = np.zeros(pool.desc.n, dtype=np.float32)
    x0[2] = pool.gait["height"]
    return x0 + np.random.default_rng(seed).normal(0, 0.02, pool.desc.n).astype(np.float32)


def test_mixed_server_same_results_one_launch_per_step(cuda):
    """Both models' ticks go out in one launch (one stream is enough to run
    them all at once), and every episode's results equal those of the server
    that launches each model's batch on its own."""
    runs = {}
    for mixed in (False, True):
        s = _server(mixed, streams=1)
        eps = []
        for k in range(4):
            s.admit("q%d" % k, "quadruped", _x0(s, "quadruped", 10 + k), 20 + 9 * k, v_ref=0.1 * k, phase=0.2 * k)
            s.admit("b%d" % k, "biped", _x0(s, "biped", 20 + k), 25 + 8 * k, v_ref=-0.1 * k, phase=0.3)
            eps += ["q%d" % k, "b%d" % k]
        running = []
        for _ in range(3):
            for e in eps:
                s.submit(e)
            s.launch_pending()
            running.append(s.stats()[1])
            s.drain()
        runs[mixed] = (sorted((d[1], tuple(np.asarray(d[3]).tolist())) for d in s.completed), running)
    assert runs[True][1] == [8, 8, 8]     # one launch holds both models' ticks
    assert runs[False][1] == [4, 4, 4]    # one stream: one model's batch at a time
    assert runs[True][0] == runs[False][0]
