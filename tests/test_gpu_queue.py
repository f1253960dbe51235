"""Device work queue: a persistent kernel solves pool rows while the host
pushes them, with the bits mpxg_solve gives; its waits are bounded and end
in a timeout status that the host reads (no trap, the context stays usable)."""
import time

import numpy as np
import pytest
import torch

from mpx_gb300 import problem as P
from mpx_gb300._lib import MpxgError
from mpx_gb300.solver import SolveQueue, Solver

pytestmark = pytest.mark.gpu


def _pool(B=24, seed=8):
    wl = P.quadruped_workload(B, horizons=(20, 30, 40), seed=seed, model=P.MODEL_SRBD_RPY12, v_range=(-0.5, 0.5),
                              random_phase=True)
    return wl, (wl.x0, wl.X0, wl.U0, wl.V0, wl.reference, wl.parameter, wl.W, wl.horizon)


def _wait(q, tickets, limit_s=20.0):
    got, t0 = {}, time.time()
    while len(got) < len(tickets):
        assert time.time() - t0 < limit_s, "queue results did not arrive"
        for t in tickets:
            if t not in got:
                r = q.result(t)
                if r is not None:
                    got[t] = r
        time.sleep(0.001)
    return got


def test_queue_solves_rows_pushed_while_it_runs(cuda):
    wl, pool = _pool()
    s = Solver(wl.desc, P.SolverOptions(sqp_iters=3), n_max=wl.n_max, batch_max=wl.batch)
    ref = s.solve(*pool)
    torch.cuda.synchronize()
    q = SolveQueue(s, pool, capacity=16, idle_timeout_s=5.0)
    first = [q.push(r) for r in range(12)]
    res = _wait(q, first)                       # the kernel solved these before the rest was pushed
    second = []
    for r in range(12, wl.batch):
        t = None
        while t is None:                         # ring of 16: wait for a free entry
            t = q.push(r)
        second.append(t)
    res.update(_wait(q, second))
    q.finish()
    m = wl.desc.m
    U0 = ref["U"][:, 0].cpu().numpy()
    kkt = ref["kkt"].cpu().numpy()
    status = ref["status"].cpu().numpy()
    for row, t in enumerate(first + second):
        r = res[t]
        assert np.array_equal(r[:m], U0[row]) and np.array_equal(r[m:m + 3], kkt[row]) and int(r[m + 3]) == status[row]
    for i, N in enumerate(wl.horizon):  # the full trajectories too
        for k, rows in (("X", N + 1), ("U", N), ("V", N + 1)):
            assert torch.equal(q.out[k][i, :rows], ref[k][i, :rows]), (k, i)


def test_queue_wait_times_out_with_a_status(cuda):
    """A queue that gets no work within its idle timeout stops its warps and
    reports MPXG_ERR_TIMEOUT; the context stays usable."""
    wl, pool = _pool(B=4, seed=9)
    s = Solver(wl.desc, P.SolverOptions(sqp_iters=2), n_max=wl.n_max, batch_max=wl.batch)
    q = SolveQueue(s, pool, capacity=4, idle_timeout_s=0.02)
    time.sleep(0.3)  # nothing pushed: every warp's wait runs out
    with pytest.raises(MpxgError, match="timeout"):
        q.push(0)
    with pytest.raises(MpxgError, match="timeout"):
        q.finish()
    out = s.solve(*pool)  # the device is fine
    torch.cuda.synchronize()
    assert torch.isfinite(out["U"]).all()


def test_queue_rejects_rows_outside_the_pool(cuda):
    wl, pool = _pool(B=4, seed=10)
    s = Solver(wl.desc, P.SolverOptions(sqp_iters=2), n_max=wl.n_max, batch_max=wl.batch)
    q = SolveQueue(s, pool, capacity=4, idle_timeout_s=5.0)
    with pytest.raises(MpxgError):
        q.push(4)
    t = q.push(3)
    _wait(q, [t])
    q.finish()
