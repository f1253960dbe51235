"""Serving: continuous batching over resident episode slots."""
import time

import numpy as np
import pytest
import torch

from mpx_gb300 import problem as P
from mpx_gb300.server import BudgetError, MPCServer, default_models, served_workload

pytestmark = pytest.mark.gpu


def make_server(**kw):
    return MPCServer(default_models(), n_max=60, budget_bytes=kw.pop("budget", 2 << 30),
                     opts=P.SolverOptions(sqp_iters=3), drift_std=0.0, **kw)


def x0_of(server, name, seed):
    pool = server.pools[name]
    rng = np.random.default_rng(seed)
    x0 = np.zeros(pool.desc.n, dtype=np.float32)
    x0[2] = pool.gait["height"]
    return x0 + rng.normal(0, 0.02, pool.desc.n).astype(np.float32)


def test_result_same_alone_and_in_mix(cuda):
    """An episode's ticks give the same controls whether it is served alone or
    batched with other episodes of both models."""
    alone = make_server()
    alone.admit("A", "quadruped", x0_of(alone, "quadruped", 1), 40, v_ref=0.3, phase=0.2)
    res_alone = []
    for _ in range(3):
        alone.submit("A"); alone.launch_pending(); alone.drain()
    res_alone = [d[3] for d in alone.completed]
    mix = make_server()
    mix.admit("A", "quadruped", x0_of(mix, "quadruped", 1), 40, v_ref=0.3, phase=0.2)
    for k in range(5):
        mix.admit("q%d" % k, "quadruped", x0_of(mix, "quadruped", 10 + k), 20 + 7 * k, v_ref=0.1 * k, phase=0.1 * k)
        mix.admit("b%d" % k, "biped", x0_of(mix, "biped", 20 + k), 25 + 5 * k, v_ref=-0.1 * k, phase=0.3)
    eps = ["A"] + ["q%d" % k for k in range(5)] + ["b%d" % k for k in range(5)]
    for _ in range(3):
        for e in eps:
            mix.submit(e)
        mix.launch_pending(); mix.drain()
    res_mix = [d[3] for d in mix.completed if d[1] == "A"]
    assert len(res_alone) == len(res_mix) == 3
    for a, b in zip(res_alone, res_mix):
        np.testing.assert_array_equal(a, b)


def test_admission_budget_and_release(cuda):
    s = make_server(max_slots=3)
    for k in range(3):
        s.admit(k, "quadruped", x0_of(s, "quadruped", k), 30)
    with pytest.raises(BudgetError):
        s.admit(99, "quadruped", x0_of(s, "quadruped", 9), 30)
    s.release(1)
    s.admit(99, "quadruped", x0_of(s, "quadruped", 9), 30)


def test_served_stream_reports_latency(cuda):
    s = MPCServer(default_models(), n_max=120, budget_bytes=4 << 30, opts=P.SolverOptions(sqp_iters=5),
                  drift_std=0.01)
    lat, wall = served_workload(s, n_episodes=40, rate_hz=2000.0, duration_s=0.5, horizon_range=(20, 120),
                                episode_ticks=30)
    assert len(lat) > 500
    assert np.all(np.isfinite(lat)) and np.percentile(lat, 99) < 1.0
    assert len(s.last_status) == len(lat) and not np.any(s.last_status & 1)
    # both models served (alternating episodes), each result tagged with its model
    assert len(s.last_model) == len(lat)
    assert set(np.unique(s.last_model).tolist()) == {0, 1} and s.model_names == ["quadruped", "biped"]


def test_c_poll_returns_each_result_once(cuda):
    """mpxg_poll: NOT_READY before the batch ran, the result row once after,
    then the ticket is gone (MPXG_ERR_INVALID_ARG)."""
    import ctypes
    from mpx_gb300 import _lib
    s = make_server()
    s.admit("E", "quadruped", x0_of(s, "quadruped", 3), 30, v_ref=0.2)
    L = s.L
    t = ctypes.c_longlong()
    assert L.mpxg_submit(s.handle, s.episodes["E"], ctypes.byref(t)) == 0
    r = _lib.Result()
    assert L.mpxg_poll(s.handle, t.value, ctypes.byref(r)) == 7     # not launched yet
    for _ in range(1000):
        assert L.mpxg_server_step(s.handle, 1, None, None) == 0
        st = L.mpxg_poll(s.handle, t.value, ctypes.byref(r))
        if st == 0:
            break
    assert st == 0 and r.ticket == t.value and r.episode == s.episodes["E"]
    assert np.all(np.isfinite(np.array(r.u0[:12]))) and r.status & 1 == 0
    assert L.mpxg_poll(s.handle, t.value, ctypes.byref(r)) == 1
    s.close()


def test_nan_result_then_reset_recovers(cuda):
    """A non-finite state makes the solve report MPXG_INST_NAN; after
    reset_slot with a valid state the episode's next tick is cold-started and
    finite (the NaN fallback of mpc_wrapper.py:79-98)."""
    s = make_server()
    bad = x0_of(s, "quadruped", 5)
    bad[3] = np.nan
    s.admit("N", "quadruped", bad, 25)
    s.submit("N"); s.drain()
    assert s.completed[-1][5] & 1
    s.reset_slot("N", x0_of(s, "quadruped", 5))
    s.submit("N"); s.drain()
    last = s.completed[-1]
    assert last[5] & 1 == 0 and np.all(np.isfinite(last[3]))
    s.close()


def test_release_waits_for_queued_tick(cuda):
    """A released episode keeps its slot until its queued tick has run."""
    s = make_server(max_slots=1)
    s.admit("A", "quadruped", x0_of(s, "quadruped", 1), 30)
    s.submit("A")
    s.release("A")                      # tick still queued: slot stays taken
    with pytest.raises(BudgetError):
        s.admit("B", "quadruped", x0_of(s, "quadruped", 2), 30)
    s.drain()
    assert len(s.completed) == 1 and s.completed[0][1] == "A"
    s.admit("B", "quadruped", x0_of(s, "quadruped", 2), 30)   # freed once the tick completed
    s.close()


def test_each_ticket_is_delivered_when_its_own_solve_ends(cuda):
    """A short-horizon tick and a long one in the same batch: the short one's
    result reaches the host while the long one is still being solved (the
    rows land in mapped host memory, status entry last), and each result
    equals the one a second server gives after draining."""
    def run(early):
        s = MPCServer(default_models(), n_max=200, budget_bytes=8 << 30, opts=P.SolverOptions(sqp_iters=5),
                      drift_std=0.0)
        s.admit("long", "quadruped", x0_of(s, "quadruped", 1), 200, v_ref=0.3, phase=0.2)
        s.admit("short", "quadruped", x0_of(s, "quadruped", 2), 20, v_ref=0.3, phase=0.6)
        s.submit("long")
        s.submit("short")
        s.launch_pending()
        got = {}
        if early:
            deadline = time.perf_counter() + 10.0
            while "short" not in got and time.perf_counter() < deadline:
                for d in s.poll():
                    got[d[1]] = d
            assert "short" in got
            assert "long" not in got  # the N = 200 solve takes ms longer than the N = 20 one
        s.drain()
        for d in s.completed:
            got[d[1]] = d
        s.close()
        return got

    early, late = run(True), run(False)
    for k in ("long", "short"):
        np.testing.assert_array_equal(early[k][3], late[k][3])
        np.testing.assert_array_equal(early[k][4], late[k][4])
        assert early[k][5] == late[k][5]
