"""Launch-geometry autotuner: measures every candidate and keeps the fastest;
every geometry gives the same results."""
import numpy as np
import pytest
import torch

from mpx_gb300 import problem as P
from mpx_gb300.autotune import time_geometry, tune
from mpx_gb300.solver import Solver

pytestmark = pytest.mark.gpu


def test_tune_picks_the_fastest_measured_candidate(cuda, tmp_path, monkeypatch):
    monkeypatch.setenv("MPXG_TUNE_CACHE", str(tmp_path / "tune.json"))
    wl = P.quadruped_workload(64, horizons=(20, 40), seed=3, model=P.MODEL_SRBD_RPY12)
    opts = P.SolverOptions(sqp_iters=2)
    r = tune(wl, opts, candidates=[(2, 0), (4, 0), (1, 2), (4, 0, 8, 16)], reps=2)
    ms = [t["ms"] for t in r["table"]]
    assert None not in ms  # the team candidate (8 warps per instance from N = 16 on) ran too
    assert r["ms"] == min(ms) and not r["cached"]
    assert tune(wl, opts, candidates=[(2, 0)], reps=1)["cached"]     # second call: from the cache


def test_create_rejects_blocks_wider_than_the_kernel(cuda):
    from mpx_gb300._lib import MpxgError
    wl = P.quadruped_workload(4, horizons=(10,), seed=5, model=P.MODEL_SRBD_RPY12)
    with pytest.raises(MpxgError):
        Solver(wl.desc, P.SolverOptions(), n_max=wl.n_max, batch_max=4, warps_per_block=8)


def test_geometry_does_not_change_results(cuda):
    wl = P.quadruped_workload(40, horizons=(15, 30), seed=4, model=P.MODEL_SRBD_RPY12)
    opts = P.SolverOptions(sqp_iters=3)
    res = []
    for wpb, bps in ((4, 0), (2, 2), (1, 1)):
        s = Solver(wl.desc, opts, n_max=wl.n_max, batch_max=wl.batch, warps_per_block=wpb, blocks_per_sm=bps)
        o = s.solve(wl.x0, wl.X0, wl.U0, wl.V0, wl.reference, wl.parameter, wl.W, wl.horizon)
        torch.cuda.synchronize()
        res.append(o["U"].cpu().numpy())
        s.close()
    for i, N in enumerate(wl.horizon):
        for r in res[1:]:
            assert np.array_equal(r[i, :N], res[0][i, :N])
