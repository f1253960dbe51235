"""mpxg_evaluate (the reference's model_evaluator_helper) vs the oracle's
stage cost and dynamics on the same trajectories."""
import numpy as np
import pytest
import torch

from mpx_gb300 import problem as P
from mpx_gb300.solver import Solver

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("model", [P.MODEL_SRBD_RPY12, P.MODEL_SRBD_QUAT13, P.MODEL_BIPED_WRENCH12])
def test_evaluate_matches_oracle(oracle, cuda, model):
    if model == P.MODEL_BIPED_WRENCH12:
        wl = P.biped_workload(5, horizons=(20, 35), seed=21)
    else:
        wl = P.quadruped_workload(5, horizons=(20, 35), seed=21, model=model, v_range=(-1, 1), random_phase=True)
    s = Solver(wl.desc, P.SolverOptions(), n_max=wl.n_max, batch_max=wl.batch)
    g, c = s.evaluate(wl.x0, wl.X0, wl.U0, wl.reference, wl.parameter, wl.W, wl.horizon)
    torch.cuda.synchronize()
    g, c = g.cpu().numpy(), c.cpu().numpy()
    s.close()
    for b in range(wl.batch):
        N = int(wl.horizon[b])
        for t in range(N + 1):
            u = wl.U0[b, t] if t < N else np.zeros(wl.desc.m)
            l = oracle.cost(wl.desc, wl.X0[b, t], u, wl.reference[b, t], wl.W[b], terminal=(t == N))
            assert abs(g[b, t] - l) <= 1e-4 * max(1.0, abs(l)), (b, t, g[b, t], l)
            if t == 0:
                ref_c = wl.x0[b] - wl.X0[b, 0]
            else:
                ref_c = oracle.dynamics(wl.desc, wl.X0[b, t - 1], wl.U0[b, t - 1], wl.parameter[b, t - 1]) - wl.X0[b, t]
            np.testing.assert_allclose(c[b, t], ref_c, atol=2e-5, rtol=1e-4)
        assert np.all(g[b, N + 1:] == 0) and np.all(c[b, N + 1:] == 0)
