"""The drop-in wrappers on the GPU against the oracle's version of the same
per-tick pipeline (timer -> reference generator -> SQP -> shift)."""
import numpy as np
import pytest
import torch

from mpx_gb300 import configs
from mpx_gb300 import problem as P
from mpx_gb300.solver import Solver
from mpx_gb300.wrappers import BatchedDataMPCWrapper, BatchedMPCControllerWrapper, MPCControllerWrapper, make_mpc

pytestmark = pytest.mark.gpu


def tick_inputs(cfg, B, rng):
    x0 = np.tile(np.concatenate([cfg.p0, cfg.quat0, np.zeros(6)]), (B, 1)).astype(np.float32)
    x0[:, 7:13] += rng.normal(0, 0.05, (B, 6)).astype(np.float32)
    inp = np.tile(np.array([0.3, 0.0, 0.0, 0.0, 0.0, 0.1, cfg.robot_height], dtype=np.float32), (B, 1))
    foot = (np.tile(cfg.p_legs0, (B, 1)) + np.tile(x0[:, :3], (1, 4)) * np.tile([1, 1, 0], 4)).astype(np.float32)
    contact = np.ones((B, 4), dtype=np.float32)
    return x0, inp, foot, contact


def test_srbd_wrapper_matches_oracle_pipeline(oracle, cuda):
    cfg = configs.srbd_quadruped()
    B, ticks = 3, 3
    rng = np.random.default_rng(0)
    opts = P.SolverOptions(sqp_iters=2)
    wr = BatchedMPCControllerWrapper(cfg, B, opts=opts)
    desc = P.quadruped_quat13(cfg)
    # oracle state
    ct = np.tile(cfg.timer_t, (B, 1)).astype(np.float32)
    lo = np.zeros((B, 12), dtype=np.float32)
    X0 = np.tile(np.concatenate([cfg.p0, cfg.quat0, np.zeros(6)]), (B, cfg.N + 1, 1)).astype(np.float32)
    U0 = np.zeros((B, cfg.N, 12), dtype=np.float32)
    V0 = np.zeros((B, cfg.N + 1, 13), dtype=np.float32)
    W = np.tile(cfg.W, (B, 1, 1))
    for k in range(ticks):
        x0, inp, foot, contact = tick_inputs(cfg, B, rng)
        wr.run(x0, inp, foot, contact)
        torch.cuda.synchronize()
        refs, pars = [], []
        for b in range(B):
            _, ct[b] = oracle.timer_run(cfg.duty_factor, cfg.step_freq, 1.0 / cfg.mpc_frequency, ct[b])
            r, p, lo[b], _ = oracle.refgen_srbd(cfg.N, cfg.dt, cfg.mass, cfg.p_legs0, cfg.duty_factor, cfg.step_freq,
                                                cfg.step_height, cfg.clearence_speed, ct[b], x0[b], foot[b], inp[b],
                                                contact[b], lo[b])
            refs.append(r); pars.append(p)
        ref, par = np.stack(refs), np.stack(pars)
        g_ref = wr.reference.cpu().numpy()
        assert np.array_equal(g_ref[:, :, 13:17], ref[:, :, 13:17])
        np.testing.assert_allclose(g_ref, ref, rtol=2e-6, atol=2e-6)
        np.testing.assert_allclose(wr.contact_time.cpu().numpy(), ct, rtol=0, atol=0)
        o = oracle.sqp_solve(desc, opts, x0, X0, U0, V0, ref, par, W, precision=32)
        g_grf = wr.grf.cpu().numpy()
        scale = np.abs(o["U"][:, 0]).max()
        assert np.abs(g_grf - o["U"][:, 0]).max() <= 1e-3 * max(scale, 1.0), (k, np.abs(g_grf - o["U"][:, 0]).max())
        X0, U0, V0 = [a.astype(np.float32) for a in P.shift_warm_start(o["X"], o["U"], o["V"], np.full(B, cfg.N))]
        np.testing.assert_allclose(wr.batch_X0.cpu().numpy(), X0, rtol=1e-3, atol=1e-3)


def test_make_mpc_single_and_batched(cuda):
    wl = P.quadruped_workload(5, horizons=(30,), seed=4)
    solve = make_mpc(wl.desc, P.SolverOptions(sqp_iters=3))
    X, U, V = solve(wl.reference, wl.parameter, wl.W, wl.x0, wl.X0, wl.U0, wl.V0)
    s = Solver(wl.desc, P.SolverOptions(sqp_iters=3), n_max=30, batch_max=5)
    ref = s.solve(wl.x0, wl.X0, wl.U0, wl.V0, wl.reference, wl.parameter, wl.W)
    torch.cuda.synchronize()
    assert torch.equal(X, ref["X"]) and torch.equal(U, ref["U"]) and torch.equal(V, ref["V"])
    X1, U1, V1 = solve(wl.reference[2], wl.parameter[2], wl.W[2], wl.x0[2], wl.X0[2], wl.U0[2], wl.V0[2])
    assert X1.shape == (31, 12) and torch.equal(X1, ref["X"][2])


def test_single_instance_wrapper_and_nan_fallback(cuda):
    cfg = configs.srbd_quadruped()
    wr = MPCControllerWrapper(cfg, opts=P.SolverOptions(sqp_iters=2))
    qpos = np.concatenate([cfg.p0, cfg.quat0, cfg.q0])
    qvel = np.zeros(18, dtype=np.float32)
    grf, q, dq = wr.run(qpos, qvel, np.array([0.2, 0, 0, 0, 0, 0, 0.35], dtype=np.float32), np.ones(4))
    assert np.all(np.isfinite(grf)) and grf.shape == (12,) and not wr._nan
    bad = qpos.copy(); bad[0] = np.nan
    grf, q, dq = wr.run(bad, qvel, np.array([0.2, 0, 0, 0, 0, 0, 0.35], dtype=np.float32), np.ones(4))
    assert wr._nan  # the NaN fallback reset the warm start (mpc_wrapper.py:271-278)
    assert torch.all(wr.V0 == 0)


def test_data_wrapper_two_ticks(cuda):
    cfg = configs.srbd_quadruped()
    B = 4
    wr = BatchedDataMPCWrapper(cfg, B, opts=P.SolverOptions(sqp_iters=2))
    data = wr.make_data()
    x0 = np.tile(np.concatenate([cfg.p0, cfg.quat0, np.zeros(6)]), (B, 1)).astype(np.float32)
    inp = np.tile(np.array([0.3, 0, 0, 0, 0, 0, cfg.robot_height], dtype=np.float32), (B, 1))
    for _ in range(2):
        data, grf = wr.run(data, x0, inp)
    torch.cuda.synchronize()
    assert grf.shape == (B, 12) and bool(torch.isfinite(grf).all())
    data = wr.reset(data, x0)
    assert torch.all(data["V0"] == 0)
