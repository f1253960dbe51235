"""The whole-body controllers of mpc_wrapper.py on the GPU: the whole-body
reference generator (mpxg_refgen_wb) against vectors from the reference's own
reference_generator (tests/golden/wb_refgen.npz, tests/golden/make_golden.py
--wbref), and MPCControllerWrapper / BatchedMPCControllerWrapper with the
aliengo configuration returning (tau, q, dq) / (data, tau) as the reference
does (mpc_wrapper.py:115-170, 297-365).

Tolerances: the generator follows the reference's float32 arithmetic step
by step; the contact schedule and the liftoff bookkeeping must match exactly.
The float rows go through sin and cos of the yaw (and asin of the terrain
pitch), whose float32 results differ by an ulp between CUDA, glibc and numpy,
so the floats are held to 2e-6 relative (a few ulps)."""
import os

import numpy as np
import pytest
import torch

from mpx_gb300 import _lib, configs, mjcf
from mpx_gb300.mpc_wrapper import BatchedMPCControllerWrapper, MPCControllerWrapper
from mpx_gb300.solver import _ptr
from mpx_gb300.wholebody import WholeBodyModel, WholeBodySQP

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(__file__)
FIX = os.path.join(HERE, "golden", "aliengo_wb.npz")
REF = os.path.join(HERE, "golden", "wb_refgen.npz")


def run_refgen(g, terrain, cuda):
    L = _lib.load()
    d = {k: torch.as_tensor(g["wbref_in_" + k]).to(cuda).contiguous() for k in
         ("t_timer", "x", "foot", "input", "contact", "liftoff")}
    cfg = g["wbref_cfg"]
    N, B = int(cfg[0]), d["x"].shape[0]
    ref = torch.empty(B, N + 1, 53, device=cuda)
    par = torch.empty(B, N + 1, 4, device=cuda)
    f0 = (_lib.ctypes.c_float * 12)(*g["wbref_foot0"].tolist())
    q0 = (_lib.ctypes.c_float * 12)(*g["wbref_q0"].tolist())
    _lib.check(L.mpxg_refgen_wb(None, B, N, 12, float(cfg[1]), float(cfg[2]), f0, q0, float(cfg[3]), float(cfg[4]),
                                float(cfg[5]), float(cfg[6]), int(terrain), _ptr(d["t_timer"]), _ptr(d["x"]),
                                _ptr(d["foot"]), _ptr(d["input"]), _ptr(d["contact"]), _ptr(d["liftoff"]),
                                _ptr(ref), _ptr(par)), None, "mpxg_refgen_wb")
    torch.cuda.synchronize()
    return ref.cpu().numpy(), par.cpu().numpy(), d["liftoff"].cpu().numpy()


@pytest.mark.parametrize("terrain", [False, True])
def test_refgen_wb_matches_golden(cuda, terrain):
    g = np.load(REF)
    tag = "terrain" if terrain else "flat"
    ref, par, lo = run_refgen(g, terrain, cuda)
    want = g["wbref_%s_reference" % tag]
    assert np.array_equal(par, g["wbref_%s_parameter" % tag])
    assert np.array_equal(ref[:, :, 37:41], want[:, :, 37:41])  # contact columns
    err = np.abs(ref - want) / (1.0 + np.abs(want))
    assert err.max() < 2e-6, err.max()
    assert np.abs(lo - g["wbref_%s_liftoff" % tag]).max() < 2e-6


def test_refgen_wb_matches_oracle_on_seeded_inputs(cuda):
    """64 seeded instances per terrain setting (tilted liftoff planes, any
    heading, velocities up to 1 m/s) against the float32 oracle
    (oracle/refgen.hpp refgen_wb)."""
    from oracle import oracle as O
    rng = np.random.default_rng(12)
    B, N = 64, 25
    cfg = configs.aliengo_wb()
    foot0, q0 = np.asarray(cfg.p_legs0, np.float32), np.asarray(cfg.q0, np.float32)
    ins = dict(t_timer=rng.uniform(0, 1, (B, 4)), x=np.zeros((B, 61)), foot=np.zeros((B, 12)),
               input=np.zeros((B, 7)), contact=rng.integers(0, 2, (B, 4)), liftoff=np.zeros((B, 12)))
    for b in range(B):
        yaw = rng.uniform(-np.pi, np.pi)
        q = np.array([np.cos(yaw / 2), 0, 0, np.sin(yaw / 2)]) + rng.normal(0, 0.05, 4)
        ins["x"][b] = np.concatenate([rng.normal(0, 0.2, 3) + [0, 0, 0.33], q / np.linalg.norm(q),
                                      q0 + rng.normal(0, 0.1, 12), rng.normal(0, 0.5, 18), foot0, np.zeros(12)])
        ins["foot"][b] = foot0 + rng.normal(0, 0.03, 12)
        ins["input"][b] = np.concatenate([rng.uniform(-1, 1, 3), rng.uniform(-0.5, 0.5, 3), [0.1]])
        ins["liftoff"][b] = ins["foot"][b] + np.repeat([0.0, 0.0, 1.0], 4) * rng.normal(0, 0.05, 12)
    ins = {k: v.astype(np.float32) for k, v in ins.items()}
    L = _lib.load()
    for terrain in (0, 1):
        d = {k: torch.as_tensor(v).to(cuda).contiguous() for k, v in ins.items()}
        ref = torch.empty(B, N + 1, 53, device=cuda)
        par = torch.empty(B, N + 1, 4, device=cuda)
        f0 = (_lib.ctypes.c_float * 12)(*foot0.tolist())
        qq = (_lib.ctypes.c_float * 12)(*q0.tolist())
        _lib.check(L.mpxg_refgen_wb(None, B, N, 12, cfg.dt, 40.0, f0, qq, cfg.duty_factor, cfg.step_freq,
                                    cfg.step_height, 0.4, terrain, _ptr(d["t_timer"]), _ptr(d["x"]), _ptr(d["foot"]),
                                    _ptr(d["input"]), _ptr(d["contact"]), _ptr(d["liftoff"]), _ptr(ref), _ptr(par)),
                   None, "mpxg_refgen_wb")
        ref, par, lo = ref.cpu().numpy(), par.cpu().numpy(), d["liftoff"].cpu().numpy()
        for b in range(B):
            r2, p2, l2 = O.refgen_wb(N, 12, cfg.dt, 40.0, foot0, q0, cfg.duty_factor, cfg.step_freq, cfg.step_height,
                                     0.4, terrain, ins["t_timer"][b], ins["x"][b], ins["foot"][b], ins["input"][b],
                                     ins["contact"][b], ins["liftoff"][b])
            assert np.array_equal(par[b], p2), (terrain, b)
            err = np.abs(ref[b] - r2) / (1.0 + np.abs(r2))
            assert err.max() < 2e-6, (terrain, b, err.max())
            assert np.abs(lo[b] - l2).max() < 2e-6


def standing(cfg, model, rng, B=1):
    qpos = np.concatenate([np.asarray(cfg.p0) + rng.normal(0, 0.01, 3), [1.0, 0.0, 0.0, 0.0],
                           np.asarray(cfg.q0) + rng.normal(0, 0.02, 12)])
    qvel = rng.normal(0, 0.05, 18)
    return np.tile(qpos, (B, 1)).astype(np.float32), np.tile(qvel, (B, 1)).astype(np.float32)


def test_single_controller_returns_tau_q_dq(cuda):
    """run(qpos, qvel, input, contact) -> (tau, q, dq): tau = U[0, :12]
    clipped to [min_torque, max_torque], q = X[0, 7:19], dq = X[1, 25:37] of
    the solve the controller ran, and the warm start is that solve shifted by
    one stage (mpc_wrapper.py:261-282, 361)."""
    cfg = configs.aliengo_wb()
    model = mjcf.load_npz(FIX)
    ctrl = MPCControllerWrapper(cfg, model=model, device=cuda)
    rng = np.random.default_rng(4)
    qpos, qvel = standing(cfg, model, rng)
    inp = np.array([0.3, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0], dtype=np.float32)
    contact = np.ones(4, dtype=np.float32)
    ctrl.reset(qpos[0], qvel[0])
    # the same tick by hand: feet by forward kinematics, timer, generator, solve
    wb = ctrl._wb
    st = wb.save_state()
    tau, q, dq = ctrl.run(qpos[0], qvel[0], inp, contact)
    assert tau.shape == (12,) and q.shape == (12,) and dq.shape == (12,)
    assert np.all(tau <= cfg.max_torque) and np.all(tau >= cfg.min_torque)
    feet = WholeBodyModel(model, device=cuda).terms(qpos, np.zeros((1, 18), np.float32))["cpos"]
    x0 = torch.cat([torch.as_tensor(qpos, device=cuda), torch.as_tensor(qvel, device=cuda), feet,
                    torch.zeros(1, 12, device=cuda)], 1)
    ct = st["contact_time"].to(cuda).clone()
    wb._timer(1, ct, cfg.duty_factor, cfg.step_freq)
    assert torch.equal(ct, wb.contact_time)
    inp2 = torch.as_tensor(inp, device=cuda).reshape(1, 7).clone()
    inp2[0, 6] = cfg.initial_height
    lo = st["liftoff"].to(cuda).clone()
    ref, par = wb._refgen(1, ct, x0, feet, inp2, torch.ones(1, 4, device=cuda), lo, cfg.duty_factor,
                          cfg.step_freq, cfg.step_height)
    sqp = WholeBodySQP(WholeBodyModel(model, device=cuda), cfg.N, batch_max=1, dt=cfg.dt)
    out = sqp.solve(x0, st["X0"].to(cuda), st["U0"].to(cuda), st["V0"].to(cuda), ref, par.to(torch.int32),
                    cfg.W_diag)
    U, X = out["U"].cpu().numpy()[0], out["X"].cpu().numpy()[0]
    assert np.array_equal(tau, np.clip(U[0, :12], cfg.min_torque, cfg.max_torque))
    assert np.array_equal(q, X[0, 7:19]) and np.array_equal(dq, X[1, 25:37])
    assert np.array_equal(wb.X0.cpu().numpy()[0, :-1], X[1:])
    assert np.array_equal(wb.X0.cpu().numpy()[0, -1], X[-1])
    # ticks of a running controller stay finite and keep the torques in range
    for _ in range(5):
        tau, q, dq = ctrl.run(qpos[0], qvel[0], inp, contact)
        assert np.all(np.isfinite(tau)) and np.all(np.abs(tau) <= cfg.max_torque)


def test_single_controller_nan_fallback(cuda):
    """A non-finite solve (a NaN warm start) returns the previous plan's
    second row and resets the warm start to x0 / u_ref / 0 (mpc_wrapper.py:
    272-282)."""
    cfg = configs.aliengo_wb()
    ctrl = MPCControllerWrapper(cfg, model=mjcf.load_npz(FIX), device=cuda)
    rng = np.random.default_rng(6)
    qpos, qvel = standing(cfg, None, rng)
    ctrl.reset(qpos[0], qvel[0])
    st = ctrl.save_state()
    st["U0"][0, 1, :] = torch.arange(12, dtype=torch.float32)
    st["X0"][0, 3:, 0] = float("nan")
    ctrl.load_state(st)
    tau, q, dq = ctrl.run(qpos[0], qvel[0], np.zeros(7, np.float32), np.ones(4, np.float32))
    assert np.array_equal(tau, np.clip(np.arange(12, dtype=np.float32), cfg.min_torque, cfg.max_torque))
    assert np.array_equal(q, st["X0"][0, 1, 7:19].numpy())
    X0 = ctrl._wb.X0.cpu().numpy()[0]
    assert np.all(X0 == X0[0]) and np.all(np.isfinite(X0))
    assert np.all(ctrl._wb.V0.cpu().numpy() == 0.0)


def test_batched_data_wrapper_matches_single_solves(cuda):
    """BatchedMPCControllerWrapper (make_data / run(data, x0, input) ->
    (data, tau) / reset): each environment's tau is that of a one-instance
    solve on the same tables, and data carries the shifted warm start, the
    stepped timers and grf = the force entries of X0[0] (mpc_wrapper.py:
    160-170)."""
    cfg = configs.aliengo_wb()
    model = mjcf.load_npz(FIX)
    B = 3
    w = BatchedMPCControllerWrapper(cfg, B, model=model, device=cuda)
    data = w.make_data()
    rng = np.random.default_rng(8)
    qpos, qvel = standing(cfg, model, rng, B)
    qpos[:, :3] += rng.normal(0, 0.01, (B, 3)).astype(np.float32)
    feet = WholeBodyModel(model, device=cuda).terms(qpos, np.zeros((B, 18), np.float32))["cpos"].cpu().numpy()
    data = w.reset(data, qpos, qvel, feet)
    x0 = np.concatenate([qpos, qvel, feet, np.zeros((B, 12), np.float32)], 1)
    inp = np.tile(np.array([0.2, 0.0, 0.0, 0.0, 0.0, 0.1, cfg.initial_height], np.float32), (B, 1))
    data2, tau = w.run(data, x0, inp)
    assert tau.shape == (B, 12)
    tau = tau.cpu().numpy()
    wb = w._wb
    for b in range(B):
        lo = data["liftoff"][b:b + 1].clone()
        xb = torch.as_tensor(x0[b:b + 1], device=cuda)
        ref, par = wb._refgen(1, data["contact_time"][b:b + 1].contiguous(), xb, xb[:, 37:49].contiguous(),
                              torch.as_tensor(inp[b:b + 1], device=cuda), torch.zeros(1, 4, device=cuda), lo,
                              cfg.duty_factor, cfg.step_freq, cfg.step_height)
        sqp = WholeBodySQP(WholeBodyModel(model, device=cuda), cfg.N, batch_max=1, dt=cfg.dt)
        out = sqp.solve(xb, data["X0"][b:b + 1], data["U0"][b:b + 1], data["V0"][b:b + 1], ref,
                        par.to(torch.int32), cfg.W_diag)
        assert np.array_equal(tau[b], out["U"].cpu().numpy()[0, 0, :12])
        assert torch.equal(data2["liftoff"][b], lo[0])
        X = out["X"].cpu().numpy()[0]
        assert np.array_equal(data2["X0"][b].cpu().numpy()[:-1], X[1:])
        assert np.array_equal(data2["grf"][b].cpu().numpy(), X[1, 49:61])
    assert not torch.equal(data2["contact_time"], data["contact_time"])
