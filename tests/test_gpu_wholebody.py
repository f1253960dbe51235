"""The whole-body kernel (mpxg_wb_terms / mpxg_wb_interface) against the
float64 oracle (oracle/wholebody.py) on the aliengo model of the reference's
SRBD configuration (tests/golden/aliengo_wb.npz).

Tolerances: float32 evaluation of the interface formula alone moves tau by
up to 2.2e-6 relative (cond(J'J) ~ 130 for these states); the bounds below
are about 20x that, relative to each quantity's own scale."""
import os

import numpy as np
import pytest
import torch

from mpx_gb300 import configs, mjcf
from mpx_gb300.wholebody import WholeBodyModel
from mpx_gb300.wrappers import BatchedMPCControllerWrapper
from oracle import wholebody as W

pytestmark = pytest.mark.gpu

FIX = os.path.join(os.path.dirname(__file__), "golden", "aliengo_wb.npz")


def states(B, seed, spread=0.3):
    rng = np.random.default_rng(seed)
    q0 = np.load(FIX)["q0"]
    quat = rng.normal(size=(B, 4))
    quat /= np.linalg.norm(quat, axis=1, keepdims=True)
    qpos = np.concatenate([rng.normal(size=(B, 3)) * spread + [0, 0, 0.3], quat,
                           q0 + rng.normal(size=(B, 12)) * 0.2], axis=1)
    return qpos, rng.normal(size=(B, 18)), rng


def close(got, ref, rel):
    got = np.asarray(got, dtype=np.float64)
    return np.abs(got - ref).max() <= rel * (1.0 + np.abs(ref).max())


@pytest.mark.parametrize("B", [1, 33, 256])
def test_terms_match_oracle(cuda, B):
    model = mjcf.load_npz(FIX)
    wb = WholeBodyModel(model, device=cuda)
    qpos, qvel, _ = states(B, B)
    out = {k: v.cpu().numpy() for k, v in wb.terms(qpos.astype(np.float32), qvel.astype(np.float32)).items()}
    for b in range(B):
        ref = W.terms(model, qpos[b].astype(np.float32), qvel[b].astype(np.float32))
        assert close(out["M"][b], ref["M"], 2e-5), b
        assert close(out["bias"][b], ref["bias"], 2e-5), b
        assert close(out["cpos"][b], ref["cpos"], 2e-6), b
        assert close(out["J"][b], ref["J"], 2e-6), b
        assert close(out["cvel"][b], ref["cvel"], 2e-5), b
    M = out["M"]
    assert np.array_equal(M, np.transpose(M, (0, 2, 1)))          # written symmetric


def test_terms_of_a_model_with_slide_and_offset_anchor(cuda):
    model = mjcf.parse(os.path.join(os.path.dirname(__file__), "golden", "slider_arm.xml"), ["tip"], ["slider"])
    wb = WholeBodyModel(model, device=cuda)
    rng = np.random.default_rng(5)
    quat = rng.normal(size=(16, 4))
    quat /= np.linalg.norm(quat, axis=1, keepdims=True)
    qpos = np.concatenate([rng.normal(size=(16, 3)), quat, rng.normal(size=(16, 2))], axis=1).astype(np.float32)
    qvel = rng.normal(size=(16, 8)).astype(np.float32)
    out = {k: v.cpu().numpy() for k, v in wb.terms(qpos, qvel).items()}
    for b in range(16):
        ref = W.terms(model, qpos[b], qvel[b])
        for k in ("M", "bias", "cpos", "J", "cvel"):
            assert close(out[k][b], ref[k], 2e-5), (k, b)


@pytest.mark.parametrize("B", [1, 33, 512])
def test_interface_matches_oracle(cuda, B):
    model = mjcf.load_npz(FIX)
    wb = WholeBodyModel(model, device=cuda)
    qpos, qvel, rng = states(B, 100 + B)
    grf = rng.normal(size=(B, 12)) * 30
    fr = rng.normal(size=(B, 12)) * 0.05
    frd = rng.normal(size=(B, 12)) * 0.2
    contact = rng.integers(0, 2, size=(B, 4)).astype(np.int32)
    cfg = configs.srbd_quadruped()
    f32 = lambda a: np.asarray(a, dtype=np.float32)
    tau, J = wb.interface(f32(qpos), f32(qvel), f32(grf), f32(fr), f32(frd), contact, cfg.Kp, cfg.Kd)
    tau, J = tau.cpu().numpy(), J.cpu().numpy()
    for b in range(B):
        rt, rJ = W.interface(model, cfg.Kp, cfg.Kd, f32(qpos[b]), f32(qvel[b]), f32(grf[b]), f32(fr[b]),
                             f32(frd[b]), contact[b])
        assert close(tau[b], rt, 5e-5), b
        assert close(J[b], rJ, 2e-6), b


def test_interface_in_contact_is_the_force_mapping(cuda):
    """With every leg in contact tau = -(J grf)[6:] exactly as the float32
    product the kernel forms; it does not depend on the PD terms."""
    model = mjcf.load_npz(FIX)
    wb = WholeBodyModel(model, device=cuda)
    B = 64
    qpos, qvel, rng = states(B, 7)
    grf = (rng.normal(size=(B, 12)) * 30).astype(np.float32)
    ones = np.ones((B, 4), dtype=np.int32)
    cfg = configs.srbd_quadruped()
    z = np.zeros((B, 12), dtype=np.float32)
    t1, J = wb.interface(qpos.astype(np.float32), qvel.astype(np.float32), grf, z, z, ones, cfg.Kp, cfg.Kd)
    t2, _ = wb.interface(qpos.astype(np.float32), qvel.astype(np.float32), grf, z + 1, z - 1, ones, cfg.Kp * 3,
                         cfg.Kd * 3)
    assert torch.equal(t1, t2)
    ref = -(J.double() @ torch.as_tensor(grf, device=cuda).double().unsqueeze(-1)).squeeze(-1)[:, 6:]
    assert (t1.double() - ref).abs().max().item() < 1e-4 * (1 + ref.abs().max().item())


def test_identical_environments_give_identical_results(cuda):
    """Every warp runs the same instruction sequence: a batch of copies of one
    state (4096, several waves of blocks) returns bitwise-equal rows."""
    model = mjcf.load_npz(FIX)
    wb = WholeBodyModel(model, device=cuda)
    qpos, qvel, _ = states(1, 3)
    B = 4096
    out = wb.terms(np.tile(qpos, (B, 1)).astype(np.float32), np.tile(qvel, (B, 1)).astype(np.float32))
    for k, v in out.items():
        assert torch.equal(v, v[:1].expand_as(v)), k


def test_srbd_wrapper_whole_body_run(cuda):
    """BatchedMPCControllerWrapper.whole_body_run after an MPC tick uses that
    tick's grf, foot references and contact flags (mpc_wrapper_srbd.py:153-154)."""
    cfg = configs.srbd_quadruped()
    model = mjcf.load_npz(FIX)
    B = 4
    wr = BatchedMPCControllerWrapper(cfg, B, wb_model=model)
    x0 = np.tile(np.concatenate([cfg.p0, cfg.quat0, np.zeros(6)]), (B, 1)).astype(np.float32)
    inp = np.tile(np.array([0.3, 0.0, 0.0, 0.0, 0.0, 0.0, cfg.robot_height], dtype=np.float32), (B, 1))
    foot = np.tile(cfg.p_legs0, (B, 1)).astype(np.float32)
    wr.run(x0, inp, foot, np.ones((B, 4), dtype=np.float32))
    qpos, qvel, _ = states(B, 11)
    qpos = qpos.astype(np.float32)
    qvel = qvel.astype(np.float32)
    tau, J = wr.whole_body_run(qpos, qvel)
    tau = tau.cpu().numpy()
    grf, fr, frd = (t.cpu().numpy() for t in (wr.grf, wr.foot_ref, wr.foot_ref_dot))
    contact = wr.contact.cpu().numpy()
    for b in range(B):
        rt, _ = W.interface(model, cfg.Kp, cfg.Kd, qpos[b], qvel[b], grf[b], fr[b], frd[b], contact[b])
        assert close(tau[b], rt, 5e-5), b
    assert torch.equal(wr.torch_whole_body_run(torch.as_tensor(qpos), torch.as_tensor(qvel)),
                       torch.as_tensor(tau, device=cuda))


def hexapod_mjcf():
    """A floating base with six 3-joint legs (19 bodies, 24 dofs, 6 feet):
    larger than the compact kernel capacity, so the general one runs."""
    legs = []
    for i in range(6):
        ang = 60.0 * i + 30.0
        x, y = 0.25 * np.cos(np.radians(ang)), 0.15 * np.sin(np.radians(ang))
        legs.append('''
      <body name="L%d_hip" pos="%.4f %.4f 0" euler="0 0 %.1f">
        <joint name="L%d_a" axis="0 0 1"/>
        <inertial pos="0.03 0 0" mass="0.4" diaginertia="0.001 0.0012 0.0009"/>
        <body name="L%d_thigh" pos="0.06 0 0">
          <joint name="L%d_b" axis="0 1 0"/>
          <inertial pos="0.05 0 -0.01" quat="0.9 0.1 0 0.2" mass="0.3" diaginertia="0.002 0.0021 0.0004"/>
          <body name="L%d_shin" pos="0.12 0 0" euler="0 30 0">
            <joint name="L%d_c" axis="0 1 0" pos="0 0 0.01"/>
            <inertial pos="0 0 -0.08" mass="0.15" diaginertia="0.0015 0.0015 0.0001"/>
            <geom name="F%d" size="0.02" pos="0 0 -0.16"/>
          </body>
        </body>
      </body>''' % (i, x, y, ang, i, i, i, i, i, i))
    return '''<mujoco><compiler angle="degree"/><default><joint armature="0.005"/></default><worldbody>
      <body name="torso" pos="0 0 0.3"><freejoint/>
        <inertial pos="0.01 0 0" mass="4" diaginertia="0.05 0.08 0.1"/>%s
      </body></worldbody></mujoco>''' % "".join(legs)


def test_general_capacity_model_matches_oracle(cuda):
    model = mjcf.parse(hexapod_mjcf(), ["F%d" % i for i in range(6)], ["L%d_shin" % i for i in range(6)])
    assert model.nbody == 19 and model.nv == 24 and len(model.contact_point_body) == 6
    wb = WholeBodyModel(model, device=cuda)
    B = 41
    rng = np.random.default_rng(9)
    quat = rng.normal(size=(B, 4))
    quat /= np.linalg.norm(quat, axis=1, keepdims=True)
    qpos = np.concatenate([rng.normal(size=(B, 3)) * 0.3, quat,
                           np.tile([0.0, 0.5, -1.2], (B, 6)) + rng.normal(size=(B, 18)) * 0.3], axis=1)
    qpos, qvel = qpos.astype(np.float32), rng.normal(size=(B, 24)).astype(np.float32)
    out = {k: v.cpu().numpy() for k, v in wb.terms(qpos, qvel).items()}
    Kp, Kd = np.diag([80.0] * 18), np.diag([4.0] * 18)
    grf = (rng.normal(size=(B, 18)) * 10).astype(np.float32)
    fr = (rng.normal(size=(B, 18)) * 0.05).astype(np.float32)
    frd = (rng.normal(size=(B, 18)) * 0.2).astype(np.float32)
    contact = rng.integers(0, 2, size=(B, 6)).astype(np.int32)
    tau, _ = wb.interface(qpos, qvel, grf, fr, frd, contact, Kp, Kd)
    tau = tau.cpu().numpy()
    for b in range(B):
        ref = W.terms(model, qpos[b], qvel[b])
        for k in ("M", "bias", "cpos", "J", "cvel"):
            assert close(out[k][b], ref[k], 2e-5), (k, b)
        rt, _ = W.interface(model, Kp, Kd, qpos[b], qvel[b], grf[b], fr[b], frd[b], contact[b])
        # cond(J'J) reaches 5.5e3 on these states: float32 evaluation of the
        # interface formula alone moves tau by up to 5e-5 relative
        assert close(tau[b], rt, 5e-4), b


def step_states(B, seed):
    rng = np.random.default_rng(seed)
    q0 = np.load(FIX)["q0"]
    quat = rng.normal(0, 0.2, (B, 4))
    quat[:, 0] += 1
    quat /= np.linalg.norm(quat, axis=1, keepdims=True)
    qpos = np.concatenate([rng.normal(0, 0.05, (B, 3)) + [0, 0, 0.33], quat, q0 + rng.normal(0, 0.2, (B, 12))], 1)
    x = np.concatenate([qpos, rng.normal(0, 0.5, (B, 18)), np.zeros((B, 24))], 1).astype(np.float32)
    return x, rng.normal(0, 10, (B, 12)).astype(np.float32), rng


def test_step_matches_oracle(cuda):
    """mpxg_wb_step against the oracle's quadruped_wb_dynamics (which is
    pinned to the reference's source, tests/test_oracle_wholebody.py).
    float32 evaluation alone moves v+ and the forces by up to 9e-7 relative."""
    model = mjcf.load_npz(FIX)
    wb = WholeBodyModel(model, device=cuda)
    B = 67
    x, u, rng = step_states(B, 21)
    contact = rng.integers(0, 2, (B, 4)).astype(np.int32)
    xn = wb.step(x, u, contact, 0.02).cpu().numpy()
    for b in range(B):
        ref = W.wb_dynamics(model, 0.02, x[b], u[b], contact[b])
        assert close(xn[b, :19], ref[:19], 2e-6), b          # qpos+
        assert close(xn[b, 19:37], ref[19:37], 2e-5), b      # qvel+
        assert close(xn[b, 37:49], ref[37:49], 2e-6), b      # contact points
        assert close(xn[b, 49:], ref[49:], 2e-5), b          # forces


def test_step_with_every_foot_in_contact_stops_the_feet(cuda):
    """2 alpha dt = 1 for the reference's alpha = 25, dt = 0.02: the feet's
    velocities after the step, J(x)' v+, vanish."""
    model = mjcf.load_npz(FIX)
    wb = WholeBodyModel(model, device=cuda)
    B = 32
    x, u, _ = step_states(B, 22)
    xn = wb.step(x, u, np.ones((B, 4), dtype=np.int32), 0.02)
    J = wb.terms(x[:, :19], x[:, 19:37])["J"]
    jv0 = (J.transpose(1, 2) @ torch.as_tensor(x[:, 19:37], device=cuda).unsqueeze(-1)).abs().amax(dim=(1, 2))
    jv1 = (J.transpose(1, 2) @ xn[:, 19:37].unsqueeze(-1)).abs().amax(dim=(1, 2))
    assert bool((jv1 <= 1e-4 * (1 + jv0)).all())
