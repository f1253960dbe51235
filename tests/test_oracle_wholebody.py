"""The whole-body oracle (oracle/wholebody.py) and the MJCF reader.

The oracle is pinned by the reference's own numbers for its model (the
aliengo foot positions at q0 that mpx/config/config_srbd.py:38-43 lists,
x to 8 digits) and by identities of the mechanics that hold whatever
algorithm computes M and qfrc_bias."""
import copy
import os

import numpy as np
import pytest

from mpx_gb300 import mjcf
from oracle import wholebody as W

FIX = os.path.join(os.path.dirname(__file__), "golden", "aliengo_wb.npz")


@pytest.fixture(scope="module")
def model():
    return mjcf.load_npz(FIX)


def random_state(model, rng, spread=0.3):
    q0 = np.load(FIX)["q0"]
    quat = rng.normal(size=4)
    qpos = np.concatenate([rng.normal(size=3) * spread, quat / np.linalg.norm(quat), q0 + rng.normal(size=12) * 0.2])
    return qpos, rng.normal(size=model.nv)


def test_feet_at_q0_match_the_reference_config(model):
    z = np.load(FIX)
    qpos = np.concatenate([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0, 0.0], z["q0"]])
    feet = W.terms(model, qpos, np.zeros(model.nv))["cpos"].reshape(4, 3)
    ref = z["p_legs0"].reshape(4, 3)
    assert np.abs(feet[:, 0] - ref[:, 0]).max() < 1e-8      # listed to 8 digits
    assert np.abs(feet[:, 1] - ref[:, 1]).max() < 1e-3      # listed to 3 digits


def test_model_totals(model):
    assert model.nbody == 13 and model.nv == 18 and model.nq == 19
    assert abs(model.mass.sum() - 24.638) < 1e-9
    assert np.allclose(model.armature, [0.0] * 6 + [0.01] * 12)   # <freejoint/> takes no armature
    assert np.allclose(model.gravity, [0.0, 0.0, -9.806])


@pytest.mark.parametrize("seed", range(3))
def test_mass_matrix_is_the_kinetic_energy(model, seed):
    """1/2 v'(M - armature)v equals the kinetic energy of the finite-differenced
    body motion, for several velocities (which pins the quadratic form)."""
    rng = np.random.default_rng(seed)
    qpos, _ = random_state(model, rng)
    M = W.terms(model, qpos, np.zeros(model.nv))["M"]
    assert np.abs(M - M.T).max() < 1e-12
    assert np.linalg.eigvalsh(M).min() > 0
    Mb = M - np.diag(model.armature)
    for _ in range(4):
        v = rng.normal(size=model.nv)
        ke = W.kinetic_energy_fd(model, qpos, v)
        assert abs(0.5 * v @ Mb @ v - ke) <= 1e-7 * ke


@pytest.mark.parametrize("seed", range(3))
def test_velocity_product_terms_match_second_differences(model, seed):
    """dJ qdot of every contact point and every body's centre of mass equals
    the second difference of the point along the qacc = 0 motion."""
    rng = np.random.default_rng(10 + seed)
    qpos, qvel = random_state(model, rng)
    T = W.kinematics(model, qpos)
    Wb, _ = W._body_velocity(model, T, qvel)
    h = 1e-4
    Tp, Tm = W.kinematics(model, W.integrate(model, qpos, qvel, h)), W.kinematics(model, W.integrate(model, qpos, qvel, -h))
    for b in range(model.nbody):
        pt = lambda TT: TT[b][:3, :3] @ model.com[b] + TT[b][:3, 3]
        a_fd = (pt(Tp) - 2 * pt(T) + pt(Tm)) / h ** 2
        a_an, w_an = W._dJ_qdot(model, T, qvel, Wb, b, pt(T))
        assert np.abs(a_fd - a_an).max() < 1e-5 * (1 + np.abs(a_an).max())
        # angular: d/dt of the body's angular velocity
        def omega(s):
            TT = W.kinematics(model, W.integrate(model, qpos, qvel, s))
            return W._body_velocity(model, TT, qvel)[0][b]
        wd_fd = (omega(h) - omega(-h)) / (2 * h)
        assert np.abs(wd_fd - w_an).max() < 1e-5 * (1 + np.abs(w_an).max())


@pytest.mark.parametrize("seed", range(3))
def test_gravity_forces_are_the_potential_gradient(model, seed):
    rng = np.random.default_rng(20 + seed)
    qpos, _ = random_state(model, rng)
    bias = W.terms(model, qpos, np.zeros(model.nv))["bias"]
    h = 1e-6
    grad = np.array([(W.potential_energy(model, W.integrate(model, qpos, e, h)) -
                      W.potential_energy(model, W.integrate(model, qpos, e, -h))) / (2 * h) for e in np.eye(model.nv)])
    assert np.abs(bias - grad).max() < 1e-6 * np.abs(grad).max()


@pytest.mark.parametrize("seed", range(3))
def test_power_balance(model, seed):
    """qdot' bias(g = 0) = 1/2 qdot' (dM/dt) qdot at qacc = 0."""
    rng = np.random.default_rng(30 + seed)
    qpos, qvel = random_state(model, rng)
    m0 = copy.deepcopy(model)
    m0.gravity = np.zeros(3)
    b0 = W.terms(m0, qpos, qvel)["bias"]
    h = 1e-5
    dM = (W.terms(model, W.integrate(model, qpos, qvel, h), qvel)["M"] -
          W.terms(model, W.integrate(model, qpos, qvel, -h), qvel)["M"]) / (2 * h)
    lhs, rhs = qvel @ b0, 0.5 * qvel @ dM @ qvel
    assert abs(lhs - rhs) < 1e-6 * (1 + abs(rhs))


def test_jacobian_is_the_point_velocity(model):
    rng = np.random.default_rng(40)
    qpos, qvel = random_state(model, rng)
    t = W.terms(model, qpos, qvel)
    h = 1e-6
    fd = (W.terms(model, W.integrate(model, qpos, qvel, h), qvel)["cpos"] -
          W.terms(model, W.integrate(model, qpos, qvel, -h), qvel)["cpos"]) / (2 * h)
    assert np.abs(fd - t["cvel"]).max() < 1e-7


def test_interface_pinv_equals_normal_equations(model):
    """pinv(J') a = J (J'J)^-1 a for the full-rank J' of a standing robot: the
    kernel's formula gives the reference's jnp.linalg.pinv result."""
    rng = np.random.default_rng(50)
    for _ in range(5):
        qpos, qvel = random_state(model, rng)
        J = W.terms(model, qpos, qvel)["J"]
        a = rng.normal(size=12)
        assert np.allclose(np.linalg.pinv(J.T) @ a, J @ np.linalg.solve(J.T @ J, a), rtol=1e-9, atol=1e-10)


def test_interface_mask_selects_mpc_or_feedback(model):
    rng = np.random.default_rng(60)
    qpos, qvel = random_state(model, rng)
    Kp, Kd = np.diag([100.0] * 12), np.diag([5.0] * 12)
    grf, fr, frd = rng.normal(size=12) * 50, rng.normal(size=12) * 0.1, rng.normal(size=12) * 0.1
    t_all, J = W.interface(model, Kp, Kd, qpos, qvel, grf, fr, frd, [1, 1, 1, 1])
    t_none, _ = W.interface(model, Kp, Kd, qpos, qvel, grf, fr, frd, [0, 0, 0, 0])
    t_mix, _ = W.interface(model, Kp, Kd, qpos, qvel, grf, fr, frd, [1, 0, 0, 1])
    assert np.allclose(t_all, -(J @ grf)[6:])
    assert np.allclose(t_mix, np.concatenate([t_all[:3], t_none[3:9], t_all[9:]]))


MJCF = open(os.path.join(os.path.dirname(__file__), "golden", "slider_arm.xml")).read()


def test_reader_resolves_defaults_orientations_and_geoms():
    m = mjcf.parse(MJCF, ["tip"], ["slider"])
    assert m.body_names == ["base", "link", "slider"]
    assert list(m.jnt_type) == [mjcf.JNT_FREE, mjcf.JNT_HINGE, mjcf.JNT_SLIDE]
    assert np.allclose(m.armature, [0.0] * 6 + [0.05, 0.02])      # childclass, then class="main"
    assert np.allclose(m.jnt_axis[1], [0, 1, 0]) and np.allclose(m.jnt_pos[1], [0, 0, 0.05])
    assert np.allclose(m.body_quat[0], [np.cos(np.pi / 4), 0, 0, np.sin(np.pi / 4)])
    assert np.allclose(m.inertia[0], [[0.1, 0.01, 0], [0.01, 0.2, 0], [0, 0, 0.3]])
    assert np.allclose(m.contact_point_pos[0], [0, 0, -0.05])
    assert m.nq == 9 and m.nv == 8


def test_reader_rejects_what_it_cannot_represent():
    two = MJCF.replace('<joint name="j1" pos="0 0 0.05"/>', '<joint name="j1"/><joint name="j1b"/>')
    with pytest.raises(NotImplementedError):
        mjcf.parse(two)
    no_inertial = MJCF.replace('<inertial pos="0 0 -0.1" mass="1" diaginertia="0.01 0.01 0.001"/>', '<geom size="0.1"/>')
    with pytest.raises(NotImplementedError):
        mjcf.parse(no_inertial)


def test_reader_folds_joint_ref_into_the_rest_pose():
    """A hinge (slide) with `ref` at coordinate q places its body as the same
    joint without `ref` at q - ref (MuJoCo's qpos - qpos0)."""
    with_ref = MJCF.replace('<joint name="j1" pos="0 0 0.05"/>', '<joint name="j1" pos="0 0 0.05" ref="25"/>')
    with_ref = with_ref.replace('type="slide" axis="0 0 1"', 'type="slide" axis="0 0 1" ref="0.03"')
    a, b = mjcf.parse(with_ref, ["tip"], ["slider"]), mjcf.parse(MJCF, ["tip"], ["slider"])
    rng = np.random.default_rng(70)
    for _ in range(3):
        quat = rng.normal(size=4)
        qpos = np.concatenate([rng.normal(size=3), quat / np.linalg.norm(quat), rng.normal(size=2)])
        shifted = qpos.copy()
        shifted[7] -= np.radians(25.0)
        shifted[8] -= 0.03
        qvel = rng.normal(size=8)
        ta, tb = W.terms(a, qpos, qvel), W.terms(b, shifted, qvel)
        for k in ("M", "bias", "cpos", "J"):
            assert np.allclose(ta[k], tb[k], atol=1e-12), k


def test_reader_orientation_forms():
    """quat, axisangle and euler (intrinsic lower case, extrinsic upper case,
    degrees or radians) give the same frames."""
    base = '<mujoco><compiler angle="%s" %s/><worldbody><body name="b" %s>' \
           '<inertial pos="0 0 0" mass="1" diaginertia="1 1 1"/></body></worldbody></mujoco>'
    q_xyz = mjcf._quat_mul(mjcf._quat_mul(mjcf._axis_quat([1, 0, 0], 0.3), mjcf._axis_quat([0, 1, 0], -0.2)),
                           mjcf._axis_quat([0, 0, 1], 0.5))
    forms = [base % ("radian", "", 'quat="%.17g %.17g %.17g %.17g"' % tuple(q_xyz)),
             base % ("radian", "", 'euler="0.3 -0.2 0.5"'),
             base % ("degree", "", 'euler="%.17g %.17g %.17g"' % tuple(np.degrees([0.3, -0.2, 0.5]))),
             base % ("radian", 'eulerseq="ZYX"', 'euler="0.5 -0.2 0.3"')]
    for f in forms:
        q = mjcf.parse(f).body_quat[0]
        assert np.allclose(mjcf.quat_to_mat(q), mjcf.quat_to_mat(q_xyz), atol=1e-12), f
    aa = mjcf.parse(base % ("degree", "", 'axisangle="0 0 1 90"')).body_quat[0]
    assert np.allclose(mjcf.quat_to_mat(aa), [[0, -1, 0], [1, 0, 0], [0, 0, 1]], atol=1e-12)


def test_reader_default_classes_inherit():
    xml = '''<mujoco><default><joint armature="0.1" axis="1 0 0"/>
      <default class="a"><joint armature="0.2"/><default class="b"><joint axis="0 1 0"/></default></default>
    </default><worldbody><body name="r"><freejoint/><inertial pos="0 0 0" mass="1" diaginertia="1 1 1"/>
      <body name="c1" childclass="b"><joint/><inertial pos="0 0 0" mass="1" diaginertia="1 1 1"/>
        <body name="c2"><joint class="a"/><inertial pos="0 0 0" mass="1" diaginertia="1 1 1"/></body>
      </body></body></worldbody></mujoco>'''
    m = mjcf.parse(xml)
    assert np.allclose(m.armature[6:], [0.2, 0.2])           # b inherits a's armature
    assert np.allclose(m.jnt_axis[1], [0, 1, 0]) and np.allclose(m.jnt_axis[2], [1, 0, 0])


# ----------------------------------------------------------------- the whole-body MPC model
WBG = np.load(os.path.join(os.path.dirname(__file__), "golden", "wb_golden.npz"))


def test_wb_dynamics_matches_the_reference_code(model):
    """quadruped_wb_dynamics (models.py:39-117) executed from the reference's
    source over the oracle's rigid-body terms (tests/golden/make_golden.py
    --wb): the contact-force solve, masking and integration agree."""
    dt = float(WBG["wb_dt"])
    for x, u, c, xn in zip(WBG["wbdyn_x"], WBG["wbdyn_u"], WBG["wbdyn_contact"], WBG["wbdyn_xnext"]):
        assert np.abs(W.wb_dynamics(model, dt, x, u, c) - xn).max() < 1e-9 * (1 + np.abs(xn).max())


def test_wb_dynamics_identities(model):
    """All feet in contact: 2 alpha dt = 1 (alpha = 25, dt = 0.02), so the
    Baumgarte term brings the feet to rest, J'v+ = 0.  No contact: a free
    semi-implicit Euler step, v+ = v + M^-1 (tau - bias) dt."""
    dt = float(WBG["wb_dt"])
    rng = np.random.default_rng(80)
    for _ in range(3):
        qpos, qvel = random_state(model, rng)
        x = np.concatenate([qpos, qvel, np.zeros(24)])
        u = rng.normal(0, 10, 12)
        x1 = W.wb_dynamics(model, dt, x, u, np.ones(4))
        J1 = W.terms(model, qpos, qvel)["J"]
        assert np.abs(J1.T @ x1[19:37]).max() < 1e-9 * (1 + np.abs(qvel).max())
        x0 = W.wb_dynamics(model, dt, x, u, np.zeros(4))
        t = W.terms(model, qpos, qvel)
        v = qvel + np.linalg.solve(t["M"], np.concatenate([np.zeros(6), u]) - t["bias"]) * dt
        assert np.allclose(x0[19:37], v, rtol=1e-12, atol=1e-12)
        assert np.allclose(x0[49:], 0.0)
        assert np.allclose(x0[37:49], t["cpos"])
        assert np.allclose(x0[7:19], qpos[7:] + v[6:] * dt)
        assert abs(np.linalg.norm(x0[3:7]) - 1) < 1e-12


def test_wb_cost_matches_the_reference_code():
    """quadruped_wb_obj (objectives.py:77-144), float32 in the reference,
    with config_aliengo's W, stage and terminal, both swing-tracking modes."""
    Wm = WBG["wb_W"].astype(np.float32)
    for x, u, r, v, t, s in zip(WBG["wbcost_x"], WBG["wbcost_u"], WBG["wbcost_ref"], WBG["wbcost_val"],
                                WBG["wbcost_terminal"], WBG["wbcost_swing"]):
        o = W.wb_stage_cost(bool(s), 12, 4, Wm, r, x, u, bool(t))
        assert abs(o - v) <= 1e-6 * max(1.0, abs(v))


def test_wb_hessian_matches_the_reference_code():
    """quadruped_wb_hessian_gn (objectives.py:146-203), float64 with
    finite-difference autodiff in the generator: the analytic restatement
    agrees to the differences' accuracy."""
    for x, u, r, s, Q, R, M in zip(WBG["wbhess_x"], WBG["wbhess_u"], WBG["wbhess_ref"], WBG["wbhess_swing"],
                                   WBG["wbhess_Q"], WBG["wbhess_R"], WBG["wbhess_M"]):
        Hx, Hu, Hxu = W.wb_hessian_gn(bool(s), 12, 4, WBG["wb_W"], r, x, u)
        assert np.abs(Hx - Q).max() <= 1e-7 * np.abs(Q).max()
        assert np.abs(Hu - R).max() <= 1e-6 * np.abs(R).max()
        assert np.abs(Hxu - M).max() <= 1e-9


def test_quat_sub_jacobian():
    rng = np.random.default_rng(90)
    for _ in range(10):
        u, v = rng.normal(size=4), rng.normal(size=4)
        u, v = u / np.linalg.norm(u), v / np.linalg.norm(v)
        h = 1e-7
        fd = np.column_stack([(W.quat_sub(u + h * e, v) - W.quat_sub(u - h * e, v)) / (2 * h) for e in np.eye(4)])
        assert np.abs(W.quat_sub_jacobian(u, v) - fd).max() < 1e-6


def test_reader_follows_includes_and_repeated_sections():
    """<include> splices the included file's sections in place; a second
    <worldbody> adds its bodies after the first (here a welded box)."""
    here = os.path.join(os.path.dirname(__file__), "golden")
    arm = mjcf.parse(os.path.join(here, "slider_arm.xml"), ["tip"], ["slider"])
    scene = mjcf.parse(os.path.join(here, "slider_scene.xml"), ["tip"], ["slider"])
    assert scene.body_names == arm.body_names + ["box"]
    assert scene.jnt_type[-1] == mjcf.JNT_NONE and scene.parent[-1] == -1
    for k in ("body_pos", "body_quat", "mass", "com", "inertia", "armature", "gravity", "contact_point_pos"):
        a, b = getattr(arm, k), getattr(scene, k)
        assert np.array_equal(a, b[:len(a)] if k in ("body_pos", "body_quat", "mass", "com", "inertia") else b), k
    with pytest.raises(ValueError):
        mjcf.parse(open(os.path.join(here, "slider_scene.xml")).read())   # text has no directory for the include


@pytest.mark.parametrize("name,kw", [("h1", dict(alpha=5.0, eps=1e-3)), ("talos", dict(forces_in_u=True))])
def test_humanoid_dynamics_match_the_reference_code(name, kw):
    """h1_wb_dynamics (models.py:119-168: alpha = 5, J'M^-1 J regularised by
    1e-3 I) and talos_wb_dynamics (models.py:170-216: the contact forces are
    controls), run from the reference's source over the oracle's rigid-body
    terms, against the oracle's restatement."""
    hm = mjcf.load_npz(os.path.join(os.path.dirname(__file__), "golden", "%s_wb.npz" % name))
    dt = float(WBG["wb_dt"])
    for x, u, c, xn in zip(WBG[name + "dyn_x"], WBG[name + "dyn_u"], WBG[name + "dyn_contact"],
                           WBG[name + "dyn_xnext"]):
        out = W.wb_dynamics(hm, dt, x, u, c, **kw)
        assert out.shape == xn.shape
        assert np.abs(out - xn).max() < 1e-9 * (1 + np.abs(xn).max())


@pytest.mark.parametrize("name", ["h1", "talos"])
def test_humanoid_models_are_consistent(name):
    """The h1 and talos fixtures pass the mechanics checks the aliengo model
    passes: M is the kinetic energy, gravity forces the potential gradient."""
    hm = mjcf.load_npz(os.path.join(os.path.dirname(__file__), "golden", "%s_wb.npz" % name))
    fx = np.load(os.path.join(os.path.dirname(__file__), "golden", "%s_wb.npz" % name))
    rng = np.random.default_rng(3)
    quat = rng.normal(0, 0.1, 4); quat[0] += 1; quat /= np.linalg.norm(quat)
    qpos = np.concatenate([fx["p0"], quat, fx["q0"] + rng.normal(0, 0.1, hm.nv - 6)])
    M = W.terms(hm, qpos, np.zeros(hm.nv))["M"]
    v = rng.normal(size=hm.nv)
    ke = W.kinetic_energy_fd(hm, qpos, v)
    assert abs(0.5 * v @ (M - np.diag(hm.armature)) @ v - ke) <= 1e-7 * ke
    bias = W.terms(hm, qpos, np.zeros(hm.nv))["bias"]
    h = 1e-6
    grad = np.array([(W.potential_energy(hm, W.integrate(hm, qpos, e, h)) -
                      W.potential_energy(hm, W.integrate(hm, qpos, e, -h))) / (2 * h) for e in np.eye(hm.nv)])
    assert np.abs(bias - grad).max() < 1e-6 * np.abs(grad).max()


@pytest.mark.parametrize("name,forces_in_u", [("h1", False), ("talos", True)])
def test_humanoid_cost_and_hessian_match_the_reference_code(name, forces_in_u):
    """h1_wb_obj / talos_wb_obj (float32 in the reference) and
    h1_wb_hessian_gn / talos_wb_hessian_gn (float64, finite-difference
    autodiff in the generator) with config_h1 / config_talos's W."""
    Wh = WBG[name + "_W"]
    nc = 4 if name == "h1" else 8
    nj = (WBG[name + "cost_ref"].shape[1] - 13 - 7 * nc)
    for i, (x, u, r, v, t) in enumerate(zip(WBG[name + "cost_x"], WBG[name + "cost_u"], WBG[name + "cost_ref"],
                                            WBG[name + "cost_val"], WBG[name + "cost_terminal"])):
        o = W.humanoid_stage_cost(forces_in_u, nj, nc, Wh.astype(np.float32), r.astype(np.float32),
                                  x.astype(np.float32), u.astype(np.float32), bool(t))
        assert abs(o - v) <= 2e-6 * max(1.0, abs(v)), i
        Hx, Hu, Hxu = W.humanoid_hessian_gn(forces_in_u, nj, nc, Wh, r, x, u)
        Q, R, M = WBG[name + "hess_Q"][i], WBG[name + "hess_R"][i], WBG[name + "hess_M"][i]
        assert np.abs(Hx - Q).max() <= 1e-7 * np.abs(Q).max(), i
        assert np.abs(Hu - R).max() <= 1e-7 * np.abs(R).max(), i
        assert np.abs(Hxu - M).max() <= 1e-7 * (1 + np.abs(M).max()), i
