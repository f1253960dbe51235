"""Configuration objects with the attribute schema of the reference's config
modules (plain attributes read by the wrappers).

srbd_quadruped(): the values of mpx/config/config_srbd.py:19-90 (the SRBD
quadruped the reference's SRBD wrapper is built for).  Any object with these
attributes -- including the reference's own config module -- can be passed to
the wrappers instead.
"""
import types

import numpy as np


def srbd_quadruped():
    c = types.SimpleNamespace()
    c.contact_frame = ["FL", "FR", "RL", "RR"]
    c.body_name = ["FL_calf", "FR_calf", "RL_calf", "RR_calf"]
    c.dt = 0.02
    c.N = 25
    c.mpc_frequency = 50
    c.whole_body_frequency = 200
    c.timer_t = np.array([0.5, 0.0, 0.0, 0.5], dtype=np.float32)
    c.duty_factor = 0.65
    c.step_freq = 1.35
    c.step_height = 0.065
    c.robot_height = 0.35
    c.clearence_speed = 0.4
    c.use_terrain_estimator = False
    c.p0 = np.array([0.0, 0.0, 0.33], dtype=np.float32)
    c.quat0 = np.array([1.0, 0.0, 0.0, 0.0], dtype=np.float32)
    c.q0 = np.array([0.2, 0.8, -1.8, -0.2, 0.8, -1.8, 0.2, 0.8, -1.8, -0.2, 0.8, -1.8], dtype=np.float32)
    c.p_legs0 = np.array([0.27092872, 0.193, 0.0, 0.27092872, -0.193, 0.0,
                          -0.20887128, 0.193, 0.0, -0.20887128, -0.193, 0.0], dtype=np.float32)
    c.n_joints = 12
    c.n_contact = 4
    c.n = 13
    c.m = 12
    c.mass = 24.637
    c.inertia = np.array([[0.2310941359705289, -0.0014987128245817424, -0.021400468992761768],
                          [-0.0014987128245817424, 1.4485084687476608, 0.0004641447134275615],
                          [-0.021400468992761768, 0.0004641447134275615, 1.503217877350808]])
    c.grf_ref = np.zeros(12, dtype=np.float32)
    c.u_ref = c.grf_ref.copy()
    c.Kp = np.diag(np.tile([100.0, 100.0, 100.0], 4))
    c.Kd = np.diag(np.tile([5.0, 5.0, 5.0], 4))
    c.W = np.diag(np.concatenate([[0.0, 0.0, 1e4], [1e3, 1e3, 0.0], [1e3] * 3, [1e1] * 3, [1e-2] * 12]))
    c.initial_height = c.robot_height
    return c


def aliengo_wb():
    """The values of mpx/config/config_aliengo.py:11-76 (the whole-body
    quadruped that mpc_wrapper.py's wrappers are built for): 61 states
    [qpos (19), qvel (18), contact points (12), contact forces (12)], 12 joint
    torques, N = 25, dt = 0.02, the diagonal of its block-diagonal W.  The
    MJCF model itself is read separately (mjcf.parse of data/aliengo/aliengo.xml,
    or its parsed copy tests/golden/aliengo_wb.npz)."""
    c = types.SimpleNamespace()
    c.contact_frame = ["FL", "FR", "RL", "RR"]
    c.body_name = ["FL_calf", "FR_calf", "RL_calf", "RR_calf"]
    c.dt = 0.02
    c.N = 25
    c.mpc_frequency = 50
    c.timer_t = np.array([0.5, 0.0, 0.0, 0.5], dtype=np.float32)
    c.duty_factor = 0.65
    c.step_freq = 1.35
    c.step_height = 0.14
    c.initial_height = 0.1
    c.robot_height = 0.36
    c.p0 = np.array([0.0, 0.0, c.robot_height], dtype=np.float32)
    c.quat0 = np.array([1.0, 0.0, 0.0, 0.0], dtype=np.float32)
    c.q0 = np.array([0.2, 0.8, -1.8, -0.2, 0.8, -1.8, 0.2, 0.8, -1.8, -0.2, 0.8, -1.8], dtype=np.float32)
    c.p_legs0 = np.array([0.27092872, 0.193, 0.0, 0.27092872, -0.193, 0.0,
                          -0.20887128, 0.193, 0.0, -0.20887128, -0.193, 0.0], dtype=np.float32)
    c.n_joints = 12
    c.n_contact = 4
    c.n = 13 + 2 * c.n_joints + 6 * c.n_contact
    c.m = c.n_joints
    c.grf_as_state = True
    c.u_ref = np.zeros(c.m, dtype=np.float32)
    c.W_diag = np.concatenate([[0.0, 0.0, 1e4], [1000.0, 1000.0, 0.0], [1e-1] * 12, [5e3] * 3, [1e2] * 3,
                               [1e-1] * 12, np.tile([1e4, 1e4, 1e5], 4), [1e-1] * 12, [1e-2] * 12]).astype(np.float32)
    c.W = np.diag(c.W_diag.astype(np.float64))
    c.use_terrain_estimation = True
    c.max_torque = 35.0
    c.min_torque = -35.0
    c.swing_tracking = True
    return c
