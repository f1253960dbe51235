"""Whole-body rigid-body terms and torque interface, CPU oracle (test
infrastructure, not the product).  Only tests/ and bench.py's CPU baseline
import it.

Restates, in float64 and from the mechanics rather than from MuJoCo's
recursive algorithms, what the reference takes from MuJoCo XLA in
mpx/utils/mpc_utils.py:276-313 (whole_body_interface):

  * forward kinematics with 4x4 homogeneous transforms (body frame in the
    parent, then the joint: a hinge rotates about its axis through its anchor,
    a slide translates along it, a free joint sets position and orientation);
  * for every body b its centre-of-mass Jacobian Jv_b and angular Jacobian
    Jw_b (geometric columns: hinge a x (p - anchor) / a, slide a / 0, free
    translation e_k / 0, free rotation R e_k x (p - x_root) / R e_k: qvel's
    angular part is in the free body's frame);
  * M = sum_b m_b Jv_b' Jv_b + Jw_b' I_b Jw_b + diag(armature)      (mjx qM)
  * bias = sum_b Jv_b' m_b (dJv_b qdot - g) + Jw_b' (I_b dJw_b qdot + w_b x I_b w_b)
    with dJ qdot the analytic time derivative of the columns at qacc = 0
    (axes fixed in a body turn with that body's angular velocity; anchors
    move with their body)                                            (mjx qfrc_bias)
  * contact points: geom positions, translational Jacobians of the point
    attached to the named body                                       (mjx.jac)
  * the interface formula of mpc_utils.py:300-311 with numpy's pinv, as the
    reference uses jnp.linalg.pinv.

MuJoCo cannot run here, so parity is pinned (tests/test_oracle_wholebody.py)
by the reference's own numbers for this model -- the foot positions
config_srbd.py:38-43 lists for aliengo at q0 -- and by identities of the
mechanics: M against the kinetic energy of finite-differenced body motion,
dJ qdot against the second difference of the point trajectory at qacc = 0,
gravity forces against the potential energy gradient, and the power balance
qdot' bias(g = 0) = 1/2 qdot' (dM/dt) qdot.
"""
import numpy as np

FREE, HINGE, SLIDE = 1, 2, 3
_NDOF = {0: 0, 1: 6, 2: 1, 3: 1}


def _qmat(q):
    w, x, y, z = np.asarray(q, dtype=np.float64) / np.linalg.norm(q)
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                     [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])


def _rot_axis(a, th):
    """Rodrigues rotation about unit axis a by th."""
    a = np.asarray(a, dtype=np.float64)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    return np.eye(3) + np.sin(th) * K + (1 - np.cos(th)) * (K @ K)


def _T(R, p):
    T = np.eye(4)
    T[:3, :3] = R
    T[:3, 3] = p
    return T


def kinematics(model, qpos):
    """World transforms [nb,4,4] of the body frames."""
    nb = model.nbody
    qadr = model.qpos_adr
    T = np.zeros((nb, 4, 4))
    for b in range(nb):
        p = model.parent[b]
        Tp = np.eye(4) if p < 0 else T[p]
        jt = int(model.jnt_type[b])
        if jt == FREE:
            a = qadr[b]
            T[b] = _T(_qmat(qpos[a + 3:a + 7]), qpos[a:a + 3])
            continue
        Tb = Tp @ _T(_qmat(model.body_quat[b]), model.body_pos[b])
        if jt == HINGE:
            th = qpos[qadr[b]]
            # rotate about the joint axis through the joint position (body frame)
            Tj = _T(np.eye(3), model.jnt_pos[b]) @ _T(_rot_axis(model.jnt_axis[b], th), np.zeros(3)) @ \
                _T(np.eye(3), -model.jnt_pos[b])
            Tb = Tb @ Tj
        elif jt == SLIDE:
            Tb = Tb @ _T(np.eye(3), model.jnt_axis[b] * qpos[qadr[b]])
        T[b] = Tb
    return T


def _chain(model, b):
    out = []
    while b >= 0:
        out.append(b)
        b = int(model.parent[b])
    return out


def _columns(model, T, b, point):
    """Geometric Jacobian columns of a point attached to body b:
    list of (dof, angular axis, linear column, kind, anchor, owner body)."""
    dadr = model.dof_adr
    cols = []
    for a in _chain(model, b):
        jt = int(model.jnt_type[a])
        R, x = T[a][:3, :3], T[a][:3, 3]
        d = dadr[a]
        if jt == FREE:
            for k in range(3):
                e = np.zeros(3); e[k] = 1.0
                cols.append((d + k, np.zeros(3), e, "ft", x, a))
            for k in range(3):
                ax = R[:, k]
                cols.append((d + 3 + k, ax, np.cross(ax, point - x), "rot", x, a))
        elif jt == HINGE:
            ax = R @ model.jnt_axis[a]
            anchor = x + R @ model.jnt_pos[a]
            cols.append((d, ax, np.cross(ax, point - anchor), "rot", anchor, a))
        elif jt == SLIDE:
            ax = R @ model.jnt_axis[a]
            cols.append((d, np.zeros(3), ax, "slide", x, a))
    return cols


def point_jacobian(model, T, b, point):
    """(Jp [3,nv], Jr [3,nv]) of a world point attached to body b."""
    nv = model.nv
    Jp, Jr = np.zeros((3, nv)), np.zeros((3, nv))
    for d, w, v, _, _, _ in _columns(model, T, b, point):
        Jp[:, d] = v
        Jr[:, d] = w
    return Jp, Jr


def _body_velocity(model, T, qvel):
    """Angular velocity and origin-point linear velocity of every body."""
    nb = model.nbody
    W, Vx = np.zeros((nb, 3)), np.zeros((nb, 3))
    for b in range(nb):
        Jp, Jr = point_jacobian(model, T, b, T[b][:3, 3])
        W[b], Vx[b] = Jr @ qvel, Jp @ qvel
    return W, Vx


def _point_velocity(model, T, qvel, b, p):
    Jp, _ = point_jacobian(model, T, b, p)
    return Jp @ qvel


def _dJ_qdot(model, T, qvel, W, b, p):
    """(dJp qdot, dJr qdot) of a point p attached to body b at qacc = 0."""
    vp = _point_velocity(model, T, qvel, b, p)
    ap, aw = np.zeros(3), np.zeros(3)
    for d, w, v, kind, anchor, owner in _columns(model, T, b, p):
        qd = qvel[d]
        if kind == "ft":
            continue
        if kind == "slide":
            ap += np.cross(W[owner], v) * qd
            continue
        wdot = np.cross(W[owner], w)               # the axis turns with its body
        van = _point_velocity(model, T, qvel, owner, anchor)
        ap += (np.cross(wdot, p - anchor) + np.cross(w, vp - van)) * qd
        aw += wdot * qd
    return ap, aw


def terms(model, qpos, qvel):
    """dict M [nv,nv], bias [nv], cpos [3C], J [nv,3C], cvel [3C] (float64)."""
    qpos = np.asarray(qpos, dtype=np.float64)
    qvel = np.asarray(qvel, dtype=np.float64)
    nb, nv = model.nbody, model.nv
    T = kinematics(model, qpos)
    W, _ = _body_velocity(model, T, qvel)
    M = np.diag(np.asarray(model.armature, dtype=np.float64)).copy()
    bias = np.zeros(nv)
    g = np.asarray(model.gravity, dtype=np.float64)
    for b in range(nb):
        R, x = T[b][:3, :3], T[b][:3, 3]
        c = x + R @ model.com[b]
        Iw = R @ model.inertia[b] @ R.T
        m = float(model.mass[b])
        Jv, Jw = point_jacobian(model, T, b, c)
        M += m * Jv.T @ Jv + Jw.T @ Iw @ Jw
        av, aw = _dJ_qdot(model, T, qvel, W, b, c)
        w = Jw @ qvel
        bias += Jv.T @ (m * (av - g)) + Jw.T @ (Iw @ aw + np.cross(w, Iw @ w))
    nc = 0 if model.contact_point_body is None else len(model.contact_point_body)
    cpos = np.zeros(3 * nc)
    J = np.zeros((nv, 3 * nc))
    for ci in range(nc):
        gb = int(model.contact_point_body[ci])
        p = T[gb][:3, :3] @ model.contact_point_pos[ci] + T[gb][:3, 3]
        cpos[3 * ci:3 * ci + 3] = p
        Jp, _ = point_jacobian(model, T, int(model.contact_jac_body[ci]), p)
        J[:, 3 * ci:3 * ci + 3] = Jp.T
    return dict(M=M, bias=bias, cpos=cpos, J=J, cvel=J.T @ qvel, T=T)


def interface(model, Kp, Kd, qpos, qvel, grf, foot_ref, foot_ref_dot, contact):
    """mpx/utils/mpc_utils.py:276-313 for one environment -> (tau, J)."""
    t = terms(model, qpos, qvel)
    M, D, J = t["M"], t["bias"], t["J"]
    current_leg, current_leg_dot = t["cpos"], J.T @ np.asarray(qvel, dtype=np.float64)
    a = np.asarray(Kp) @ (np.asarray(foot_ref) - current_leg) + np.asarray(Kd) @ (np.asarray(foot_ref_dot) -
                                                                                  current_leg_dot)
    tau_fb_lin = D[6:] + (M @ np.linalg.pinv(J.T) @ a)[6:]
    tau_mpc = -(J @ np.asarray(grf, dtype=np.float64))[6:]
    mask = np.repeat(np.asarray(contact, dtype=np.float64), 3)
    return tau_mpc * mask + (1 - mask) * tau_fb_lin, J


# ----------------------------------------------------------------- identities used to pin the oracle
def integrate(model, qpos, qvel, h):
    """qpos after time h at constant qvel (MuJoCo's qacc = 0 motion): free
    position + h v, orientation q * exp(h w_body / 2), joints + h qdot."""
    q = np.array(qpos, dtype=np.float64)
    qadr, dadr = model.qpos_adr, model.dof_adr
    for b in range(model.nbody):
        jt = int(model.jnt_type[b])
        a, d = qadr[b], dadr[b]
        if jt == FREE:
            q[a:a + 3] += h * qvel[d:d + 3]
            w = np.asarray(qvel[d + 3:d + 6], dtype=np.float64)
            th = np.linalg.norm(w) * h
            dq = np.array([1.0, 0, 0, 0]) if th == 0 else np.concatenate([[np.cos(th / 2)],
                                                                           np.sin(th / 2) * w / np.linalg.norm(w)])
            w1, x1, y1, z1 = q[a + 3:a + 7]
            w2, x2, y2, z2 = dq
            q[a + 3:a + 7] = [w1 * w2 - x1 * x2 - y1 * y2 - z1 * z2, w1 * x2 + x1 * w2 + y1 * z2 - z1 * y2,
                              w1 * y2 - x1 * z2 + y1 * w2 + z1 * x2, w1 * z2 + x1 * y2 - y1 * x2 + z1 * w2]
        elif jt in (HINGE, SLIDE):
            q[a] += h * qvel[d]
    return q


def kinetic_energy_fd(model, qpos, qvel, h=1e-5):
    """Kinetic energy from central differences of the body motion."""
    Tm, Tp = kinematics(model, integrate(model, qpos, qvel, -h)), kinematics(model, integrate(model, qpos, qvel, h))
    T0 = kinematics(model, qpos)
    E = 0.0
    for b in range(model.nbody):
        cm = Tm[b][:3, :3] @ model.com[b] + Tm[b][:3, 3]
        cp = Tp[b][:3, :3] @ model.com[b] + Tp[b][:3, 3]
        v = (cp - cm) / (2 * h)
        dR = (Tp[b][:3, :3] - Tm[b][:3, :3]) / (2 * h)
        R = T0[b][:3, :3]
        Wx = dR @ R.T
        w = np.array([Wx[2, 1] - Wx[1, 2], Wx[0, 2] - Wx[2, 0], Wx[1, 0] - Wx[0, 1]]) / 2
        Iw = R @ model.inertia[b] @ R.T
        E += 0.5 * model.mass[b] * v @ v + 0.5 * w @ Iw @ w
    return E


def potential_energy(model, qpos):
    T = kinematics(model, qpos)
    g = np.asarray(model.gravity, dtype=np.float64)
    return -sum(model.mass[b] * g @ (T[b][:3, :3] @ model.com[b] + T[b][:3, 3]) for b in range(model.nbody))


# ----------------------------------------------------------------- the whole-body MPC model
# quadruped_wb_dynamics (mpx/utils/models.py:39-117) and its cost and
# Gauss-Newton Hessian (mpx/utils/objectives.py:77-203), the model the
# reference's whole-body configurations (config_aliengo.py:66-68,
# config_go2.py:67-69) hand to its solver.  State x = [p (3), quat (4),
# q (nj), v (3), omega (3, body frame), dq (nj), foot positions (3C),
# grf (3C)], control u = joint torques (nj).


def _qmul(a, b):
    w1, x1, y1, z1 = a
    w2, x2, y2, z2 = b
    return np.array([w1 * w2 - x1 * x2 - y1 * y2 - z1 * z2, w1 * x2 + x1 * w2 + y1 * z2 - z1 * y2,
                     w1 * y2 - x1 * z2 + y1 * w2 + z1 * x2, w1 * z2 + x1 * y2 - y1 * x2 + z1 * w2])


def quat_integrate(q, w, dt):
    """q * exp(w dt / 2) renormalised, w in the body frame (mjx math)."""
    w = np.asarray(w, dtype=np.float64)
    n = np.linalg.norm(w)
    axis = w / n if n > 0 else np.zeros(3)
    half = 0.5 * n * dt
    out = _qmul(np.asarray(q, dtype=np.float64), np.concatenate([[np.cos(half)], np.sin(half) * axis]))
    return out / np.linalg.norm(out)


def quat_sub(u, v):
    """The rotation vector of conj(v) * u, angle in (-pi, pi] (mjx math)."""
    q = _qmul(np.asarray(v, dtype=np.float64) * [1, -1, -1, -1], np.asarray(u, dtype=np.float64))
    n = np.linalg.norm(q[1:])
    axis = q[1:] / n if n > 0 else np.zeros(3)
    ang = 2 * np.arctan2(n, q[0])
    if ang > np.pi:
        ang -= 2 * np.pi
    return axis * ang


def quat_sub_jacobian(u, v):
    """d quat_sub(u, v) / du (3 x 4), from the chain rule through conj(v) * u
    and the logarithm (theta = 2 atan2(|w|, s), result theta w / |w|); at a
    zero vector part w the limit (2 / s) I of d/dw (d/ds = 0)."""
    vc = np.asarray(v, dtype=np.float64) * [1, -1, -1, -1]
    a0, a1, a2, a3 = vc
    L = np.array([[a0, -a1, -a2, -a3], [a1, a0, -a3, a2], [a2, a3, a0, -a1], [a3, -a2, a1, a0]])
    q = L @ np.asarray(u, dtype=np.float64)
    s, w = q[0], q[1:]
    n = np.linalg.norm(w)
    th = 2 * np.arctan2(n, s)
    if th > np.pi:
        th -= 2 * np.pi
    if n == 0.0:  # the limit of the smooth map at a zero vector part
        return np.column_stack([np.zeros(3), np.eye(3) * (2.0 / s)]) @ L
    a = w / n
    r2 = s * s + n * n
    d_ds = a * (-2 * n / r2)
    d_dw = np.outer(a, a) * (2 * s / r2) + th * (np.eye(3) - np.outer(a, a)) / n
    return np.column_stack([d_ds, d_dw]) @ L


def wb_dynamics(model, dt, x, u, contact, alpha=25.0, eps=0.0, forces_in_u=False):
    """One step of the reference's whole-body models, with
    nj = nv - 6 joints and C contact points:
      quadruped_wb_dynamics (models.py:39-117): alpha = 25, eps = 0;
      h1_wb_dynamics (models.py:119-168): alpha = 5, eps = 1e-3;
      talos_wb_dynamics (models.py:170-216): forces_in_u (the forces are the
        controls u[nj:]; no force solve; the next state carries no forces).
    Otherwise the contact forces hold the feet, stabilised at the velocity
    level (Baumgarte, -2 alpha J'v), from (J'M^-1 J + eps I) f = rhs, masked
    by contact; then a semi-implicit Euler step.  The new state carries the
    contact points at the current configuration (and the forces)."""
    x = np.asarray(x, dtype=np.float64)
    u = np.asarray(u, dtype=np.float64)
    nv = model.nv
    nq, nj = nv + 1, nv - 6
    qpos, qvel = x[:nq], x[nq:nq + nv]
    t = terms(model, qpos, qvel)
    M, D, J, feet = t["M"], t["bias"], t["J"], t["cpos"]
    tau = np.concatenate([np.zeros(6), u[:nj]])
    mask = np.repeat(np.asarray(contact, dtype=np.float64), 3)
    solve = lambda b: np.linalg.solve(M, b)
    if forces_in_u:
        grf = u[nj:] * mask
    else:
        A = J.T @ solve(J) + eps * np.eye(J.shape[1])
        rhs = -J.T @ solve(tau - D) - 2 * alpha * (J.T @ qvel)
        grf = np.linalg.solve(A, rhs) * mask
    v = qvel + solve(tau - D + J @ grf) * dt
    p = qpos[:3] + v[:3] * dt
    quat = quat_integrate(qpos[3:7], v[3:6], dt)
    q = qpos[7:] + v[6:] * dt
    return np.concatenate([p, quat, q, v, feet] + ([] if forces_in_u else [grf]))


def penalty(c, alpha=0.1, sigma=5.0):
    """objectives.py:7-13: relaxed log barrier, clipped to [0, 1e8]."""
    c = np.asarray(c, dtype=np.float64)
    logb = -alpha * np.log(np.clip(c, 1e-10, 1e6))
    quad = alpha / 2 * (np.square((c - 2 * sigma) / sigma) - 1)
    return np.clip(np.where(c > sigma, logb, quad + logb), 0, 1e8)


def penalty_dd(c, alpha=0.1, sigma=5.0):
    """Second derivative of penalty() where it is smooth (0 where clipped)."""
    c = np.asarray(c, dtype=np.float64)
    logdd = np.where((c > 1e-10) & (c < 1e6), alpha / np.square(c), 0.0)
    dd = np.where(c > sigma, logdd, alpha / sigma ** 2 + logdd)
    raw = np.where(c > sigma, -alpha * np.log(np.clip(c, 1e-10, 1e6)),
                   alpha / 2 * (np.square((c - 2 * sigma) / sigma) - 1) - alpha * np.log(np.clip(c, 1e-10, 1e6)))
    return np.where((raw > 0) & (raw < 1e8), dd, 0.0)


def _wb_split(nj, nc, x, u):
    o = {}
    o["p"], o["quat"], o["q"] = x[:3], x[3:7], x[7:7 + nj]
    o["dp"], o["omega"], o["dq"] = x[7 + nj:10 + nj], x[10 + nj:13 + nj], x[13 + nj:13 + 2 * nj]
    o["p_leg"], o["grf"] = x[13 + 2 * nj:13 + 2 * nj + 3 * nc], x[13 + 2 * nj + 3 * nc:]
    o["tau"] = u[:nj]
    return o


def _wb_ref(nj, nc, r):
    return dict(p=r[:3], quat=r[3:7], q=r[7:7 + nj], dp=r[7 + nj:10 + nj], omega=r[10 + nj:13 + nj],
                p_leg=r[13 + nj:13 + nj + 3 * nc], contact=r[13 + nj + 3 * nc:13 + nj + 4 * nc],
                grf=r[13 + nj + 4 * nc:13 + nj + 7 * nc])


def _limits(nj, v, bound):
    """kron(I, [-1, 1])' v + bound + 1e-2: [bound - v_0, bound + v_0, ...]."""
    out = np.empty(2 * nj)
    out[0::2], out[1::2] = -v, v
    return out + bound + 1e-2


def wb_stage_cost(swing_tracking, nj, nc, W, ref_row, x, u, terminal):
    """objectives.py:77-144 (one stage; terminal = the t == N branch)."""
    W = np.asarray(W, dtype=np.float64)
    s = _wb_split(nj, nc, np.asarray(x, dtype=np.float64), np.asarray(u, dtype=np.float64))
    r = _wb_ref(nj, nc, np.asarray(ref_row, dtype=np.float64))
    quad = lambda e, a, b: e @ W[a:b, a:b] @ e
    eq = quat_sub(s["quat"], r["quat"])
    cost = quad(s["p"] - r["p"], 0, 3) + quad(eq, 3, 6) + quad(s["q"] - r["q"], 6, 6 + nj) + \
        quad(s["dp"] - r["dp"], 6 + nj, 9 + nj) + quad(s["omega"] - r["omega"], 9 + nj, 12 + nj) + \
        quad(s["dq"], 12 + nj, 12 + 2 * nj)
    if terminal:
        return 0.5 * cost
    cmap = np.ones(3 * nc) if swing_tracking else np.repeat(r["contact"], 3)
    a = 12 + 2 * nj
    cost += quad(cmap * (s["p_leg"] - r["p_leg"]), a, a + 3 * nc)
    a += 3 * nc
    cost += quad(s["tau"], a, a + nj)
    a += nj
    cost += quad(s["grf"] - r["grf"], a, a + 3 * nc)
    g = s["grf"]
    cone = penalty(0.5 * g[2::3] - np.sqrt(np.square(g[1::3]) + np.square(g[0::3]) + 1e-2))
    cost += np.sum(penalty(_limits(nj, s["tau"], 44.0), 1, 1)) + np.sum(cone * r["contact"]) + \
        np.sum(penalty(_limits(nj, s["dq"], 10.0), 1, 1))
    return 0.5 * cost


def wb_hessian_gn(swing_tracking, nj, nc, W, ref_row, x, u):
    """objectives.py:146-203: (H_xx, H_uu, H_xu) = J_x'W J_x + barrier terms,
    J_u'W J_u + torque barrier, J_x'W J_u, with the residual's Jacobians
    formed analytically."""
    W = np.asarray(W, dtype=np.float64)
    x = np.asarray(x, dtype=np.float64)
    u = np.asarray(u, dtype=np.float64)
    r = _wb_ref(nj, nc, np.asarray(ref_row, dtype=np.float64))
    n, m, R = x.size, u.size, W.shape[0]
    Jx, Ju = np.zeros((R, n)), np.zeros((R, m))
    Jx[0:3, 0:3] = np.eye(3)
    Jx[3:6, 3:7] = quat_sub_jacobian(x[3:7], r["quat"])
    Jx[6:6 + nj, 7:7 + nj] = np.eye(nj)
    Jx[6 + nj:12 + nj, 7 + nj:13 + nj] = np.eye(6)
    Jx[12 + nj:12 + 2 * nj, 13 + nj:13 + 2 * nj] = np.eye(nj)
    cmap = np.ones(3 * nc) if swing_tracking else np.repeat(r["contact"], 3)
    a = 12 + 2 * nj
    Jx[a:a + 3 * nc, 13 + 2 * nj:13 + 2 * nj + 3 * nc] = np.diag(cmap)
    Ju[a + 3 * nc:a + 3 * nc + nj, :nj] = np.eye(nj)
    b = a + 3 * nc + nj
    Jx[b:b + 3 * nc, 13 + 2 * nj + 3 * nc:] = np.eye(3 * nc)
    Hx, Hu, Hxu = Jx.T @ W @ Jx, Ju.T @ W @ Ju, Jx.T @ W @ Ju
    # friction cone (with 1e-1 under the root here, objectives.py:184-188)
    g0 = 13 + 2 * nj + 3 * nc
    g = x[g0:]
    sq = np.sqrt(np.square(g[1::3]) + np.square(g[0::3]) + 1e-1)
    cone = 0.5 * g[2::3] - sq
    Jf = np.zeros((nc, n))
    for i in range(nc):
        Jf[i, g0 + 3 * i] = -g[3 * i] / sq[i]
        Jf[i, g0 + 3 * i + 1] = -g[3 * i + 1] / sq[i]
        Jf[i, g0 + 3 * i + 2] = 0.5
    Hx += Jf.T @ np.diag(np.clip(penalty_dd(cone), -1e6, 1e6) * r["contact"]) @ Jf
    K = np.zeros((2 * nj, nj))
    K[0::2, :], K[1::2, :] = -np.eye(nj), np.eye(nj)
    Hu += K.T @ np.diag(np.clip(penalty_dd(_limits(nj, u[:nj], 44.0), 1, 1), -1e6, 1e6)) @ K
    Js = np.zeros((2 * nj, n))
    Js[:, 13 + nj:13 + 2 * nj] = K
    Hx += Js.T @ np.diag(np.clip(penalty_dd(_limits(nj, x[13 + nj:13 + 2 * nj], 10.0)), -1e6, 1e6)) @ Js
    return Hx, Hu, Hxu


def humanoid_residual_jacobians(forces_in_u, nj, nc, ref_row, x, u):
    """Residual r = [p - p_ref, quat_sub(quat, quat_ref), q - q_ref,
    v - v_ref, w - w_ref, dq, p_leg - p_leg_ref, tau, grf - grf_ref] of
    h1_wb_obj / talos_wb_obj (objectives.py:204-250, 325-376), with its
    Jacobians.  The forces are state entries (h1) or controls u[nj:]
    (talos, forces_in_u)."""
    x = np.asarray(x, dtype=np.float64)
    u = np.asarray(u, dtype=np.float64)
    rr = _wb_ref(nj, nc, np.asarray(ref_row, dtype=np.float64))
    grf = u[nj:] if forces_in_u else x[13 + 2 * nj + 3 * nc:]
    r = np.concatenate([x[:3] - rr["p"], quat_sub(x[3:7], rr["quat"]), x[7:7 + nj] - rr["q"],
                        x[7 + nj:10 + nj] - rr["dp"], x[10 + nj:13 + nj] - rr["omega"], x[13 + nj:13 + 2 * nj],
                        x[13 + 2 * nj:13 + 2 * nj + 3 * nc] - rr["p_leg"], u[:nj], grf - rr["grf"]])
    R = r.size
    Jx, Ju = np.zeros((R, x.size)), np.zeros((R, u.size))
    Jx[0:3, 0:3] = np.eye(3)
    Jx[3:6, 3:7] = quat_sub_jacobian(x[3:7], rr["quat"])
    Jx[6:12 + 2 * nj, 7:13 + 2 * nj] = np.eye(6 + 2 * nj)
    a = 12 + 2 * nj
    Jx[a:a + 3 * nc, 13 + 2 * nj:13 + 2 * nj + 3 * nc] = np.eye(3 * nc)
    Ju[a + 3 * nc:a + 3 * nc + nj, :nj] = np.eye(nj)
    b = a + 3 * nc + nj
    if forces_in_u:
        Ju[b:b + 3 * nc, nj:] = np.eye(3 * nc)
    else:
        Jx[b:b + 3 * nc, 13 + 2 * nj + 3 * nc:] = np.eye(3 * nc)
    return r, Jx, Ju


def humanoid_stage_cost(forces_in_u, nj, nc, W, ref_row, x, u, terminal):
    """h1_wb_obj / talos_wb_obj: 1/2 r'W r (stage), or its first six blocks
    (terminal, the t == N branch).  Their barriers are commented out in the
    reference; the friction cone is computed but unused."""
    W = np.asarray(W, dtype=np.float64)
    r, _, _ = humanoid_residual_jacobians(forces_in_u, nj, nc, ref_row, x, u)
    if terminal:
        k = 12 + 2 * nj
        return 0.5 * r[:k] @ W[:k, :k] @ r[:k]
    return 0.5 * r @ W @ r


def humanoid_hessian_gn(forces_in_u, nj, nc, W, ref_row, x, u):
    """h1_wb_hessian_gn / talos_wb_hessian_gn (objectives.py:252-323,
    378-450): J_x'W J_x, J_u'W J_u, J_x'W J_u.  The friction-cone term they
    compute is not added to what they return."""
    W = np.asarray(W, dtype=np.float64)
    _, Jx, Ju = humanoid_residual_jacobians(forces_in_u, nj, nc, ref_row, x, u)
    return Jx.T @ W @ Jx, Ju.T @ W @ Ju, Jx.T @ W @ Ju
