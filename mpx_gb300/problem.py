"""Model descriptions, solver options and synthetic SRBD workloads.

The model set mirrors what the reference's SRBD path compiles in through
`functools.partial` (mpx/utils/mpc_wrapper_srbd.py:61-68): a dynamics model,
a tracking cost with a relaxed friction-cone barrier and a Gauss-Newton
Hessian.  Across the C ABI the model is selected by id:

  MODEL_SRBD_QUAT13     the reference's quadruped SRBD, x = [p, quat(wxyz), v, omega]
                        (mpx/utils/models.py:6-37, mpx/config/config_srbd.py:60-61)
  MODEL_SRBD_RPY12      the same body with roll-pitch-yaw orientation (n = 12),
                        Euler-rate map of mpx/utils/rotation.py:26-35
  MODEL_BIPED_WRENCH12  SRBD biped, two rectangular feet with 6-D contact wrenches
  MODEL_GENERIC_LQ      time-varying LQ data supplied per stage

Array layouts (all float32, row-major, padded to a horizon N_max):
  x0 [B, n], X [B, N_max+1, n], U [B, N_max, m], V [B, N_max+1, n],
  reference [B, N_max+1, ref_cols], parameter [B, N_max+1, par_cols],
  W [B, 24, 24], horizon [B] (int32, per-instance N <= N_max).
"""
import dataclasses

import numpy as np

MODEL_SRBD_QUAT13 = 1
MODEL_SRBD_RPY12 = 2
MODEL_BIPED_WRENCH12 = 3
MODEL_GENERIC_LQ = 4

NW = 24  # residual dimension of the SRBD tracking cost (12 state + 12 control)

_REF_COLS = {MODEL_SRBD_QUAT13: 17, MODEL_SRBD_RPY12: 16, MODEL_BIPED_WRENCH12: 14, MODEL_GENERIC_LQ: 0}
_PAR_COLS = {MODEL_SRBD_QUAT13: 16, MODEL_SRBD_RPY12: 16, MODEL_BIPED_WRENCH12: 8, MODEL_GENERIC_LQ: 0}
_DIMS = {MODEL_SRBD_QUAT13: (13, 12), MODEL_SRBD_RPY12: (12, 12), MODEL_BIPED_WRENCH12: (12, 12)}


def ref_cols(model):
    return _REF_COLS[model]


def par_cols(model):
    return _PAR_COLS[model]


@dataclasses.dataclass
class ModelDesc:
    """Physical description of one compiled-in model."""
    model: int
    n: int
    m: int
    dt: float = 0.02
    mass: float = 1.0
    inertia: np.ndarray = dataclasses.field(default_factory=lambda: np.eye(3))
    n_contact: int = 4
    gravity: float = 9.81
    mu: float = 0.7                 # friction coefficient (objectives.py:28 uses 0.7)
    barrier_alpha: float = 0.1      # objectives.py:7
    barrier_sigma: float = 5.0      # objectives.py:7
    foot_length: float = 0.0        # biped plate extent along x
    foot_width: float = 0.0         # biped plate extent along y
    barrier_kind: int = 0           # 0: penalty() of objectives.py:7-13; 1: C2 relaxed log barrier
    barrier_masked: int = 0         # 1: barrier cost multiplied by the stage contact flag
    barrier_hess_scale: float = 1.0 # factor on the barrier's Gauss-Newton curvature
    cone_eps2: float = 1e-2         # friction cone sqrt(fx^2 + fy^2 + cone_eps2) (objectives.py:29: 1e-2)

    @property
    def inertia_inv(self):
        # host-side inversion, as mpx/utils/mpc_wrapper_srbd.py:66 does
        return np.linalg.inv(np.asarray(self.inertia, dtype=np.float64))

    @property
    def ref_cols(self):
        return ref_cols(self.model)

    @property
    def par_cols(self):
        return par_cols(self.model)


@dataclasses.dataclass
class SolverOptions:
    """Settings of the primal-dual SQP.  The reference's solver module is not
    present in its tree, so these constants are this implementation's own
    (documented defaults; parity of these choices is unpinned)."""
    sqp_iters: int = 5          # SQP iterations per solve call
    ls_max_trials: int = 8      # backtracking trials of the merit line search
    ls_beta: float = 0.5        # step shrink factor
    ls_eta: float = 1e-4        # Armijo constant
    reg: float = 1e-6           # added to the diagonal of Q_uu
    rho0: float = 1.0           # initial augmented-Lagrangian penalty
    ls_skip_tol: float = 1e-7   # |predicted merit change| below this x (1+|merit|): take the full step
    compute_kkt: bool = True    # evaluate the KKT residual of the result on the device
    team_warps: int = 0         # 4 or 8: horizons >= team_min_horizon are solved time-parallel by 4 or 8 warps each
    team_min_horizon: int = 64
    team_exact_last: bool = False  # the team kernel's last KKT step as one sequential sweep (accurate duals)


# ----------------------------------------------------------------- models
def quadruped_quat13(config=None, mu=0.7):
    """The reference's SRBD quadruped.  `config` is a module or object with the
    attributes of mpx/config/config_srbd.py (dt, mass, inertia); defaults are
    that file's values."""
    if config is None:
        dt, mass = 0.02, 24.637
        inertia = np.array([[0.2310941359705289, -0.0014987128245817424, -0.021400468992761768],
                            [-0.0014987128245817424, 1.4485084687476608, 0.0004641447134275615],
                            [-0.021400468992761768, 0.0004641447134275615, 1.503217877350808]])
    else:
        dt, mass = float(config.dt), float(config.mass)
        inertia = np.asarray(config.inertia, dtype=np.float64)
    return ModelDesc(MODEL_SRBD_QUAT13, 13, 12, dt=dt, mass=mass, inertia=inertia, n_contact=4, mu=mu)


def quadruped_rpy12(mu=0.6):
    """Quadruped SRBD with roll-pitch-yaw state: mass 15 kg, inertia
    diag(0.10, 0.25, 0.30) kg m^2, dt 0.02 s, friction 0.6.  The friction
    cone enters as a C2 relaxed log barrier (quadratic below delta = 5 N),
    applied to legs in stance, with its exact curvature in the Hessian.  The
    cone's tangential norm is smoothed over 1 N, sqrt(fx^2 + fy^2 + 1), where
    the reference smooths over 0.1 N (objectives.py:29): at 0.1 N the cone's
    curvature near zero tangential force is 10 per N, Newton steps on forces
    of a few N overshoot it, and the merit line search then cuts them to a
    quarter iteration after iteration."""
    return ModelDesc(MODEL_SRBD_RPY12, 12, 12, dt=0.02, mass=15.0, inertia=np.diag([0.10, 0.25, 0.30]),
                     n_contact=4, mu=mu, barrier_kind=1, barrier_masked=1, cone_eps2=1.0)


def biped_wrench12(mu=0.6):
    """SRBD biped: mass 60 kg, inertia diag(6, 5, 1.5) kg m^2, two 0.2 x 0.1 m
    foot plates each carrying a 6-D wrench [F, tau].  The cone is smoothed
    over 1 N, as for the roll-pitch-yaw quadruped."""
    return ModelDesc(MODEL_BIPED_WRENCH12, 12, 12, dt=0.02, mass=60.0, inertia=np.diag([6.0, 5.0, 1.5]),
                     n_contact=2, mu=mu, foot_length=0.2, foot_width=0.1, barrier_kind=1, barrier_masked=1,
                     cone_eps2=1.0)


def generic_lq(n, m):
    return ModelDesc(MODEL_GENERIC_LQ, n, m, n_contact=0)


# ----------------------------------------------------------------- gait timer
def timer_run_np(duty_factor, step_freq, leg_time, dt):
    """mpx/utils/mpc_utils.py:7-14 in float32 (no fused multiply-add):
    leg_time += dt*step_freq; wrap once above 1; contact = leg_time < duty."""
    lt = np.asarray(leg_time, dtype=np.float32)
    inc = np.float32(dt) * np.float32(step_freq)
    lt = (lt + inc).astype(np.float32)
    lt = np.where(lt > np.float32(1.0), (lt - np.float32(1.0)).astype(np.float32), lt).astype(np.float32)
    contact = (lt < np.float32(duty_factor)).astype(np.int32)
    return contact, lt


# ----------------------------------------------------------------- workloads
HIP_OFFSETS = np.array([[0.20, 0.12, -0.30], [0.20, -0.12, -0.30], [-0.20, 0.12, -0.30], [-0.20, -0.12, -0.30]])
TROT_PHASE = np.array([0.0, 0.5, 0.5, 0.0])


def quadruped_weights(model=MODEL_SRBD_RPY12):
    """W = diag(pos 50, orientation 20, velocity 5, angular velocity 1, forces 1e-4)."""
    w = np.array([50.0] * 3 + [20.0] * 3 + [5.0] * 3 + [1.0] * 3 + [1e-4] * 12)
    return np.diag(w)


@dataclasses.dataclass
class Workload:
    desc: ModelDesc
    x0: np.ndarray
    X0: np.ndarray
    U0: np.ndarray
    V0: np.ndarray
    reference: np.ndarray
    parameter: np.ndarray
    W: np.ndarray
    horizon: np.ndarray
    # gait state carried between control ticks
    leg_time: np.ndarray = None
    v_ref: np.ndarray = None
    duty: float = 0.6
    step_freq: float = 2.0
    height: float = 0.30

    @property
    def batch(self):
        return self.x0.shape[0]

    @property
    def n_max(self):
        return self.X0.shape[1] - 1


def quadruped_tables(desc, x0, leg_time, v_ref, horizon, n_max, duty=0.6, step_freq=2.0, height=0.30):
    """Reference and parameter tables of the quadruped trot workload.

    The contact schedule comes from the gait timer exactly as the reference
    generator does it (one timer step per stage, mpc_utils.py:187-189); the CoM
    reference moves at v_ref along x at constant height with zero attitude and
    angular rate; the feet sit at the hip offsets (+-0.20, +-0.12, -0.30) m
    below the CoM reference."""
    B = x0.shape[0]
    rc, pc = desc.ref_cols, desc.par_cols
    ref = np.zeros((B, n_max + 1, rc), dtype=np.float32)
    par = np.zeros((B, n_max + 1, pc), dtype=np.float32)
    lt = leg_time.astype(np.float32).copy()
    t = np.arange(n_max + 1, dtype=np.float32)
    px = x0[:, 0:1] + t[None, :] * np.float32(desc.dt) * v_ref[:, None]
    py = np.repeat(x0[:, 1:2], n_max + 1, axis=1)
    contacts = np.zeros((B, n_max + 1, 4), dtype=np.float32)
    for k in range(n_max + 1):
        c, lt = timer_run_np(duty, step_freq, lt, desc.dt)
        contacts[:, k, :] = c
    ref[:, :, 0] = px
    ref[:, :, 1] = py
    ref[:, :, 2] = height
    if desc.model == MODEL_SRBD_QUAT13:
        ref[:, :, 3] = 1.0
        ref[:, :, 7] = v_ref[:, None]
        ref[:, :, 13:17] = contacts
    else:
        ref[:, :, 6] = v_ref[:, None]
        ref[:, :, 12:16] = contacts
    par[:, :, 0:4] = contacts
    off = HIP_OFFSETS.astype(np.float32)  # float32 sums, as the device tables
    for i in range(4):
        par[:, :, 4 + 3 * i] = px + off[i, 0]
        par[:, :, 5 + 3 * i] = py + off[i, 1]
        par[:, :, 6 + 3 * i] = np.float32(height) + off[i, 2]
    # beyond each instance's horizon the rows are left as computed (never read)
    return ref, par


def nominal_grf(desc, parameter):
    """Gravity-compensating forces split over the legs in stance."""
    c = parameter[:, :-1, 0:4]
    ns = np.maximum(c.sum(-1, keepdims=True), 1.0)
    U = np.zeros(parameter.shape[:2] + (12,), dtype=np.float32)[:, :-1]
    fz = desc.mass * desc.gravity * c / ns
    U[:, :, 2::3] = fz
    return U.astype(np.float32)


def quadruped_workload(batch, horizons=(50,), seed=0, model=MODEL_SRBD_RPY12, v_range=(0.5, 0.5), random_phase=False,
                       noise=0.05, mu=0.6):
    """Seeded synthetic quadruped trot MPC batch.

    horizons: a tuple of horizon lengths drawn uniformly per instance;
    v_range: forward reference speed range; random_phase: uniform gait phase
    offset per instance; noise: std of the N(0, noise^2) initial-state
    perturbation around the nominal standing state."""
    rng = np.random.default_rng(seed)
    desc = quadruped_rpy12(mu) if model == MODEL_SRBD_RPY12 else quadruped_quat13(mu=mu)
    n, m = desc.n, desc.m
    horizon = rng.choice(np.asarray(horizons, dtype=np.int32), size=batch).astype(np.int32)
    n_max = int(max(horizons))
    v_ref = rng.uniform(v_range[0], v_range[1], size=batch).astype(np.float32)
    phase = rng.uniform(0.0, 1.0, size=batch) if random_phase else np.zeros(batch)
    leg_time = np.mod(TROT_PHASE[None, :] + phase[:, None], 1.0).astype(np.float32)
    height = 0.30
    x0 = np.zeros((batch, n), dtype=np.float32)
    x0[:, 2] = height
    if model == MODEL_SRBD_QUAT13:
        x0[:, 3] = 1.0
        pert = rng.normal(0.0, noise, size=(batch, 12))
        x0[:, 0:3] += pert[:, 0:3]
        # small attitude perturbation through the exponential map
        half = 0.5 * pert[:, 3:6]
        ang = np.linalg.norm(half, axis=1, keepdims=True)
        s = np.where(ang > 1e-12, np.sin(ang) / np.maximum(ang, 1e-12), 1.0)
        x0[:, 3] = np.cos(ang[:, 0])
        x0[:, 4:7] = half * s
        x0[:, 7:13] += pert[:, 6:12]
    else:
        x0 += rng.normal(0.0, noise, size=(batch, n)).astype(np.float32)
    x0 = x0.astype(np.float32)
    ref, par = quadruped_tables(desc, x0, leg_time, v_ref, horizon, n_max, height=height)
    W = np.tile(quadruped_weights(model)[None], (batch, 1, 1)).astype(np.float32)
    X0 = np.repeat(x0[:, None, :], n_max + 1, axis=1).astype(np.float32)
    U0 = nominal_grf(desc, par)
    V0 = np.zeros((batch, n_max + 1, n), dtype=np.float32)
    return Workload(desc, x0, X0, U0, V0, ref, par, W, horizon, leg_time=leg_time, v_ref=v_ref, height=height)


def shift_warm_start(X, U, V, horizon, shift=1):
    """Warm start for the next tick (mpx/utils/mpc_wrapper_srbd.py:135-137):
    drop the first `shift` rows and repeat the last row, per instance horizon."""
    X = np.array(X, copy=True); U = np.array(U, copy=True); V = np.array(V, copy=True)
    for b, N in enumerate(np.asarray(horizon)):
        N = int(N)
        X[b, :N + 1 - shift] = X[b, shift:N + 1]; X[b, N + 1 - shift:N + 1] = X[b, N]
        V[b, :N + 1 - shift] = V[b, shift:N + 1]; V[b, N + 1 - shift:N + 1] = V[b, N]
        U[b, :N - shift] = U[b, shift:N]; U[b, N - shift:N] = U[b, N - 1]
    return X, U, V


def random_lq(batch, n, m, N, seed=0, rho=0.98):
    """Isolated KKT/LQR workload: A_t = I + 0.05 G, G ~ N(0, 1/n) rescaled to
    spectral radius `rho`; B_t ~ N(0, 1/m); Q_t = M M^T / n + 0.1 I;
    R_t = 0.1 I; S_t = 0; affine terms and x0 ~ N(0, 1).  float64 arrays."""
    rng = np.random.default_rng(seed)
    G = rng.normal(0.0, 1.0 / np.sqrt(n), size=(batch, N, n, n))
    A = np.eye(n) + 0.05 * G
    ev = np.abs(np.linalg.eigvals(A)).max(-1)
    A = A * (rho / ev)[..., None, None]
    Bm = rng.normal(0.0, 1.0 / np.sqrt(m), size=(batch, N, n, m))
    Mq = rng.normal(0.0, 1.0, size=(batch, N + 1, n, n))
    Q = Mq @ np.swapaxes(Mq, -1, -2) / n + 0.1 * np.eye(n)
    R = np.broadcast_to(0.1 * np.eye(m), (batch, N, m, m)).copy()
    M = np.zeros((batch, N, n, m))
    q = rng.normal(size=(batch, N + 1, n))
    r = rng.normal(size=(batch, N, m))
    c = rng.normal(size=(batch, N, n))
    x0 = rng.normal(size=(batch, n))
    return dict(A=A, B=Bm, c=c, Q=Q, R=R, M=M, q=q, r=r, x0=x0)


def random_lq_eq(batch, n=72, m=30, n_eq=12, N=100, seed=0, dt=0.1, rho_cap=1.01):
    """Large linearised whole-body-sized LQ workload with stage equality
    constraints C_t x_t + D_t u_t = e_t: A_t = I + dt J_t, J_t ~ N(0, 1/n),
    spectral radius capped at rho_cap; B_t ~ N(0, 0.1/m); Q_t diagonal,
    log-uniform in [1e-2, 1e2]; R_t = 1e-3 I; M_t = 0; n_eq constraint rows
    [C_t D_t] ~ N(0, 1); c_t ~ N(0, 0.1^2), q_t ~ N(0, 1), r_t = 0,
    e_t ~ N(0, 1), x0 ~ N(0, 1).  float64 arrays."""
    rng = np.random.default_rng(seed)
    J = rng.normal(0.0, 1.0 / np.sqrt(n), size=(batch, N, n, n))
    A = np.eye(n) + dt * J
    ev = np.abs(np.linalg.eigvals(A)).max(-1)
    A = A * np.minimum(1.0, rho_cap / ev)[..., None, None]
    Bm = rng.normal(0.0, np.sqrt(0.1 / m), size=(batch, N, n, m))
    Q = np.zeros((batch, N + 1, n, n))
    di = np.arange(n)
    Q[..., di, di] = 10.0 ** rng.uniform(-2.0, 2.0, size=(batch, N + 1, n))
    R = np.broadcast_to(1e-3 * np.eye(m), (batch, N, m, m)).copy()
    M = np.zeros((batch, N, n, m))
    CD = rng.normal(size=(batch, N, n_eq, n + m))
    return dict(A=A, B=Bm, c=rng.normal(0.0, 0.1, size=(batch, N, n)), Q=Q, R=R, M=M,
                q=rng.normal(size=(batch, N + 1, n)), r=np.zeros((batch, N, m)),
                C=CD[..., :n].copy(), D=CD[..., n:].copy(), e=rng.normal(size=(batch, N, n_eq)),
                x0=rng.normal(size=(batch, n)))


BIPED_HIP_OFFSETS = np.array([[0.0, 0.10, -0.90], [0.0, -0.10, -0.90]])
WALK_PHASE = np.array([0.0, 0.5])


def biped_tables(desc, x0, leg_time, v_ref, n_max, duty=0.6, step_freq=1.25, height=0.90):
    """Reference / parameter tables of the biped walking workload: alternating
    feet (gait timer per foot), CoM reference at v_ref along x, feet 0.10 m left
    and right of the CoM reference on the ground."""
    B = x0.shape[0]
    ref = np.zeros((B, n_max + 1, desc.ref_cols), dtype=np.float32)
    par = np.zeros((B, n_max + 1, desc.par_cols), dtype=np.float32)
    lt = leg_time.astype(np.float32).copy()
    t = np.arange(n_max + 1, dtype=np.float32)
    px = x0[:, 0:1] + t[None, :] * np.float32(desc.dt) * v_ref[:, None]
    py = np.repeat(x0[:, 1:2], n_max + 1, axis=1)
    for k in range(n_max + 1):
        c, lt = timer_run_np(duty, step_freq, lt, desc.dt)
        ref[:, k, 12:14] = c
        par[:, k, 0:2] = c
    ref[:, :, 0] = px
    ref[:, :, 1] = py
    ref[:, :, 2] = height
    ref[:, :, 6] = v_ref[:, None]
    for i in range(2):
        off = BIPED_HIP_OFFSETS.astype(np.float32)  # float32 sums, as the device tables
        par[:, :, 2 + 3 * i] = px + off[i, 0]
        par[:, :, 3 + 3 * i] = py + off[i, 1]
        par[:, :, 4 + 3 * i] = np.float32(height) + off[i, 2]
    return ref, par


def biped_weights():
    w = np.array([50.0] * 3 + [20.0] * 3 + [5.0] * 3 + [1.0] * 3 + ([1e-4] * 3 + [1e-3] * 3) * 2)
    return np.diag(w)


def biped_workload(batch, horizons=(50,), seed=0, v_range=(-0.5, 0.5), random_phase=True, noise=0.02, mu=0.6):
    """Seeded synthetic biped walking MPC batch (SRBD with 6-D foot wrenches)."""
    rng = np.random.default_rng(seed)
    desc = biped_wrench12(mu)
    horizon = rng.choice(np.asarray(horizons, dtype=np.int32), size=batch).astype(np.int32)
    n_max = int(max(horizons))
    v_ref = rng.uniform(v_range[0], v_range[1], size=batch).astype(np.float32)
    phase = rng.uniform(0.0, 1.0, size=batch) if random_phase else np.zeros(batch)
    leg_time = np.mod(WALK_PHASE[None, :] + phase[:, None], 1.0).astype(np.float32)
    height = 0.90
    x0 = np.zeros((batch, 12), dtype=np.float32)
    x0[:, 2] = height
    x0 += rng.normal(0.0, noise, size=(batch, 12)).astype(np.float32)
    ref, par = biped_tables(desc, x0, leg_time, v_ref, n_max, height=height)
    W = np.tile(biped_weights()[None], (batch, 1, 1)).astype(np.float32)
    X0 = np.repeat(x0[:, None, :], n_max + 1, axis=1).astype(np.float32)
    c = par[:, :-1, 0:2]
    ns = np.maximum(c.sum(-1, keepdims=True), 1.0)
    U0 = np.zeros((batch, n_max, 12), dtype=np.float32)
    U0[:, :, 2] = desc.mass * desc.gravity * c[:, :, 0] / ns[:, :, 0]
    U0[:, :, 8] = desc.mass * desc.gravity * c[:, :, 1] / ns[:, :, 0]
    V0 = np.zeros((batch, n_max + 1, 12), dtype=np.float32)
    wl = Workload(desc, x0, X0, U0, V0, ref, par, W, horizon, leg_time=leg_time, v_ref=v_ref, duty=0.6,
                  step_freq=1.25, height=height)
    return wl


def wb_workload(batch, N, q0, feet0, mass, seed=0, dt=0.02, duty=0.65, step_freq=1.35, height=0.33, noise=0.02,
                v_range=(-0.5, 0.5), step_height=0.06):
    """Seeded synthetic whole-body MPC instances (aliengo-shaped: 12 joints,
    4 feet), in the layouts mpxg_wb_sqp takes:
      x0 [B,61] = [p, quat, q, v, omega, dq, feet (3C), forces (3C)]: a
        standing pose (q0, height) with N(0, noise) perturbations of the base
        position, orientation (unit quaternion), joints and velocities;
      reference [B,N+1,53] rows [p, quat, q, dp, omega, feet, contact, forces]:
        base moving at v ~ U(v_range) along x at `height`, identity
        orientation, q0, feet at feet0 (nominal, base frame at the origin)
        shifted with the base, lifted by step_height along a sine in swing,
        a trot contact schedule with a random phase, contact forces
        m g / (feet in contact) on the feet in contact;
      contact [B,N+1,4] int32 (the same schedule, the dynamics' mask);
      X0 [B,N+1,61] = tiles of x0, U0 [B,N,12] = 0, V0 [B,N+1,61] = 0."""
    rng = np.random.default_rng(seed)
    nj, nc = len(q0), len(feet0) // 3
    nx = 13 + 2 * nj + 6 * nc
    q0 = np.asarray(q0, dtype=np.float64)
    feet0 = np.asarray(feet0, dtype=np.float64).reshape(nc, 3)
    x0 = np.zeros((batch, nx))
    x0[:, 0:3] = np.array([0.0, 0.0, height]) + rng.normal(size=(batch, 3)) * noise
    quat = np.array([1.0, 0.0, 0.0, 0.0]) + rng.normal(size=(batch, 4)) * noise
    x0[:, 3:7] = quat / np.linalg.norm(quat, axis=1, keepdims=True)
    x0[:, 7:7 + nj] = q0 + rng.normal(size=(batch, nj)) * noise
    x0[:, 7 + nj:13 + 2 * nj] = rng.normal(size=(batch, 6 + nj)) * noise
    x0[:, 13 + 2 * nj:13 + 2 * nj + 3 * nc] = (feet0 + [0.0, 0.0, 0.0]).reshape(-1)
    v = rng.uniform(v_range[0], v_range[1], size=batch)
    phase = rng.uniform(0.0, 1.0, size=batch)
    offs = np.array([0.0, 0.5, 0.5, 0.0])[:nc]
    t = np.arange(N + 1) * dt
    ph = (phase[:, None, None] + offs[None, None, :] + step_freq * t[None, :, None]) % 1.0  # [B,N+1,C]
    contact = (ph < duty).astype(np.int32)
    ref = np.zeros((batch, N + 1, 13 + nj + 7 * nc))
    ref[:, :, 0] = x0[:, None, 0] + v[:, None] * t[None, :]
    ref[:, :, 1] = x0[:, None, 1]
    ref[:, :, 2] = height
    ref[:, :, 3] = 1.0
    ref[:, :, 7:7 + nj] = q0
    ref[:, :, 7 + nj] = v[:, None]
    feet = np.broadcast_to(feet0[None, None], (batch, N + 1, nc, 3)).copy()
    feet[..., 0] += ref[:, :, 0:1] - x0[:, None, 0:1]
    swing = np.where(contact == 0, np.sin(np.pi * np.clip((ph - duty) / (1.0 - duty), 0.0, 1.0)), 0.0)
    feet[..., 2] += step_height * swing
    ref[:, :, 13 + nj:13 + nj + 3 * nc] = feet.reshape(batch, N + 1, 3 * nc)
    ref[:, :, 13 + nj + 3 * nc:13 + nj + 4 * nc] = contact
    grf = np.zeros((batch, N + 1, nc, 3))
    grf[..., 2] = contact * mass * 9.81 / (contact.sum(axis=2, keepdims=True) + 1e-5)
    ref[:, :, 13 + nj + 4 * nc:] = grf.reshape(batch, N + 1, 3 * nc)
    f32 = lambda a: np.ascontiguousarray(a, dtype=np.float32)
    x0 = f32(x0)
    return dict(x0=x0, reference=f32(ref), contact=contact, X0=f32(np.repeat(x0[:, None], N + 1, axis=1)),
                U0=np.zeros((batch, N, nj), dtype=np.float32), V0=np.zeros((batch, N + 1, nx), dtype=np.float32))
