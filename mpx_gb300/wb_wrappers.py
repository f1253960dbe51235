"""The whole-body controllers of mpx/utils/mpc_wrapper.py (the reference's
MPCControllerWrapper and BatchedMPCControllerWrapper are built for whole-body
configurations such as config_aliengo.py: 13 + 2 nj + 6 C states, joint
torques as controls, quadruped_wb_dynamics / quadruped_wb_obj /
quadruped_wb_hessian_gn).

  WholeBodyController         <- MPCControllerWrapper, mpc_wrapper.py:194-468
  WholeBodyBatchedController  <- BatchedMPCControllerWrapper, mpc_wrapper.py:29-192

mpx_gb300.wrappers.MPCControllerWrapper and BatchedDataMPCWrapper (exported by
mpx_gb300.mpc_wrapper under the reference's names) hand a whole-body
configuration to these classes, so the reference's call sites run unchanged.
Every per-tick step -- forward kinematics of the feet (mj_kinematics,
mpc_wrapper.py:313-316), gait timer, whole-body reference generator, the SQP
solve, the warm-start shift with its NaN fallback -- runs as libmpxg kernels
on device-resident tensors; the host sees only the returned torques.
"""
import numpy as np
import torch

from . import _lib
from . import mjcf
from .solver import _ptr, _stream_handle
from .wholebody import WholeBodyModel, WholeBodySQP


def is_whole_body(config):
    """A configuration of the reference's whole-body wrappers: its state holds
    qpos, qvel, the contact points and (grf_as_state) the contact forces."""
    nj, nc, n = getattr(config, "n_joints", None), getattr(config, "n_contact", None), getattr(config, "n", None)
    if nj is None or nc is None or n is None:
        return False
    return int(n) in (13 + 2 * int(nj) + 6 * int(nc), 13 + 2 * int(nj) + 3 * int(nc)) and int(n) > 13


def _dev(a, dev, dtype=torch.float32):
    if isinstance(a, torch.Tensor):
        return a.to(device=dev, dtype=dtype).contiguous()
    return torch.as_tensor(np.asarray(a), dtype=dtype, device=dev).contiguous()


def _w_diag(config):
    W = np.asarray(config.W, dtype=np.float64)
    if W.ndim == 2:
        if np.any(W - np.diag(np.diag(W))):
            raise ValueError("the whole-body solve takes a diagonal W (config_aliengo / config_go2 build a "
                             "block-diagonal W of diagonal blocks)")
        W = np.diag(W)
    return W.astype(np.float32)


def _sqp_kwargs(opts):
    """WholeBodySQP's options from a dict of them or from the SolverOptions
    the wrappers take for the SRBD models (iterations, line search, reg, rho0)."""
    if opts is None:
        return {}
    if isinstance(opts, dict):
        return dict(opts)
    return dict(iters=int(opts.sqp_iters), reg=float(opts.reg), rho0=float(opts.rho0), ls_beta=float(opts.ls_beta),
                ls_eta=float(opts.ls_eta), ls_skip_tol=float(opts.ls_skip_tol), ls_max_trials=int(opts.ls_max_trials))


def _model(config, model):
    if model is not None:
        return model
    return mjcf.parse(config.model_path, list(config.contact_frame), list(config.body_name))


class _WbCommon:
    def _setup(self, config, model, batch, device, opts, clearence_speed):
        if not bool(getattr(config, "grf_as_state", True)):
            raise ValueError("the whole-body solve is built with the contact forces as states (grf_as_state)")
        self.config = config
        self.dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.wb = WholeBodyModel(_model(config, model), device=self.dev)
        self.nj, self.nc, self.N = int(config.n_joints), int(config.n_contact), int(config.N)
        self.nx = 13 + 2 * self.nj + 6 * self.nc
        # the reference's robot_mass = qM[0] (mpc_wrapper.py:46,208): the
        # free body's translational inertia, the model's total mass
        self.mass = float(np.sum(self.wb.model.mass))
        self.mpc_frequency = float(config.mpc_frequency)
        self.shift = int(1 / (config.dt * config.mpc_frequency))
        self.sqp = WholeBodySQP(self.wb, self.N, batch_max=batch, dt=float(config.dt), **_sqp_kwargs(opts))
        self.W = _dev(_w_diag(config), self.dev)
        self.foot0 = np.asarray(config.p_legs0, dtype=np.float32)
        self.q0 = np.asarray(config.q0, dtype=np.float32)
        self.u_ref = _dev(np.asarray(config.u_ref, dtype=np.float32), self.dev)
        self.terrain = int(bool(getattr(config, "use_terrain_estimation", False)))
        self.clearence_speed = clearence_speed
        self.L = _lib.load()

    def _refgen(self, B, t_timer, x0, foot, inp, contact, liftoff, duty, freq, height):
        ref = torch.empty(B, self.N + 1, 13 + self.nj + 7 * self.nc, device=self.dev)
        par = torch.empty(B, self.N + 1, self.nc, device=self.dev)
        f0 = (_lib.ctypes.c_float * 12)(*self.foot0.tolist())
        q0 = (_lib.ctypes.c_float * self.nj)(*self.q0.tolist())
        _lib.check(self.L.mpxg_refgen_wb(_stream_handle(None), B, self.N, self.nj, float(self.config.dt), self.mass,
                                         f0, q0, float(duty), float(freq), float(height),
                                         float(self.clearence_speed), self.terrain, _ptr(t_timer), _ptr(x0),
                                         _ptr(foot), _ptr(inp), _ptr(contact), _ptr(liftoff), _ptr(ref),
                                         _ptr(par)), None, "mpxg_refgen_wb")
        return ref, par

    def _timer(self, B, leg_time, duty, freq):
        cont = torch.empty(B, self.nc, dtype=torch.int32, device=self.dev)
        _lib.check(self.L.mpxg_timer_run(_stream_handle(None), B, self.nc, float(duty), float(freq),
                                         1.0 / self.mpc_frequency, _ptr(leg_time), _ptr(cont)), None,
                   "mpxg_timer_run")
        return cont

    def _feet(self, qpos):
        """Contact points at qpos (the reference's mj_kinematics + geom_xpos)."""
        qpos = _dev(qpos, self.dev).reshape(-1, self.wb.nq)
        return self.wb.terms(qpos, torch.zeros(qpos.shape[0], self.wb.nv, device=self.dev))["cpos"]

    def _solve_and_shift(self, x0, X0, U0, V0, ref, par):
        """The solve and update_and_extract (mpc_wrapper.py:81-98, 261-282):
        the shifted warm start, or on NaN in U[0, 0] tiles of u_ref / x0 and
        zero duals; tau = U[0, :nj], q = X[0, 7:7+nj], dq = X[1, 13+nj:13+2nj]
        (from the previous warm start where the result is NaN)."""
        B, N, nj = x0.shape[0], self.N, self.nj
        out = self.sqp.solve(x0, X0, U0, V0, ref, par.to(torch.int32), self.W)
        X, U, V = out["X"], out["U"], out["V"]
        nan = torch.isnan(U[:, 0, 0])
        s = self.shift
        sh = lambda a: torch.cat([a[:, s:], a[:, -1:].expand(-1, s, -1)], 1)
        Xn, Un, Vn = sh(X), sh(U), sh(V)
        tau = torch.where(nan[:, None], U0[:, 1, :nj], U[:, 0, :nj])
        q = torch.where(nan[:, None], X0[:, 1, 7:7 + nj], X[:, 0, 7:7 + nj])
        dq = torch.where(nan[:, None], X0[:, 1, 13 + nj:13 + 2 * nj], X[:, 1, 13 + nj:13 + 2 * nj])
        if bool(nan.any()):
            k = int(nan.sum())
            Xn[nan] = x0[nan].unsqueeze(1).expand(-1, N + 1, -1)
            Un[nan] = self.u_ref.reshape(1, 1, -1).expand(k, N, -1)
            Vn[nan] = 0.0
        return Xn.contiguous(), Un.contiguous(), Vn.contiguous(), tau, q, dq, out


class WholeBodyController(_WbCommon):
    """MPCControllerWrapper of mpc_wrapper.py:194-468 for a whole-body
    configuration: run(qpos, qvel, input, contact) -> (tau, q, dq) with tau
    clipped to [min_torque, max_torque]; reset(qpos, qvel).  `model`: a parsed
    mjcf.RigidBodyModel with the configuration's contacts (default: parsed
    from config.model_path); `opts`: WholeBodySQP options."""

    STATE = ("X0", "U0", "V0", "contact_time", "liftoff")

    def __init__(self, config, limited_memory=False, model=None, device=None, opts=None):
        self._setup(config, model, 1, device, opts, clearence_speed=0.4)  # mpc_wrapper.py:292
        self.duty_factor = float(config.duty_factor)
        self.step_freq = float(config.step_freq)
        self.step_height = float(config.step_height)
        self.robot_height = float(config.initial_height)  # mpc_wrapper.py:288
        init = np.concatenate([np.asarray(config.p0, np.float32), np.asarray(config.quat0, np.float32), self.q0,
                               np.zeros(6 + self.nj, np.float32), self.foot0, np.zeros(3 * self.nc, np.float32)])
        self._set_warm(_dev(init, self.dev).reshape(1, -1))
        self.contact_time = _dev(np.asarray(config.timer_t, np.float32).reshape(1, self.nc), self.dev)
        self.liftoff = _dev(self.foot0.reshape(1, -1), self.dev)

    def _set_warm(self, x0):
        N = self.N
        self.X0 = x0.reshape(1, 1, -1).expand(1, N + 1, -1).contiguous()
        self.U0 = self.u_ref.reshape(1, 1, -1).expand(1, N, -1).contiguous()
        self.V0 = torch.zeros(1, N + 1, self.nx, device=self.dev)

    def _x0(self, qpos, qvel, feet):
        return torch.cat([_dev(qpos, self.dev).reshape(1, -1), _dev(qvel, self.dev).reshape(1, -1),
                          feet.reshape(1, -1), torch.zeros(1, 3 * self.nc, device=self.dev)], 1).contiguous()

    def run(self, qpos, qvel, input, contact):
        """mpc_wrapper.py:297-365."""
        feet = self._feet(qpos)
        inp = _dev(input, self.dev).reshape(1, 7).clone()
        inp[0, 6] = self.robot_height                                                  # :318
        x0 = self._x0(qpos, qvel, feet)
        cont = _dev(contact, self.dev).reshape(1, self.nc)
        self._timer(1, self.contact_time, self.duty_factor, self.step_freq)             # :332
        ref, par = self._refgen(1, self.contact_time, x0, feet, inp, cont, self.liftoff, self.duty_factor,
                                self.step_freq, self.step_height)                       # :335-346
        X0, U0, V0, tau, q, dq, _ = self._solve_and_shift(x0, self.X0, self.U0, self.V0, ref, par)
        self.X0, self.U0, self.V0 = X0, U0, V0
        tau = torch.clamp(tau, float(self.config.min_torque), float(self.config.max_torque))  # :361
        return tau[0].cpu().numpy(), q[0].cpu().numpy(), dq[0].cpu().numpy()

    def reset(self, qpos, qvel):
        """mpc_wrapper.py:367-385."""
        feet = self._feet(qpos)
        self.contact_time = _dev(np.asarray(self.config.timer_t, np.float32).reshape(1, self.nc), self.dev)
        self.liftoff = feet.reshape(1, -1).clone()
        self._set_warm(self._x0(qpos, qvel, feet))
        print("MPC Controller Reset")

    def runOffline(self, qpos, qvel, reference=None, parameter=None, max_iter=100):
        """mpc_wrapper.py:387-468 on caller-given whole-body tables
        (reference [N+1, 13+nj+7C], parameter [N+1, C]; the reference takes
        them from config.reference): single SQP iterations, the warm start's
        first 13 + nj columns set to the reference's (:419), until the
        reference's stop rule (:465) holds with the KKT residual standing in
        for its objective: the residual changed by less than 1e-3 and
        max |c|^2 < 1e-5 (the reference's sum of c^2 over its defects).
        Returns (X, U, reference, the iterates' X)."""
        if reference is None or parameter is None:
            make = getattr(self.config, "reference", None)
            if make is None:
                raise ValueError("runOffline needs reference and parameter tables (config.reference is absent)")
            reference, parameter = make(self.N + 1, self.config.dt, self.nj, self.nc, self.foot0, self.q0)
        feet = self._feet(qpos)
        x0 = self._x0(qpos, qvel, feet)
        ref = _dev(reference, self.dev).reshape(1, self.N + 1, -1)
        par = _dev(parameter, self.dev).reshape(1, self.N + 1, -1)[:, :, :self.nc].to(torch.int32)
        X = self.X0.clone()
        X[:, :, :13 + self.nj] = ref[:, :, :13 + self.nj]                            # :419
        U, V = self.U0.clone(), self.V0.clone()
        outputs, last = [X[0].cpu().numpy()], 1e10
        for _ in range(max_iter):
            out = self.sqp.solve(x0, X, U, V, ref, par, self.W, iters=1)
            X, U, V = out["X"], out["U"], out["V"]
            outputs.append(X[0].cpu().numpy())
            kkt = out["kkt"][0].cpu().numpy()
            res = float(kkt[2])
            if last - res < 1e-3 and float(kkt[0]) ** 2 < 1e-5:
                break
            last = res
        self.X0, self.U0, self.V0 = X, U, V
        return X, U, ref, outputs

    def save_state(self):
        return {k: getattr(self, k).detach().to("cpu", copy=True) for k in self.STATE}

    def load_state(self, state):
        for k in self.STATE:
            cur = getattr(self, k)
            src = torch.as_tensor(state[k])
            if tuple(src.shape) != tuple(cur.shape):
                raise ValueError("load_state: %s has shape %s, this controller holds %s"
                                 % (k, tuple(src.shape), tuple(cur.shape)))
            setattr(self, k, src.to(device=cur.device, dtype=cur.dtype).contiguous().clone())


class WholeBodyBatchedController(_WbCommon):
    """BatchedMPCControllerWrapper of mpc_wrapper.py:29-192 for a whole-body
    configuration: make_data(), run(data, x0, input) -> (data, tau),
    reset(data, qpos, qvel, foot), with `data` an mpx_data record of device
    tensors with a leading env dimension."""

    def __init__(self, config, n_env, limited_memory=False, model=None, device=None, opts=None):
        self.n_env = int(n_env)
        self._setup(config, model, self.n_env, device, opts, clearence_speed=0.2)  # mpc_wrapper.py:75
        self.initial_state = np.concatenate([np.asarray(config.p0, np.float32), np.asarray(config.quat0, np.float32),
                                             self.q0, np.zeros(6 + self.nj, np.float32), self.foot0,
                                             np.zeros(3 * self.nc, np.float32)])

    def make_data(self):
        """mpc_wrapper.py:100-113, for all environments."""
        from .wrappers import mpx_data
        B, N, dev, c = self.n_env, self.N, self.dev, self.config
        return mpx_data(
            dt=float(c.dt), duty_factor=float(c.duty_factor), step_freq=float(c.step_freq),
            step_height=float(c.step_height),
            contact_time=_dev(np.tile(np.asarray(c.timer_t, np.float32), (B, 1)), dev),
            liftoff=torch.zeros(B, 3 * self.nc, device=dev),
            X0=_dev(np.tile(self.initial_state, (B, N + 1, 1)), dev),
            U0=self.u_ref.reshape(1, 1, -1).expand(B, N, -1).contiguous(),
            V0=torch.zeros(B, N + 1, self.nx, device=dev),
            W=self.W.reshape(1, -1).expand(B, -1).contiguous(),
            grf=torch.zeros(B, 3 * self.nc, device=dev))

    def run(self, data, x0, input):
        """mpc_wrapper.py:115-170: timer, reference (with the feet of x0 and
        no measured contact), solve, NaN-guarded warm start; returns
        (data, tau)."""
        from .wrappers import mpx_data
        B, nj, nc = self.n_env, self.nj, self.nc
        x0 = _dev(x0, self.dev).reshape(B, self.nx)
        inp = _dev(input, self.dev).reshape(B, 7)
        ct = data["contact_time"].clone()
        self._timer(B, ct, data["duty_factor"], data["step_freq"])
        foot = x0[:, 13 + 2 * nj:13 + 2 * nj + 3 * nc].contiguous()
        lo = data["liftoff"].clone()
        ref, par = self._refgen(B, data["contact_time"], x0, foot, inp, torch.zeros(B, nc, device=self.dev), lo,
                                data["duty_factor"], data["step_freq"], data["step_height"])
        X0, U0, V0, tau, _, _, _ = self._solve_and_shift(x0, data["X0"], data["U0"], data["V0"], ref, par)
        g0 = 13 + 2 * nj + 3 * nc
        data = mpx_data(data, X0=X0, U0=U0, V0=V0, contact_time=ct, liftoff=lo,
                        grf=X0[:, 0, g0:g0 + 3 * nc].contiguous())
        return data, tau

    def reset(self, data, qpos, qvel, foot):
        """mpc_wrapper.py:172-192."""
        from .wrappers import mpx_data
        B, N, dev = self.n_env, self.N, self.dev
        foot = _dev(foot, dev).reshape(B, 3 * self.nc)
        x0 = torch.cat([_dev(qpos, dev).reshape(B, -1), _dev(qvel, dev).reshape(B, -1), foot,
                        torch.zeros(B, 3 * self.nc, device=dev)], 1)
        return mpx_data(data, contact_time=_dev(np.tile(np.asarray(self.config.timer_t, np.float32), (B, 1)), dev),
                        liftoff=foot.clone(), X0=x0.unsqueeze(1).expand(-1, N + 1, -1).contiguous(),
                        U0=self.u_ref.reshape(1, 1, -1).expand(B, N, -1).contiguous(),
                        V0=torch.zeros(B, N + 1, self.nx, device=dev),
                        grf=torch.zeros(B, 3 * self.nc, device=dev))
