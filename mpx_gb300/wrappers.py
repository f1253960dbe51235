"""Drop-in controller wrappers with the reference's API.

  BatchedMPCControllerWrapper  <- mpx/utils/mpc_wrapper_srbd.py:19-175  (SRBD, batched)
  MPCControllerWrapper         <- mpx/utils/mpc_wrapper.py:194-468      (single instance)
  BatchedDataMPCWrapper        <- mpx/utils/mpc_wrapper.py:29-192       (make_data + run(data, x0, input))
  mpx_data                     <- mpx/utils/mpc_wrapper.py:16-27        (the data record)
  mpc(...) / make_mpc(...)     <- optimizers.mpc as bound with functools.partial
                                  (mpx/utils/mpc_wrapper_srbd.py:68,77)

mpx_gb300.mpc_wrapper and mpx_gb300.mpc_wrapper_srbd export these classes
under the reference modules' own names.

Every per-tick step of the reference's `run()` -- gait timer, reference
generator, solve, warm-start shift -- runs as a CUDA kernel of libmpxg on
device-resident tensors; there is no host round trip unless the caller reads
a result.  Inputs may be numpy arrays, torch tensors (any device) or any
DLPack-capable array; they are copied to the solver's device as float32.

Differences from the reference, by necessity:
  * Python callables (cost, dynamics, hessian_approx) cannot cross the C ABI:
    the model is one of the compiled ids (problem.ModelDesc).
  * `limited_memory` is accepted and ignored.
  * MuJoCo is not available.  With a whole-body configuration (the
    reference's config_aliengo / config_go2), MPCControllerWrapper and
    BatchedDataMPCWrapper hand over to mpx_gb300.wb_wrappers, which computes
    the feet by libmpxg's own rigid-body kernel over the robot's MJCF
    (`config.model_path`, read by mpx_gb300.mjcf, or a parsed `model=`) and
    returns the reference's (tau, q, dq) / (data, tau).  With a compiled SRBD
    model the foot positions (mpc_wrapper.py:313-316) are passed in by the
    caller (`foot_op`).  The SRBD wrapper's whole-body torque mapping
    (mpc_utils.py:275-313) runs on the same rigid-body kernel
    (mpx_gb300.wholebody) over the MJCF or a model passed as `wb_model`.
"""
import os

import numpy as np
import torch

from . import _lib
from . import mjcf
from . import problem as P
from .solver import Solver, _ptr, _stream_handle
from .wb_wrappers import WholeBodyBatchedController, WholeBodyController, is_whole_body
from .wholebody import WholeBodyModel


def _to_dev(a, dev, dtype=torch.float32):
    if a is None:
        return None
    if isinstance(a, torch.Tensor):
        return a.to(device=dev, dtype=dtype).contiguous()
    if hasattr(a, "__dlpack__") and not isinstance(a, np.ndarray):
        return torch.from_dlpack(a).to(device=dev, dtype=dtype).contiguous()
    return torch.as_tensor(np.asarray(a), dtype=dtype, device=dev).contiguous()


def _cfg(config, name, default=None):
    v = getattr(config, name, default)
    if hasattr(v, "__array__") and not isinstance(v, (float, int)):
        return np.asarray(v)
    return v


def _save_state(obj, names):
    return {k: getattr(obj, k).detach().to("cpu", copy=True) for k in names}


def _load_state(obj, names, state):
    new = {}
    for k in names:
        cur = getattr(obj, k)
        src = torch.as_tensor(state[k])
        if tuple(src.shape) != tuple(cur.shape):
            raise ValueError("load_state: %s has shape %s, this controller holds %s"
                             % (k, tuple(src.shape), tuple(cur.shape)))
        new[k] = src.to(device=cur.device, dtype=cur.dtype).contiguous().clone()
    for k, v in new.items():
        setattr(obj, k, v)


# ----------------------------------------------------------------- functional API
def make_mpc(desc, opts=None, n_max=None, batch_max=1, device=None):
    """The equivalent of `jax.vmap(partial(optimizers.mpc, cost, dynamics,
    hessian_approx, limited_memory))`: returns solve(reference, parameter, W,
    x0, X0, U0, V0) -> (X, U, V) for batched (leading batch dim) or single
    (no batch dim) inputs.  The model is the compiled `desc`."""
    cache = {}

    def solve(reference, parameter, W, x0, X0, U0, V0):
        dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        x0t = _to_dev(x0, dev)
        single = x0t.dim() == 1
        add = (lambda t: t.unsqueeze(0)) if single else (lambda t: t)
        x0t, X0t, U0t, V0t = add(x0t), add(_to_dev(X0, dev)), add(_to_dev(U0, dev)), add(_to_dev(V0, dev))
        ref, par = add(_to_dev(reference, dev)), add(_to_dev(parameter, dev))
        Wt = _to_dev(W, dev)
        B, Np1 = X0t.shape[0], X0t.shape[1]
        key = (Np1 - 1, max(B, batch_max))
        if key not in cache:
            cache.clear()
            cache[key] = Solver(desc, opts or P.SolverOptions(), n_max=key[0] if n_max is None else n_max,
                                batch_max=key[1], device=dev)
        out = cache[key].solve(x0t, X0t, U0t, V0t, ref, par, Wt)
        X, U, V = out["X"], out["U"], out["V"]
        if single:
            X, U, V = X[0], U[0], V[0]
        return X, U, V

    return solve


def mpc(desc, reference, parameter, W, x0, X0, U0, V0, opts=None):
    """One call of optimizers.mpc with the model given by its compiled id."""
    return make_mpc(desc, opts)(reference, parameter, W, x0, X0, U0, V0)


# ----------------------------------------------------------------- SRBD wrapper
class BatchedMPCControllerWrapper:
    """SRBD quadruped MPC for n_env environments (mpc_wrapper_srbd.py:19-175).

    `config` has the attributes of mpx/config/config_srbd.py (dt, N,
    mpc_frequency, timer_t, duty_factor, step_freq, step_height,
    clearence_speed, p0, quat0, p_legs0, n, mass, inertia, u_ref, W, ...)."""

    def __init__(self, config, n_env, opts=None, device=None, limited_memory=False, wb_model=None, desc=None):
        """wb_model: an mjcf.RigidBodyModel for whole_body_run (default: the
        MJCF at config.model_path with config.contact_frame / body_name).
        desc: the quaternion model's description (default: the reference's
        own, problem.quadruped_quat13(config), with its penalty barrier); a
        description with barrier_kind=1, barrier_masked=1 and cone_eps2=1
        selects the smooth, stance-masked barrier with which the SQP
        converges (the reference's clipped, unmasked penalty defeats the
        merit line search)."""
        self.config = config
        self.n_env = int(n_env)
        self.dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        path = getattr(config, "model_path", None)
        if wb_model is None and path and os.path.exists(path):
            wb_model = mjcf.parse(path, list(config.contact_frame), list(config.body_name))
        self.wb = WholeBodyModel(wb_model, device=self.dev) if wb_model is not None else None
        self.Kp = _to_dev(np.asarray(getattr(config, "Kp", np.zeros((12, 12))), dtype=np.float32), self.dev)
        self.Kd = _to_dev(np.asarray(getattr(config, "Kd", np.zeros((12, 12))), dtype=np.float32), self.dev)
        self.mpc_frequency = float(config.mpc_frequency)
        self.shift = int(1 / (config.dt * config.mpc_frequency))
        self.N = int(config.N)
        self.n = int(getattr(config, "n", 13))
        self.foot0 = np.asarray(config.p_legs0, dtype=np.float32).copy()
        self.q0 = np.asarray(getattr(config, "q0", np.zeros(12)), dtype=np.float32).copy()
        self.initial_state = np.concatenate([np.asarray(config.p0, dtype=np.float32),
                                             np.asarray(config.quat0, dtype=np.float32),
                                             np.zeros(6, dtype=np.float32)])
        self.desc = desc or P.quadruped_quat13(config, mu=float(getattr(config, "mu", 0.7)))
        if self.desc.model != P.MODEL_SRBD_QUAT13:
            raise ValueError("the SRBD wrapper runs the quaternion model (MODEL_SRBD_QUAT13)")
        self.opts = opts or P.SolverOptions()
        self.solver = Solver(self.desc, self.opts, n_max=self.N, batch_max=self.n_env, device=self.dev)
        self.L = _lib.load()
        self.duty_factor = float(config.duty_factor)
        self.step_freq = float(config.step_freq)
        self.step_height = float(config.step_height)
        self.clearence_speed = float(config.clearence_speed)
        self.w = _to_dev(np.diag(np.asarray(config.W, dtype=np.float64)).astype(np.float32), self.dev)
        self.w = self.w.reshape(1, -1).expand(self.n_env, -1).contiguous()
        W = np.asarray(config.W, dtype=np.float64)
        if np.count_nonzero(W - np.diag(np.diag(W))):
            raise ValueError("config.W must be diagonal for the compiled SRBD model")
        self._alloc()
        self.reset(verbose=False)

    def _alloc(self):
        B, N, n, m, dev = self.n_env, self.N, self.n, 12, self.dev
        z = lambda *s: torch.zeros(*s, device=dev)
        self.reference = z(B, N + 1, 17)
        self.parameter = z(B, N + 1, 16)
        self._foot_ref_dot_all = z(B, N + 1, 12)
        self.contact = torch.zeros(B, 4, dtype=torch.int32, device=dev)
        self.kkt = z(B, 3)
        self.status = torch.zeros(B, dtype=torch.int32, device=dev)
        self.X = z(B, N + 1, n)
        self.U = z(B, N, m)
        self.V = z(B, N + 1, n)

    def reset(self, verbose=True):
        """mpc_wrapper_srbd.py:162-175."""
        B, N = self.n_env, self.N
        self.contact_time = _to_dev(np.tile(np.asarray(self.config.timer_t, dtype=np.float32), (B, 1)), self.dev)
        self.liftoff = torch.zeros(B, 12, device=self.dev)
        u_ref = np.asarray(self.config.u_ref, dtype=np.float32)
        self.batch_U0 = _to_dev(np.tile(u_ref, (B, N, 1)), self.dev)
        self.batch_X0 = _to_dev(np.tile(self.initial_state, (B, N + 1, 1)), self.dev)
        self.batch_V0 = torch.zeros(B, N + 1, self.n, device=self.dev)
        self.foot_ref = torch.zeros(B, 12, device=self.dev)
        self.foot_ref_dot = torch.zeros(B, 12, device=self.dev)
        self.grf = torch.zeros(B, 12, device=self.dev)
        if verbose:
            print("MPC Controller Reset")

    def run(self, x0, input, foot_op, contact):
        """One MPC tick for all environments (mpc_wrapper_srbd.py:91-141).
        Returns 0; the first control of every environment is in self.grf."""
        dev, B = self.dev, self.n_env
        x0 = _to_dev(x0, dev).reshape(B, 13)
        inp = _to_dev(input, dev).reshape(B, 7)
        foot = _to_dev(foot_op, dev).reshape(B, 12)
        cont = _to_dev(contact, dev).reshape(B, 4)
        st = _stream_handle(None)
        # gait timer at the MPC rate (:106)
        _lib.check(self.L.mpxg_timer_run(st, B, 4, self.duty_factor, self.step_freq, 1.0 / self.mpc_frequency,
                                         _ptr(self.contact_time), _ptr(self.contact)), None, "mpxg_timer_run")
        # reference generator (:110-120)
        f0 = (_lib.ctypes.c_float * 12)(*self.foot0.tolist())
        _lib.check(self.L.mpxg_refgen_srbd(st, B, self.N, self.N, float(self.config.dt), f0, self.duty_factor,
                                           self.step_freq, self.step_height, self.clearence_speed,
                                           _ptr(self.contact_time), _ptr(x0), _ptr(foot), _ptr(inp), _ptr(cont),
                                           _ptr(self.liftoff), _ptr(self.reference), _ptr(self.parameter),
                                           _ptr(self._foot_ref_dot_all)), None, "mpxg_refgen_srbd")
        self.foot_ref = self.parameter[:, 0, 4:]
        self.foot_ref_dot = self._foot_ref_dot_all[:, 0, :]
        # solve (:124-132)
        out = dict(X=self.X, U=self.U, V=self.V, kkt=self.kkt, status=self.status)
        io = self.solver.io(x0, self.batch_X0, self.batch_U0, self.batch_V0, self.reference, self.parameter, self.w,
                            None, out)
        _lib.check(self.L.mpxg_solve(self.solver.handle, st, _lib.ctypes.byref(io)), self.solver.handle,
                   "mpxg_solve")
        # warm start for the next call (:135-137), then the first control (:139)
        self.solver.shift(self.X, self.U, self.V, None, self.shift, out=(self.batch_X0, self.batch_U0,
                                                                        self.batch_V0))
        self.grf = self.U[:, 0, :]
        self._keep = (x0, inp, foot, cont)
        return 0

    # resident state carried from tick to tick (warm start, gait timers,
    # liftoff positions) and the last tick's outputs
    STATE = ("batch_X0", "batch_U0", "batch_V0", "contact_time", "liftoff", "contact", "grf", "foot_ref",
             "foot_ref_dot")

    def save_state(self):
        """Checkpoint of the controller between ticks as host tensors.  The
        reference keeps the same state in wrapper attributes
        (mpc_wrapper_srbd.py:56-58,82-88) and writes no files.
        load_state() resumes from it here or on another wrapper with the same
        config and n_env (another process or GPU)."""
        return _save_state(self, self.STATE)

    def load_state(self, state):
        """Resume from save_state(); the next run() continues that episode."""
        _load_state(self, self.STATE, state)

    def torch_run(self, x0_torch, input_torch, foot_op_torch, contact_torch=None):
        """mpc_wrapper_srbd.py:143-151 (which calls run() without `contact`);
        here contact defaults to the gait schedule's current contact."""
        if contact_torch is None:
            contact_torch = self.contact.float()
        return self.run(x0_torch, input_torch, foot_op_torch, contact_torch)

    def whole_body_run(self, qpos, qvel):
        """mpc_wrapper_srbd.py:153-154: joint torques for every environment from
        the last tick's grf, foot references and contact flags
        (mpc_utils.py:276-313).  qpos [n_env,nq], qvel [n_env,nv] ->
        (tau [n_env,nv-6], J [n_env,nv,12])."""
        if self.wb is None:
            raise RuntimeError("no whole-body model: set config.model_path to the robot's MJCF or pass wb_model=")
        return self.wb.interface(qpos, qvel, self.grf, self.foot_ref, self.foot_ref_dot, self.contact, self.Kp,
                                 self.Kd)

    def torch_whole_body_run(self, qpos, qvel):
        """mpc_wrapper_srbd.py:156-160 (which hands the (tau, J) pair to DLPack);
        returns the torque tensor."""
        return self.whole_body_run(qpos, qvel)[0]


# ----------------------------------------------------------------- single-instance wrapper
class MPCControllerWrapper:
    """Single-instance controller with the API of mpx/utils/mpc_wrapper.py:194-468,
    on a compiled SRBD model.  The state is the floating base [p, quat, v, omega]
    read from qpos[:7] and qvel[:6]; foot positions are given by the caller."""

    def __init__(self, config, limited_memory=False, opts=None, device=None, desc=None, model=None):
        self._wb = None
        if is_whole_body(config):  # the reference's own whole-body configurations (config_aliengo, config_go2)
            self._wb = WholeBodyController(config, limited_memory, model=model, device=device, opts=opts)
            self.config = config
            return
        self.config = config
        self.dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.mpc_frequency = float(config.mpc_frequency)
        self.shift = int(1 / (config.dt * config.mpc_frequency))
        self.N = int(config.N)
        self.desc = desc or P.quadruped_quat13(config, mu=float(getattr(config, "mu", 0.7)))
        self.n = self.desc.n
        self.opts = opts or P.SolverOptions()
        self.solver = Solver(self.desc, self.opts, n_max=self.N, batch_max=1, device=self.dev)
        self.L = _lib.load()
        self.duty_factor = float(config.duty_factor)
        self.step_freq = float(config.step_freq)
        self.step_height = float(config.step_height)
        self.robot_height = float(getattr(config, "initial_height", getattr(config, "robot_height", 0.3)))
        self.clearence_speed = 0.4  # mpc_wrapper.py:292
        self.foot0 = np.asarray(config.p_legs0, dtype=np.float32)
        W = np.asarray(config.W, dtype=np.float64)
        self.w = _to_dev(np.diag(W).astype(np.float32).reshape(1, -1), self.dev)
        self.contact_time = _to_dev(np.asarray(config.timer_t, dtype=np.float32).reshape(1, 4), self.dev)
        self.liftoff = _to_dev(self.foot0.reshape(1, 12), self.dev)
        x_init = np.concatenate([np.asarray(config.p0, dtype=np.float32), np.asarray(config.quat0, dtype=np.float32),
                                 np.zeros(6, dtype=np.float32)])
        self._set_warm(x_init)
        self.ref = torch.zeros(1, self.N + 1, 17, device=self.dev)
        self.par = torch.zeros(1, self.N + 1, 16, device=self.dev)
        self.frd = torch.zeros(1, self.N + 1, 12, device=self.dev)
        self.cont = torch.zeros(1, 4, dtype=torch.int32, device=self.dev)

    def _set_warm(self, x0):
        N = self.N
        u_ref = np.asarray(self.config.u_ref, dtype=np.float32)
        self.U0 = _to_dev(np.tile(u_ref, (1, N, 1)), self.dev)
        self.X0 = _to_dev(np.tile(np.asarray(x0, dtype=np.float32), (1, N + 1, 1)), self.dev)
        self.V0 = torch.zeros(1, N + 1, self.n, device=self.dev)

    def _state(self, qpos, qvel):
        qpos = np.asarray(qpos, dtype=np.float32)
        qvel = np.asarray(qvel, dtype=np.float32)
        return np.concatenate([qpos[:7], qvel[:6]])

    def run(self, qpos, qvel, input, contact, foot_op=None):
        """mpc_wrapper.py:297-365.  With a whole-body configuration this is the
        reference's controller (wb_wrappers.WholeBodyController): returns
        (tau, q, dq), the joint torques clipped to the configuration's limits
        and the planned joint positions and velocities.  With a compiled SRBD
        model it returns (grf, q, dq): the first control and the floating-base
        pose/velocity of the plan."""
        if getattr(self, "_wb", None) is not None:
            return self._wb.run(qpos, qvel, input, contact)
        x0 = self._state(qpos, qvel)
        foot = np.asarray(foot_op if foot_op is not None else self.foot0 + np.tile(x0[:3], 4), dtype=np.float32)
        inp = np.asarray(input, dtype=np.float32).copy()
        inp[6] = self.robot_height  # :318
        dev, st = self.dev, _stream_handle(None)
        x0d, footd, inpd = _to_dev(x0.reshape(1, -1), dev), _to_dev(foot.reshape(1, -1), dev), _to_dev(inp.reshape(1, -1), dev)
        contd = _to_dev(np.asarray(contact, dtype=np.float32).reshape(1, 4), dev)
        _lib.check(self.L.mpxg_timer_run(st, 1, 4, self.duty_factor, self.step_freq, 1.0 / self.mpc_frequency,
                                         _ptr(self.contact_time), _ptr(self.cont)), None, "mpxg_timer_run")
        f0 = (_lib.ctypes.c_float * 12)(*self.foot0.tolist())
        _lib.check(self.L.mpxg_refgen_srbd(st, 1, self.N, self.N, float(self.config.dt), f0, self.duty_factor,
                                           self.step_freq, self.step_height, self.clearence_speed,
                                           _ptr(self.contact_time), _ptr(x0d), _ptr(footd), _ptr(inpd), _ptr(contd),
                                           _ptr(self.liftoff), _ptr(self.ref), _ptr(self.par), _ptr(self.frd)),
                   None, "mpxg_refgen_srbd")
        out = self.solver.solve(x0d, self.X0, self.U0, self.V0, self.ref, self.par, self.w)
        X, U, V = out["X"], out["U"], out["V"]
        self._update_and_extract(X, U, V, x0)
        grf = U[0, 0].cpu().numpy() if not self._nan else self.U0[0, 1].cpu().numpy()
        q = (X[0, 0] if not self._nan else self.X0[0, 1]).cpu().numpy()[:7]
        dq = (X[0, 1] if not self._nan else self.X0[0, 1]).cpu().numpy()[7:13]
        return grf, q, dq

    STATE = ("X0", "U0", "V0", "contact_time", "liftoff")

    def save_state(self):
        """Checkpoint of the warm start and gait state as host tensors (the
        reference keeps them in attributes, mpc_wrapper.py:367-385)."""
        if getattr(self, "_wb", None) is not None:
            return self._wb.save_state()
        return _save_state(self, self.STATE)

    def load_state(self, state):
        """Resume from save_state()."""
        if getattr(self, "_wb", None) is not None:
            return self._wb.load_state(state)
        _load_state(self, self.STATE, state)

    def _update_and_extract(self, X, U, V, x0):
        """mpc_wrapper.py:261-282: shift the warm start, or on NaN in U[0,0]
        reset it to tiles of u_ref / x0 and zero duals."""
        self._nan = bool(torch.isnan(U[0, 0, 0]).item())
        if self._nan:
            self._set_warm(x0)
        else:
            self.solver.shift(X, U, V, None, self.shift, out=(self.X0, self.U0, self.V0))

    def reset(self, qpos, qvel, foot=None):
        """mpc_wrapper.py:367-385."""
        if getattr(self, "_wb", None) is not None:
            return self._wb.reset(qpos, qvel)
        x0 = self._state(qpos, qvel)
        self.contact_time = _to_dev(np.asarray(self.config.timer_t, dtype=np.float32).reshape(1, 4), self.dev)
        lo = self.foot0 if foot is None else np.asarray(foot, dtype=np.float32)
        self.liftoff = _to_dev(lo.reshape(1, 12), self.dev)
        self._set_warm(x0)
        print("MPC Controller Reset")

    def runOffline(self, qpos, qvel, reference=None, parameter=None, max_iter=100):
        """mpc_wrapper.py:387-468: repeat single SQP iterations until the
        reference's stop rule  last_cost - cost < 1e-3 and sum(c^2) < 1e-5
        (:465), with cost the objective (sum of the stage costs) and c the
        defects.  `reference`/`parameter` are the offline tables
        ([N+1, 17] and [N+1, 16] for the compiled SRBD model); by default
        they come, as in the reference (:411), from
        config.reference(N+1, dt, n_joints, n_contact, p_legs0, q0)."""
        if getattr(self, "_wb", None) is not None:
            return self._wb.runOffline(qpos, qvel, reference, parameter, max_iter)
        if reference is None or parameter is None:
            make = getattr(self.config, "reference", None)
            if make is None:
                raise ValueError("runOffline needs the offline tables: pass reference and parameter, or give the "
                                 "config a reference(N+1, dt, n_joints, n_contact, p_legs0, q0) function")
            reference, parameter = make(self.N + 1, self.config.dt, getattr(self.config, "n_joints", 12),
                                        getattr(self.config, "n_contact", 4), self.config.p_legs0,
                                        getattr(self.config, "q0", None))
        x0 = _to_dev(self._state(qpos, qvel).reshape(1, -1), self.dev)
        ref = _to_dev(reference, self.dev).reshape(1, self.N + 1, -1)
        par = _to_dev(parameter, self.dev).reshape(1, self.N + 1, -1)
        one = Solver(self.desc, P.SolverOptions(sqp_iters=1), n_max=self.N, batch_max=1, device=self.dev)
        X, U, V = self.X0.clone(), self.U0.clone(), self.V0.clone()
        last = 1e10
        outputs = [X.clone()]
        for it in range(max_iter + 1):
            out = one.solve(x0, X, U, V, ref, par, self.w, out=dict(X=X, U=U, V=V, kkt=torch.zeros(1, 3, device=self.dev),
                                                                   status=torch.zeros(1, dtype=torch.int32, device=self.dev)))
            outputs.append(X.clone())
            g, c = one.evaluate(x0, X, U, ref, par, self.w)   # model_evaluator_helper (:452)
            cost = float(torch.sum(g).item())
            csq = float(torch.sum(c * c).item())
            if last - cost < 1e-3 and csq < 1e-5:
                break
            last = cost
        self.X0, self.U0, self.V0 = X, U, V
        return X, U, reference, outputs


class mpx_data(dict):
    """The controller record of mpx/utils/mpc_wrapper.py:16-27 (dt,
    duty_factor, step_freq, step_height, contact_time, liftoff, X0, U0, V0, W,
    grf), for all environments at once: the array fields are device tensors
    with a leading env dimension.  Fields read as items (data["X0"]) or, as
    on the reference's flax PyTreeNode, as attributes (data.X0), and
    replace(**fields) returns an updated copy."""

    FIELDS = ("dt", "duty_factor", "step_freq", "step_height", "contact_time", "liftoff", "X0", "U0", "V0", "W",
              "grf")

    def __getattr__(self, name):
        try:
            return self[name]
        except KeyError:
            raise AttributeError(name) from None

    def replace(self, **fields):
        return mpx_data(self, **fields)


class BatchedDataMPCWrapper:
    """The mpx_data API of mpx/utils/mpc_wrapper.py:16-192: a per-environment
    data record and run(data, x0, input) -> (data, grf), on a compiled SRBD
    model.  `data` is an mpx_data (a dict of device tensors with a leading env
    dimension); a plain dict with the same keys is accepted too."""

    def __init__(self, config, n_env, limited_memory=False, opts=None, device=None, desc=None, model=None):
        self.config = config
        self.n_env = int(n_env)
        self._wb = None
        if is_whole_body(config):  # the reference's own whole-body configurations
            self._wb = WholeBodyBatchedController(config, n_env, limited_memory, model=model, device=device,
                                                  opts=opts)
            return
        self.dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.N = int(config.N)
        self.shift = int(1 / (config.dt * config.mpc_frequency))
        self.mpc_frequency = float(config.mpc_frequency)
        self.desc = desc or P.quadruped_quat13(config, mu=float(getattr(config, "mu", 0.7)))
        self.solver = Solver(self.desc, opts or P.SolverOptions(), n_max=self.N, batch_max=self.n_env, device=self.dev)
        self.L = _lib.load()
        self.foot0 = np.asarray(config.p_legs0, dtype=np.float32)
        self.initial_state = np.concatenate([np.asarray(config.p0, dtype=np.float32),
                                             np.asarray(config.quat0, dtype=np.float32),
                                             np.zeros(6, dtype=np.float32)])

    def make_data(self):
        """mpc_wrapper.py:100-113, for all environments at once."""
        if getattr(self, "_wb", None) is not None:
            return self._wb.make_data()
        B, N = self.n_env, self.N
        dev = self.dev
        W = np.diag(np.asarray(self.config.W, dtype=np.float64)).astype(np.float32)
        return mpx_data(
            dt=float(self.config.dt), duty_factor=float(self.config.duty_factor),
            step_freq=float(self.config.step_freq), step_height=float(self.config.step_height),
            contact_time=_to_dev(np.tile(np.asarray(self.config.timer_t, dtype=np.float32), (B, 1)), dev),
            liftoff=torch.zeros(B, 12, device=dev),
            X0=_to_dev(np.tile(self.initial_state, (B, N + 1, 1)), dev),
            U0=_to_dev(np.tile(np.asarray(self.config.u_ref, dtype=np.float32), (B, N, 1)), dev),
            V0=torch.zeros(B, N + 1, self.desc.n, device=dev),
            W=_to_dev(np.tile(W, (B, 1)), dev),
            grf=torch.zeros(B, 12, device=dev))

    def run(self, data, x0, input, foot_op=None):
        """mpc_wrapper.py:115-170: timer, reference, solve, NaN-guarded warm
        start; returns (data, grf), or with a whole-body configuration
        (data, tau) as the reference does."""
        if getattr(self, "_wb", None) is not None:
            return self._wb.run(data, x0, input)
        B, N, dev, st = self.n_env, self.N, self.dev, _stream_handle(None)
        x0 = _to_dev(x0, dev).reshape(B, -1)
        inp = _to_dev(input, dev).reshape(B, 7)
        foot = _to_dev(foot_op, dev).reshape(B, 12) if foot_op is not None else \
            (x0[:, :3].repeat(1, 4) + _to_dev(self.foot0, dev).reshape(1, 12))
        ct = data["contact_time"].clone()
        cont = torch.zeros(B, 4, dtype=torch.int32, device=dev)
        ref = torch.zeros(B, N + 1, 17, device=dev)
        par = torch.zeros(B, N + 1, 16, device=dev)
        frd = torch.zeros(B, N + 1, 12, device=dev)
        lo = data["liftoff"].clone()
        f0 = (_lib.ctypes.c_float * 12)(*self.foot0.tolist())
        zero_contact = torch.zeros(B, 4, device=dev)  # mpc_wrapper.py:134
        _lib.check(self.L.mpxg_refgen_srbd(st, B, N, N, float(data["dt"]), f0, data["duty_factor"],
                                           data["step_freq"], data["step_height"], 0.2,
                                           _ptr(data["contact_time"]), _ptr(x0), _ptr(foot), _ptr(inp),
                                           _ptr(zero_contact), _ptr(lo), _ptr(ref), _ptr(par), _ptr(frd)),
                   None, "mpxg_refgen_srbd")
        _lib.check(self.L.mpxg_timer_run(st, B, 4, data["duty_factor"], data["step_freq"], 1.0 / self.mpc_frequency,
                                         _ptr(ct), _ptr(cont)), None, "mpxg_timer_run")
        out = self.solver.solve(x0, data["X0"], data["U0"], data["V0"], ref, par, data["W"])
        X, U, V = out["X"], out["U"], out["V"]
        nan = torch.isnan(U[:, 0, 0])
        X0n, U0n, V0n = X.clone(), U.clone(), V.clone()
        self.solver.shift(X0n, U0n, V0n, None, self.shift)
        if bool(nan.any()):
            u_ref = _to_dev(np.asarray(self.config.u_ref, dtype=np.float32), dev)
            X0n[nan] = x0[nan].unsqueeze(1).expand(-1, N + 1, -1)
            U0n[nan] = u_ref.reshape(1, 1, -1).expand(int(nan.sum()), N, -1)
            V0n[nan] = 0.0
        grf = torch.where(nan.unsqueeze(1), data["U0"][:, 1, :], U[:, 0, :])
        data = mpx_data(data, X0=X0n, U0=U0n, V0=V0n, contact_time=ct, liftoff=lo, grf=grf)
        return data, grf

    def reset(self, data, qpos, qvel=None, foot=None):
        """mpc_wrapper.py:172-192, called as there with (data, qpos, qvel,
        foot): the compiled model's state is the floating base, qpos[:, :7]
        followed by qvel[:, :6].  Called as (data, x0), qpos is that state.
        With a whole-body configuration the state is [qpos, qvel, foot, 0]."""
        if getattr(self, "_wb", None) is not None:
            return self._wb.reset(data, qpos, qvel, foot)
        B, N, dev = self.n_env, self.N, self.dev
        x0 = _to_dev(qpos, dev).reshape(B, -1)
        if qvel is not None:
            x0 = torch.cat([x0[:, :7], _to_dev(qvel, dev).reshape(B, -1)[:, :6]], 1).contiguous()
        return mpx_data(data, contact_time=_to_dev(np.tile(np.asarray(self.config.timer_t, dtype=np.float32), (B, 1)), dev),
                    liftoff=_to_dev(foot, dev).reshape(B, 12) if foot is not None else torch.zeros(B, 12, device=dev),
                    X0=x0.unsqueeze(1).expand(-1, N + 1, -1).contiguous(),
                    U0=_to_dev(np.tile(np.asarray(self.config.u_ref, dtype=np.float32), (B, N, 1)), dev),
                    V0=torch.zeros(B, N + 1, self.desc.n, device=dev), grf=torch.zeros(B, 12, device=dev))
