"""Whole-body rigid-body terms and the SRBD controller's whole-body torque
interface on the GPU (mpx/utils/mpc_utils.py:275-313), through
mpxg_wb_terms / mpxg_wb_interface of libmpxg.

    wb = WholeBodyModel.from_mjcf("aliengo.xml", ["FL", "FR", "RL", "RR"],
                                  ["FL_calf", "FR_calf", "RL_calf", "RR_calf"])
    tau, J = wb.interface(qpos, qvel, grf, foot_ref, foot_ref_dot, contact, Kp, Kd)

All arrays are batched over environments on the model's device (float32;
contact int32).  There is no CPU path: without the library the calls raise.
"""
import torch

from . import _lib
from . import mjcf
from .solver import _ptr, _stream_handle


def _dev(a, dev, dtype=torch.float32):
    if isinstance(a, torch.Tensor):
        return a.to(device=dev, dtype=dtype).contiguous()
    return torch.as_tensor(a, dtype=dtype, device=dev).contiguous()


class WholeBodyModel:
    def __init__(self, model, device=None):
        """model: an mjcf.RigidBodyModel with contacts set."""
        if model.contact_point_body is None:
            raise ValueError("the model needs contact points (mjcf.RigidBodyModel.with_contacts)")
        self.model = model
        self.struct = model.to_struct()
        self.dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.nq, self.nv, self.nc = model.nq, model.nv, len(model.contact_point_body)
        self.L = _lib.load()

    @classmethod
    def from_mjcf(cls, path, contact_geoms, contact_bodies, device=None):
        return cls(mjcf.parse(path, contact_geoms, contact_bodies), device=device)

    def terms(self, qpos, qvel, stream=None):
        """dict M [B,nv,nv], bias [B,nv], cpos [B,3C], J [B,nv,3C], cvel [B,3C]."""
        qpos = _dev(qpos, self.dev).reshape(-1, self.nq)
        qvel = _dev(qvel, self.dev).reshape(-1, self.nv)
        B, nv, nr = qpos.shape[0], self.nv, 3 * self.nc
        if qvel.shape[0] != B:
            raise ValueError("qpos and qvel batch sizes differ")
        out = dict(M=torch.empty(B, nv, nv, device=self.dev), bias=torch.empty(B, nv, device=self.dev),
                   cpos=torch.empty(B, nr, device=self.dev), J=torch.empty(B, nv, nr, device=self.dev),
                   cvel=torch.empty(B, nr, device=self.dev))
        _lib.check(self.L.mpxg_wb_terms(_stream_handle(stream), _lib.ctypes.byref(self.struct), B, _ptr(qpos),
                                        _ptr(qvel), _ptr(out["M"]), _ptr(out["bias"]), _ptr(out["cpos"]),
                                        _ptr(out["J"]), _ptr(out["cvel"])), None, "mpxg_wb_terms")
        return out

    def interface(self, qpos, qvel, grf, foot_ref, foot_ref_dot, contact, Kp, Kd, stream=None, with_jacobian=True):
        """mpc_utils.py:276-313 for every environment -> (tau [B,nv-6], J [B,nv,3C] or None)."""
        qpos = _dev(qpos, self.dev).reshape(-1, self.nq)
        B, nr = qpos.shape[0], 3 * self.nc
        qvel = _dev(qvel, self.dev).reshape(B, self.nv)
        grf = _dev(grf, self.dev).reshape(B, nr)
        foot_ref = _dev(foot_ref, self.dev).reshape(B, nr)
        foot_ref_dot = _dev(foot_ref_dot, self.dev).reshape(B, nr)
        contact = _dev(contact, self.dev, torch.int32).reshape(B, self.nc)
        Kp = _dev(Kp, self.dev).reshape(nr, nr)
        Kd = _dev(Kd, self.dev).reshape(nr, nr)
        tau = torch.empty(B, self.nv - 6, device=self.dev)
        J = torch.empty(B, self.nv, nr, device=self.dev) if with_jacobian else None
        _lib.check(self.L.mpxg_wb_interface(_stream_handle(stream), _lib.ctypes.byref(self.struct), B, _ptr(qpos),
                                            _ptr(qvel), _ptr(grf), _ptr(foot_ref), _ptr(foot_ref_dot),
                                            _ptr(contact), _ptr(Kp), _ptr(Kd), _ptr(tau), _ptr(J)), None,
                   "mpxg_wb_interface")
        return tau, J

    def step(self, x, u, contact, dt, alpha=25.0, stream=None):
        """One step of the whole-body MPC model (mpx/utils/models.py:39-117)
        for every row: x [B, nq + nv + 6C], u [B, nv - 6], contact [B, C] ->
        x_next [B, nq + nv + 6C]."""
        nr = 3 * self.nc
        nx = self.nq + self.nv + 2 * nr
        x = _dev(x, self.dev).reshape(-1, nx)
        B = x.shape[0]
        u = _dev(u, self.dev).reshape(B, self.nv - 6)
        contact = _dev(contact, self.dev, torch.int32).reshape(B, self.nc)
        out = torch.empty(B, nx, device=self.dev)
        _lib.check(self.L.mpxg_wb_step(_stream_handle(stream), _lib.ctypes.byref(self.struct), B, float(dt),
                                       float(alpha), _ptr(x), _ptr(u), _ptr(contact), _ptr(out)), None,
                   "mpxg_wb_step")
        return out


class WholeBodySQP:
    """Batched SQP solve of the whole-body MPC (mpxg_wb_sqp): the solve that
    mpc_wrapper.py's wrappers call each tick (optimizers.mpc over
    quadruped_wb_dynamics / quadruped_wb_obj / quadruped_wb_hessian_gn,
    mpc_wrapper.py:67,150-158,236,346-354).

        sqp = WholeBodySQP(WholeBodyModel.from_mjcf(...), N=25, batch_max=64)
        out = sqp.solve(x0, X0, U0, V0, reference, contact, W)

    x0 [B,nx], X0 [B,N+1,nx], U0 [B,N,nj], V0 [B,N+1,nx], reference
    [B,N+1,13+nj+7C], contact [B,N+1,C], W [B,12+3nj+6C] or [12+3nj+6C]
    (the diagonal of the reference's W) -> dict X, U, V, kkt [B,3], status
    [B].  The workspace is allocated once, for batch_max instances."""

    def __init__(self, wb, N, batch_max, dt=0.02, alpha=25.0, swing_tracking=True, iters=5, reg=1e-6, rho0=1.0,
                 ls_beta=0.5, ls_eta=1e-4, ls_skip_tol=1e-7, ls_max_trials=8):
        self.wb, self.N, self.batch_max, self.iters = wb, int(N), int(batch_max), int(iters)
        self.nj, self.nc = wb.nv - 6, wb.nc
        self.nx = wb.nq + wb.nv + 6 * wb.nc
        self.nR = 12 + 3 * self.nj + 6 * self.nc
        self.ncol = 13 + self.nj + 7 * self.nc
        self.dev, self.L = wb.dev, wb.L
        nbytes = self.L.mpxg_wb_sqp_workspace_bytes(_lib.ctypes.byref(wb.struct), self.batch_max, self.N)
        if nbytes == 0:
            raise ValueError("mpxg_wb_sqp does not take this model or size: %s" %
                             self.L.mpxg_last_error(None).decode())
        self.workspace = torch.empty(int(nbytes), dtype=torch.uint8, device=self.dev)
        self.opts = dict(dt=float(dt), alpha=float(alpha), swing_tracking=int(bool(swing_tracking)), reg=float(reg),
                         rho0=float(rho0), ls_beta=float(ls_beta), ls_eta=float(ls_eta),
                         ls_skip_tol=float(ls_skip_tol), ls_max_trials=int(ls_max_trials))

    def solve(self, x0, X, U, V, reference, contact, W, iters=None, stream=None, inplace=False, kkt=True):
        N, nx, nj = self.N, self.nx, self.nj
        x0 = _dev(x0, self.dev).reshape(-1, nx)
        B = x0.shape[0]
        if B > self.batch_max:
            raise ValueError("batch %d exceeds batch_max %d" % (B, self.batch_max))

        def state(a, shape):
            t = _dev(a, self.dev)
            if t.numel() != int(torch.tensor(shape).prod()):
                raise ValueError("expected %s elements for shape %s, got %s" % (int(torch.tensor(shape).prod()),
                                                                               shape, tuple(t.shape)))
            t = t.reshape(shape)
            return t if inplace else t.clone()

        X, U, V = state(X, (B, N + 1, nx)), state(U, (B, N, nj)), state(V, (B, N + 1, nx))
        ref = _dev(reference, self.dev).reshape(B, N + 1, self.ncol)
        cont = _dev(contact, self.dev, torch.int32).reshape(B, N + 1, self.nc)
        Wd = _dev(W, self.dev)
        Wd = (Wd.reshape(1, self.nR).expand(B, self.nR) if Wd.numel() == self.nR else Wd.reshape(B, self.nR))
        Wd = Wd.contiguous()
        kk = torch.empty(B, 3, device=self.dev) if kkt else None
        st = torch.empty(B, dtype=torch.int32, device=self.dev)
        io = _lib.WbSqpIO(model=_lib.ctypes.pointer(self.wb.struct), batch=B, N=N,
                          iters=self.iters if iters is None else int(iters), **self.opts)
        for k, t in (("x0", x0), ("X", X), ("U", U), ("V", V), ("reference", ref), ("contact", cont), ("W", Wd),
                     ("kkt", kk), ("status", st), ("workspace", self.workspace)):
            setattr(io, k, _ptr(t))
        _lib.check(self.L.mpxg_wb_sqp(_stream_handle(stream), _lib.ctypes.byref(io)), None, "mpxg_wb_sqp")
        return dict(X=X, U=U, V=V, kkt=kk, status=st)
