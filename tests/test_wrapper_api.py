"""The wrapper API against the reference's (CPU; no kernel runs).

A caller of the reference switches by its import line: mpx_gb300.mpc_wrapper
and mpx_gb300.mpc_wrapper_srbd export the reference modules' names, and each
method takes the reference's parameters, in the reference's order, first.
"""
import inspect
import types

import numpy as np
import torch

from mpx_gb300 import mpc_wrapper, mpc_wrapper_srbd, wrappers

# (class, method) -> the reference's parameters after self
REFERENCE_SIGNATURES = {
    # mpx/utils/mpc_wrapper_srbd.py:20,91,143,153,156,162
    (mpc_wrapper_srbd.BatchedMPCControllerWrapper, "__init__"): ["config", "n_env"],
    (mpc_wrapper_srbd.BatchedMPCControllerWrapper, "run"): ["x0", "input", "foot_op", "contact"],
    (mpc_wrapper_srbd.BatchedMPCControllerWrapper, "torch_run"): ["x0_torch", "input_torch", "foot_op_torch"],
    (mpc_wrapper_srbd.BatchedMPCControllerWrapper, "whole_body_run"): ["qpos", "qvel"],
    (mpc_wrapper_srbd.BatchedMPCControllerWrapper, "torch_whole_body_run"): ["qpos", "qvel"],
    (mpc_wrapper_srbd.BatchedMPCControllerWrapper, "reset"): [],
    # mpx/utils/mpc_wrapper.py:30,100,115,172
    (mpc_wrapper.BatchedMPCControllerWrapper, "__init__"): ["config", "n_env", "limited_memory"],
    (mpc_wrapper.BatchedMPCControllerWrapper, "make_data"): [],
    (mpc_wrapper.BatchedMPCControllerWrapper, "run"): ["data", "x0", "input"],
    (mpc_wrapper.BatchedMPCControllerWrapper, "reset"): ["data", "qpos", "qvel", "foot"],
    # mpx/utils/mpc_wrapper.py:195,297,367,387
    (mpc_wrapper.MPCControllerWrapper, "__init__"): ["config", "limited_memory"],
    (mpc_wrapper.MPCControllerWrapper, "run"): ["qpos", "qvel", "input", "contact"],
    (mpc_wrapper.MPCControllerWrapper, "reset"): ["qpos", "qvel"],
    (mpc_wrapper.MPCControllerWrapper, "runOffline"): ["qpos", "qvel"],
}


def test_reference_module_names():
    assert mpc_wrapper_srbd.BatchedMPCControllerWrapper is wrappers.BatchedMPCControllerWrapper
    assert mpc_wrapper.BatchedMPCControllerWrapper is wrappers.BatchedDataMPCWrapper
    assert mpc_wrapper.MPCControllerWrapper is wrappers.MPCControllerWrapper
    assert mpc_wrapper.mpx_data is wrappers.mpx_data


def test_reference_parameters_come_first_in_order():
    for (cls, name), ref in REFERENCE_SIGNATURES.items():
        params = list(inspect.signature(getattr(cls, name)).parameters.values())[1:]
        assert [p.name for p in params[:len(ref)]] == ref, (cls.__name__, name)
        # anything we add after the reference's parameters has a default
        for p in params[len(ref):]:
            assert p.default is not inspect.Parameter.empty, (cls.__name__, name, p.name)


def test_mpx_data_record():
    # mpx/utils/mpc_wrapper.py:16-27
    assert wrappers.mpx_data.FIELDS == ("dt", "duty_factor", "step_freq", "step_height", "contact_time", "liftoff",
                                        "X0", "U0", "V0", "W", "grf")
    d = wrappers.mpx_data(dt=0.02, X0=torch.zeros(2, 3, 4))
    assert d.dt == 0.02 and d["dt"] == 0.02 and d.X0 is d["X0"]
    e = d.replace(dt=0.01)
    assert isinstance(e, wrappers.mpx_data) and e.dt == 0.01 and d.dt == 0.02 and e.X0 is d.X0
    try:
        d.grf
    except AttributeError:
        pass
    else:
        raise AssertionError("a missing field must raise AttributeError")
    # copies and pickles as a record of the same type
    import copy
    import pickle
    for e2 in (copy.copy(e), copy.deepcopy(e), pickle.loads(pickle.dumps(e))):
        assert isinstance(e2, wrappers.mpx_data) and e2.dt == 0.01 and torch.equal(e2.X0, e.X0)


def _cpu_data_wrapper(B=3, N=5):
    """A BatchedDataMPCWrapper with its host state on the CPU (no solver)."""
    w = object.__new__(wrappers.BatchedDataMPCWrapper)
    w.n_env, w.N, w.dev = B, N, torch.device("cpu")
    w.config = types.SimpleNamespace(timer_t=np.array([0.5, 0.0, 0.0, 0.5]), u_ref=np.arange(12.0))
    w.desc = types.SimpleNamespace(n=13)
    return w


def test_data_reset_with_the_reference_arguments():
    """reset(data, qpos, qvel, foot) as in mpc_wrapper.py:172-192: the state
    is the floating base qpos[:, :7] ++ qvel[:, :6]; the same as reset(data,
    x0) with that state."""
    B, N = 3, 5
    w = _cpu_data_wrapper(B, N)
    rng = np.random.default_rng(0)
    qpos = rng.normal(size=(B, 19)).astype(np.float32)
    qvel = rng.normal(size=(B, 18)).astype(np.float32)
    foot = rng.normal(size=(B, 12)).astype(np.float32)
    d = w.reset(wrappers.mpx_data(dt=0.02), qpos, qvel, foot)
    x0 = np.concatenate([qpos[:, :7], qvel[:, :6]], 1)
    assert isinstance(d, wrappers.mpx_data) and d.dt == 0.02
    assert d.X0.shape == (B, N + 1, 13)
    assert np.array_equal(d.X0.numpy(), np.repeat(x0[:, None], N + 1, 1))
    assert np.array_equal(d.liftoff.numpy(), foot)
    assert np.array_equal(d.U0.numpy(), np.tile(np.arange(12.0, dtype=np.float32), (B, N, 1)))
    assert np.array_equal(d.contact_time.numpy(), np.tile(np.float32([0.5, 0, 0, 0.5]), (B, 1)))
    assert not d.V0.any() and not d.grf.any()
    d2 = w.reset(wrappers.mpx_data(dt=0.02), x0, foot=foot)
    for k in ("X0", "U0", "V0", "liftoff", "contact_time", "grf"):
        assert torch.equal(d[k], d2[k]), k


def test_run_offline_without_tables_says_what_it_needs():
    w = object.__new__(wrappers.MPCControllerWrapper)
    w.config = types.SimpleNamespace(dt=0.02, p_legs0=np.zeros(12))
    w.N = 5
    try:
        w.runOffline(np.zeros(19), np.zeros(18))
    except ValueError as e:
        assert "reference and parameter" in str(e)
    else:
        raise AssertionError("runOffline without tables must raise ValueError")


def test_save_and_load_state_round_trip():
    """save_state() checkpoints the tick-to-tick state as host tensors;
    load_state() restores it with the holder's device and dtype, into a
    wrapper of the same shape, and refuses a checkpoint of another shape."""
    rng = np.random.default_rng(1)
    B, N = 3, 6

    def srbd():
        w = object.__new__(wrappers.BatchedMPCControllerWrapper)
        w.batch_X0, w.batch_U0, w.batch_V0 = (torch.zeros(B, N + 1, 13), torch.zeros(B, N, 12),
                                              torch.zeros(B, N + 1, 13))
        w.contact_time, w.liftoff = torch.zeros(B, 4), torch.zeros(B, 12)
        w.contact = torch.zeros(B, 4, dtype=torch.int32)
        w.grf, w.foot_ref, w.foot_ref_dot = torch.zeros(B, 12), torch.zeros(B, 12), torch.zeros(B, 12)
        return w

    a = srbd()
    for k in a.STATE:
        t = getattr(a, k)
        setattr(a, k, torch.as_tensor(rng.normal(size=t.shape) * 5).to(t.dtype))
    st = a.save_state()
    assert set(st) == set(a.STATE) and all(v.device.type == "cpu" for v in st.values())
    b = srbd()
    b.load_state(st)
    for k in a.STATE:
        assert torch.equal(getattr(a, k), getattr(b, k)) and getattr(b, k).dtype == getattr(a, k).dtype, k
    a.batch_X0 += 1  # the checkpoint is a copy
    assert not torch.equal(a.batch_X0, st["batch_X0"])
    small = srbd()
    small.batch_X0 = torch.zeros(B, N, 13)
    try:
        small.load_state(st)
    except ValueError as e:
        assert "batch_X0" in str(e)
    else:
        raise AssertionError("a checkpoint of another shape must be refused")
    # nothing was replaced by the refused load
    assert small.batch_X0.shape == (B, N, 13) and not small.contact_time.any()

    s = object.__new__(wrappers.MPCControllerWrapper)
    s.X0, s.U0, s.V0 = torch.ones(1, N + 1, 13), torch.ones(1, N, 12), torch.ones(1, N + 1, 13)
    s.contact_time, s.liftoff = torch.full((1, 4), 0.25), torch.ones(1, 12)
    st = s.save_state()
    s.X0 = torch.zeros(1, N + 1, 13)
    s.load_state(st)
    assert torch.equal(s.X0, torch.ones(1, N + 1, 13))


def test_whole_body_configurations_are_recognised():
    """mpc_wrapper.py's controllers hand whole-body configurations (13 + 2 nj
    + 6 C states, config_aliengo / config_go2) to the whole-body solve and
    keep the SRBD ones; W must be diagonal; SolverOptions map onto the
    whole-body solve's options."""
    import numpy as np
    from mpx_gb300 import configs, problem as P, wb_wrappers
    wb, srbd = configs.aliengo_wb(), configs.srbd_quadruped()
    assert wb_wrappers.is_whole_body(wb) and not wb_wrappers.is_whole_body(srbd)
    assert wb.n == 61 and wb_wrappers._w_diag(wb).shape == (72,)
    W = np.diag(wb.W_diag.astype(np.float64))
    W[0, 1] = 1.0
    bad = types.SimpleNamespace(W=W)
    try:
        wb_wrappers._w_diag(bad)
        raise AssertionError("a W with off-diagonal entries was accepted")
    except ValueError:
        pass
    kw = wb_wrappers._sqp_kwargs(P.SolverOptions(sqp_iters=3, ls_max_trials=6))
    assert kw["iters"] == 3 and kw["ls_max_trials"] == 6
    assert wb_wrappers._sqp_kwargs(None) == {} and wb_wrappers._sqp_kwargs({"iters": 2}) == {"iters": 2}
