"""Gait timer (bit-exact), reference generator and warm-start shift on the GPU."""
import ctypes

import numpy as np
import pytest
import torch

from mpx_gb300 import _lib
from mpx_gb300 import problem as P
from mpx_gb300.solver import Solver

pytestmark = pytest.mark.gpu


def test_timer_bit_exact(oracle, cuda):
    L = _lib.load()
    rng = np.random.default_rng(0)
    lt0 = rng.uniform(0, 1, size=(257, 4)).astype(np.float32)
    duty, freq, dt = 0.65, 1.35, 0.02
    lt = torch.tensor(lt0, device="cuda")
    ct = torch.empty(257, 4, dtype=torch.int32, device="cuda")
    ref_lt = lt0.copy()
    for step in range(300):
        st = L.mpxg_timer_run(None, 257, 4, duty, freq, dt, ctypes.c_void_p(lt.data_ptr()), ctypes.c_void_p(ct.data_ptr()))
        assert st == 0
        c_ref = np.zeros((257, 4), dtype=np.int32)
        for b in range(257):
            c_ref[b], ref_lt[b] = oracle.timer_run(duty, freq, dt, ref_lt[b])
        torch.cuda.synchronize()
        assert np.array_equal(ct.cpu().numpy(), c_ref)
        assert np.array_equal(lt.cpu().numpy().view(np.uint32), ref_lt.view(np.uint32))


def test_refgen_matches_oracle(oracle, cuda):
    L = _lib.load()
    rng = np.random.default_rng(1)
    B, N = 16, 25
    foot0 = np.array([0.27092872, 0.193, 0.0, 0.27092872, -0.193, 0.0, -0.20887128, 0.193, 0.0,
                      -0.20887128, -0.193, 0.0], dtype=np.float32)
    t_timer = rng.uniform(0, 1, (B, 4)).astype(np.float32)
    x = np.zeros((B, 13), dtype=np.float32)
    x[:, 0:3] = rng.normal(0, 0.1, (B, 3)); x[:, 2] += 0.33
    q = rng.normal(0, 0.1, (B, 4)); q[:, 0] += 1; q /= np.linalg.norm(q, axis=1, keepdims=True)
    x[:, 3:7] = q; x[:, 7:13] = rng.normal(0, 0.3, (B, 6))
    foot = (np.tile(foot0, (B, 1)) + rng.normal(0, 0.02, (B, 12))).astype(np.float32)
    inp = np.concatenate([rng.uniform(-1, 1, (B, 3)), rng.uniform(-0.5, 0.5, (B, 3)), np.full((B, 1), 0.35)], 1).astype(np.float32)
    contact = rng.integers(0, 2, (B, 4)).astype(np.float32)
    liftoff = (foot + rng.normal(0, 0.01, (B, 12))).astype(np.float32)
    args = dict(duty_factor=0.65, step_freq=1.35, step_height=0.065, clearence_speed=0.4)
    dev = lambda a: torch.tensor(a, device="cuda")
    tl = [dev(a) for a in (t_timer, x, foot, inp, contact, liftoff)]
    refd = torch.zeros(B, N + 1, 17, device="cuda"); pard = torch.zeros(B, N + 1, 16, device="cuda")
    frdd = torch.zeros(B, N + 1, 12, device="cuda")
    f0 = (ctypes.c_float * 12)(*foot0.tolist())
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    st = L.mpxg_refgen_srbd(None, B, N, N, 0.02, f0, args["duty_factor"], args["step_freq"], args["step_height"],
                            args["clearence_speed"], *[p(t) for t in tl], p(refd), p(pard), p(frdd))
    assert st == 0
    torch.cuda.synchronize()
    for b in range(B):
        r, pa, lo, frd = oracle.refgen_srbd(N, 0.02, 24.637, foot0, args["duty_factor"], args["step_freq"],
                                            args["step_height"], args["clearence_speed"], t_timer[b], x[b], foot[b],
                                            inp[b], contact[b], liftoff[b])
        g_ref, g_par, g_frd = refd[b].cpu().numpy(), pard[b].cpu().numpy(), frdd[b].cpu().numpy()
        assert np.array_equal(g_ref[:, 13:17], r[:, 13:17])  # contact schedule: bit-exact
        assert np.array_equal(g_par[:, 0:4], pa[:, 0:4])
        np.testing.assert_allclose(g_ref, r, rtol=2e-6, atol=2e-6)
        np.testing.assert_allclose(g_par, pa, rtol=2e-6, atol=2e-6)
        np.testing.assert_allclose(g_frd, frd, rtol=1e-5, atol=1e-5)
        np.testing.assert_allclose(tl[5][b].cpu().numpy(), lo, rtol=2e-6, atol=2e-6)


def test_shift_matches_host(cuda):
    wl = P.quadruped_workload(5, horizons=(10, 20), seed=3)
    s = Solver(wl.desc, P.SolverOptions(), n_max=wl.n_max, batch_max=5)
    rng = np.random.default_rng(2)
    X = rng.standard_normal(wl.X0.shape).astype(np.float32)
    U = rng.standard_normal(wl.U0.shape).astype(np.float32)
    V = rng.standard_normal(wl.V0.shape).astype(np.float32)
    Xe, Ue, Ve = P.shift_warm_start(X, U, V, wl.horizon)
    Xd, Ud, Vd = (torch.tensor(a, device="cuda") for a in (X, U, V))
    hz = torch.tensor(wl.horizon, device="cuda")
    s.shift(Xd, Ud, Vd, hz)
    torch.cuda.synchronize()
    for b, N in enumerate(wl.horizon):
        assert np.array_equal(Xd[b, :N + 1].cpu().numpy(), Xe[b, :N + 1])
        assert np.array_equal(Ud[b, :N].cpu().numpy(), Ue[b, :N])
        assert np.array_equal(Vd[b, :N + 1].cpu().numpy(), Ve[b, :N + 1])


def test_refgen_and_timer_match_golden(cuda):
    """CUDA gait timer and reference generator against vectors produced by the
    reference's own source (tests/golden/make_golden.py)."""
    import os
    G = np.load(os.path.join(os.path.dirname(__file__), "golden", "srbd_golden.npz"))
    L = _lib.load()
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    for tag in ("srbd", "trot"):
        duty, freq, dt = [float(v) for v in G["timer_%s_params" % tag]]
        lt = torch.tensor(G["timer_%s_init" % tag], device="cuda")
        ct = torch.empty(lt.shape, dtype=torch.int32, device="cuda")
        for k in range(G["timer_%s_contact" % tag].shape[0]):
            assert L.mpxg_timer_run(None, lt.shape[0], 4, duty, freq, dt, p(lt), p(ct)) == 0
            torch.cuda.synchronize()
            assert np.array_equal(ct.cpu().numpy(), G["timer_%s_contact" % tag][k])
            assert np.array_equal(lt.cpu().numpy().view(np.uint32), G["timer_%s_time" % tag][k].view(np.uint32))
    N, dt, mass, duty, freq, sh, cl = [float(v) for v in G["refgen_cfg"]]
    N = int(N)
    R = G["refgen_in_x"].shape[0]
    tl = [torch.tensor(G["refgen_in_" + k], device="cuda") for k in ("t_timer", "x", "foot", "input", "contact", "liftoff")]
    refd = torch.zeros(R, N + 1, 17, device="cuda"); pard = torch.zeros(R, N + 1, 16, device="cuda")
    frdd = torch.zeros(R, N + 1, 12, device="cuda")
    f0 = (ctypes.c_float * 12)(*G["refgen_foot0"].tolist())
    assert L.mpxg_refgen_srbd(None, R, N, N, dt, f0, duty, freq, sh, cl, *[p(t) for t in tl], p(refd), p(pard),
                              p(frdd)) == 0
    torch.cuda.synchronize()
    gref, gpar = G["refgen_out_reference"], G["refgen_out_parameter"]
    assert np.array_equal(refd.cpu().numpy()[:, :, 13:17], gref[:, :, 13:17])
    assert np.array_equal(pard.cpu().numpy()[:, :, 0:4], gpar[:, :, 0:4])
    np.testing.assert_allclose(refd.cpu().numpy(), gref, rtol=2e-6, atol=2e-6)
    np.testing.assert_allclose(pard.cpu().numpy(), gpar, rtol=2e-6, atol=2e-6)
    np.testing.assert_allclose(frdd.cpu().numpy(), G["refgen_out_foot_ref_dot"], rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(tl[5].cpu().numpy(), G["refgen_out_liftoff"], rtol=2e-6, atol=2e-6)


@pytest.mark.parametrize("mode", [0, 1])
def test_gait_tables_match_host_tables(cuda, mode):
    """mpxg_gait_tables (warp per entry, lane per stage) reproduces the host
    trot tables bit for bit, through a slot subset of a pool; mode 0 also
    cold-starts X, V, U; mode 1 first takes x0 from the warm start and
    advances the gait timers one tick."""
    from mpx_gb300.solver import gait_tables
    rng = np.random.default_rng(9)
    desc = P.quadruped_rpy12()
    pool, n_max = 7, 70
    slots = np.array([5, 0, 3, 6], dtype=np.int32)
    horizon = rng.integers(1, n_max + 1, size=pool).astype(np.int32)
    horizon[5] = n_max
    x0 = rng.normal(0, 0.1, (pool, desc.n)).astype(np.float32)
    Xw = rng.normal(0, 0.1, (pool, n_max + 1, desc.n)).astype(np.float32)
    lt = rng.uniform(0, 1, (pool, 4)).astype(np.float32)
    v = rng.uniform(-1, 1, pool).astype(np.float32)
    d = lambda a, dt=torch.float32: torch.as_tensor(a).to("cuda", dt).contiguous()
    tx0, tX, tlt, tv = d(x0), d(Xw), d(lt), d(v)
    tU = torch.zeros(pool, n_max, desc.m, device="cuda")
    tV = torch.ones(pool, n_max + 1, desc.n, device="cuda")
    ref = torch.zeros(pool, n_max + 1, desc.ref_cols, device="cuda")
    par = torch.zeros(pool, n_max + 1, desc.par_cols, device="cuda")
    gait = dict(duty=0.6, step_freq=2.0, height=0.30, offsets=P.HIP_OFFSETS)
    gait_tables(None, desc, len(slots), n_max, tx0, tX, tU, tV, tv, tlt, ref, par, gait, mode,
                slot=d(slots, torch.int32), horizon=d(horizon, torch.int32))
    torch.cuda.synchronize()
    xs = x0.copy()
    lts = lt.copy()
    if mode == 1:
        xs = Xw[:, 0, :].copy()
        _, lts = P.timer_run_np(0.6, 2.0, lts, desc.dt)
    href, hpar = P.quadruped_tables(desc, xs, lts, v, horizon, n_max)
    gref, gpar, gx0, glt = ref.cpu().numpy(), par.cpu().numpy(), tx0.cpu().numpy(), tlt.cpu().numpy()
    for s in slots:
        N = horizon[s]
        assert np.array_equal(gref[s, :N + 1], href[s, :N + 1]), s
        assert np.array_equal(gpar[s, :N + 1], hpar[s, :N + 1]), s
        assert np.array_equal(gx0[s], xs[s])
        assert np.array_equal(glt[s], lts[s] if mode == 1 else lt[s])
        if mode == 0:
            gX, gV, gU = tX.cpu().numpy(), tV.cpu().numpy(), tU.cpu().numpy()
            assert np.array_equal(gX[s, :N + 1], np.repeat(xs[s][None], N + 1, 0))
            assert not gV[s, :N + 1].any()
            fz = gU[s, :N, 2::3]
            assert np.all((fz > 0) == (href[s, :N, 12:16] > 0))
    untouched = np.setdiff1d(np.arange(pool), slots)
    assert not gref[untouched].any() and not gpar[untouched].any()
