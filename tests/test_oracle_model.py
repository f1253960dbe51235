"""Finite-difference checks of the oracle's SRBD linearisation (CPU)."""
import numpy as np
import pytest

from mpx_gb300 import problem as P


def _stage(model, seed):
    if model == P.MODEL_BIPED_WRENCH12:
        wl = P.biped_workload(1, horizons=(10,), seed=seed)
    else:
        wl = P.quadruped_workload(1, horizons=(10,), seed=seed, model=model)
    rng = np.random.default_rng(seed)
    x = wl.X0[0, 3].astype(np.float64) + 0.05 * rng.standard_normal(wl.desc.n)
    if model == P.MODEL_SRBD_QUAT13:
        x[3:7] /= np.linalg.norm(x[3:7])
    u = wl.U0[0, 3].astype(np.float64) + rng.standard_normal(12)
    return wl, x, u, wl.reference[0, 3].astype(np.float64), wl.parameter[0, 3].astype(np.float64)


@pytest.mark.parametrize("model", [P.MODEL_SRBD_QUAT13, P.MODEL_SRBD_RPY12, P.MODEL_BIPED_WRENCH12])
def test_dynamics_jacobian_fd(oracle, model):
    wl, x, u, ref, par = _stage(model, 3)
    A, B, fx, g, H, l = oracle.linearize(wl.desc, x, u, ref, par, wl.W[0])
    h = 1e-6
    for j in range(wl.desc.n):
        e = np.zeros(wl.desc.n); e[j] = h
        col = (oracle.dynamics(wl.desc, x + e, u, par) - oracle.dynamics(wl.desc, x - e, u, par)) / (2 * h)
        np.testing.assert_allclose(A[:, j], col, atol=1e-6, rtol=1e-5)
    for j in range(12):
        e = np.zeros(12); e[j] = h
        col = (oracle.dynamics(wl.desc, x, u + e, par) - oracle.dynamics(wl.desc, x, u - e, par)) / (2 * h)
        np.testing.assert_allclose(B[:, j], col, atol=1e-6, rtol=1e-5)


@pytest.mark.parametrize("model", [P.MODEL_SRBD_QUAT13, P.MODEL_SRBD_RPY12, P.MODEL_BIPED_WRENCH12])
def test_cost_gradient_fd(oracle, model):
    wl, x, u, ref, par = _stage(model, 4)
    A, B, fx, g, H, l = oracle.linearize(wl.desc, x, u, ref, par, wl.W[0])
    h = 1e-6
    z = np.concatenate([x, u])
    n = wl.desc.n
    for j in range(n + 12):
        e = np.zeros(n + 12); e[j] = h
        zp, zm = z + e, z - e
        fd = (oracle.cost(wl.desc, zp[:n], zp[n:], ref, wl.W[0]) - oracle.cost(wl.desc, zm[:n], zm[n:], ref, wl.W[0])) / (2 * h)
        assert abs(g[j] - fd) <= 1e-5 * max(1.0, abs(fd)), j


@pytest.mark.parametrize("model", [P.MODEL_SRBD_RPY12, P.MODEL_BIPED_WRENCH12])
def test_relaxed_barrier_hessian_is_exact(oracle, model):
    """For the relaxed barrier (kind 1) the control block of the Hessian model
    is the exact second derivative of the cost (the tracking part is quadratic).
    The biped's constraints add the centre-of-pressure and torsion bounds of
    its foot plates, linear in the wrench."""
    wl, x, u, ref, par = _stage(model, 5)
    ref = ref.copy()
    if model == P.MODEL_BIPED_WRENCH12:
        ref[12:14] = 1.0  # both feet in stance
        u[2::6] = np.abs(u[2::6]) + 300.0
        u[3::6] *= 0.1; u[4::6] *= 0.1; u[5::6] *= 0.1
    else:
        ref[12:16] = 1.0  # all legs in stance
        u[2::3] = np.abs(u[2::3]) + 20.0
    A, B, fx, g, H, l = oracle.linearize(wl.desc, x, u, ref, par, wl.W[0])
    n = wl.desc.n
    h = 1e-5
    for j in range(12):
        e = np.zeros(12); e[j] = h
        gp = oracle.linearize(wl.desc, x, u + e, ref, par, wl.W[0])[3][n:]
        gm = oracle.linearize(wl.desc, x, u - e, ref, par, wl.W[0])[3][n:]
        np.testing.assert_allclose(H[n:, n + j], (gp - gm) / (2 * h), atol=1e-6, rtol=1e-4)


def test_reference_penalty_matches_formula(oracle):
    """penalty() of objectives.py:7-13 (alpha 0.1, sigma 5) and its curvature."""
    d = P.quadruped_quat13()
    a, s = 0.1, 5.0
    for c in (1e-3, 0.5, 1.0, 1.9, 3.0, 7.0, -2.0):
        logb = -a * np.log(np.clip(c, 1e-10, 1e6))
        raw = logb if c > s else a / 2 * (((c - 2 * s) / s) ** 2 - 1) + logb
        assert abs(oracle.penalty(d, c) - np.clip(raw, 0, 1e8)) < 1e-12
        h = 1e-5
        if 0 < raw < 1e8 and abs(c - s) > 1e-3 and c > 1e-3:
            fd = (oracle.penalty(d, c + h) - 2 * oracle.penalty(d, c) + oracle.penalty(d, c - h)) / h ** 2
            assert abs(oracle.penalty_dd(d, c) - fd) < 1e-3 * max(1, abs(fd))
