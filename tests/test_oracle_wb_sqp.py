"""The float64 whole-body SQP oracle (oracle/wb_sqp.py), which the GPU's
mpxg_wb_sqp is checked against: its exact cost gradient against central
differences of the reference's stage cost (wb_stage_cost, pinned to the
reference's source by tests/golden), the quaternion Jacobian's limit at a
zero rotation, and one iteration's decrease of the KKT residual."""
import os

import numpy as np
import pytest

from mpx_gb300 import configs, mjcf, problem
from oracle.wb_sqp import WbProblem, wb_cost_grad, wb_kkt, wb_sqp_iteration
from oracle.wholebody import quat_sub, quat_sub_jacobian, wb_stage_cost

FIX = os.path.join(os.path.dirname(__file__), "golden", "aliengo_wb.npz")


def stage_point(rng, nj=12, nc=4, terminal=False):
    q = rng.normal(0, 0.1, 4)
    q[0] += 1
    q /= np.linalg.norm(q)
    x = np.concatenate([rng.normal(0, 0.05, 3) + [0, 0, 0.33], q, rng.normal(0, 0.2, nj), rng.normal(0, 0.3, 6),
                        rng.normal(0, 1.0, nj), rng.normal(0, 0.05, 3 * nc),
                        np.tile([5.0, -3.0, 90.0], nc) + rng.normal(0, 5, 3 * nc)])
    u = rng.normal(0, 8, nj)
    qr = rng.normal(0, 0.1, 4)
    qr[0] += 1
    qr /= np.linalg.norm(qr)
    ref = np.concatenate([rng.normal(0, 0.05, 3) + [0, 0, 0.33], qr, rng.normal(0, 0.2, nj), rng.normal(0, 0.3, 6),
                          rng.normal(0, 0.05, 3 * nc), rng.integers(0, 2, nc), rng.normal(0, 30, 3 * nc)])
    return x, u, ref


@pytest.mark.parametrize("terminal", [False, True])
def test_cost_gradient_is_the_derivative_of_the_stage_cost(terminal):
    cfg = configs.aliengo_wb()
    rng = np.random.default_rng(3 if terminal else 4)
    for _ in range(4):
        x, u, ref = stage_point(rng)
        gx, gu = wb_cost_grad(True, 12, 4, cfg.W, ref, x, u, terminal)
        f = lambda xx, uu: wb_stage_cost(True, 12, 4, cfg.W, ref, xx, uu, terminal)
        for j in range(x.size):
            h = 1e-6 * max(1.0, abs(x[j]))
            xp, xm = x.copy(), x.copy()
            xp[j] += h
            xm[j] -= h
            d = (f(xp, u) - f(xm, u)) / (2 * h)
            assert abs(d - gx[j]) <= 1e-5 * (1.0 + abs(d)), (terminal, "x", j, d, gx[j])
        if not terminal:
            for j in range(u.size):
                h = 1e-6 * max(1.0, abs(u[j]))
                up, um = u.copy(), u.copy()
                up[j] += h
                um[j] -= h
                d = (f(x, up) - f(x, um)) / (2 * h)
                assert abs(d - gu[j]) <= 1e-5 * (1.0 + abs(d)), ("u", j, d, gu[j])


def test_quaternion_jacobian_limit_at_zero_rotation():
    """At u = v the rotation vector's Jacobian is the limit (2/s) I of the
    smooth map (s the scalar part of conj(v) u): it matches differences of
    quat_sub taken across the zero rotation."""
    rng = np.random.default_rng(5)
    for _ in range(3):
        v = rng.normal(size=4)
        v /= np.linalg.norm(v)
        J = quat_sub_jacobian(v, v)
        assert np.all(np.isfinite(J))
        for k in range(4):
            h = 1e-7
            up, um = v.copy(), v.copy()
            up[k] += h
            um[k] -= h
            d = (quat_sub(up, v) - quat_sub(um, v)) / (2 * h)
            assert np.abs(d - J[:, k]).max() < 1e-6, (k, d, J[:, k])


def test_one_iteration_reduces_the_kkt_residual():
    model = mjcf.load_npz(FIX)
    d = np.load(FIX)
    cfg = configs.aliengo_wb()
    wl = problem.wb_workload(1, 3, d["q0"], d["p_legs0"], float(np.sum(model.mass)), seed=9)
    pb = WbProblem(model, cfg.dt, cfg.W, wl["reference"][0], wl["contact"][0])
    x0 = wl["x0"][0].astype(np.float64)
    X, U, V = [wl[k][0].astype(np.float64) for k in ("X0", "U0", "V0")]
    k0 = wb_kkt(pb, x0, X, U, V)
    r = wb_sqp_iteration(pb, x0, X, U, V, 1.0)
    k1 = wb_kkt(pb, x0, r["X"], r["U"], r["V"])
    assert r["status"] == 0 and 0.0 < r["alpha"] <= 1.0
    assert k1[0] < k0[0] and k1[1] < k0[1], (k0, k1)  # primal and dual parts both fall
    # the step satisfies the linearised dynamics it was computed from
    assert np.abs(r["dX"][0] - r["c"][0]).max() < 1e-9


def _dense_lq_kkt(A, B, c, Q, R, M, q, r, x0):
    """The LQ step problem as one dense KKT system: variables [x_0..x_N,
    u_0..u_{N-1}], constraints x_0 = x0 and x_{t+1} - A_t x_t - B_t u_t = c_t,
    cost sum 1/2 x'Qx + x'Mu + 1/2 u'Ru + q'x + r'u.  Returns X, U and the
    constraints' multipliers nu (stationarity H z + g + E' nu = 0)."""
    N, n, m = len(A), x0.size, B[0].shape[1]
    nz = (N + 1) * n + N * m
    xi = lambda t: slice(t * n, (t + 1) * n)
    ui = lambda t: slice((N + 1) * n + t * m, (N + 1) * n + (t + 1) * m)
    H, g = np.zeros((nz, nz)), np.zeros(nz)
    for t in range(N + 1):
        H[xi(t), xi(t)] = Q[t]
        g[xi(t)] = q[t]
        if t < N:
            H[ui(t), ui(t)] = R[t]
            H[xi(t), ui(t)] = M[t]
            H[ui(t), xi(t)] = M[t].T
            g[ui(t)] = r[t]
    E, e = np.zeros(((N + 1) * n, nz)), np.zeros((N + 1) * n)
    E[xi(0), xi(0)] = np.eye(n)
    e[xi(0)] = x0
    for t in range(N):
        E[xi(t + 1), xi(t + 1)] = np.eye(n)
        E[xi(t + 1), xi(t)] = -A[t]
        E[xi(t + 1), ui(t)] = -B[t]
        e[xi(t + 1)] = c[t]
    K = np.block([[H, E.T], [E, np.zeros((E.shape[0], E.shape[0]))]])
    sol = np.linalg.solve(K, np.concatenate([-g, e]))
    z, nu = sol[:nz], sol[nz:]
    X = np.stack([z[xi(t)] for t in range(N + 1)])
    U = np.stack([z[ui(t)] for t in range(N)])
    return X, U, nu.reshape(N + 1, n)


@pytest.mark.parametrize("structured", [False, True])
def test_step_riccati_equals_dense_kkt(structured):
    """The oracle's Riccati step (the one the GPU's 61-state Riccati is
    checked against) equals a dense KKT solve of the same LQ problem, with
    its costates the negated constraint multipliers; both for a general
    problem and for the whole-body structure (the contact-point and force
    columns of A zero, M = 0)."""
    from oracle.wb_sqp import _riccati
    rng = np.random.default_rng(31 if structured else 30)
    N, n, m, nzc = 5, 61, 12, 37
    A, B, c, Q, R, M, q, r = [], [], [], [], [], [], [], []
    for t in range(N + 1):
        L = rng.normal(size=(n, n))
        Q.append(L @ L.T / n + 0.1 * np.eye(n))
        q.append(rng.normal(size=n))
        if t == N:
            break
        a = np.eye(n) + 0.05 * rng.normal(size=(n, n))
        if structured:
            a[:, nzc:] = 0.0
        A.append(a)
        B.append(0.1 * rng.normal(size=(n, m)))
        c.append(0.1 * rng.normal(size=n))
        R.append(np.eye(m))
        M.append(np.zeros((n, m)) if structured else 0.02 * rng.normal(size=(n, m)))
        r.append(rng.normal(size=m))
    x0 = rng.normal(size=n)
    dX, dU, lam = _riccati(A, B, c, Q, R, M, q, r, x0)
    X, U, nu = _dense_lq_kkt(A, B, c, Q, R, M, q, r, x0)
    scale = lambda a: 1.0 + np.abs(a).max()
    assert np.abs(dX - X).max() < 1e-9 * scale(X)
    assert np.abs(dU - U).max() < 1e-9 * scale(U)
    assert np.abs(lam + nu).max() < 1e-9 * scale(nu)
