"""Differentiable solve: mpxg_solve_vjp against a dense FP64 solve of the same
adjoint (implicit-function) system, assembled from the oracle's Gauss-Newton
linearisation at the GPU's converged solution."""
import numpy as np
import pytest
import torch

from mpx_gb300 import problem as P
from mpx_gb300.solver import Solver

pytestmark = pytest.mark.gpu


def dense_adjoint(oracle, desc, X, U, ref, par, W, N, gX, gU, reg):
    """Solve H w + C'mu = g, C w = 0 (C: dx_0 = 0 and the linearised
    dynamics); returns (wX, wU, mu_0)."""
    n, m = desc.n, desc.m
    nv = (N + 1) * n + N * m
    xi = lambda t: t * (n + m)
    ui = lambda t: t * (n + m) + n
    H = np.zeros((nv, nv)); g = np.zeros(nv)
    C = np.zeros(((N + 1) * n, nv))
    C[0:n, 0:n] = np.eye(n)
    for t in range(N + 1):
        term = t == N
        u = U[t] if not term else np.zeros(m)
        A, Bm, fx, grad, Ht, l = oracle.linearize(desc, X[t], u, ref[t], par[t], W, terminal=term)
        H[xi(t):xi(t) + n, xi(t):xi(t) + n] = Ht[:n, :n]
        g[xi(t):xi(t) + n] = gX[t]
        if not term:
            H[xi(t):xi(t) + n, ui(t):ui(t) + m] = Ht[:n, n:]
            H[ui(t):ui(t) + m, xi(t):xi(t) + n] = Ht[n:, :n]
            H[ui(t):ui(t) + m, ui(t):ui(t) + m] = Ht[n:, n:] + reg * np.eye(m)
            g[ui(t):ui(t) + m] = gU[t]
            rows = slice((t + 1) * n, (t + 2) * n)
            C[rows, xi(t + 1):xi(t + 1) + n] = np.eye(n)
            C[rows, xi(t):xi(t) + n] = -A
            C[rows, ui(t):ui(t) + m] = -Bm
    K = np.block([[H, C.T], [C, np.zeros((C.shape[0], C.shape[0]))]])
    sol = np.linalg.solve(K, np.concatenate([g, np.zeros(C.shape[0])]))
    w, mu = sol[:nv], sol[nv:]
    wX = np.stack([w[xi(t):xi(t) + n] for t in range(N + 1)])
    wU = np.stack([w[ui(t):ui(t) + m] for t in range(N)])
    return wX, wU, mu[:n]


@pytest.mark.parametrize("model", [P.MODEL_SRBD_RPY12, P.MODEL_BIPED_WRENCH12])
def test_vjp_matches_dense_adjoint(oracle, cuda, model):
    if model == P.MODEL_BIPED_WRENCH12:
        wl = P.biped_workload(4, horizons=(15,), seed=41)
    else:
        wl = P.quadruped_workload(4, horizons=(15,), seed=41, model=model, v_range=(-1, 1), random_phase=True)
    opts = P.SolverOptions(sqp_iters=8)
    s = Solver(wl.desc, opts, n_max=wl.n_max, batch_max=wl.batch)
    sol = s.solve(wl.x0, wl.X0, wl.U0, wl.V0, wl.reference, wl.parameter, wl.W, wl.horizon)
    torch.cuda.synchronize()
    X, U, V = sol["X"].clone(), sol["U"].clone(), sol["V"].clone()
    rng = np.random.default_rng(7)
    gX = rng.normal(size=X.shape).astype(np.float32)
    gU = rng.normal(size=U.shape).astype(np.float32)
    out = s.vjp(wl.x0, X, U, V, wl.reference, wl.parameter, wl.W, gX, gU, wl.horizon)
    torch.cuda.synchronize()
    Xn, Un = X.cpu().double().numpy(), U.cpu().double().numpy()
    for b in range(wl.batch):
        N = int(wl.horizon[b])
        wX, wU, mu0 = dense_adjoint(oracle, wl.desc, Xn[b], Un[b], wl.reference[b], wl.parameter[b], wl.W[b], N,
                                    gX[b, :N + 1].astype(np.float64), gU[b, :N].astype(np.float64), opts.reg)
        for got, ref in ((out["wX"][b, :N + 1], wX), (out["wU"][b, :N], wU), (out["gx0"][b], mu0)):
            got = got.cpu().double().numpy()
            err = np.abs(got - ref).max() / np.abs(ref).max()
            assert err < 2e-3, err
        w = np.asarray(wl.W[b]).diagonal()[:12] if np.ndim(wl.W[b]) == 2 else np.asarray(wl.W[b])[:12]
        assert np.allclose(out["gref"][b, :N + 1].cpu().numpy(), w * out["wX"][b, :N + 1, :12].cpu().numpy(),
                           rtol=1e-5, atol=1e-6)
    s.close()
