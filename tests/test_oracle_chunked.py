"""The time-parallel LQR restatement (oracle/chunked_lqr.py) against the
sequential Riccati recursion and a dense KKT solve, in float64: the chunk
elements, their combination and the chunk-local sweeps give the same gains,
value functions, steps and costates for any chunking.  The CUDA team kernel
(mpx_gb300/csrc/sqp_team.cuh) implements this algebra."""
import numpy as np
import pytest

from mpx_gb300 import problem as P
from oracle import chunked_lqr as C


def random_lq(n, m, N, seed):
    rng = np.random.default_rng(seed)
    A = [np.eye(n) + 0.05 * rng.normal(size=(n, n)) for _ in range(N)]
    B = [0.1 * rng.normal(size=(n, m)) for _ in range(N)]
    c = [rng.normal(size=n) for _ in range(N + 1)]
    H, g = [], []
    for _ in range(N + 1):
        Mq = rng.normal(size=(n + m, n + m))
        H.append(Mq @ Mq.T / (n + m) + 0.1 * np.eye(n + m))
        g.append(rng.normal(size=n + m))
    return H, g, A, B, c


def max_diff(a, b, keys):
    return max(float(np.abs(a[t] - b[t]).max()) for t in keys)


@pytest.mark.parametrize("bounds", [[0, 10, 20, 30, 45, 57], [0, 1, 2, 57], [0, 30, 57],
                                    [0, 5, 11, 17, 23, 29, 35, 41, 57]])
def test_chunked_equals_sequential_riccati(bounds):
    N = 57
    H, g, A, B, c = random_lq(12, 12, N, seed=3)
    K, k, Ps, ps = C.riccati(H, g, A, B, c)
    dx, du, lam = C.forward(A, B, c, K, k, Ps, ps, c[0], 0, N)
    o = C.chunked_solve(H, g, A, B, c, bounds)
    assert max_diff(o["K"], K, range(N)) < 1e-10
    assert max_diff(o["k"], k, range(N)) < 1e-10
    assert max_diff(o["P"], Ps, range(N + 1)) < 1e-10
    assert max_diff(o["dx"], dx, range(N + 1)) < 1e-10
    assert max_diff(o["du"], du, range(N)) < 1e-10
    assert max_diff(o["lam"], lam, range(N + 1)) < 1e-10


def test_chunked_equals_dense_kkt():
    """Against one dense KKT solve of the whole LQ problem (no cross term)."""
    from oracle import oracle as O
    n, m, N = 6, 3, 20
    rng = np.random.default_rng(5)
    A = np.eye(n) + 0.1 * rng.normal(size=(N, n, n))
    Bm = rng.normal(size=(N, n, m))
    cc = rng.normal(size=(N, n))
    Q = np.stack([np.eye(n) * (1 + t % 3) for t in range(N + 1)])
    R = np.stack([np.eye(m) * 0.5 for _ in range(N)])
    M = np.zeros((N, n, m))
    q = rng.normal(size=(N + 1, n))
    r = rng.normal(size=(N, m))
    x0 = rng.normal(size=n)
    X, U, lam = O.dense_lqr(A, Bm, cc, Q, R, M, q, r, x0)
    # the same problem in step form around x = 0, u = 0: H, g per stage, c_0 = x0, c_{t+1} = c_t
    H = [np.block([[Q[t], M[t]], [M[t].T, R[t]]]) for t in range(N)] + [np.block([[Q[N], np.zeros((n, m))],
                                                                                  [np.zeros((m, n)), np.eye(m)]])]
    g = [np.concatenate([q[t], r[t]]) for t in range(N)] + [np.concatenate([q[N], np.zeros(m)])]
    c = [x0] + [cc[t] for t in range(N)]
    o = C.chunked_solve(H, g, list(A), list(Bm), c, [0, 4, 9, 13, N])
    assert max(np.abs(o["dx"][t] - X[t]).max() for t in range(N + 1)) < 1e-9
    assert max(np.abs(o["du"][t] - U[t]).max() for t in range(N)) < 1e-9
    assert max(np.abs(o["lam"][t] - lam[t]).max() for t in range(N + 1)) < 1e-9


def test_chunked_on_srbd_linearisation(oracle):
    """The KKT step of an actual SQP iterate of the roll-pitch-yaw quadruped
    (N = 100, tracking weights up to 50, control weights 1e-4 and the cone
    barrier): the chunked solve equals the sequential one in float64, and in
    float32 stays within a few times the sequential float32 error."""
    N = 100
    wl = P.quadruped_workload(1, horizons=(N,), seed=5, model=P.MODEL_SRBD_RPY12, v_range=(-1, 1), random_phase=True)
    o = oracle.sqp_solve(wl.desc, P.SolverOptions(sqp_iters=3), wl.x0, wl.X0, wl.U0, wl.V0, wl.reference,
                         wl.parameter, wl.W, wl.horizon)
    X, U = o["X"][0], o["U"][0]
    A, B, H, g, c = [], [], [], [], [wl.x0[0] - X[0]]
    for t in range(N + 1):
        term = t == N
        a, bm, fx, gg, hh, _ = oracle.linearize(wl.desc, X[t], U[t] if not term else np.zeros(12), wl.reference[0, t],
                                                wl.parameter[0, t], wl.W[0], term)
        H.append(hh); g.append(gg)
        if not term:
            A.append(a); B.append(bm); c.append(fx - X[t + 1])
    K, k, Ps, ps = C.riccati(H, g, A, B, c, reg=1e-6)
    dx, du, lam = C.forward(A, B, c, K, k, Ps, ps, c[0], 0, N)
    bounds = [0, 12, 24, 36, 48, 60, 71, 83, N]
    od = C.chunked_solve(H, g, A, B, c, bounds, reg=1e-6)
    scale = lambda d: max(np.abs(v).max() for v in d.values())
    for key, ref in (("dx", dx), ("du", du), ("lam", lam)):
        assert max_diff(od[key], ref, ref.keys()) <= 1e-9 * scale(ref), key
    f32 = lambda L: [np.asarray(v, np.float32) for v in L]
    H3, g3, A3, B3, c3 = f32(H), f32(g), f32(A), f32(B), f32(c)
    K3, k3, P3, p3 = C.riccati(H3, g3, A3, B3, c3, reg=1e-6)
    dx3, du3, lam3 = C.forward(A3, B3, c3, K3, k3, P3, p3, c3[0], 0, N)
    o3 = C.chunked_solve(H3, g3, A3, B3, c3, bounds, reg=1e-6)
    for key, ref, seq in (("dx", dx, dx3), ("du", du, du3), ("lam", lam, lam3)):
        e_seq = max_diff(seq, ref, ref.keys()) / scale(ref)
        e_chk = max_diff(o3[key], ref, ref.keys()) / scale(ref)
        assert e_chk <= 10.0 * e_seq + 1e-6, (key, e_chk, e_seq)
