"""The algebra of the time-parallel LQR (mpxg_lqr_solve method 1), restated
in numpy: the element product is associative, and the suffix products of the
stage elements carry the Riccati value functions (CPU, no GPU)."""
import numpy as np

from mpx_gb300 import problem as P


def element(A, B, c, Q, R, M, q, r):
    """Stage element (A, b, C, eta, J) after eliminating the cross term."""
    Ri = np.linalg.inv(R)
    return (A - B @ Ri @ M.T, c - B @ Ri @ r, B @ Ri @ B.T, M @ Ri @ r - q, Q - M @ Ri @ M.T)


def combine(ei, ej):
    """e_i (x) e_j, e_i the earlier element."""
    Ai, bi, Ci, etai, Ji = ei
    Aj, bj, Cj, etaj, Jj = ej
    n = Ai.shape[0]
    Z = np.eye(n) + Ci @ Jj
    Zi = np.linalg.inv(Z)
    T1 = Zi @ Ai
    return (Aj @ T1, Aj @ Zi @ (bi + Ci @ etaj) + bj, Aj @ Zi @ Ci @ Aj.T + Cj,
            T1.T @ (etaj - Jj @ bi) + etai, T1.T @ Jj @ Ai + Ji)


def riccati(d, b):
    """Value functions (P_t, p_t) of the sequential recursion, t = 0..N."""
    A, B, c, Q, R, M, q, r = (d[k][b] for k in ("A", "B", "c", "Q", "R", "M", "q", "r"))
    N = A.shape[0]
    P_, p_ = Q[N].copy(), q[N].copy()
    out = [None] * (N + 1)
    out[N] = (P_, p_)
    for t in range(N - 1, -1, -1):
        w = P_ @ c[t] + p_
        Qxx, Qux, Quu = Q[t] + A[t].T @ P_ @ A[t], M[t].T + B[t].T @ P_ @ A[t], R[t] + B[t].T @ P_ @ B[t]
        qx, qu = q[t] + A[t].T @ w, r[t] + B[t].T @ w
        K, k = -np.linalg.solve(Quu, Qux), -np.linalg.solve(Quu, qu)
        P_ = Qxx + Qux.T @ K
        P_ = 0.5 * (P_ + P_.T)
        p_ = qx + Qux.T @ k
        out[t] = (P_, p_)
    return out


def lq(seed):
    d = P.random_lq(1, 6, 3, 9, seed=seed)
    d["M"] = 0.05 * np.random.default_rng(seed).normal(size=d["M"].shape)
    return d


def stage_elements(d, b):
    N = d["A"].shape[1]
    es = [element(*(d[k][b, t] for k in ("A", "B", "c", "Q", "R", "M", "q", "r"))) for t in range(N)]
    n = d["A"].shape[-1]
    es.append((np.zeros((n, n)), np.zeros(n), np.zeros((n, n)), -d["q"][b, N], d["Q"][b, N]))
    return es


def test_element_product_is_associative():
    es = stage_elements(lq(1), 0)
    for i in range(len(es) - 3):
        x = combine(combine(es[i], es[i + 1]), es[i + 2])
        y = combine(es[i], combine(es[i + 1], es[i + 2]))
        for a, b in zip(x, y):
            assert np.abs(a - b).max() <= 1e-9 * max(1.0, np.abs(a).max())


def test_suffix_products_are_the_riccati_value_functions():
    d = lq(2)
    es = stage_elements(d, 0)
    ref = riccati(d, 0)
    N = len(es) - 1
    acc = es[N]
    for t in range(N, -1, -1):
        if t < N:
            acc = combine(es[t], acc)
        J, eta = acc[4], acc[3]
        P_, p_ = ref[t]
        assert np.abs(J - P_).max() <= 1e-8 * np.abs(P_).max()
        assert np.abs(-eta - p_).max() <= 1e-8 * max(1.0, np.abs(p_).max())


def test_chunked_scan_equals_sequential():
    """Fold chunks, scan across chunk elements, Riccati inside each chunk: the
    schedule of the GPU kernel gives the sequential value functions."""
    d = lq(3)
    es = stage_elements(d, 0)
    ref = riccati(d, 0)
    N = len(es) - 1
    chunks = [(s, min(N, s + 3)) for s in range(0, N, 3)]
    folded = []
    for s0, s1 in chunks:
        n = es[0][0].shape[0]
        e = (np.eye(n), np.zeros(n), np.zeros((n, n)), np.zeros(n), np.zeros((n, n)))  # identity element
        for t in range(s1 - 1, s0 - 1, -1):
            e = combine(es[t], e)
        folded.append(e)
    V = es[N]  # value at the end of the last chunk: the terminal element
    for ci in range(len(chunks) - 1, -1, -1):
        V = combine(folded[ci], V)
        s0 = chunks[ci][0]
        assert np.abs(V[4] - ref[s0][0]).max() <= 1e-8 * np.abs(ref[s0][0]).max()
