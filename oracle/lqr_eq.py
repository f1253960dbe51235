"""Equality-constrained time-varying LQR, CPU oracle (test infrastructure,
not the product).  Only tests/ and bench.py's CPU baseline import it.

Problem (the large linearised whole-body-sized LQ workload, n = 72, m = 30,
12 equality rows per stage):

    min  sum_t 1/2 x'Q x + x'M u + 1/2 u'R u + q'x + r'u  +  1/2 x_N'Q_N x_N + q_N'x_N
    s.t. x_0 = x0,  x_{t+1} = A_t x_t + B_t u_t + c_t,  C_t x_t + D_t u_t = e_t.

It stands in for the LQ/KKT step of the absent primal_dual_ilqr solver
(mpx/primal_dual_ilqr is an empty, unpinned submodule, .gitmodules:1-3): the
reference has no code or tests for it, so parity is unpinned and anchored on
a dense KKT solve of the same problem (dense_lqr_eq below).

riccati_eq restates the stagewise equality-constrained Riccati recursion
(the control QP of each stage solved by a Schur complement):
    Q_xx = Q + A'P A,  Q_ux = M' + B'P A,  Q_uu = R + B'P B,
    q_x = q + A'(P c + p),  q_u = r + B'(P c + p),
    Z = Q_uu^-1 Q_ux, g = Q_uu^-1 q_u, W = Q_uu^-1 D', S = D W,
    K_nu = S^-1 (C - D Z),  k_nu = -S^-1 (D g + e),
    K = -Z - W K_nu,  k = -g - W k_nu,
    P <- Q_xx + Q_ux'K + C'K_nu,  p <- q_x + Q_ux'k + C'k_nu   (using D K = -C),
and the forward pass u = K x + k, nu = K_nu x + k_nu, lam = P x + p.
"""
import numpy as np


def riccati_eq(A, B, c, Q, R, M, q, r, C, D, e, x0, dtype=np.float64):
    """One instance.  A [N,n,n], B [N,n,m], c [N,n], Q [N+1,n,n], R [N,m,m],
    M [N,n,m], q [N+1,n], r [N,m], C [N,p,n], D [N,p,m], e [N,p], x0 [n].
    Returns dict K [N,m,n], k [N,m], Knu [N,p,n], knu [N,p], X [N+1,n],
    U [N,m], lam [N+1,n], nu [N,p] (nu: multipliers of C x + D u = e in the
    convention of the stationarity condition l_u + B'lam_{t+1} + D'nu = 0)."""
    f = lambda a: np.asarray(a, dtype=dtype)
    A, B, c, Q, R, M, q, r, C, D, e, x0 = map(f, (A, B, c, Q, R, M, q, r, C, D, e, x0))
    N, n, _ = A.shape
    m, pq = B.shape[-1], C.shape[1]
    K = np.zeros((N, m, n), dtype); k = np.zeros((N, m), dtype)
    Kn = np.zeros((N, pq, n), dtype); kn = np.zeros((N, pq), dtype)
    Ps = np.zeros((N + 1, n, n), dtype); ps = np.zeros((N + 1, n), dtype)
    P, p = Q[N].copy(), q[N].copy()
    Ps[N], ps[N] = P, p
    for t in range(N - 1, -1, -1):
        PA, PB = P @ A[t], P @ B[t]
        w = P @ c[t] + p
        Qxx = Q[t] + A[t].T @ PA
        Qux = M[t].T + B[t].T @ PA
        Quu = R[t] + B[t].T @ PB
        qx = q[t] + A[t].T @ w
        qu = r[t] + B[t].T @ w
        Z = np.linalg.solve(Quu, Qux)
        g = np.linalg.solve(Quu, qu)
        W = np.linalg.solve(Quu, D[t].T)
        S = D[t] @ W
        Kn[t] = np.linalg.solve(S, C[t] - D[t] @ Z)
        kn[t] = -np.linalg.solve(S, D[t] @ g + e[t])
        K[t] = -Z - W @ Kn[t]
        k[t] = -g - W @ kn[t]
        P = Qxx + Qux.T @ K[t] + C[t].T @ Kn[t]
        P = 0.5 * (P + P.T)
        p = qx + Qux.T @ k[t] + C[t].T @ kn[t]
        Ps[t], ps[t] = P, p
    X = np.zeros((N + 1, n), dtype); U = np.zeros((N, m), dtype)
    lam = np.zeros((N + 1, n), dtype); nu = np.zeros((N, pq), dtype)
    x = x0.copy()
    for t in range(N + 1):
        X[t] = x
        lam[t] = Ps[t] @ x + ps[t]
        if t == N:
            break
        U[t] = K[t] @ x + k[t]
        nu[t] = Kn[t] @ x + kn[t]
        x = A[t] @ x + B[t] @ U[t] + c[t]
    return dict(K=K, k=k, Knu=Kn, knu=kn, X=X, U=U, lam=lam, nu=nu)


def dense_lqr_eq(A, B, c, Q, R, M, q, r, C, D, e, x0):
    """The same problem as one dense KKT solve (FP64, small sizes):
    returns (X, U, lam, nu) with lam_t = dV_t/dx_t."""
    N, n, _ = A.shape
    m, pq = B.shape[-1], C.shape[1]
    nv = (N + 1) * n + N * m
    nd = (N + 1) * n
    ne = N * pq
    xi = lambda t: t * (n + m)
    ui = lambda t: t * (n + m) + n
    H = np.zeros((nv, nv)); g = np.zeros(nv)
    for t in range(N):
        H[xi(t):xi(t) + n, xi(t):xi(t) + n] = Q[t]
        H[xi(t):xi(t) + n, ui(t):ui(t) + m] = M[t]
        H[ui(t):ui(t) + m, xi(t):xi(t) + n] = M[t].T
        H[ui(t):ui(t) + m, ui(t):ui(t) + m] = R[t]
        g[xi(t):xi(t) + n] = q[t]
        g[ui(t):ui(t) + m] = r[t]
    H[xi(N):xi(N) + n, xi(N):xi(N) + n] = Q[N]
    g[xi(N):xi(N) + n] = q[N]
    G = np.zeros((nd + ne, nv)); h = np.zeros(nd + ne)
    G[0:n, xi(0):xi(0) + n] = np.eye(n)
    h[0:n] = x0
    for t in range(N):
        rows = slice((t + 1) * n, (t + 2) * n)
        G[rows, xi(t + 1):xi(t + 1) + n] = np.eye(n)
        G[rows, xi(t):xi(t) + n] = -A[t]
        G[rows, ui(t):ui(t) + m] = -B[t]
        h[rows] = c[t]
        er = slice(nd + t * pq, nd + (t + 1) * pq)
        G[er, xi(t):xi(t) + n] = C[t]
        G[er, ui(t):ui(t) + m] = D[t]
        h[er] = e[t]
    Kkt = np.block([[H, G.T], [G, np.zeros((nd + ne, nd + ne))]])
    sol = np.linalg.solve(Kkt, np.concatenate([-g, h]))
    z, mult = sol[:nv], sol[nv:]
    X = np.stack([z[xi(t):xi(t) + n] for t in range(N + 1)])
    U = np.stack([z[ui(t):ui(t) + m] for t in range(N)])
    lam = -mult[:nd].reshape(N + 1, n)
    nu = mult[nd:].reshape(N, pq)
    return X, U, lam, nu


def step_data(A, B, c, Q, R, M, q, r, C, D, e, x0, X, U):
    """The step problem's data at the iterate (X, U): defects
    c' = A x + B u + c - x+, cost gradients q' = Q x + M u + q (terminal
    Q_N x_N + q_N), r' = M'x + R u + r, constraint residuals
    e' = e - C x - D u, and x0' = x0 - x_0.  The step (dX, dU) solves the LQ
    problem with the same matrices and these vectors."""
    N = A.shape[0]
    cs = np.einsum("tij,tj->ti", A, X[:N]) + np.einsum("tij,tj->ti", B, U) + c - X[1:]
    qs = np.einsum("tij,tj->ti", Q, X).copy()
    qs[:N] += np.einsum("tij,tj->ti", M, U)
    qs += q
    rs = np.einsum("tji,tj->ti", M, X[:N]) + np.einsum("tij,tj->ti", R, U) + r
    es = e - np.einsum("tij,tj->ti", C, X[:N]) - np.einsum("tij,tj->ti", D, U)
    return cs, qs, rs, es, x0 - X[0]


def sqp_eq(A, B, c, Q, R, M, q, r, C, D, e, x0, X, U, iters=1, dtype=np.float64):
    """SQP on the constrained LQ problem from the iterate (X, U): each
    iteration solves the step problem (step_data) with riccati_eq and takes
    the full step.  The problem is linear-quadratic, so one iteration lands
    on riccati_eq's direct solution up to rounding.  Returns dict X, U, lam,
    nu (multipliers of the result) and K, k, Knu, knu of the last step."""
    f = lambda a: np.asarray(a, dtype=dtype)
    A, B, c, Q, R, M, q, r, C, D, e, x0, X, U = map(f, (A, B, c, Q, R, M, q, r, C, D, e, x0, X, U))
    X, U = X.copy(), U.copy()
    for _ in range(iters):
        cs, qs, rs, es, xs = step_data(A, B, c, Q, R, M, q, r, C, D, e, x0, X, U)
        s = riccati_eq(A, B, cs, Q, R, M, qs, rs, C, D, es, xs, dtype=dtype)
        X, U = X + s["X"], U + s["U"]
    return dict(s, X=X, U=U)


def kkt_eq(A, B, c, Q, R, M, q, r, C, D, e, x0, X, U, lam, nu):
    """KKT residual of (X, U, lam, nu): primal = max |defect|, |C x + D u - e|,
    |x0 - x_0|; dual = max |g_x + A'lam+ + C'nu - lam| (t = 1..N-1),
    |g_N - lam_N|, |g_u + B'lam+ + D'nu| (t = 0..N-1), relative to
    1 + max |gradient| (g_x = Q x + M u + q, g_u = M'x + R u + r).  lam_0 is
    the multiplier of x_0 = x0 and has no stationarity row.  Returns
    (primal, relative dual, max of the two)."""
    N = A.shape[0]
    cs, qs, rs, es, xs = step_data(A, B, c, Q, R, M, q, r, C, D, e, x0, X, U)
    primal = max(np.abs(cs).max(), np.abs(es).max(), np.abs(xs).max())
    dx = qs[:N] + np.einsum("tji,tj->ti", A, lam[1:]) + np.einsum("tji,tj->ti", C, nu) - lam[:N]
    du = rs + np.einsum("tji,tj->ti", B, lam[1:]) + np.einsum("tji,tj->ti", D, nu)
    dual = max(np.abs(dx[1:]).max() if N > 1 else 0.0, np.abs(qs[N] - lam[N]).max(), np.abs(du).max())
    rel = dual / (1.0 + max(np.abs(qs).max(), np.abs(rs).max()))
    return primal, rel, max(primal, rel)
