"""Time-parallel (chunked) LQR solve in float64 (test infrastructure, not the product).

The KKT step of the SQP is a time-varying LQR:

    min  sum_t 1/2 [dx;du]' H_t [dx;du] + g_t' [dx;du]  +  1/2 dx_N' H_N dx_N + g_N' dx_N
    s.t. dx_0 = c_0,  dx_{t+1} = A_t dx_t + B_t du_t + c_{t+1}.

The reference's solver module (mpx/primal_dual_ilqr, absent from its tree;
README.md:23-24,29) solves it by associative scans over time.  This file
restates the time-parallel method the CUDA team kernel implements, after
Saerkkae and Garcia-Fernandez, "Temporal parallelization of dynamic
programming and linear quadratic control" (IEEE TAC 2023), with the chunk
elements obtained from a chunk-local Riccati sweep:

1. Split [0, N] into chunks [s_c, e_c).  For every chunk but the last, run
   the Riccati recursion from a zero terminal cost at e_c.  Besides the value
   function (J, eta) at s_c this gives the closed-loop affine map of that
   policy, x_e = Phi x_s + phi, and the Gramian
       G = sum_t Phi_{t+1->e} B_t Quu_t^-1 B_t' Phi_{t+1->e}',
   the cost of steering the chunk's end away from phi + Phi x_s being
   1/2 d' G^-1 d.  (Phi, phi, G, eta, J) is the chunk's element.  The last
   chunk runs from the true terminal cost and is exact.
2. Combine the elements from the last chunk backwards (one element per
   chunk, so a short sequential scan): given the true value (P_e, p_e) at
   e_c,
       Z = (I + G P_e)^-1 [Phi | phi - G p_e]
       P_s = J + Phi' P_e Z_Phi,   p_s = eta + Phi' (P_e z + p_e)
   (the chunk's optimal end state would be x_e = Z_Phi x_s + z).
3. Each chunk re-runs its Riccati sweep from its true terminal value and
   composes the closed-loop affine map of its true gains, x_e = Phi' x_s +
   phi'.  The boundary states follow forwards from dx_0 = c_0 through those
   maps (the forward pass as composed affine maps; in exact arithmetic the
   same as Z_Phi x_s + z, and in float32 consistent with each chunk's own
   forward sweep), and each chunk runs its forward sweep from its boundary
   state.

riccati() is the sequential recursion (the oracle's riccati_solve,
oracle.hpp) on the same data, for comparison.
"""
import numpy as np


def riccati_stage(H, g, A, B, c_next, P, p, reg=0.0):
    """One backward Riccati step from the value (P, p) of stage t+1.
    Returns (K, k, P_t, p_t, Quu)."""
    n, m = A.shape[0], B.shape[1]
    Pc = P @ c_next + p
    Qxx = H[:n, :n] + A.T @ P @ A
    Qux = H[n:, :n] + B.T @ P @ A
    Quu = H[n:, n:] + B.T @ P @ B + (reg * np.eye(m)).astype(A.dtype)
    qx = g[:n] + A.T @ Pc
    qu = g[n:] + B.T @ Pc
    K = -np.linalg.solve(Quu, Qux)
    k = -np.linalg.solve(Quu, qu)
    Pt = Qxx + Qux.T @ K
    Pt = (Pt + Pt.T) * Pt.dtype.type(0.5)
    pt = qx + Qux.T @ k
    return K, k, Pt, pt, Quu


def riccati(H, g, A, B, c, reg=0.0, lo=0, hi=None, PN=None, pN=None):
    """Sequential Riccati over stages [lo, hi) from the value (PN, pN) at hi
    (default: the terminal cost H[N], g[N])."""
    N = len(A)
    hi = N if hi is None else hi
    n = A[0].shape[0]
    if PN is None:
        PN, pN = H[N][:n, :n].copy(), g[N][:n].copy()
    P, p = PN, pN
    K, k, Ps, ps = {}, {}, {hi: P}, {hi: p}
    for t in range(hi - 1, lo - 1, -1):
        K[t], k[t], P, p, _ = riccati_stage(H[t], g[t], A[t], B[t], c[t + 1], P, p, reg)
        Ps[t], ps[t] = P, p
    return K, k, Ps, ps


def forward(A, B, c, K, k, Ps, ps, x_lo, lo, hi):
    """Forward sweep over [lo, hi] from dx_lo: states, controls, costates."""
    dx, du, lam = {lo: x_lo}, {}, {}
    for t in range(lo, hi + 1):
        lam[t] = Ps[t] @ dx[t] + ps[t]
        if t == hi:
            break
        du[t] = K[t] @ dx[t] + k[t]
        dx[t + 1] = A[t] @ dx[t] + B[t] @ du[t] + c[t + 1]
    return dx, du, lam


def chunk_element(H, g, A, B, c, lo, hi, reg=0.0):
    """Step 1: the element (Phi, phi, G, eta, J) of chunk [lo, hi), from the
    Riccati sweep with a zero terminal cost at hi."""
    n, dt = A[0].shape[0], A[0].dtype
    P, p = np.zeros((n, n), dt), np.zeros(n, dt)
    Phi, phi, G = np.eye(n, dtype=dt), np.zeros(n, dt), np.zeros((n, n), dt)   # maps from stage t+1 to hi
    for t in range(hi - 1, lo - 1, -1):
        K, k, P, p, Quu = riccati_stage(H[t], g[t], A[t], B[t], c[t + 1], P, p, reg)
        PB = Phi @ B[t]
        G = G + PB @ np.linalg.solve(Quu, PB.T)
        phi = phi + Phi @ (B[t] @ k + c[t + 1])
        Phi = Phi @ (A[t] + B[t] @ K)
    return Phi, phi, G, p, P


def combine(elem, Pe, pe):
    """Step 2 for one chunk: its start value (P_s, p_s) and end-state map
    (Z_Phi, z) from the true value (P_e, p_e) at its end."""
    Phi, phi, G, eta, J = elem
    n = Phi.shape[0]
    S = np.eye(n, dtype=Phi.dtype) + G @ Pe
    Z = np.linalg.solve(S, np.concatenate([Phi, (phi - G @ pe)[:, None]], axis=1))
    ZPhi, z = Z[:, :n], Z[:, n]
    Ps = J + Phi.T @ Pe @ ZPhi
    Ps = (Ps + Ps.T) * Ps.dtype.type(0.5)
    ps = eta + Phi.T @ (Pe @ z + pe)
    return Ps, ps, ZPhi, z


def chunked_solve(H, g, A, B, c, bounds, reg=0.0):
    """The full time-parallel solve over chunks bounds = [0, s_1, ..., N]:
    returns dict(K, k, P, p, dx, du, lam) over all stages, as riccati() +
    forward() would."""
    N = len(A)
    W = len(bounds) - 1
    n = A[0].shape[0]
    # step 1 (parallel over chunks); the last chunk is solved from the true terminal cost
    elems = [chunk_element(H, g, A, B, c, bounds[w], bounds[w + 1], reg) for w in range(W - 1)]
    Kl, kl, Pl, pl = riccati(H, g, A, B, c, reg, bounds[W - 1], N)
    # step 2: values at the chunk starts, backwards
    Pv, pv = {N: Pl[N]}, {N: pl[N]}
    Pv[bounds[W - 1]], pv[bounds[W - 1]] = Pl[bounds[W - 1]], pl[bounds[W - 1]]
    for w in range(W - 2, -1, -1):
        e = bounds[w + 1]
        Pv[bounds[w]], pv[bounds[w]], _, _ = combine(elems[w], Pv[e], pv[e])
    # step 3 (parallel over chunks): local Riccati from the true end value and its closed-loop map
    local, maps = {}, {}
    for w in range(W):
        lo, hi = bounds[w], bounds[w + 1]
        if w == W - 1:
            local[w] = (Kl, kl, Pl, pl)
            continue
        K, k, Ps, ps = riccati(H, g, A, B, c, reg, lo, hi, Pv[hi], pv[hi])
        local[w] = (K, k, Ps, ps)
        Phi, phi = np.eye(n, dtype=A[0].dtype), np.zeros(n, A[0].dtype)  # map from stage t+1 to hi
        for t in range(hi - 1, lo - 1, -1):
            phi = phi + Phi @ (B[t] @ k[t] + c[t + 1])
            Phi = Phi @ (A[t] + B[t] @ K[t])
        maps[w] = (Phi, phi)
    # boundary states forwards through the composed maps
    xb = {0: c[0].copy()}
    for w in range(W - 1):
        Phi, phi = maps[w]
        xb[bounds[w + 1]] = Phi @ xb[bounds[w]] + phi
    out = dict(K={}, k={}, P={}, p={}, dx={}, du={}, lam={})
    for w in range(W):
        lo, hi = bounds[w], bounds[w + 1]
        K, k, Ps, ps = local[w]
        dx, du, lam = forward(A, B, c, K, k, Ps, ps, xb[lo], lo, hi)
        for t in range(lo, hi):
            out["K"][t], out["k"][t], out["du"][t] = K[t], k[t], du[t]
        for t in range(lo, hi + (1 if w == W - 1 else 0)):
            out["P"][t], out["p"][t], out["dx"][t], out["lam"][t] = Ps[t], ps[t], dx[t], lam[t]
    return out
