"""Whole-body SQP, CPU oracle in float64 (test infrastructure, not the
product; only tests/ import it).

The reference runs its whole-body MPC (mpx/utils/mpc_wrapper.py:150-158,
346-354 with mpx/config/config_aliengo.py: quadruped_wb_dynamics,
quadruped_wb_obj(True, ...), quadruped_wb_hessian_gn(True, ...)) through
optimizers.mpc, whose module (mpx/primal_dual_ilqr) is absent from the
reference tree, so the iteration below is this implementation's and its
parity is unpinned; the model functions it calls (oracle/wholebody.py) are
pinned to the reference's own source.

One iteration at (X, U, V), x = [qpos, qvel, feet, forces], u = joint torques:
  defects  c_0 = x0 - X_0,  c_{t+1} = f(X_t, U_t, contact_t) - X_{t+1};
  Jacobians A_t, B_t of f by central differences, h_j = 1e-6 max(1, |z_j|),
    over qpos, qvel and u (f does not read the feet and force states: their
    columns are zero);
  the cost gradient (wb_cost_grad, exact) and the reference's Gauss-Newton
    blocks (wb_hessian_gn) with reg added to H_uu;
  the step problem (defects, gradients, x0 - X_0) solved by Riccati;
  merit phi(a) = sum l_t(X + a dX, U + a dU) + sum V_t(a).c_t(a)
                 + rho/2 sum |c_t(a)|^2,  V(a) = V + a (lam - V);
  G = sum g.(dx, du) + sum (lam - 2V).c;  rho <- max(rho, 2G / sum|c|^2) when
    both are positive (at most 1e12);  dphi = G - rho sum|c|^2;
  alpha = 1 if dphi >= -skip_tol (1 + |phi(0)|), else the first of
    1, beta, beta^2, ... (max_trials values) with
    phi(alpha) - phi(0) <= eta alpha dphi, else the last one (status 4);
  X += alpha dX,  U += alpha dU,  V += alpha (lam - V).
"""
import numpy as np

from oracle.wholebody import penalty, wb_dynamics, wb_hessian_gn, wb_stage_cost, quat_sub, quat_sub_jacobian


def _penalty_d(c, alpha=0.1, sigma=5.0):
    """First derivative of penalty() where it is smooth (0 where clipped)."""
    c = np.asarray(c, dtype=np.float64)
    inside = (c > 1e-10) & (c < 1e6)
    logd = np.where(inside, -alpha / np.where(inside, c, 1.0), 0.0)
    d = np.where(c > sigma, logd, alpha * (c - 2 * sigma) / sigma ** 2 + logd)
    raw = penalty(c, alpha, sigma)
    return np.where((raw > 0) & (raw < 1e8), d, 0.0)


def wb_residual(swing_tracking, nj, nc, ref_row, x, u, terminal):
    """The weighted residual of quadruped_wb_obj (objectives.py:77-144), in
    the order of W's blocks; the terminal stage keeps its first 12 + 2 nj."""
    r = np.asarray(ref_row, dtype=np.float64)
    rq = r[3:7]
    p_leg_ref, contact, grf_ref = r[13 + nj:13 + nj + 3 * nc], r[13 + nj + 3 * nc:13 + nj + 4 * nc], \
        r[13 + nj + 4 * nc:13 + nj + 7 * nc]
    res = [x[:3] - r[:3], quat_sub(x[3:7], rq), x[7:7 + nj] - r[7:7 + nj], x[7 + nj:10 + nj] - r[7 + nj:10 + nj],
           x[10 + nj:13 + nj] - r[10 + nj:13 + nj], x[13 + nj:13 + 2 * nj]]
    if terminal:
        return np.concatenate(res)
    cmap = np.ones(3 * nc) if swing_tracking else np.repeat(contact, 3)
    a = 13 + 2 * nj
    res += [cmap * (x[a:a + 3 * nc] - p_leg_ref), np.asarray(u[:nj], dtype=np.float64), x[a + 3 * nc:] - grf_ref]
    return np.concatenate(res)


def wb_cost_grad(swing_tracking, nj, nc, W, ref_row, x, u, terminal):
    """Exact gradient of wb_stage_cost (0.5 x the cost sum) w.r.t. x and u."""
    W = np.asarray(W, dtype=np.float64)
    x, u = np.asarray(x, dtype=np.float64), np.asarray(u, dtype=np.float64)
    r = np.asarray(ref_row, dtype=np.float64)
    n, m = x.size, u.size
    res = wb_residual(swing_tracking, nj, nc, r, x, u, terminal)
    R = res.size
    Jx, Ju = np.zeros((R, n)), np.zeros((R, m))
    Jx[0:3, 0:3] = np.eye(3)
    Jx[3:6, 3:7] = quat_sub_jacobian(x[3:7], r[3:7])
    Jx[6:6 + nj, 7:7 + nj] = np.eye(nj)
    Jx[6 + nj:12 + nj, 7 + nj:13 + nj] = np.eye(6)
    Jx[12 + nj:12 + 2 * nj, 13 + nj:13 + 2 * nj] = np.eye(nj)
    if not terminal:
        contact = r[13 + nj + 3 * nc:13 + nj + 4 * nc]
        cmap = np.ones(3 * nc) if swing_tracking else np.repeat(contact, 3)
        a = 12 + 2 * nj
        Jx[a:a + 3 * nc, 13 + 2 * nj:13 + 2 * nj + 3 * nc] = np.diag(cmap)
        Ju[a + 3 * nc:a + 3 * nc + nj, :nj] = np.eye(nj)
        b = a + 3 * nc + nj
        Jx[b:b + 3 * nc, 13 + 2 * nj + 3 * nc:] = np.eye(3 * nc)
    Wr = W[:R, :R] @ res
    gx, gu = Jx.T @ Wr, Ju.T @ Wr
    if terminal:
        return gx, gu
    contact = r[13 + nj + 3 * nc:13 + nj + 4 * nc]
    g0 = 13 + 2 * nj + 3 * nc
    g = x[g0:]
    s = np.sqrt(np.square(g[1::3]) + np.square(g[0::3]) + 1e-2)
    dc = 0.5 * _penalty_d(0.5 * g[2::3] - s) * contact
    gx[g0 + 0::3][:nc] += dc * (-g[0::3] / s)
    gx[g0 + 1::3][:nc] += dc * (-g[1::3] / s)
    gx[g0 + 2::3][:nc] += dc * 0.5
    for vec, off, bound, tgt in ((u[:nj], None, 44.0, gu), (x[13 + nj:13 + 2 * nj], 13 + nj, 10.0, gx)):
        lo = bound + 1e-2 - vec   # the -v entries of _limits
        hi = bound + 1e-2 + vec
        d = 0.5 * (-_penalty_d(lo, 1, 1) + _penalty_d(hi, 1, 1))
        if off is None:
            tgt[:nj] += d
        else:
            tgt[off:off + nj] += d
    return gx, gu


def _riccati(A, B, c, Q, R, M, q, r, x0):
    N, n = len(A), x0.size
    P, p = Q[N].copy(), q[N].copy()
    K, k = [None] * N, [None] * N
    Ps, ps = [None] * (N + 1), [None] * (N + 1)
    Ps[N], ps[N] = P, p
    for t in range(N - 1, -1, -1):
        w = P @ c[t] + p
        Qxx = Q[t] + A[t].T @ P @ A[t]
        Qux = M[t].T + B[t].T @ P @ A[t]
        Quu = R[t] + B[t].T @ P @ B[t]
        qx = q[t] + A[t].T @ w
        qu = r[t] + B[t].T @ w
        K[t] = -np.linalg.solve(Quu, Qux)
        k[t] = -np.linalg.solve(Quu, qu)
        P = Qxx + Qux.T @ K[t]
        P = 0.5 * (P + P.T)
        p = qx + Qux.T @ k[t]
        Ps[t], ps[t] = P, p
    dX, dU, lam = np.zeros((N + 1, n)), np.zeros((N, B[0].shape[1])), np.zeros((N + 1, n))
    x = x0.copy()
    for t in range(N + 1):
        dX[t] = x
        lam[t] = Ps[t] @ x + ps[t]
        if t == N:
            break
        dU[t] = K[t] @ x + k[t]
        x = A[t] @ x + B[t] @ dU[t] + c[t]
    return dX, dU, lam


class WbProblem:
    """One whole-body MPC instance: model (oracle.wholebody model record),
    dt, Baumgarte alpha, W [72, 72] (block diagonal), reference rows
    [N+1, 13 + nj + 7C], contact [N+1, C] (the dynamics' mask, parameter[t])."""

    def __init__(self, model, dt, W, reference, contact, swing_tracking=True, alpha=25.0):
        self.model, self.dt, self.alpha = model, float(dt), float(alpha)
        self.W = np.asarray(W, dtype=np.float64)
        self.ref = np.asarray(reference, dtype=np.float64)
        self.contact = np.asarray(contact, dtype=np.float64)
        self.swing = bool(swing_tracking)
        self.nv = model.nv
        self.nq = self.nv + 1
        self.nj = self.nv - 6
        self.nc = len(model.contact_point_body)
        self.nx = self.nq + self.nv + 6 * self.nc
        self.N = self.ref.shape[0] - 1

    def f(self, x, u, t):
        return wb_dynamics(self.model, self.dt, x, u, self.contact[t], alpha=self.alpha)

    def cost(self, t, x, u):
        return wb_stage_cost(self.swing, self.nj, self.nc, self.W, self.ref[t], x, u, t == self.N)

    def jacobians(self, x, u, t):
        nz = self.nq + self.nv
        A, B = np.zeros((self.nx, self.nx)), np.zeros((self.nx, self.nj))
        for j in range(nz + self.nj):
            xp, xm, up, um = x.copy(), x.copy(), u.copy(), u.copy()
            if j < nz:
                h = 1e-6 * max(1.0, abs(x[j]))
                xp[j] += h
                xm[j] -= h
                A[:, j] = (self.f(xp, u, t) - self.f(xm, u, t)) / (2 * h)
            else:
                a = j - nz
                h = 1e-6 * max(1.0, abs(u[a]))
                up[a] += h
                um[a] -= h
                B[:, a] = (self.f(x, up, t) - self.f(x, um, t)) / (2 * h)
        return A, B

    def defects(self, x0, X, U):
        c = np.zeros((self.N + 1, self.nx))
        c[0] = x0 - X[0]
        for t in range(self.N):
            c[t + 1] = self.f(X[t], U[t], t) - X[t + 1]
        return c


def wb_sqp_iteration(pb, x0, X, U, V, rho, reg=1e-6, beta=0.5, eta=1e-4, max_trials=8, skip_tol=1e-7):
    """One iteration as in the module docstring.  Returns dict X, U, V, rho,
    alpha, status, dX, dU, lam, phi0, dphi."""
    N, nx, nj = pb.N, pb.nx, pb.nj
    c = pb.defects(x0, X, U)
    A, B, Q, R, M, q, r = [], [], [], [], [], [], []
    for t in range(N + 1):
        u = U[t] if t < N else np.zeros(nj)
        gx, gu = wb_cost_grad(pb.swing, nj, pb.nc, pb.W, pb.ref[t], X[t], u, t == N)
        Hx, Hu, Hxu = wb_hessian_gn(pb.swing, nj, pb.nc, pb.W, pb.ref[t], X[t], u)
        if t == N:  # the terminal cost's blocks: the first 12 + 2 nj residual rows only
            from oracle.wholebody import quat_sub_jacobian as _qj
            Jx = np.zeros((12 + 2 * nj, nx))
            Jx[0:3, 0:3] = np.eye(3)
            Jx[3:6, 3:7] = _qj(X[t][3:7], pb.ref[t][3:7])
            Jx[6:6 + nj, 7:7 + nj] = np.eye(nj)
            Jx[6 + nj:12 + nj, 7 + nj:13 + nj] = np.eye(6)
            Jx[12 + nj:12 + 2 * nj, 13 + nj:13 + 2 * nj] = np.eye(nj)
            Hx = Jx.T @ pb.W[:12 + 2 * nj, :12 + 2 * nj] @ Jx
        Q.append(Hx)
        q.append(gx)
        if t < N:
            a_, b_ = pb.jacobians(X[t], U[t], t)
            A.append(a_)
            B.append(b_)
            R.append(Hu + reg * np.eye(nj))
            M.append(Hxu)
            r.append(gu)
    dX, dU, lam = _riccati(A, B, c[1:], Q, R, M, q, r, c[0])
    gd = sum(q[t] @ dX[t] for t in range(N + 1)) + sum(r[t] @ dU[t] for t in range(N))
    lc = float(np.sum((lam - 2 * V) * c))
    cs = float(np.sum(c * c))
    Jc = sum(pb.cost(t, X[t], U[t] if t < N else np.zeros(nj)) for t in range(N + 1))
    vc = float(np.sum(V * c))
    G = gd + lc
    if cs > 0 and G > 0:
        rho = min(max(rho, 2 * G / cs), 1e12)
    dphi = G - rho * cs
    phi0 = Jc + vc + 0.5 * rho * cs

    def phi(a):
        Xa, Ua, Va = X + a * dX, U + a * dU, V + a * (lam - V)
        ca = pb.defects(x0, Xa, Ua)
        J = sum(pb.cost(t, Xa[t], Ua[t] if t < N else np.zeros(nj)) for t in range(N + 1))
        return J + float(np.sum(Va * ca)) + 0.5 * rho * float(np.sum(ca * ca))

    alpha, status = 1.0, 0
    if dphi < -skip_tol * (1 + abs(phi0)):
        ok = False
        for tr in range(max_trials):
            if phi(alpha) - phi0 <= eta * alpha * dphi:
                ok = True
                break
            if tr + 1 < max_trials:
                alpha *= beta
        status = 0 if ok else 4
    return dict(X=X + alpha * dX, U=U + alpha * dU, V=V + alpha * (lam - V), rho=rho, alpha=alpha, status=status,
                dX=dX, dU=dU, lam=lam, phi0=phi0, dphi=dphi, c=c)


def wb_kkt(pb, x0, X, U, V):
    """(primal, dual / (1 + max |gradient|), max): primal = max |c|; dual =
    max |g_x + A'V_{t+1} - V_t| (t = 1..N-1), |g_N - V_N|, |g_u + B'V_{t+1}|."""
    N, nj = pb.N, pb.nj
    c = pb.defects(x0, X, U)
    rd, gm = 0.0, 0.0
    for t in range(N + 1):
        u = U[t] if t < N else np.zeros(nj)
        gx, gu = wb_cost_grad(pb.swing, nj, pb.nc, pb.W, pb.ref[t], X[t], u, t == N)
        gm = max(gm, np.abs(gx).max(), np.abs(gu).max() if t < N else 0.0)
        if t == N:
            rd = max(rd, np.abs(gx - V[N]).max())
            continue
        A, B = pb.jacobians(X[t], U[t], t)
        if t >= 1:
            rd = max(rd, np.abs(gx + A.T @ V[t + 1] - V[t]).max())
        rd = max(rd, np.abs(gu + B.T @ V[t + 1]).max())
    rp = float(np.abs(c).max())
    return rp, rd / (1 + gm), max(rp, rd / (1 + gm))
