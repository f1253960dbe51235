// Fused primal-dual SQP solve of one MPC instance per warp.
//
// One warp owns one instance for the whole solve (all SQP iterations):
//   backward sweep  t = N..0: per stage, lane j evaluates the dynamics with a
//                   dual number seeded on direction j (column j of [A|B]),
//                   lane JA = n+m evaluates the defect c = f(x,u) - x_{t+1};
//                   the warp forms the augmented stage matrix
//                       H = G + F^T P F      (F = [A B c; 0 0 1], G = cost model)
//                   with lane j holding column j, and eliminates the m control
//                   pivots by Gauss-Jordan: what remains is the new value
//                   function (P, p) and the gains (K, k) -- one Riccati step.
//   forward sweep   t = 0..N: du = K dx + k, dx+ = A dx + B du + c, and the
//                   costates lam = P dx + p (the new duals).
//   merit search    stage-parallel evaluation (lane = stage) of the augmented
//                   Lagrangian merit phi = J + V.c + rho/2 |c|^2 at trial steps.
// The reference solves the same Newton-KKT system of its multiple-shooting SQP
// (call sites mpx/utils/mpc_wrapper_srbd.py:124-132; the solver module itself is
// absent from the reference tree).
#pragma once
#include "models.cuh"

namespace mpxg {

enum { ST_NAN = 1, ST_NON_PD = 2, ST_LS_FAIL = 4, ST_BAD_HORIZON = 8 };

struct SqpParams {
  int sqp_iters, ls_max_trials;
  float ls_beta, ls_eta, reg, rho0, ls_skip_tol;
  int compute_kkt;
};

struct BatchPtrs {
  int batch, n_max;
  const int* horizon;
  const float *x0, *X_in, *U_in, *V_in, *ref, *par, *w;
  float *X, *U, *V, *K, *k, *kkt;
  int* status;
  int* counter;            // work-queue head (zeroed before each launch)
  float* scratch;          // per-warp scratch
  long long scratch_stride;  // floats per warp
  int single_instance;     // >= 0: solve only this instance with warp 0 (plain path)
};

template <class M>
struct Dims {
  static constexpr int NX = M::NX, NU = M::NU;
  static constexpr int NZ = NX + NU + 1;   // augmented columns: x, u, affine
  static constexpr int JA = NX + NU;       // affine column / lane
  static constexpr int NP = NX + 1;        // value-function rows: x, affine
  static constexpr int LDP = (NP + 3) / 4 * 4;
};

// Per-warp shared memory.
template <class M>
struct __align__(16) WarpSmem {
  typedef Dims<M> D;
  float xs[16], us[16], xn[16], ref[20], par[16];
  float w[24];
  float P[D::NP * D::LDP];     // value function of stage t+1, column-major
  float Praw[D::NP * D::LDP];  // unsymmetrised new value function
  float F[D::NZ * D::LDP];     // columns of the augmented dynamics F
  float col[32];               // pivot column broadcast
  float g[32];                 // cost gradient gather
  float J[D::NX * 12];         // state-residual Jacobian columns
  float dx[16], du[16];
};

// Floats of per-warp scratch for horizon n_max.
template <class M>
__host__ __device__ inline long long scratch_floats(int n_max) {
  typedef Dims<M> D;
  long long f = 0;
  f += (long long)n_max * D::NZ * D::NX;          // F columns (rows 0..NX-1)
  f += (long long)n_max * D::NP * M::NU;          // [K | k] column-major
  f += (long long)(n_max + 1) * D::NP * D::NP;    // value functions
  f += (long long)(n_max + 1) * (D::NX + D::NU);  // cost gradients
  f += (long long)(n_max + 1) * D::NX * 2;        // dX, lam
  f += (long long)n_max * M::NU;                  // dU
  return (f + 31) / 32 * 32;
}

template <class M>
struct Scratch {
  typedef Dims<M> D;
  float *F, *K, *P, *G, *dX, *L, *dU;
  __device__ Scratch(float* base, int n_max) {
    F = base;
    K = F + (size_t)n_max * D::NZ * D::NX;
    P = K + (size_t)n_max * D::NP * M::NU;
    G = P + (size_t)(n_max + 1) * D::NP * D::NP;
    dX = G + (size_t)(n_max + 1) * (D::NX + D::NU);
    L = dX + (size_t)(n_max + 1) * D::NX;
    dU = L + (size_t)(n_max + 1) * D::NX;
  }
};

// Merit contribution of constraint/stage index t (0..N) at step alpha:
// l_t + V~_t . c~_t + rho/2 |c~_t|^2 (double-free, one lane).
template <class M>
__device__ __forceinline__ float merit_stage(const ModelConst& mc, int t, int N, float alpha, float rho,
                                             const float* x0, const float* X, const float* U, const float* V,
                                             const Scratch<M>& s, const float* ref, const float* par, const float* w,
                                             float* cmax) {
  constexpr int NX = M::NX, NU = M::NU;
  float xt[NX], ut[NU], ct[NX];
#pragma unroll
  for (int i = 0; i < NX; ++i) xt[i] = X[t * NX + i] + alpha * s.dX[t * NX + i];
  float l;
  if (t < N) {
#pragma unroll
    for (int a = 0; a < NU; ++a) ut[a] = U[t * NU + a] + alpha * s.dU[t * NU + a];
    l = stage_cost<M>(mc, xt, ut, ref + t * M::NREF, w, false);
  } else {
    l = stage_cost<M>(mc, xt, ut, ref + t * M::NREF, w, true);
  }
  if (t == 0) {
#pragma unroll
    for (int i = 0; i < NX; ++i) ct[i] = x0[i] - xt[i];
  } else {
    float xp[NX], up[NU], fx[NX];
#pragma unroll
    for (int i = 0; i < NX; ++i) xp[i] = X[(t - 1) * NX + i] + alpha * s.dX[(t - 1) * NX + i];
#pragma unroll
    for (int a = 0; a < NU; ++a) up[a] = U[(t - 1) * NU + a] + alpha * s.dU[(t - 1) * NU + a];
    M::template dynamics<float>(mc, xp, up, par + (t - 1) * M::NPAR, fx);
#pragma unroll
    for (int i = 0; i < NX; ++i) ct[i] = fx[i] - xt[i];
  }
  float vc = 0.0f, cs = 0.0f, cm = 0.0f;
#pragma unroll
  for (int i = 0; i < NX; ++i) {
    const float vt = V[t * NX + i] + alpha * (s.L[t * NX + i] - V[t * NX + i]);
    vc += vt * ct[i];
    cs += ct[i] * ct[i];
    cm = fmaxf(cm, fabsf(ct[i]));
  }
  *cmax = cm;
  return l + vc + 0.5f * rho * cs;
}

// Lane j's column of the stage cost model G (rows 0..NZ-1 except the affine
// row, which the caller fills with the gradient) and gradient entry g_j.
// Diagonal weights w[24].  terminal: state block only.
template <class M>
__device__ __forceinline__ void cost_column(const ModelConst& mc, WarpSmem<M>& sm, int j, bool terminal,
                                            float* gcol, float* gj) {
  typedef Dims<M> D;
  constexpr int NX = D::NX, NU = D::NU, NZ = D::NZ;
#pragma unroll
  for (int i = 0; i < NZ; ++i) gcol[i] = 0.0f;
  *gj = 0.0f;
  if (j < NX) {
    // residual Jacobian column j and residual value
    float rj[12], rv[12];
    if (M::IDENT_RES) {
#pragma unroll
      for (int a = 0; a < 12; ++a) { rv[a] = sm.xs[a] - sm.ref[a]; rj[a] = (a == j) ? 1.0f : 0.0f; }
    } else {
      DF xd[NX], r[12];
#pragma unroll
      for (int i = 0; i < NX; ++i) xd[i] = mkd(sm.xs[i], i == j ? 1.0f : 0.0f);
      M::template state_residual<DF>(xd, sm.ref, r);
#pragma unroll
      for (int a = 0; a < 12; ++a) { rv[a] = r[a].v; rj[a] = r[a].d; }
    }
    float g = 0.0f;
#pragma unroll
    for (int a = 0; a < 12; ++a) g += sm.w[a] * rv[a] * rj[a];
    *gj = g;
    if (M::IDENT_RES) {
      const float wj = sm.w[j];
#pragma unroll
      for (int i = 0; i < NX; ++i) gcol[i] = (i == j) ? wj : 0.0f;
    } else {
#pragma unroll
      for (int a = 0; a < 12; ++a) sm.J[j * 12 + a] = rj[a];
    }
  } else if (j < NX + NU && !terminal) {
    const int a = j - NX;
    constexpr int LD = (M::LEGS == 4) ? 3 : 6;
    float hb[LD];
    float gb;
    int leg;
    barrier_lane<M>(mc, a, sm.us, sm.ref, &gb, hb, &leg);
    const float wa = sm.w[12 + a];
    *gj = wa * sm.us[a] + gb;
#pragma unroll
    for (int b = 0; b < NU; ++b) {
      float v = 0.0f;
#pragma unroll
      for (int r = 0; r < LD; ++r) v = (b == LD * leg + r) ? hb[r] : v;
      gcol[NX + b] = v + ((b == a) ? wa : 0.0f);
    }
  }
}

// Gauss-Newton state block for non-identity residuals (needs every lane's
// column in sm.J; call after __syncwarp()).
template <class M>
__device__ __forceinline__ void cost_column_state_block(WarpSmem<M>& sm, int j, float* gcol) {
  constexpr int NX = M::NX;
  if (M::IDENT_RES || j >= NX) return;
  float wr[12];
#pragma unroll
  for (int a = 0; a < 12; ++a) wr[a] = sm.w[a] * sm.J[j * 12 + a];
#pragma unroll
  for (int i = 0; i < NX; ++i) {
    float s = 0.0f;
#pragma unroll
    for (int a = 0; a < 12; ++a) s += sm.J[i * 12 + a] * wr[a];
    gcol[i] = s;
  }
}

template <class M>
__device__ void solve_instance(const ModelConst& mc, const SqpParams& sp, const BatchPtrs& bp, int b,
                               WarpSmem<M>& sm, float* scr) {
  typedef Dims<M> D;
  constexpr int NX = D::NX, NU = D::NU, NZ = D::NZ, JA = D::JA, NP = D::NP, LDP = D::LDP;
  const int lane = threadIdx.x & 31;
  const int n_max = bp.n_max;
  const int N = bp.horizon ? bp.horizon[b] : n_max;
  if (N < 1 || N > n_max) {  // invalid horizon: report, touch nothing else
    if (bp.status && lane == 0) bp.status[b] = ST_BAD_HORIZON;
    return;
  }
  const size_t xo = (size_t)b * (n_max + 1) * NX, uo = (size_t)b * n_max * NU;
  float* X = bp.X + xo;
  float* U = bp.U + uo;
  float* V = bp.V + xo;
  const float* x0 = bp.x0 + (size_t)b * NX;
  const float* ref = bp.ref + (size_t)b * (n_max + 1) * M::NREF;
  const float* par = bp.par + (size_t)b * (n_max + 1) * M::NPAR;
  Scratch<M> s(scr, n_max);

  // warm start into the outputs (in place when they alias)
  if (bp.X_in != bp.X)
    for (int e = lane; e < (N + 1) * NX; e += 32) X[e] = bp.X_in[xo + e];
  if (bp.V_in != bp.V)
    for (int e = lane; e < (N + 1) * NX; e += 32) V[e] = bp.V_in[xo + e];
  if (bp.U_in != bp.U)
    for (int e = lane; e < N * NU; e += 32) U[e] = bp.U_in[uo + e];
  if (lane < 24) sm.w[lane] = bp.w[(size_t)b * 24 + lane];
  __syncwarp();

  float rho = sp.rho0;
  int status = 0;
  const int j = lane;

  for (int it = 0; it < sp.sqp_iters; ++it) {
    // ================================================ backward sweep
    float J0 = 0.0f;  // stage costs, accumulated on lane JA
    {
      // terminal value function P_N = G_N, p_N = g_N
      for (int e = lane; e < NX; e += 32) sm.xs[e] = X[N * NX + e];
      for (int e = lane; e < M::NREF; e += 32) sm.ref[e] = ref[N * M::NREF + e];
      __syncwarp();
      float gcol[NZ], gj;
      cost_column<M>(mc, sm, j, true, gcol, &gj);
      __syncwarp();
      cost_column_state_block<M>(sm, j, gcol);
      if (j < NX) {
#pragma unroll
        for (int i = 0; i < NX; ++i) sm.P[j * LDP + i] = gcol[i];
        sm.P[j * LDP + NX] = gj;
        sm.P[NX * LDP + j] = gj;
        s.G[N * (NX + NU) + j] = gj;
      }
      if (j == JA) {
        sm.P[NX * LDP + NX] = 0.0f;
        J0 += stage_cost<M>(mc, sm.xs, sm.us, sm.ref, sm.w, true);
      }
      __syncwarp();
      if (j < NP) {
#pragma unroll
        for (int i = 0; i < NP; ++i) s.P[(size_t)N * NP * NP + j * NP + i] = sm.P[j * LDP + i];
      }
    }
    for (int t = N - 1; t >= 0; --t) {
      __syncwarp();
      for (int e = lane; e < NX; e += 32) { sm.xs[e] = X[t * NX + e]; sm.xn[e] = X[(t + 1) * NX + e]; }
      for (int e = lane; e < NU; e += 32) sm.us[e] = U[t * NU + e];
      for (int e = lane; e < M::NREF; e += 32) sm.ref[e] = ref[t * M::NREF + e];
      for (int e = lane; e < M::NPAR; e += 32) sm.par[e] = par[t * M::NPAR + e];
      __syncwarp();
      // ---- linearisation: column j of F and of the cost model G
      float fcol[NP];
      if (j < NX + NU) {
        DF xd[NX], ud[NU], fd[NX];
#pragma unroll
        for (int i = 0; i < NX; ++i) xd[i] = mkd(sm.xs[i], i == j ? 1.0f : 0.0f);
#pragma unroll
        for (int a = 0; a < NU; ++a) ud[a] = mkd(sm.us[a], NX + a == j ? 1.0f : 0.0f);
        M::template dynamics<DF>(mc, xd, ud, sm.par, fd);
#pragma unroll
        for (int i = 0; i < NX; ++i) fcol[i] = fd[i].d;
        fcol[NX] = 0.0f;
      } else if (j == JA) {
        float fx[NX];
        M::template dynamics<float>(mc, sm.xs, sm.us, sm.par, fx);
#pragma unroll
        for (int i = 0; i < NX; ++i) fcol[i] = fx[i] - sm.xn[i];
        fcol[NX] = 1.0f;
        J0 += stage_cost<M>(mc, sm.xs, sm.us, sm.ref, sm.w, false);
      } else {
#pragma unroll
        for (int i = 0; i < NP; ++i) fcol[i] = 0.0f;
      }
      float gcol[NZ], gj;
      cost_column<M>(mc, sm, j, false, gcol, &gj);
      if (j < NZ) {
#pragma unroll
        for (int i = 0; i < NP; ++i) sm.F[j * LDP + i] = fcol[i];
      }
      if (j < JA) sm.g[j] = gj;
      __syncwarp();
      cost_column_state_block<M>(sm, j, gcol);
      if (j < JA) {
        gcol[JA] = gj;
        s.G[t * (NX + NU) + j] = gj;
      } else if (j == JA) {
#pragma unroll
        for (int i = 0; i < JA; ++i) gcol[i] = sm.g[i];
        gcol[JA] = 0.0f;
      }
      // ---- T = P F[:, j];  H[:, j] = G[:, j] + F^T T
      float tv[NP];
#pragma unroll
      for (int i = 0; i < NP; ++i) tv[i] = 0.0f;
#pragma unroll
      for (int k = 0; k < NP; ++k) {
        const float fk = fcol[k];
#pragma unroll
        for (int i = 0; i < NP; ++i) tv[i] += sm.P[k * LDP + i] * fk;
      }
      float h[NZ];
#pragma unroll
      for (int i = 0; i < NZ; ++i) {
        float a = gcol[i];
#pragma unroll
        for (int k = 0; k < NP; ++k) a += sm.F[i * LDP + k] * tv[k];
        h[i] = a;
      }
      if (j >= NX && j < JA) {
#pragma unroll
        for (int a = NX; a < JA; ++a)
          if (a == j) h[a] += sp.reg;
      }
      // ---- Gauss-Jordan elimination of the control pivots
#pragma unroll
      for (int p = NX; p < JA; ++p) {
        __syncwarp();
        if (lane == p) {
#pragma unroll
          for (int i = 0; i < NZ; ++i) sm.col[i] = h[i];
        }
        __syncwarp();
        float d = sm.col[p];
        if (!(d > 0.0f)) { status |= ST_NON_PD; d = fmaxf(fabsf(d), 1e-12f); }
        const float hp = h[p] / d;
#pragma unroll
        for (int i = 0; i < NZ; ++i)
          if (i != p) h[i] -= sm.col[i] * hp;
        h[p] = hp;
      }
      // ---- outputs: K, k, new value function (symmetrised)
      if (j < NX) {
#pragma unroll
        for (int a = 0; a < NU; ++a) s.K[(size_t)t * NP * NU + j * NU + a] = -h[NX + a];
#pragma unroll
        for (int i = 0; i < NX; ++i) sm.Praw[j * LDP + i] = h[i];
      } else if (j == JA) {
#pragma unroll
        for (int a = 0; a < NU; ++a) s.K[(size_t)t * NP * NU + NX * NU + a] = -h[NX + a];
#pragma unroll
        for (int i = 0; i < NX; ++i) sm.Praw[NX * LDP + i] = h[i];
      }
      if (j < NZ) {
#pragma unroll
        for (int i = 0; i < NX; ++i) s.F[(size_t)t * NZ * NX + j * NX + i] = fcol[i];
      }
      __syncwarp();
      if (j < NX) {
        float* Pt = s.P + (size_t)t * NP * NP;
#pragma unroll
        for (int i = 0; i < NX; ++i) {
          const float v = 0.5f * (h[i] + sm.Praw[i * LDP + j]);
          sm.P[j * LDP + i] = v;
          Pt[j * NP + i] = v;
        }
        const float pj = 0.5f * (h[JA] + sm.Praw[NX * LDP + j]);
        sm.P[j * LDP + NX] = pj;
        sm.P[NX * LDP + j] = pj;
        Pt[j * NP + NX] = pj;
        Pt[NX * NP + j] = pj;
      }
      if (j == 0) {
        sm.P[NX * LDP + NX] = 0.0f;
        s.P[(size_t)t * NP * NP + NX * NP + NX] = 0.0f;
      }
    }
    __syncwarp();
    // ================================================ forward sweep
    double a_gd = 0.0, a_lc = 0.0, a_vc = 0.0, a_cs = 0.0;
    float c_cur = 0.0f;
    if (lane < NX) {
      c_cur = x0[lane] - X[lane];
      sm.dx[lane] = c_cur;
    }
    __syncwarp();
    for (int t = 0; t <= N; ++t) {
      const float* Pt = s.P + (size_t)t * NP * NP;
      if (lane < NX) {
        float lam = Pt[NX * NP + lane];
#pragma unroll
        for (int k = 0; k < NX; ++k) lam += Pt[k * NP + lane] * sm.dx[k];
        const float vt = V[t * NX + lane];
        a_lc += (double)((lam - 2.0f * vt) * c_cur);
        a_vc += (double)(vt * c_cur);
        a_cs += (double)(c_cur * c_cur);
        a_gd += (double)(s.G[t * (NX + NU) + lane] * sm.dx[lane]);
        s.L[t * NX + lane] = lam;
        s.dX[t * NX + lane] = sm.dx[lane];
      }
      if (t == N) break;
      const float* Kt = s.K + (size_t)t * NP * NU;
      if (lane < NU) {
        float du = Kt[NX * NU + lane];
#pragma unroll
        for (int k = 0; k < NX; ++k) du += Kt[k * NU + lane] * sm.dx[k];
        sm.du[lane] = du;
        a_gd += (double)(s.G[t * (NX + NU) + NX + lane] * du);
        s.dU[t * NU + lane] = du;
      }
      __syncwarp();
      float dxn = 0.0f;
      if (lane < NX) {
        const float* Ft = s.F + (size_t)t * NZ * NX;
        c_cur = Ft[JA * NX + lane];
        dxn = c_cur;
#pragma unroll
        for (int k = 0; k < NX; ++k) dxn += Ft[k * NX + lane] * sm.dx[k];
#pragma unroll
        for (int a = 0; a < NU; ++a) dxn += Ft[(NX + a) * NX + lane] * sm.du[a];
      }
      __syncwarp();
      if (lane < NX) sm.dx[lane] = dxn;
      __syncwarp();
    }
    __syncwarp();
    const double gd = warp_sum(a_gd), lc = warp_sum(a_lc), vc = warp_sum(a_vc), cs = warp_sum(a_cs);
    const double Jc = warp_sum((double)J0);
    // ================================================ merit line search
    const double G = gd + lc;
    if (cs > 0.0 && G > 0.0) rho = fminf(fmaxf(rho, (float)(2.0 * G / cs)), 1e12f);
    const double dphi = G - (double)rho * cs;
    const double phi0 = Jc + vc + 0.5 * (double)rho * cs;
    float alpha = 1.0f;
    bool accepted = false;
    if (!(dphi < -(double)sp.ls_skip_tol * (1.0 + fabs(phi0)))) {
      accepted = true;
    } else {
      for (int tr = 0; tr < sp.ls_max_trials; ++tr) {
        double acc = 0.0;
        for (int t = lane; t <= N; t += 32) {
          float cm;
          acc += (double)merit_stage<M>(mc, t, N, alpha, rho, x0, X, U, V, s, ref, par, sm.w, &cm);
        }
        const double phi = warp_sum(acc);
        if (phi <= phi0 + (double)sp.ls_eta * alpha * dphi) { accepted = true; break; }
        if (tr + 1 < sp.ls_max_trials) alpha *= sp.ls_beta;
      }
    }
    if (!accepted) status |= ST_LS_FAIL;
    // ================================================ step
    for (int e = lane; e < (N + 1) * NX; e += 32) {
      X[e] += alpha * s.dX[e];
      V[e] += alpha * (s.L[e] - V[e]);
    }
    for (int e = lane; e < N * NU; e += 32) U[e] += alpha * s.dU[e];
    __syncwarp();
  }

  // ================================================ gains of the last step
  if (bp.K) {
    float* Ko = bp.K + (size_t)b * n_max * NU * NX;
    for (int e = lane; e < N * NU * NX; e += 32) {
      const int t = e / (NU * NX), r = e - t * NU * NX, a = r / NX, jj = r - a * NX;
      Ko[e] = s.K[(size_t)t * NP * NU + jj * NU + a];
    }
  }
  if (bp.k) {
    float* ko = bp.k + (size_t)b * n_max * NU;
    for (int e = lane; e < N * NU; e += 32) {
      const int t = e / NU, a = e - t * NU;
      ko[e] = s.K[(size_t)t * NP * NU + NX * NU + a];
    }
  }

  // ================================================ KKT residual of the result
  if (bp.kkt && sp.compute_kkt) {
    float rp = 0.0f, rd = 0.0f, gm = 0.0f;
    if (lane < NX) rp = fabsf(x0[lane] - X[lane]);
    for (int t = 0; t <= N; ++t) {
      __syncwarp();
      for (int e = lane; e < NX; e += 32) {
        sm.xs[e] = X[t * NX + e];
        if (t < N) sm.xn[e] = X[(t + 1) * NX + e];
      }
      if (t < N) {
        for (int e = lane; e < NU; e += 32) sm.us[e] = U[t * NU + e];
        for (int e = lane; e < M::NPAR; e += 32) sm.par[e] = par[t * M::NPAR + e];
      }
      for (int e = lane; e < M::NREF; e += 32) sm.ref[e] = ref[t * M::NREF + e];
      __syncwarp();
      float gcol[NZ], gj;
      cost_column<M>(mc, sm, j, t == N, gcol, &gj);
      if (t == N) {
        if (j < NX) {
          rd = fmaxf(rd, fabsf(gj - V[t * NX + j]));
          gm = fmaxf(gm, fabsf(gj));
        }
        break;
      }
      if (j < NX + NU) {
        DF xd[NX], ud[NU], fd[NX];
#pragma unroll
        for (int i = 0; i < NX; ++i) xd[i] = mkd(sm.xs[i], i == j ? 1.0f : 0.0f);
#pragma unroll
        for (int a = 0; a < NU; ++a) ud[a] = mkd(sm.us[a], NX + a == j ? 1.0f : 0.0f);
        M::template dynamics<DF>(mc, xd, ud, sm.par, fd);
        float r = gj;
#pragma unroll
        for (int i = 0; i < NX; ++i) r += fd[i].d * V[(t + 1) * NX + i];
        if (j < NX) r -= V[t * NX + j];
        rd = fmaxf(rd, fabsf(r));
        gm = fmaxf(gm, fabsf(gj));
        if (j == 0) {
#pragma unroll
          for (int i = 0; i < NX; ++i) rp = fmaxf(rp, fabsf(fd[i].v - sm.xn[i]));
        }
      }
    }
    rp = warp_max(rp);
    rd = warp_max(rd);
    gm = warp_max(gm);
    if (lane == 0) {
      float* o = bp.kkt + (size_t)b * 3;
      o[0] = rp;
      o[1] = rd / (1.0f + gm);
      o[2] = fmaxf(o[0], o[1]);
    }
  }
  // ================================================ status
  int bad = 0;
  for (int e = lane; e < (N + 1) * NX; e += 32)
    if (!isfinite(X[e]) || !isfinite(V[e])) bad = 1;
  for (int e = lane; e < N * NU; e += 32)
    if (!isfinite(U[e])) bad = 1;
  status = warp_or(status | (bad ? ST_NAN : 0));
  if (bp.status && lane == 0) bp.status[b] = status;
}

template <class M>
__global__ void sqp_kernel(ModelConst mc, SqpParams sp, BatchPtrs bp) {
  extern __shared__ float4 smem_raw[];
  WarpSmem<M>* sms = reinterpret_cast<WarpSmem<M>*>(smem_raw);
  const int wib = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int gw = blockIdx.x * (blockDim.x >> 5) + wib;
  WarpSmem<M>& sm = sms[wib];
  float* scr = bp.scratch + (size_t)gw * bp.scratch_stride;
  if (bp.single_instance >= 0) {
    if (gw == 0) solve_instance<M>(mc, sp, bp, bp.single_instance, sm, scr);
    return;
  }
  for (;;) {
    int b = 0;
    if (lane == 0) b = atomicAdd(bp.counter, 1);
    b = __shfl_sync(0xffffffffu, b, 0);
    if (b >= bp.batch) break;
    solve_instance<M>(mc, sp, bp, b, sm, scr);
  }
}

}  // namespace mpxg
