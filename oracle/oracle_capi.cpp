// ============================================================================
// C entry points of the CPU ORACLE (test infrastructure only; see oracle.hpp).
// Loaded by tests/ and bench.py through oracle/oracle.py (ctypes).
// ============================================================================
#include <cstdio>
#include <cstdlib>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "flops.hpp"
#include "oracle.hpp"
#include "refgen.hpp"

using namespace oracle;

extern "C" {

// Mirrors the product's mpxg_problem_desc fields that the arithmetic needs.
typedef struct {
  int model, n, m, n_contact;
  double dt, mass, gravity, mu, barrier_alpha, barrier_sigma, foot_length, foot_width;
  int barrier_kind;
  int barrier_masked;
  double barrier_hess_scale;
  double inertia[9], inertia_inv[9];
  double cone_eps2;
} orc_model;

typedef struct {
  int sqp_iters, ls_max_trials;
  double ls_beta, ls_eta, reg, rho0, ls_skip_tol;
} orc_opts;

// Generic LQ stage data for a batch, all [B, ...] stage-major, double.
typedef struct {
  const double *A, *B, *c, *Q, *R, *M, *q, *r;
} orc_lq;

}  // extern "C" (types)

static ModelParams to_mp(const orc_model* d) {
  ModelParams mp;
  mp.model = d->model; mp.n = d->n; mp.m = d->m; mp.n_contact = d->n_contact;
  mp.dt = d->dt; mp.mass = d->mass; mp.gravity = d->gravity; mp.mu = d->mu;
  mp.barrier_alpha = d->barrier_alpha; mp.barrier_sigma = d->barrier_sigma;
  mp.foot_length = d->foot_length; mp.foot_width = d->foot_width;
  mp.barrier_kind = d->barrier_kind; mp.barrier_masked = d->barrier_masked; mp.barrier_hess_scale = d->barrier_hess_scale;
  for (int i = 0; i < 9; ++i) { mp.inertia[i] = d->inertia[i]; mp.inertia_inv[i] = d->inertia_inv[i]; }
  mp.cone_eps2 = d->cone_eps2 > 0.0 ? d->cone_eps2 : 1e-2;
  return mp;
}
static Opts to_opts(const orc_opts* o) {
  Opts op;
  op.sqp_iters = o->sqp_iters; op.ls_max_trials = o->ls_max_trials; op.ls_beta = o->ls_beta;
  op.ls_eta = o->ls_eta; op.reg = o->reg; op.rho0 = o->rho0; op.ls_skip_tol = o->ls_skip_tol;
  return op;
}

template <class T>
static void cvt(const double* src, size_t cnt, std::vector<T>& dst) {
  dst.resize(cnt);
  for (size_t i = 0; i < cnt; ++i) dst[i] = T(src[i]);
}

// Per-instance copies of the inputs in precision T.
template <class T>
struct InstBuf {
  std::vector<T> x0, X, U, V, ref, par, W, A, B, c, Q, R, M, q, r, K, k;
  LQData<T> lq;
};

template <class T>
static void load_instance(const ModelParams& mp, int b, int Nmax, int N, const double* x0, const double* X, const double* U,
                          const double* V, const double* ref, const double* par, const double* W, const orc_lq* lq,
                          InstBuf<T>& ib) {
  const int n = mp.n, m = mp.m;
  const int rc = ref_cols(mp.model), pc = par_cols(mp.model);
  cvt(x0 + (size_t)b * n, n, ib.x0);
  cvt(X + (size_t)b * (Nmax + 1) * n, (size_t)(N + 1) * n, ib.X);
  cvt(U + (size_t)b * Nmax * m, (size_t)N * m, ib.U);
  cvt(V + (size_t)b * (Nmax + 1) * n, (size_t)(N + 1) * n, ib.V);
  if (mp.model == MODEL_GENERIC_LQ) {
    cvt(lq->A + (size_t)b * Nmax * n * n, (size_t)N * n * n, ib.A);
    cvt(lq->B + (size_t)b * Nmax * n * m, (size_t)N * n * m, ib.B);
    cvt(lq->c + (size_t)b * Nmax * n, (size_t)N * n, ib.c);
    // terminal Q/q live at row N of the padded [Nmax+1] arrays
    ib.Q.resize((size_t)(N + 1) * n * n); ib.q.resize((size_t)(N + 1) * n);
    for (size_t i = 0; i < (size_t)N * n * n; ++i) ib.Q[i] = T(lq->Q[(size_t)b * (Nmax + 1) * n * n + i]);
    for (size_t i = 0; i < (size_t)n * n; ++i) ib.Q[(size_t)N * n * n + i] = T(lq->Q[(size_t)b * (Nmax + 1) * n * n + (size_t)Nmax * n * n + i]);
    for (size_t i = 0; i < (size_t)N * n; ++i) ib.q[i] = T(lq->q[(size_t)b * (Nmax + 1) * n + i]);
    for (size_t i = 0; i < (size_t)n; ++i) ib.q[(size_t)N * n + i] = T(lq->q[(size_t)b * (Nmax + 1) * n + (size_t)Nmax * n + i]);
    cvt(lq->R + (size_t)b * Nmax * m * m, (size_t)N * m * m, ib.R);
    cvt(lq->M + (size_t)b * Nmax * n * m, (size_t)N * n * m, ib.M);
    cvt(lq->r + (size_t)b * Nmax * m, (size_t)N * m, ib.r);
    ib.lq = LQData<T>{ib.A.data(), ib.B.data(), ib.c.data(), ib.Q.data(), ib.R.data(), ib.M.data(), ib.q.data(), ib.r.data()};
  } else {
    cvt(ref + (size_t)b * (Nmax + 1) * rc, (size_t)(N + 1) * rc, ib.ref);
    cvt(par + (size_t)b * (Nmax + 1) * pc, (size_t)(N + 1) * pc, ib.par);
    cvt(W + (size_t)b * NW * NW, (size_t)NW * NW, ib.W);
  }
}

template <class T>
static int solve_batch(const orc_model* md, const orc_opts* od, int B, int Nmax, const int* horizon, const double* x0,
                       const double* X_in, const double* U_in, const double* V_in, const double* ref, const double* par,
                       const double* W, const orc_lq* lq, double* X, double* U, double* V, double* K, double* k,
                       double* kkt, int* status, int n_threads) {
  const ModelParams mp = to_mp(md);
  const Opts op = to_opts(od);
  const int n = mp.n, m = mp.m;
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (int b = 0; b < B; ++b) {
    const int N = horizon ? horizon[b] : Nmax;
    InstBuf<T> ib;
    load_instance<T>(mp, b, Nmax, N, x0, X_in, U_in, V_in, ref, par, W, lq, ib);
    Instance<T> in{N, ib.x0.data(), ib.ref.data(), ib.par.data(), ib.W.data(), &ib.lq};
    ib.K.assign((size_t)N * m * n, T(0));
    ib.k.assign((size_t)N * m, T(0));
    int st = sqp_solve(mp, op, in, ib.X.data(), ib.U.data(), ib.V.data(), ib.K.data(), ib.k.data());
    if (status) status[b] = st;
    for (size_t i = 0; i < (size_t)(N + 1) * n; ++i) { X[(size_t)b * (Nmax + 1) * n + i] = double(ib.X[i]); V[(size_t)b * (Nmax + 1) * n + i] = double(ib.V[i]); }
    for (size_t i = 0; i < (size_t)N * m; ++i) U[(size_t)b * Nmax * m + i] = double(ib.U[i]);
    if (K) for (size_t i = 0; i < (size_t)N * m * n; ++i) K[(size_t)b * Nmax * m * n + i] = double(ib.K[i]);
    if (k) for (size_t i = 0; i < (size_t)N * m; ++i) k[(size_t)b * Nmax * m + i] = double(ib.k[i]);
    if (kkt) {
      // residual of the result, always evaluated in FP64
      InstBuf<double> jb;
      load_instance<double>(mp, b, Nmax, N, x0, X, U, V, ref, par, W, lq, jb);
      Instance<double> jn{N, jb.x0.data(), jb.ref.data(), jb.par.data(), jb.W.data(), &jb.lq};
      kkt_residual(mp, jn, jb.X.data(), jb.U.data(), jb.V.data(), kkt + 3 * (size_t)b);
    }
  }
  return 0;
}

extern "C" {

// Full SQP solve of a batch.  precision: 32 or 64.  All arrays are padded to
// Nmax: X/V [B, Nmax+1, n], U [B, Nmax, m], ref [B, Nmax+1, rc], par [B, Nmax+1, pc],
// W [B, 24, 24], K [B, Nmax, m, n], k [B, Nmax, m], kkt [B, 3], status [B].
int orc_sqp_solve(const orc_model* md, const orc_opts* od, int precision, int B, int Nmax, const int* horizon,
                  const double* x0, const double* X_in, const double* U_in, const double* V_in, const double* ref,
                  const double* par, const double* W, const orc_lq* lq, double* X, double* U, double* V, double* K,
                  double* k, double* kkt, int* status, int n_threads) {
  if (precision == 32)
    return solve_batch<float>(md, od, B, Nmax, horizon, x0, X_in, U_in, V_in, ref, par, W, lq, X, U, V, K, k, kkt, status, n_threads);
  return solve_batch<double>(md, od, B, Nmax, horizon, x0, X_in, U_in, V_in, ref, par, W, lq, X, U, V, K, k, kkt, status, n_threads);
}

// KKT residual (FP64) of given trajectories; kkt [B, 3] = (r_prim, r_dual, max).
int orc_kkt_residual(const orc_model* md, int B, int Nmax, const int* horizon, const double* x0, const double* X,
                     const double* U, const double* V, const double* ref, const double* par, const double* W,
                     const orc_lq* lq, double* kkt) {
  const ModelParams mp = to_mp(md);
  for (int b = 0; b < B; ++b) {
    const int N = horizon ? horizon[b] : Nmax;
    InstBuf<double> jb;
    load_instance<double>(mp, b, Nmax, N, x0, X, U, V, ref, par, W, lq, jb);
    Instance<double> jn{N, jb.x0.data(), jb.ref.data(), jb.par.data(), jb.W.data(), &jb.lq};
    kkt_residual(mp, jn, jb.X.data(), jb.U.data(), jb.V.data(), kkt + 3 * (size_t)b);
  }
  return 0;
}

// One dynamics step (FP64): xn = f(x, u; par).
int orc_dynamics(const orc_model* md, const double* x, const double* u, const double* par, double* xn) {
  ModelParams mp = to_mp(md);
  dynamics(mp, x, u, par, xn);
  return 0;
}
// One dynamics step in FP32.
int orc_dynamics_f32(const orc_model* md, const float* x, const float* u, const float* par, float* xn) {
  ModelParams mp = to_mp(md);
  dynamics(mp, x, u, par, xn);
  return 0;
}
// Stage cost (FP64).  terminal != 0 selects the t == N branch.
double orc_cost(const orc_model* md, const double* x, const double* u, const double* ref, const double* W, int terminal) {
  ModelParams mp = to_mp(md);
  return stage_cost(mp, x, u, ref, W, terminal != 0);
}
float orc_cost_f32(const orc_model* md, const float* x, const float* u, const float* ref, const float* W, int terminal) {
  ModelParams mp = to_mp(md);
  return stage_cost(mp, x, u, ref, W, terminal != 0);
}
// Linearisation of one SRBD stage (FP64): A [n,n], B [n,m], fx [n], g [n+m], H [(n+m)^2], l.
int orc_linearize(const orc_model* md, const double* x, const double* u, const double* ref, const double* par,
                  const double* W, int terminal, double* A, double* Bm, double* fx, double* g, double* H, double* l) {
  ModelParams mp = to_mp(md);
  StageLin<double> L;
  linearize_stage(mp, 0, terminal != 0, x, u, ref, par, W, (const LQData<double>*)nullptr, L);
  const int n = mp.n, m = mp.m, nz = n + m;
  for (int i = 0; i < n * n; ++i) A[i] = L.A[i];
  for (int i = 0; i < n * m; ++i) Bm[i] = L.B[i];
  for (int i = 0; i < n; ++i) fx[i] = L.fx[i];
  for (int i = 0; i < nz; ++i) g[i] = L.g[i];
  for (int i = 0; i < nz * nz; ++i) H[i] = L.H[i];
  *l = L.l;
  return 0;
}
// Barrier penalty and its second derivative (FP64), for tests.
double orc_penalty(const orc_model* md, double c) { ModelParams mp = to_mp(md); return penalty(mp, c); }
double orc_penalty_dd(const orc_model* md, double c) { ModelParams mp = to_mp(md); return penalty_dd(mp, c); }

// Pure LQR in absolute coordinates (config "isolated KKT/LQR"):
//   x_{t+1} = A x + B u + c, cost 1/2 x'Qx + x'Mu + 1/2 u'Ru + q'x + r'u, terminal Q_N, q_N,
// solved by the sequential Riccati recursion.  Outputs K [B,N,m,n], k [B,N,m], X [B,N+1,n],
// U [B,N,m], lam [B,N+1,n] (costates = dV/dx along the optimal trajectory).
int orc_lqr_solve(int precision, int B, int N, int n, int m, const double* A, const double* Bm, const double* c,
                  const double* Q, const double* R, const double* M, const double* q, const double* r,
                  const double* x0, double* K, double* k, double* X, double* U, double* lam, int n_threads) {
  orc_model md{};
  md.model = MODEL_GENERIC_LQ; md.n = n; md.m = m;
  orc_opts od{1, 1, 0.5, 1e-4, 0.0, 1.0, 1e300};
  std::vector<double> X0((size_t)B * (N + 1) * n, 0.0), U0((size_t)B * N * m, 0.0), V0((size_t)B * (N + 1) * n, 0.0);
  orc_lq lq{A, Bm, c, Q, R, M, q, r};
  int rc = orc_sqp_solve(&md, &od, precision, B, N, nullptr, x0, X0.data(), U0.data(), V0.data(), nullptr, nullptr,
                         nullptr, &lq, X, U, lam, K, k, nullptr, nullptr, n_threads);
  // With the zero initial guess the SQP step is the LQR solution itself: the
  // gains are the LQR gains and k is the feedforward at x = 0.
  return rc;
}

// Gait timer (mpc_utils.py:7-14), FP32.
void orc_timer_run(float duty, float step_freq, float dt, int n, float* leg_time, int* contact) {
  timer_run(duty, step_freq, dt, n, leg_time, contact);
}

// SRBD reference generator (mpc_utils.py:146-270), FP32, one instance.
int orc_refgen_srbd(int N, float dt, float mass, const float* foot0, float duty_factor, float step_freq,
                    float step_height, float clearence_speed, const float* t_timer, const float* x, const float* foot,
                    const float* input, const float* contact, float* liftoff, float* reference, float* parameter,
                    float* foot_ref_dot) {
  RefGenCfg g;
  g.N = N; g.dt = dt; g.n_contact = 4; g.mass = mass;
  for (int i = 0; i < 12; ++i) g.foot0[i] = foot0[i];
  g.duty_factor = duty_factor; g.step_freq = step_freq; g.step_height = step_height; g.clearence_speed = clearence_speed;
  refgen_srbd(g, t_timer, x, foot, input, contact, liftoff, reference, parameter, foot_ref_dot);
  return 0;
}

// Whole-body reference generator (mpc_utils.py:15-145), FP32, one instance.
int orc_refgen_wb(int N, int nj, float dt, float mass, const float* foot0, const float* q0, float duty_factor,
                  float step_freq, float step_height, float clearence_speed, int terrain, const float* t_timer,
                  const float* x, const float* foot, const float* input, const float* contact, float* liftoff,
                  float* reference, float* parameter) {
  RefGenCfg g;
  g.N = N; g.dt = dt; g.n_contact = 4; g.mass = mass;
  for (int i = 0; i < 12; ++i) g.foot0[i] = foot0[i];
  g.duty_factor = duty_factor; g.step_freq = step_freq; g.step_height = step_height; g.clearence_speed = clearence_speed;
  refgen_wb(g, nj, q0, terrain, t_timer, x, foot, input, contact, liftoff, reference, parameter);
  return 0;
}

// Model FLOPs of one non-terminal stage at (x, u) (flops.hpp): out = {f,
// f with [A B], l, the linearisation, one line-search trial}.
void orc_stage_flops(const orc_model* md, const double* x, const double* u, const double* ref, const double* par,
                     const double* W, double* out) {
  const flopcount::StageCount c = flopcount::count_stage(to_mp(md), x, u, ref, par, W);
  out[0] = c.dyn_value; out[1] = c.dyn_jacobian; out[2] = c.cost_value; out[3] = c.linearisation; out[4] = c.trial;
}

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
