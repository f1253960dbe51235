// Whole-body SQP (mpxg_wb_sqp): the whole-body MPC solve of mpc_wrapper.py's
// wrappers (quadruped_wb_dynamics, models.py:39-117; quadruped_wb_obj and
// quadruped_wb_hessian_gn, objectives.py:77-203), one SQP iteration as
// eight launches:
//   wb_lin_kernel    a warp per (instance, stage): the dynamics step in
//                    float64 at X_t, U_t (the defects' f); and in the same
//                    launch a warp per (instance, stage, column): the step on
//                    a forward-mode dual number seeded on one state or
//                    control entry, in float32: a column of A_t or B_t, exact
//                    up to float32 rounding;
//   wb_quad_kernel   a warp per (instance, stage): defects, stage cost,
//                    gradient, Gauss-Newton blocks (float64, written float32);
//   wb_riccati_kernel  a 256-thread block per instance: the float32 Riccati
//                    sweep over the dense n = 61 stage blocks, forward sweep
//                    and costates (the block products and eliminations of
//                    lqr_eq_kernel.cuh, without equality rows);
//   wb_merit_kernel  a block per instance: directional derivative, penalty
//                    update, merit at the current iterate;
//   wb_trial_kernel  a warp per (instance, trial step, stage): the merit's
//                    stage terms at X + a_k dX (dynamics step, cost, defect),
//                    launched for the full step, then for every shorter trial
//                    a_k = beta^k at once for the instances that reject it;
//   wb_accept_kernel a block per instance after each trial launch: the first
//                    trial that passes the Armijo test (the same choice as
//                    trying them in order), then the update.
// The defects and the merit take the step in float64 (the merit's changes near
// convergence are ~1e-7 of its value); the derivatives and the Riccati run in
// float32 like every other solve here.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <string>

#include "../../include/mpxg.h"
#include "internal.h"
#include "lqr_eq_kernel.cuh"
#include "wb_kernel.cuh"

using namespace mpxg;

namespace mpxg {
namespace wb {

// A forward-mode dual number with one tangent: (value, derivative) in
// float32.  The templated rigid-body and step code of wb_kernel.cuh runs on
// it unchanged; every operation carries the derivative by the chain rule.
struct D1 {
  float v, d;
  D1() = default;
  __device__ __forceinline__ D1(float a) : v(a), d(0.0f) {}
  __device__ __forceinline__ D1(double a) : v((float)a), d(0.0f) {}
  __device__ __forceinline__ D1(int a) : v((float)a), d(0.0f) {}
  __device__ __forceinline__ D1(float a, float b) : v(a), d(b) {}
};
__device__ __forceinline__ D1 operator+(D1 a, D1 b) { return D1(a.v + b.v, a.d + b.d); }
__device__ __forceinline__ D1 operator-(D1 a, D1 b) { return D1(a.v - b.v, a.d - b.d); }
__device__ __forceinline__ D1 operator*(D1 a, D1 b) { return D1(a.v * b.v, fmaf(a.v, b.d, a.d * b.v)); }
__device__ __forceinline__ D1 operator/(D1 a, D1 b) {
  const float q = a.v / b.v;
  return D1(q, (a.d - q * b.d) / b.v);
}
__device__ __forceinline__ D1 operator-(D1 a) { return D1(-a.v, -a.d); }
__device__ __forceinline__ D1 operator+(D1 a, float b) { return D1(a.v + b, a.d); }
__device__ __forceinline__ D1 operator+(float a, D1 b) { return D1(a + b.v, b.d); }
__device__ __forceinline__ D1 operator-(D1 a, float b) { return D1(a.v - b, a.d); }
__device__ __forceinline__ D1 operator-(float a, D1 b) { return D1(a - b.v, -b.d); }
__device__ __forceinline__ D1 operator*(D1 a, float b) { return D1(a.v * b, a.d * b); }
__device__ __forceinline__ D1 operator*(float a, D1 b) { return D1(a * b.v, a * b.d); }
__device__ __forceinline__ D1& operator+=(D1& a, D1 b) { return a = a + b; }
__device__ __forceinline__ D1& operator-=(D1& a, D1 b) { return a = a - b; }
__device__ __forceinline__ D1& operator*=(D1& a, D1 b) { return a = a * b; }
__device__ __forceinline__ D1& operator+=(D1& a, float b) { return a = a + b; }
__device__ __forceinline__ bool operator>(D1 a, D1 b) { return a.v > b.v; }
__device__ __forceinline__ bool operator<(D1 a, D1 b) { return a.v < b.v; }
__device__ __forceinline__ bool operator>(D1 a, float b) { return a.v > b; }
__device__ __forceinline__ bool operator<(D1 a, float b) { return a.v < b; }
__device__ __forceinline__ D1 sqrt_t(D1 a) {
  const float r = sqrtf(a.v);
  return D1(r, a.d / (2.0f * r));
}
__device__ __forceinline__ D1 rsqrt_t(D1 a) {
  const float r = rsqrtf(a.v);
  return D1(r, -0.5f * r * r * r * a.d);
}
__device__ __forceinline__ void sincos_t(D1 a, D1* s, D1* c) {
  float sv, cv;
  sincosf(a.v, &sv, &cv);
  *s = D1(sv, cv * a.d);
  *c = D1(cv, -sv * a.d);
}
__device__ __forceinline__ D1 __shfl_sync(unsigned mask, D1 a, int src) {
  return D1(::__shfl_sync(mask, a.v, src), ::__shfl_sync(mask, a.d, src));
}

}  // namespace wb
}  // namespace mpxg

namespace {

// quadruped capacity: 16 bodies, 20 dofs, 4 contacts; two warps per block
// (the float64 per-warp state is ~15 KB)
using WbCap = wb::Cap<16, 20, 4, 2, 1>;
constexpr int kNW = WbCap::NW;
constexpr int kNX = 61, kNU = 12, kNZ = 37;  // the built Riccati size (nv = 18, 4 contacts); kNZ = nq + nv
constexpr int kMaxX = 64, kMaxU = 16, kMaxRef = 64, kMaxW = 80, kMaxC = 4, kMaxTrials = 8;

struct WbDims {
  int nq, nv, nj, nc, nr, nx, nz, nR, ncol;
};

WbDims wb_dims(const mpxg_wb_model& m) {
  WbDims d{};
  d.nv = m.nv;
  d.nq = m.nq;
  d.nj = m.nv - 6;
  d.nc = m.n_contact;
  d.nr = 3 * d.nc;
  d.nx = d.nq + d.nv + 2 * d.nr;
  d.nz = d.nq + d.nv;
  d.nR = 12 + 3 * d.nj + 6 * d.nc;
  d.ncol = 13 + d.nj + 7 * d.nc;
  return d;
}

// Device view of one mpxg_wb_sqp call: the caller's arrays and the workspace.
struct WbSqp {
  int B, N, KT, first;
  int k_lo, k_hi, phase;  // trial steps of this wb_trial_kernel launch; wb_accept_kernel's pass
  // float64 steps per block (1 or kNW) of wb_lin_kernel's nominal part and
  // of wb_trial_kernel: one while a launch has fewer steps than the SMs
  // hold at kNW, so that each step has an SM's FP64 pipe to itself
  int nom_pb, trial_pb;
  WbDims d;
  double dt, alpha, beta, eta, skip_tol, rho0;
  float reg;
  int swing;
  const float *x0, *ref, *W;
  const int* contact;
  float *X, *U, *V;
  double *fnom, *cd, *sums, *ls, *trial;
  // f of every trial step at its stages [B, KT, N, nx], and per instance the
  // accepted trial + 1 (0: the iterate's f is not cached), so that the next
  // linearisation takes the accepted step's f instead of recomputing it
  double* fcache;
  int* fvalid;
  float *A, *Bm, *c, *x0s, *Q, *R, *M, *q, *r, *K, *k, *dX, *dU, *lam, *Pscr;
  unsigned* kbits;
  int* status;
  float* kkt;
};

// ---------------------------------------------------------------- cost
// The relaxed barrier of objectives.py:7-13 and its derivatives where it is
// smooth (the clipped ranges have zero derivative).
__device__ __forceinline__ double pen_raw(double c, double a, double s) {
  const double logb = -a * log(fmin(fmax(c, 1e-10), 1e6));
  const double t = (c - 2.0 * s) / s;
  return c > s ? logb : a / 2.0 * (t * t - 1.0) + logb;
}
__device__ __forceinline__ double pen(double c, double a, double s) { return fmin(fmax(pen_raw(c, a, s), 0.0), 1e8); }
__device__ __forceinline__ double pen_d(double c, double a, double s) {
  const double logd = (c > 1e-10 && c < 1e6) ? -a / c : 0.0;
  const double d = c > s ? logd : a * (c - 2.0 * s) / (s * s) + logd;
  const double v = pen(c, a, s);
  return (v > 0.0 && v < 1e8) ? d : 0.0;
}
__device__ __forceinline__ double pen_dd(double c, double a, double s) {
  const double logdd = (c > 1e-10 && c < 1e6) ? a / (c * c) : 0.0;
  const double dd = c > s ? logdd : a / (s * s) + logdd;
  const double raw = pen_raw(c, a, s);
  return (raw > 0.0 && raw < 1e8) ? fmin(fmax(dd, -1e6), 1e6) : 0.0;
}

// conj(v) * u as a left-multiplication matrix L(conj v) applied to u
__device__ __forceinline__ void qconj_mul(const double* v, const double* u, double* o, double L[4][4]) {
  const double a0 = v[0], a1 = -v[1], a2 = -v[2], a3 = -v[3];
  const double Lm[4][4] = {{a0, -a1, -a2, -a3}, {a1, a0, -a3, a2}, {a2, a3, a0, -a1}, {a3, -a2, a1, a0}};
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    o[i] = Lm[i][0] * u[0] + Lm[i][1] * u[1] + Lm[i][2] * u[2] + Lm[i][3] * u[3];
#pragma unroll
    for (int k = 0; k < 4; ++k) L[i][k] = Lm[i][k];
  }
}

// quat_sub(u, v): the rotation vector of conj(v) u (angle in (-pi, pi]) and,
// if J, its 3 x 4 Jacobian w.r.t. u (at a zero vector part the limit 2/s I
// of the smooth map).
__device__ void quat_sub_d(const double* u, const double* v, double* e, double (*J)[4]) {
  double q[4], L[4][4];
  qconj_mul(v, u, q, L);
  const double s = q[0], n = sqrt(q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  double th = 2.0 * atan2(n, s);
  if (th > M_PI) th -= 2.0 * M_PI;
  double a[3] = {0.0, 0.0, 0.0};
  if (n > 0.0) {
    a[0] = q[1] / n; a[1] = q[2] / n; a[2] = q[3] / n;
  }
#pragma unroll
  for (int i = 0; i < 3; ++i) e[i] = a[i] * th;
  if (!J) return;
  double D[3][4];  // d(result)/d(s, w)
  if (n > 0.0) {
    const double r2 = s * s + n * n;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      D[i][0] = a[i] * (-2.0 * n / r2);
#pragma unroll
      for (int k = 0; k < 3; ++k)
        D[i][1 + k] = a[i] * a[k] * (2.0 * s / r2) + th * ((i == k ? 1.0 : 0.0) - a[i] * a[k]) / n;
    }
  } else {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      D[i][0] = 0.0;
#pragma unroll
      for (int k = 0; k < 3; ++k) D[i][1 + k] = i == k ? 2.0 / s : 0.0;
    }
  }
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int k = 0; k < 4; ++k) J[i][k] = D[i][0] * L[0][k] + D[i][1] * L[1][k] + D[i][2] * L[2][k] + D[i][3] * L[3][k];
}

// Per-warp operands and results of one stage's cost.
struct CostScr {
  double x[kMaxX], u[kMaxU], r[kMaxRef], w[kMaxW];
  double gx[kMaxX], gu[kMaxU], diag[kMaxX], rdiag[kMaxU];
  double qb[4][4], cb[kMaxC][3][3];
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// One stage of quadruped_wb_obj (objectives.py:77-125; terminal: the t == N
// branch) at s.x, s.u, s.r, s.w; returns the stage cost on every lane.  With
// DERIV also its gradient (s.gx, s.gu) and the Gauss-Newton blocks of
// quadruped_wb_hessian_gn (objectives.py:127-203): the diagonal part of H_xx
// (s.diag), the quaternion block (s.qb, rows/columns 3..6), the friction-cone
// blocks (s.cb, the force entries of each contact) and the diagonal H_uu
// (s.rdiag, without reg); H_xu is zero (no residual row reads both).
template <bool DERIV>
__device__ double stage_eval(const WbDims& d, CostScr& s, bool terminal, bool swing, int lane) {
  const int nj = d.nj, nc = d.nc, nx = d.nx;
  const int a = 12 + 2 * nj, g0 = 13 + 2 * nj + 3 * nc, rc = 13 + nj + 3 * nc;
  double acc = 0.0;
  for (int i = lane; i < nx; i += 32) {
    double g = 0.0, h = 0.0;
    if (i < 3) {
      const double e = s.x[i] - s.r[i], w = s.w[i];
      acc += w * e * e; g = w * e; h = w;
    } else if (i < 7) {
      // the quaternion rows: lane 0 below
    } else if (i < 13 + nj) {  // q, dp, omega: reference entry i, weight i - 1
      const double e = s.x[i] - s.r[i], w = s.w[i - 1];
      acc += w * e * e; g = w * e; h = w;
    } else if (i < 13 + 2 * nj) {  // dq, its speed limits
      const double e = s.x[i], w = s.w[i - 1];
      acc += w * e * e; g = w * e; h = w;
      if (!terminal) {
        const double lo = 10.0 + 1e-2 - e, hi = 10.0 + 1e-2 + e;
        acc += pen(lo, 1.0, 1.0) + pen(hi, 1.0, 1.0);
        g += 0.5 * (-pen_d(lo, 1.0, 1.0) + pen_d(hi, 1.0, 1.0));
        h += pen_dd(lo, 0.1, 5.0) + pen_dd(hi, 0.1, 5.0);
      }
    } else if (!terminal) {
      if (i < g0) {  // contact points
        const int k = i - (13 + 2 * nj);
        const double cm = swing ? 1.0 : s.r[rc + k / 3];
        const double e = cm * (s.x[i] - s.r[13 + nj + k]), w = s.w[a + k];
        acc += w * e * e; g = cm * w * e; h = cm * cm * w;
      } else {  // contact forces
        const int k = i - g0;
        const double e = s.x[i] - s.r[13 + nj + 4 * nc + k], w = s.w[a + 3 * nc + nj + k];
        acc += w * e * e; g = w * e; h = w;
      }
    }
    if (DERIV) {
      s.gx[i] = g;
      s.diag[i] = h;
    }
  }
  if (!terminal) {
    for (int j = lane; j < nj; j += 32) {  // torques and their limits
      const double uu = s.u[j], w = s.w[a + 3 * nc + j];
      const double lo = 44.0 + 1e-2 - uu, hi = 44.0 + 1e-2 + uu;
      acc += w * uu * uu + pen(lo, 1.0, 1.0) + pen(hi, 1.0, 1.0);
      if (DERIV) {
        s.gu[j] = w * uu + 0.5 * (-pen_d(lo, 1.0, 1.0) + pen_d(hi, 1.0, 1.0));
        s.rdiag[j] = w + pen_dd(lo, 1.0, 1.0) + pen_dd(hi, 1.0, 1.0);
      }
    }
  }
  if (DERIV) __syncwarp();
  if (lane == 0) {  // orientation residual quat_sub(quat, quat_ref)
    double e[3], J[3][4];
    quat_sub_d(s.x + 3, s.r + 3, e, DERIV ? J : nullptr);
#pragma unroll
    for (int k = 0; k < 3; ++k) acc += s.w[3 + k] * e[k] * e[k];
    if (DERIV) {
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        double g = 0.0;
#pragma unroll
        for (int k = 0; k < 3; ++k) g += J[k][c] * s.w[3 + k] * e[k];
        s.gx[3 + c] = g;
#pragma unroll
        for (int f = 0; f < 4; ++f) {
          double h = 0.0;
#pragma unroll
          for (int k = 0; k < 3; ++k) h += J[k][c] * s.w[3 + k] * J[k][f];
          s.qb[c][f] = h;
        }
      }
    }
  }
  if (!terminal && lane >= 1 && lane <= nc) {  // friction cone of contact lane - 1
    const int c = lane - 1;
    const double on = s.r[rc + c];
    const double fx = s.x[g0 + 3 * c], fy = s.x[g0 + 3 * c + 1], fz = s.x[g0 + 3 * c + 2];
    const double sq1 = sqrt(fy * fy + fx * fx + 1e-2);
    const double cone = 0.5 * fz - sq1;
    acc += pen(cone, 0.1, 5.0) * on;
    if (DERIV) {
      const double dc = 0.5 * pen_d(cone, 0.1, 5.0) * on;
      s.gx[g0 + 3 * c] += dc * (-fx / sq1);
      s.gx[g0 + 3 * c + 1] += dc * (-fy / sq1);
      s.gx[g0 + 3 * c + 2] += dc * 0.5;
      const double sq2 = sqrt(fy * fy + fx * fx + 1e-1);
      const double hh = pen_dd(0.5 * fz - sq2, 0.1, 5.0) * on;
      const double jf[3] = {-fx / sq2, -fy / sq2, 0.5};
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int k = 0; k < 3; ++k) s.cb[c][i][k] = hh * jf[i] * jf[k];
    }
  }
  if (DERIV) __syncwarp();
  return 0.5 * warp_sum(acc);
}

// ---------------------------------------------------------------- dynamics
// Per-warp state of the float64 step.
struct StepScr {
  wb::Warp<WbCap, double> w;
  double xb[kMaxX], ub[kMaxU], f[kMaxX];
};

// f(x, u) of the step model into s.f (every lane of the warp).
__device__ __forceinline__ void eval_step(const mpxg_wb_model& m, const WbSqp& p, StepScr& s, const double* x,
                                          const double* u, const int* contact, int lane) {
  const int nq = p.d.nq, nv = p.d.nv;
  for (int i = lane; i < nq; i += 32) s.w.qpos[i] = x[i];
  if (lane < nv) s.w.qvel[lane] = x[nq + lane];
  __syncwarp();
  wb::rb_terms(m, s.w, lane);
  wb::step(m, s.w, u, contact, p.dt, p.alpha, s.f, lane);
  __syncwarp();
}

// A warp per (instance b, stage t < N): the step at (X_t, U_t) in float64,
// into fnom, and the columns of A_t that f does not depend on (points,
// forces) set to zero.
__device__ __forceinline__ void nominal_item(const mpxg_wb_model& m, const WbSqp& p, StepScr& s, long long item,
                                             int lane) {
  const WbDims& d = p.d;
  const int b = (int)(item / p.N), t = (int)(item % p.N);
  const size_t st = (size_t)b * p.N + t;
  const int nx = d.nx;
  double* fo = p.fnom + st * nx;
  const int kv = p.fvalid[b];
  if (kv > 0) {  // the accepted trial evaluated f at exactly this (X_t, U_t)
    const double* fc = p.fcache + (((size_t)b * p.KT + (kv - 1)) * p.N + t) * nx;
    for (int i = lane; i < nx; i += 32) fo[i] = fc[i];
  } else {
    const float* Xt = p.X + ((size_t)b * (p.N + 1) + t) * nx;
    for (int i = lane; i < nx; i += 32) s.xb[i] = (double)Xt[i];
    if (lane < d.nj) s.ub[lane] = (double)p.U[st * d.nj + lane];
    __syncwarp();
    eval_step(m, p, s, s.xb, s.ub, p.contact + ((size_t)b * (p.N + 1) + t) * d.nc, lane);
    for (int i = lane; i < nx; i += 32) fo[i] = s.f[i];
  }
  float* At = p.A + st * nx * nx;
  const int nzc = nx - d.nz;
  for (int e = lane; e < nx * nzc; e += 32) At[(e / nzc) * nx + d.nz + e % nzc] = 0.0f;
}

// Per-warp state of the dual-number step.
struct JacScr {
  wb::Warp<WbCap, wb::D1> w;
  wb::D1 u[kMaxU], f[kMaxX];
};

// A warp per (instance b, stage t < N, column j < nz + nj): the step at
// (X_t, U_t) on dual numbers whose tangent is state entry j (j < nz) or
// control j - nz; the tangents of the result are column j of A_t or B_t.
__device__ __forceinline__ void jac_item(const mpxg_wb_model& m, const WbSqp& p, JacScr& s, long long item, int lane) {
  using wb::D1;
  const WbDims& d = p.d;
  const int ncols = d.nz + d.nj;
  const int b = (int)(item / ((long long)p.N * ncols));
  const int rem = (int)(item % ((long long)p.N * ncols));
  const int t = rem / ncols, j = rem % ncols;
  const size_t st = (size_t)b * p.N + t;
  const int nx = d.nx, nq = d.nq, nv = d.nv;
  const float* Xt = p.X + ((size_t)b * (p.N + 1) + t) * nx;
  for (int i = lane; i < nq; i += 32) s.w.qpos[i] = D1(Xt[i], i == j ? 1.0f : 0.0f);
  if (lane < nv) s.w.qvel[lane] = D1(Xt[nq + lane], nq + lane == j ? 1.0f : 0.0f);
  if (lane < d.nj) s.u[lane] = D1(p.U[st * d.nj + lane], d.nz + lane == j ? 1.0f : 0.0f);
  __syncwarp();
  wb::rb_terms(m, s.w, lane);
  wb::step(m, s.w, s.u, p.contact + ((size_t)b * (p.N + 1) + t) * d.nc, D1((float)p.dt), D1((float)p.alpha), s.f,
           lane);
  __syncwarp();
  for (int i = lane; i < nx; i += 32) {
    if (j < d.nz) p.A[st * nx * nx + (size_t)i * nx + j] = s.f[i].d;
    else p.Bm[st * nx * d.nj + (size_t)i * d.nj + (j - d.nz)] = s.f[i].d;
  }
}

// The linearisation's dynamics in one launch: warps 0 .. B N - 1 take the
// float64 steps at (X_t, U_t) (nominal_item), the following B N (nz + nj)
// warps the dual-number columns (jac_item); the long float64 chains start
// first and the two kinds overlap on the SMs.
__global__ void __launch_bounds__(32 * kNW) wb_lin_kernel(const __grid_constant__ mpxg_wb_model m,
                                                          const __grid_constant__ WbSqp p) {
  __shared__ union Scr {
    StepScr nom[kNW];
    JacScr jac[kNW];
  } sw;
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long nom = (long long)p.B * p.N, nom_blocks = (nom + p.nom_pb - 1) / p.nom_pb;
  if (blockIdx.x < nom_blocks) {
    const long long item = (long long)blockIdx.x * p.nom_pb + wid;
    if (wid < p.nom_pb && item < nom) nominal_item(m, p, sw.nom[wid], item, lane);
    return;
  }
  const long long item = (long long)(blockIdx.x - nom_blocks) * kNW + wid;
  if (item < nom * (p.d.nz + p.d.nj)) jac_item(m, p, sw.jac[wid], item, lane);
}

__device__ __forceinline__ void load_stage(const WbSqp& p, CostScr& s, int b, int t, int lane) {
  const WbDims& d = p.d;
  const float* Xt = p.X + ((size_t)b * (p.N + 1) + t) * d.nx;
  for (int i = lane; i < d.nx; i += 32) s.x[i] = (double)Xt[i];
  for (int j = lane; j < d.nj; j += 32) s.u[j] = t < p.N ? (double)p.U[((size_t)b * p.N + t) * d.nj + j] : 0.0;
  const float* rt = p.ref + ((size_t)b * (p.N + 1) + t) * d.ncol;
  for (int i = lane; i < d.ncol; i += 32) s.r[i] = (double)rt[i];
  for (int i = lane; i < d.nR; i += 32) s.w[i] = (double)p.W[(size_t)b * d.nR + i];
}

// A warp per (instance b, stage t <= N): defect c_t (float64 in cd, float32
// as the step problem's c / x0), the merit's stage terms (cost, V.c, c.c),
// and the stage's LQ data: q_t, r_t, dense Q_t, R_t (+ reg), M_t = 0.
__global__ void __launch_bounds__(128) wb_quad_kernel(const __grid_constant__ WbSqp p) {
  __shared__ CostScr sw[4];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long item = (long long)blockIdx.x * 4 + wid;
  if (item >= (long long)p.B * (p.N + 1)) return;
  const int b = (int)(item / (p.N + 1)), t = (int)(item % (p.N + 1));
  const WbDims& d = p.d;
  const int nx = d.nx, nj = d.nj;
  CostScr& s = sw[wid];
  load_stage(p, s, b, t, lane);
  __syncwarp();
  const bool term = t == p.N;
  const double cost = stage_eval<true>(d, s, term, p.swing != 0, lane);
  // defect
  const size_t s1 = (size_t)b * (p.N + 1) + t;
  const float* Vt = p.V + s1 * nx;
  double cv = 0.0, cc = 0.0;
  for (int i = lane; i < nx; i += 32) {
    const double ci = t == 0 ? (double)p.x0[(size_t)b * nx + i] - s.x[i]
                             : p.fnom[((size_t)b * p.N + t - 1) * nx + i] - s.x[i];
    p.cd[s1 * nx + i] = ci;
    if (t == 0) p.x0s[(size_t)b * nx + i] = (float)ci;
    else p.c[((size_t)b * p.N + t - 1) * nx + i] = (float)ci;
    cv += (double)Vt[i] * ci;
    cc += ci * ci;
  }
  cv = warp_sum(cv);
  cc = warp_sum(cc);
  if (lane == 0) {
    p.sums[s1 * 4 + 0] = cost;
    p.sums[s1 * 4 + 1] = cv;
    p.sums[s1 * 4 + 2] = cc;
  }
  // gradient
  for (int i = lane; i < nx; i += 32) p.q[s1 * nx + i] = (float)s.gx[i];
  // dense Q_t: the diagonal, the quaternion block, the cone blocks
  const int g0 = 13 + 2 * nj + 3 * d.nc;
  float* Qt = p.Q + s1 * nx * nx;
  for (int e = lane; e < nx * nx; e += 32) {
    const int i = e / nx, k = e % nx;
    double v = i == k ? s.diag[i] : 0.0;
    if (i >= 3 && i < 7 && k >= 3 && k < 7) v = s.qb[i - 3][k - 3];
    if (!term && i >= g0 && k >= g0 && (i - g0) / 3 == (k - g0) / 3) v += s.cb[(i - g0) / 3][(i - g0) % 3][(k - g0) % 3];
    Qt[e] = (float)v;
  }
  if (term) return;
  const size_t sn = (size_t)b * p.N + t;
  for (int j = lane; j < nj; j += 32) p.r[sn * nj + j] = (float)s.gu[j];
  float* Rt = p.R + sn * nj * nj;
  for (int e = lane; e < nj * nj; e += 32) {
    const int i = e / nj, k = e % nj;
    Rt[e] = i == k ? (float)(s.rdiag[i] + (double)p.reg) : 0.0f;
  }
  float* Mt = p.M + sn * nx * nj;
  for (int e = lane; e < nx * nj; e += 32) Mt[e] = 0.0f;
}

// ---------------------------------------------------------------- Riccati
// Columns NZ..NX-1 of every A_t are zero (the whole-body step does not read
// the contact-point and force states), so a stage's products are taken over
// the NC = NZ + NU columns of [A_Z | B] (A_Z the first NZ columns of A) and
// one more column: c_t, which P turns into P c + p.
//
// Shared-memory layout of the Riccati block (floats): the stage matrices
// column-major with odd leading dimensions, as lqr_eq_kernel's.  T, the
// value function before symmetrisation, spans AB and PAB (both dead by then).
template <int NX, int NU, int NZ>
struct RLay {
  static constexpr int NC = NZ + NU;
  static constexpr int LX = NX + (NX % 2 == 0 ? 1 : 2), LU = NU + (NU % 2 == 0 ? 1 : 2);
  static constexpr int P = 0, AB = P + NX * LX, PAB = AB + (NC + 1) * LX, T = AB, Q = PAB + (NC + 1) * LX,
                       M = Q + NX * LX, QUU = M + NU * LX, QUX = QUU + NU * LU, ZG = QUX + NX * LU,
                       PAN = (ZG + (NX + 1) * LU + 3) / 4 * 4, V = PAN + 2 * lqeq::kGjBlock * 32;
  static constexpr int VL = NX + 4;
  static constexpr int vq = V, vr = vq + VL, vp = vr + VL, vqx = vp + VL, vqu = vqx + VL, vx = vqu + VL,
                       vu = vx + VL, FLOATS = vu + VL;
  static_assert(2 * (NC + 1) * LX >= NX * LX, "T fits in AB and PAB");
};

// out(r, c) = sum_l X(r, l) Y(l, c) over 16 x 16 threads, the tiling and
// summation order of lqeq::bmm, each result handed to ep(r, c, sum) rather
// than stored; the inner loop unrolled 4 deep, so that a warp has four
// steps' shared-memory loads in flight.  Ends with a barrier.
template <int ROWS, int INNER, int COLS, bool TX, bool TY, class Ep>
__device__ __forceinline__ void bmm_ep(const float* X, int ldx, const float* Y, int ldy, Ep ep) {
  constexpr int TR = (ROWS + 15) / 16, TC = (COLS + 15) / 16;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  float acc[TR][TC];
#pragma unroll
  for (int i = 0; i < TR; ++i)
#pragma unroll
    for (int j = 0; j < TC; ++j) acc[i][j] = 0.0f;
#pragma unroll 4
  for (int l = 0; l < INNER; ++l) {
    float xa[TR], yb[TC];
#pragma unroll
    for (int i = 0; i < TR; ++i) {
      const int r = ty + 16 * i;
      xa[i] = (r < ROWS) ? (TX ? X[r * ldx + l] : X[l * ldx + r]) : 0.0f;
    }
#pragma unroll
    for (int j = 0; j < TC; ++j) {
      const int c = tx + 16 * j;
      yb[j] = (c < COLS) ? (TY ? Y[l * ldy + c] : Y[c * ldy + l]) : 0.0f;
    }
#pragma unroll
    for (int i = 0; i < TR; ++i)
#pragma unroll
      for (int j = 0; j < TC; ++j) acc[i][j] += xa[i] * yb[j];
  }
#pragma unroll
  for (int i = 0; i < TR; ++i)
#pragma unroll
    for (int j = 0; j < TC; ++j) {
      const int r = ty + 16 * i, c = tx + 16 * j;
      if (r < ROWS && c < COLS) ep(r, c, acc[i][j]);
    }
  __syncthreads();
}

// One stage's step-problem data held in registers: issued (global loads) at
// the top of the stage before it, committed to shared memory at that
// stage's end, so the loads' latency hides behind its products.
template <int NX, int NU, int NZ>
struct StagePre {
  typedef RLay<NX, NU, NZ> L;
  static constexpr int TH = lqeq::kThreads, NC = L::NC, LX = L::LX, LU = L::LU;
  static constexpr int nA = (NX * NZ + TH - 1) / TH, nB = (NX * NU + TH - 1) / TH, nQ = (NX * NX + TH - 1) / TH,
                       nR = (NU * NU + TH - 1) / TH, nV = (NX + TH - 1) / TH;
  static_assert(NU <= TH, "one thread per entry of r");
  float a[nA], bm[nB], q[nQ], m[nB], r[nR], c[nV], vq[nV], vr;

  __device__ __forceinline__ void issue(const mpxg_lq_eq_io& io, size_t sn, size_t sn1, int t) {
    const int tid = threadIdx.x;
    const float* A = io.A + (sn + t) * NX * NX;
    const float* Bm = io.Bm + (sn + t) * NX * NU;
    const float* Q = io.Q + (sn1 + t) * NX * NX;
    const float* M = io.M + (sn + t) * NX * NU;
    const float* R = io.R + (sn + t) * NU * NU;
#pragma unroll
    for (int i = 0; i < nA; ++i) {
      const int e = tid + TH * i;
      a[i] = e < NX * NZ ? __ldg(A + (e / NZ) * NX + e % NZ) : 0.0f;
    }
#pragma unroll
    for (int i = 0; i < nB; ++i) {
      const int e = tid + TH * i;
      bm[i] = e < NX * NU ? __ldg(Bm + e) : 0.0f;
      m[i] = e < NX * NU ? __ldg(M + e) : 0.0f;
    }
#pragma unroll
    for (int i = 0; i < nQ; ++i) {
      const int e = tid + TH * i;
      q[i] = e < NX * NX ? __ldg(Q + e) : 0.0f;
    }
#pragma unroll
    for (int i = 0; i < nR; ++i) {
      const int e = tid + TH * i;
      r[i] = e < NU * NU ? __ldg(R + e) : 0.0f;
    }
#pragma unroll
    for (int i = 0; i < nV; ++i) {
      const int e = tid + TH * i;
      c[i] = e < NX ? __ldg(io.c + (sn + t) * NX + e) : 0.0f;
      vq[i] = e < NX ? __ldg(io.q + (sn1 + t) * NX + e) : 0.0f;
    }
    vr = tid < NU ? __ldg(io.r + (sn + t) * NU + tid) : 0.0f;
  }

  // row-major sources to column-major shared memory: A_Z, B and c into the
  // columns of AB, Q, M, R into Q_uu's slot, q and r
  __device__ __forceinline__ void commit(float* s) const {
    const int tid = threadIdx.x;
#pragma unroll
    for (int i = 0; i < nA; ++i) {
      const int e = tid + TH * i;
      if (e < NX * NZ) s[L::AB + (e % NZ) * LX + e / NZ] = a[i];
    }
#pragma unroll
    for (int i = 0; i < nB; ++i) {
      const int e = tid + TH * i;
      if (e < NX * NU) {
        s[L::AB + (NZ + e % NU) * LX + e / NU] = bm[i];
        s[L::M + (e % NU) * LX + e / NU] = m[i];
      }
    }
#pragma unroll
    for (int i = 0; i < nQ; ++i) {
      const int e = tid + TH * i;
      if (e < NX * NX) s[L::Q + (e % NX) * LX + e / NX] = q[i];
    }
#pragma unroll
    for (int i = 0; i < nR; ++i) {
      const int e = tid + TH * i;
      if (e < NU * NU) s[L::QUU + (e % NU) * LU + e / NU] = r[i];
    }
#pragma unroll
    for (int i = 0; i < nV; ++i) {
      const int e = tid + TH * i;
      if (e < NX) {
        s[L::AB + NC * LX + e] = c[i];
        s[L::vq + e] = vq[i];
      }
    }
    if (tid < NU) s[L::vr + tid] = vr;
  }
};

// Riccati sweep of the step problem x_{t+1} = A x + B u + c (x_0 = c_0),
// cost 1/2 x'Qx + x'Mu + 1/2 u'Ru + q'x + r'u:
//   Q_xx = Q + A'PA, Q_ux = M' + B'PA, Q_uu = R + B'PB, q_x = q + A'(Pc + p),
//   q_u = r + B'(Pc + p), [Z | g] = Q_uu^-1 [Q_ux | q_u], K = -Z, k = -g,
//   P <- Q_xx - Q_ux'Z (symmetrised), p <- q_x + Q_ux'k;
// then dX, dU by the forward sweep and lam_t = P_t dX_t + p_t.  A stage is
// four block products: [P A_Z | P B | P c + p]; [A_Z | B]' times that
// (Q_xx's A-block, Q_ux's A-columns, Q_uu, q_x's A-part, q_u); the pivot
// solve; [Q_xx - Q_ux'Z | q_x - Q_ux'g].  Off the A-columns Q_xx, Q_ux and
// q_x are Q, M' and q.
template <int NX, int NU, int NZ>
__global__ void __launch_bounds__(lqeq::kThreads, 1) wb_riccati_kernel(mpxg_lq_eq_io io, float* Pscr) {
  using namespace lqeq;
  typedef RLay<NX, NU, NZ> L;
  constexpr int LX = L::LX, LU = L::LU, NC = L::NC;
  extern __shared__ float4 smem4[];
  float* s = reinterpret_cast<float*>(smem4);
  float *P = s + L::P, *AB = s + L::AB, *PAB = s + L::PAB, *T = s + L::T, *sQ = s + L::Q, *sM = s + L::M;
  float *Quu = s + L::QUU, *Qux = s + L::QUX, *ZG = s + L::ZG, *pan = s + L::PAN;
  float *vq = s + L::vq, *vr = s + L::vr, *vp = s + L::vp, *vqx = s + L::vqx, *vqu = s + L::vqu;
  float *vx = s + L::vx, *vu = s + L::vu;
  const int b = blockIdx.x, N = io.N, tid = threadIdx.x;
  constexpr int NP = NX + 1;
  float* Ps = Pscr + (size_t)b * (N + 1) * NP * NX;
  const size_t sn = (size_t)b * N, sn1 = (size_t)b * (N + 1);

  StagePre<NX, NU, NZ> pre;
  pre.issue(io, sn, sn1, N - 1);
  load_cm<NX, NX>(P, LX, io.Q + (sn1 + N) * NX * NX);
  load_vec<NX>(vp, io.q + (sn1 + N) * NX);
  pre.commit(s);
  __syncthreads();
  for (int e = tid; e < NX * NX; e += kThreads) Ps[(size_t)N * NP * NX + e] = P[(e / NX) * LX + e % NX];
  for (int i = tid; i < NX; i += kThreads) Ps[(size_t)N * NP * NX + NX * NX + i] = vp[i];

  for (int t = N - 1; t >= 0; --t) {
    if (t > 0) pre.issue(io, sn, sn1, t - 1);
    bmm_ep<NX, NX, NC + 1, false, false>(P, LX, AB, LX, [&](int r, int c, float v) {
      PAB[c * LX + r] = c < NC ? v : v + vp[r];
    });
    for (int e = tid; e < NU * (NX - NZ); e += kThreads) {  // Q_ux = M' off the A-columns
      const int a = e % NU, i = NZ + e / NU;
      Qux[i * LU + a] = sM[a * LX + i];
    }
    for (int i = NZ + tid; i < NX; i += kThreads) vqx[i] = vq[i];  // q_x = q off the A-columns
    bmm_ep<NC, NX, NC + 1, true, false>(AB, LX, PAB, LX, [&](int r, int c, float v) {
      if (c == NC) {
        if (r < NZ) vqx[r] = v + vq[r];
        else vqu[r - NZ] = v + vr[r - NZ];
      } else if (r < NZ) {
        if (c < NZ) sQ[c * LX + r] = v + sQ[c * LX + r];
      } else if (c < NZ) {
        Qux[c * LU + (r - NZ)] = v + sM[(r - NZ) * LX + c];
      } else {
        Quu[(c - NZ) * LU + (r - NZ)] = v + Quu[(c - NZ) * LU + (r - NZ)];
      }
    });
    gj_solve<NU, NU + NX + 1, kGjBlock>(pan, [&](int j, float* v) {
#pragma unroll
      for (int i = 0; i < NU; ++i)
        v[i] = j < NU ? Quu[j * LU + i] : (j < NU + NX ? Qux[(j - NU) * LU + i] : vqu[i]);
    }, [&](int j, const float* v) {
#pragma unroll
      for (int i = 0; i < NU; ++i) ZG[(j - NU) * LU + i] = v[i];
    });
    {
      float* Ko = io.K + (sn + t) * NU * NX;
      float* ko = io.k + (sn + t) * NU;
      for (int e = tid; e < NU * NX; e += kThreads) Ko[e] = -ZG[(e % NX) * LU + e / NX];
      for (int a = tid; a < NU; a += kThreads) ko[a] = -ZG[NX * LU + a];
    }
    bmm_ep<NX, NU, NX + 1, true, false>(Qux, LU, ZG, LU, [&](int r, int c, float v) {
      if (c < NX) T[c * LX + r] = -v + sQ[c * LX + r];
      else vp[r] = -v + vqx[r];
    });
    float* Pt = Ps + (size_t)t * NP * NX;
    for (int e = tid; e < NX * NX; e += kThreads) {
      const int c = e / NX, r = e % NX;
      const float v = 0.5f * (T[c * LX + r] + T[r * LX + c]);
      P[c * LX + r] = v;
      Pt[e] = v;
    }
    for (int i = tid; i < NX; i += kThreads) Pt[NX * NX + i] = vp[i];
    __syncthreads();
    if (t > 0) {
      pre.commit(s);
      __syncthreads();
    }
  }
  static_assert(2 * FwdLay<NX, NU>::STG <= L::V, "forward staging must fit below the vectors");
  forward_sweep<NX, NU>(io, b, s, s + FwdLay<NX, NU>::STG, vx, vu, vq);
  __syncthreads();
  costates<NX, 0>(io, b, Ps, s);
}

// ---------------------------------------------------------------- merit
constexpr int kBlk = 256;

__device__ double block_sum(double v, double* red) {
  v = warp_sum(v);
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < kBlk / 32; ++w) t += red[w];
  return t;  // thread 0 only
}

// ls[b] = (rho, dphi, phi0, skip): G = g.(dX, dU) + (lam - 2V).c,
// rho <- min(max(rho, 2G / |c|^2), 1e12) when both are positive,
// dphi = G - rho |c|^2, phi0 = cost + V.c + rho/2 |c|^2.
__global__ void __launch_bounds__(kBlk) wb_merit_kernel(const __grid_constant__ WbSqp p) {
  __shared__ double red[kBlk / 32];
  const int b = blockIdx.x;
  const WbDims& d = p.d;
  const size_t nX = (size_t)(p.N + 1) * d.nx, nU = (size_t)p.N * d.nj;
  const size_t oX = (size_t)b * nX, oU = (size_t)b * nU;
  double gd = 0.0, lc = 0.0;
  for (size_t e = threadIdx.x; e < nX; e += kBlk) {
    gd += (double)p.q[oX + e] * (double)p.dX[oX + e];
    lc += ((double)p.lam[oX + e] - 2.0 * (double)p.V[oX + e]) * p.cd[oX + e];
  }
  for (size_t e = threadIdx.x; e < nU; e += kBlk) gd += (double)p.r[oU + e] * (double)p.dU[oU + e];
  const double G = block_sum(gd, red) + block_sum(lc, red);
  if (threadIdx.x != 0) return;
  double Jc = 0.0, vc = 0.0, cs = 0.0;
  for (int t = 0; t <= p.N; ++t) {
    const double* st = p.sums + ((size_t)b * (p.N + 1) + t) * 4;
    Jc += st[0];
    vc += st[1];
    cs += st[2];
  }
  double rho = p.first ? p.rho0 : p.ls[b * 8 + 0];
  if (cs > 0.0 && G > 0.0) rho = fmin(fmax(rho, 2.0 * G / cs), 1e12);
  const double dphi = G - rho * cs, phi0 = Jc + vc + 0.5 * rho * cs;
  double* ls = p.ls + b * 8;
  ls[0] = rho;
  ls[1] = dphi;
  ls[2] = phi0;
  ls[3] = (dphi < -p.skip_tol * (1.0 + fabs(phi0))) ? 0.0 : 1.0;
  if (p.first && p.status) p.status[b] = 0;
}

// A warp per (instance b, trial k in [k_lo, k_hi), stage t <= N): the
// merit's stage terms at a_k = beta^k: cost_t(X_t + a dX_t, U_t + a dU_t) +
// V_t(a).c_t(a) + rho/2 |c_t(a)|^2, c_0(a) = x0 - X_0(a),
// c_t(a) = f(X_{t-1}(a), U_{t-1}(a)) - X_t(a).  Nothing for an instance
// whose search is over (ls[3] != 0: the full step taken untested, or a step
// already accepted).
__global__ void __launch_bounds__(32 * kNW) wb_trial_kernel(const __grid_constant__ mpxg_wb_model m,
                                                            const __grid_constant__ WbSqp p) {
  __shared__ StepScr sws[kNW];
  __shared__ CostScr swc[kNW];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long item = (long long)blockIdx.x * p.trial_pb + wid;
  const int N1 = p.N + 1, nk = p.k_hi - p.k_lo;
  if (wid >= p.trial_pb || item >= (long long)p.B * nk * N1) return;
  const int b = (int)(item / ((long long)nk * N1));
  const int rem = (int)(item % ((long long)nk * N1));
  const int k = p.k_lo + rem / N1, t = rem % N1;
  const double* ls = p.ls + b * 8;
  if (ls[3] != 0.0) return;
  double al = 1.0;
  for (int i = 0; i < k; ++i) al *= p.beta;
  const WbDims& d = p.d;
  const int nx = d.nx, nj = d.nj;
  StepScr& ss = sws[wid];
  CostScr& s = swc[wid];
  const size_t oX = (size_t)b * N1 * nx, oU = (size_t)b * p.N * nj;
  load_stage(p, s, b, t, lane);
  __syncwarp();
  // the trial point as wb_accept_kernel stores it (float32 of the same fma),
  // so that the accepted trial's f is the next linearisation's
  for (int i = lane; i < nx; i += 32) s.x[i] = (double)(float)fma(al, (double)p.dX[oX + (size_t)t * nx + i], s.x[i]);
  if (t < p.N)
    for (int j = lane; j < nj; j += 32) s.u[j] = (double)(float)fma(al, (double)p.dU[oU + (size_t)t * nj + j], s.u[j]);
  __syncwarp();
  const double cost = stage_eval<false>(d, s, t == p.N, p.swing != 0, lane);
  if (t > 0) {
    const int tp = t - 1;
    for (int i = lane; i < nx; i += 32)
      ss.xb[i] = (double)(float)fma(al, (double)p.dX[oX + (size_t)tp * nx + i], (double)p.X[oX + (size_t)tp * nx + i]);
    for (int j = lane; j < nj; j += 32)
      ss.ub[j] = (double)(float)fma(al, (double)p.dU[oU + (size_t)tp * nj + j], (double)p.U[oU + (size_t)tp * nj + j]);
    __syncwarp();
    eval_step(m, p, ss, ss.xb, ss.ub, p.contact + ((size_t)b * N1 + tp) * d.nc, lane);
    double* fc = p.fcache + (((size_t)b * p.KT + k) * p.N + tp) * nx;
    for (int i = lane; i < nx; i += 32) fc[i] = ss.f[i];
  }
  double vcs = 0.0, ccs = 0.0;
  for (int i = lane; i < nx; i += 32) {
    const double ci = (t == 0 ? (double)p.x0[(size_t)b * nx + i] : ss.f[i]) - s.x[i];
    const double v = (double)p.V[oX + (size_t)t * nx + i], l = (double)p.lam[oX + (size_t)t * nx + i];
    vcs += (double)(float)fma(al, l - v, v) * ci;
    ccs += ci * ci;
  }
  vcs = warp_sum(vcs);
  ccs = warp_sum(ccs);
  if (lane == 0) p.trial[((size_t)b * p.KT + k) * N1 + t] = cost + vcs + 0.5 * ls[0] * ccs;
}

// A block per instance, in two passes around the two trial launches.
// Pass 0 (after the full step's trial): a = 1 when the iteration skips the
// search or the full step passes phi(1) - phi0 <= eta dphi; otherwise the
// instance stays searching and nothing is updated (with ls_max_trials = 1
// the full step is taken with MPXG_INST_LS_FAIL).  Pass 1 (after the trials
// k >= 1): for the instances still searching, the first a_k that passes, or
// the last trial's step and MPXG_INST_LS_FAIL.  The choice is that of
// trying 1, beta, beta^2, ... in order.  Then X += a dX, U += a dU,
// V += a (lam - V), MPXG_INST_NAN on a non-finite result.
__global__ void __launch_bounds__(kBlk) wb_accept_kernel(const __grid_constant__ WbSqp p) {
  __shared__ double s_al;
  __shared__ int s_bad, s_go;
  const int b = blockIdx.x, N1 = p.N + 1;
  double* ls = p.ls + b * 8;
  if (threadIdx.x == 0) {
    double al = 1.0;
    int fail = 0, go = 1, kv = 0;  // kv: the taken trial + 1, 0 for a step taken untested
    if (p.phase == 0) {
      if (ls[3] == 0.0) {
        double phi = 0.0;
        const double* tr = p.trial + ((size_t)b * p.KT) * N1;
        for (int t = 0; t < N1; ++t) phi += tr[t];
        if (phi - ls[2] <= p.eta * ls[1]) { ls[3] = 1.0; kv = 1; }
        else if (p.KT == 1) { fail = MPXG_INST_LS_FAIL; ls[3] = 1.0; kv = 1; }
        else go = 0;  // pass 1 decides
      }
    } else if (ls[3] != 0.0) {
      go = 0;  // decided in pass 0
    } else {
      bool ok = false;
      double a = 1.0;
      kv = p.KT;  // the last trial when none passes
      for (int k = 1; k < p.KT; ++k) {
        a *= p.beta;
        double phi = 0.0;
        const double* tr = p.trial + ((size_t)b * p.KT + k) * N1;
        for (int t = 0; t < N1; ++t) phi += tr[t];
        if (phi - ls[2] <= p.eta * a * ls[1]) {
          ok = true;
          kv = k + 1;
          break;
        }
      }
      al = a;
      fail = ok ? 0 : MPXG_INST_LS_FAIL;
      ls[3] = 1.0;
    }
    s_al = al;
    s_bad = fail;
    s_go = go;
    if (go) p.fvalid[b] = kv;
  }
  __syncthreads();
  if (!s_go) return;
  const double al = s_al;
  const WbDims& d = p.d;
  const size_t nX = (size_t)N1 * d.nx, nU = (size_t)p.N * d.nj;
  const size_t oX = (size_t)b * nX, oU = (size_t)b * nU;
  int bad = 0;
  for (size_t e = threadIdx.x; e < nX; e += kBlk) {
    const float x = (float)fma(al, (double)p.dX[oX + e], (double)p.X[oX + e]);
    const double v0 = (double)p.V[oX + e];
    const float v = (float)fma(al, (double)p.lam[oX + e] - v0, v0);
    p.X[oX + e] = x;
    p.V[oX + e] = v;
    if (!isfinite(x) || !isfinite(v)) bad = 1;
  }
  for (size_t e = threadIdx.x; e < nU; e += kBlk) {
    const float u = (float)fma(al, (double)p.dU[oU + e], (double)p.U[oU + e]);
    p.U[oU + e] = u;
    if (!isfinite(u)) bad = 1;
  }
  if (bad) atomicOr(&s_bad, MPXG_INST_NAN);
  __syncthreads();
  if (threadIdx.x == 0 && p.status) p.status[b] |= s_bad;
}

// ---------------------------------------------------------------- KKT
// A warp per (instance b, stage t <= N), after wb_lin / wb_quad at the
// result: primal max |c_t|; dual |q_t + A_t'V_{t+1} - V_t| (1 <= t < N),
// |q_N - V_N|, |r_t + B_t'V_{t+1}|; max |gradient|; maxima by atomicMax on
// the float bits (non-negative floats order as their bits).
__global__ void __launch_bounds__(128) wb_kkt_kernel(const __grid_constant__ WbSqp p) {
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long item = (long long)blockIdx.x * 4 + wid;
  const int N1 = p.N + 1;
  if (item >= (long long)p.B * N1) return;
  const int b = (int)(item / N1), t = (int)(item % N1);
  const WbDims& d = p.d;
  const int nx = d.nx, nj = d.nj;
  const size_t s1 = (size_t)b * N1 + t;
  double rp = 0.0, rd = 0.0, gm = 0.0;
  for (int i = lane; i < nx; i += 32) {
    rp = fmax(rp, fabs(p.cd[s1 * nx + i]));
    gm = fmax(gm, fabs((double)p.q[s1 * nx + i]));
  }
  const float* Vt = p.V + s1 * nx;
  if (t == p.N) {
    for (int i = lane; i < nx; i += 32) rd = fmax(rd, fabs((double)p.q[s1 * nx + i] - (double)Vt[i]));
  } else {
    const size_t sn = (size_t)b * p.N + t;
    const float* Vn = Vt + nx;
    const float* At = p.A + sn * nx * nx;
    const float* Bt = p.Bm + sn * nx * nj;
    if (t >= 1) {
      for (int j = lane; j < nx; j += 32) {
        double a = 0.0;
        for (int i = 0; i < nx; ++i) a += (double)At[(size_t)i * nx + j] * (double)Vn[i];
        rd = fmax(rd, fabs((double)p.q[s1 * nx + j] + a - (double)Vt[j]));
      }
    }
    for (int j = lane; j < nj; j += 32) {
      double a = 0.0;
      for (int i = 0; i < nx; ++i) a += (double)Bt[(size_t)i * nj + j] * (double)Vn[i];
      const double g = (double)p.r[sn * nj + j];
      gm = fmax(gm, fabs(g));
      rd = fmax(rd, fabs(g + a));
    }
  }
  rp = warp_max(rp);
  rd = warp_max(rd);
  gm = warp_max(gm);
  if (lane == 0) {
    unsigned* kb = p.kbits + (size_t)b * 3;
    atomicMax(kb + 0, __float_as_uint((float)rp));
    atomicMax(kb + 1, __float_as_uint((float)rd));
    atomicMax(kb + 2, __float_as_uint((float)gm));
  }
}

__global__ void wb_kkt_finish_kernel(int B, unsigned* bits, float* kkt) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const float rp = __uint_as_float(bits[3 * b]), rd = __uint_as_float(bits[3 * b + 1]);
  const float gm = __uint_as_float(bits[3 * b + 2]);
  const float dual = rd / (1.0f + gm);
  kkt[3 * b] = rp;
  kkt[3 * b + 1] = dual;
  kkt[3 * b + 2] = fmaxf(rp, dual);
  bits[3 * b] = bits[3 * b + 1] = bits[3 * b + 2] = 0u;
}

// ---------------------------------------------------------------- host
struct WsLayout {
  size_t fnom, cd, sums, ls, trial, fcache, fvalid, A, Bm, c, x0s, Q, R, M, q, r, K, k, dX, dU, lam, Pscr, kbits, bytes;
};

WsLayout ws_layout(const WbDims& d, int B, int N) {
  WsLayout L{};
  size_t o = 0;
  auto take = [&](size_t bytes) {
    const size_t at = o;
    o += (bytes + 255) & ~size_t(255);
    return at;
  };
  const size_t b = (size_t)B, n = (size_t)N, nx = d.nx, nj = d.nj;
  L.fnom = take(b * n * nx * 8);
  L.cd = take(b * (n + 1) * nx * 8);
  L.sums = take(b * (n + 1) * 4 * 8);
  L.ls = take(b * 8 * 8);
  L.trial = take(b * kMaxTrials * (n + 1) * 8);
  L.fcache = take(b * kMaxTrials * n * nx * 8);
  L.fvalid = take(b * 4);
  L.A = take(b * n * nx * nx * 4);
  L.Bm = take(b * n * nx * nj * 4);
  L.c = take(b * n * nx * 4);
  L.x0s = take(b * nx * 4);
  L.Q = take(b * (n + 1) * nx * nx * 4);
  L.R = take(b * n * nj * nj * 4);
  L.M = take(b * n * nx * nj * 4);
  L.q = take(b * (n + 1) * nx * 4);
  L.r = take(b * n * nj * 4);
  L.K = take(b * n * nj * nx * 4);
  L.k = take(b * n * nj * 4);
  L.dX = take(b * (n + 1) * nx * 4);
  L.dU = take(b * n * nj * 4);
  L.lam = take(b * (n + 1) * nx * 4);
  L.Pscr = take(b * (n + 1) * (nx + 1) * nx * 4);
  L.kbits = take(b * 3 * 4);
  L.bytes = o;
  return L;
}

// The launch grids stay below 2^31 blocks: a block per warp item of the
// B N (nz + nj) dual-number columns or the B (ls_max_trials - 1) (N + 1)
// line-search trials at most.
bool wb_sqp_grid_ok(const WbDims& d, int batch, int N) {
  const long long per = d.nz + d.nj > kMaxTrials ? d.nz + d.nj : kMaxTrials;
  return (long long)batch * ((long long)N + 1) * per <= 0x7fffffffLL;
}

const char* wb_sqp_model_problem(const mpxg_wb_model* m) {
  if (const char* why = wb_model_check(m)) return why;
  const int nv = m->nv, nr = 3 * m->n_contact;
  if (m->jnt_type[0] != 1 || m->nq != nv + 1 || m->n_contact < 1 || nr > nv || nv + nr + 1 > 32)
    return "needs a free root, hinge or slide joints elsewhere, 3 x contacts <= nv and nv + 3 x contacts + 1 <= 32";
  if (m->nbody > WbCap::MB || nv > WbCap::MD || m->n_contact > kMaxC)
    return "the whole-body SQP is built for up to 16 bodies, 20 dofs and 4 contacts";
  const WbDims d = wb_dims(*m);
  if (d.nx != kNX || d.nj != kNU) return "the whole-body SQP is built for nv = 18 with 4 contacts (nx = 61, nj = 12)";
  return nullptr;
}

}  // namespace

extern "C" {

size_t mpxg_wb_sqp_workspace_bytes(const mpxg_wb_model* model, int batch, int N) {
  if (!model || wb_sqp_model_problem(model) || batch < 0 || N < 1 || !wb_sqp_grid_ok(wb_dims(*model), batch, N))
    return 0;
  return ws_layout(wb_dims(*model), batch, N).bytes;
}

mpxg_status mpxg_wb_sqp(void* stream, const mpxg_wb_sqp_io* io) {
  if (!io) return lib_fail(MPXG_ERR_INVALID_ARG, "mpxg_wb_sqp: null io");
  if (const char* why = wb_sqp_model_problem(io->model))
    return lib_fail(MPXG_ERR_INVALID_ARG, std::string("mpxg_wb_sqp: ") + why);
  if (io->batch < 0 || io->N < 1 || io->iters < 0 || io->ls_max_trials < 1 || io->ls_max_trials > kMaxTrials ||
      !(io->dt > 0.0f) || !(io->ls_beta > 0.0f && io->ls_beta < 1.0f) || !(io->reg >= 0.0f))
    return lib_fail(MPXG_ERR_INVALID_ARG,
                    "mpxg_wb_sqp: needs batch >= 0, N >= 1, iters >= 0, ls_max_trials in 1..8, dt > 0, "
                    "0 < ls_beta < 1, reg >= 0");
  if (!wb_sqp_grid_ok(wb_dims(*io->model), io->batch, io->N))
    return lib_fail(MPXG_ERR_INVALID_ARG, "mpxg_wb_sqp: batch x (N + 1) x 49 must stay below 2^31 (launch grids)");
  if (io->batch == 0) return MPXG_OK;
  if (!io->x0 || !io->X || !io->U || !io->V || !io->reference || !io->contact || !io->W || !io->workspace)
    return lib_fail(MPXG_ERR_INVALID_ARG, "mpxg_wb_sqp: null array");
  if (((uintptr_t)io->workspace & 255u) != 0)
    return lib_fail(MPXG_ERR_INVALID_ARG, "mpxg_wb_sqp: workspace must be 256-byte aligned");
  const mpxg_wb_model& m = *io->model;
  const WbDims d = wb_dims(m);
  const int B = io->batch, N = io->N;
  const WsLayout L = ws_layout(d, B, N);
  char* ws = static_cast<char*>(io->workspace);
  WbSqp p{};
  p.B = B; p.N = N; p.KT = io->ls_max_trials; p.d = d;
  p.dt = io->dt; p.alpha = io->alpha; p.beta = io->ls_beta; p.eta = io->ls_eta; p.skip_tol = io->ls_skip_tol;
  p.rho0 = io->rho0; p.reg = io->reg; p.swing = io->swing_tracking;
  p.x0 = io->x0; p.ref = io->reference; p.W = io->W; p.contact = io->contact;
  p.X = io->X; p.U = io->U; p.V = io->V; p.status = io->status; p.kkt = io->kkt;
  p.fnom = (double*)(ws + L.fnom); p.cd = (double*)(ws + L.cd); p.sums = (double*)(ws + L.sums);
  p.ls = (double*)(ws + L.ls); p.trial = (double*)(ws + L.trial);
  p.fcache = (double*)(ws + L.fcache); p.fvalid = (int*)(ws + L.fvalid);
  p.A = (float*)(ws + L.A); p.Bm = (float*)(ws + L.Bm); p.c = (float*)(ws + L.c); p.x0s = (float*)(ws + L.x0s);
  p.Q = (float*)(ws + L.Q); p.R = (float*)(ws + L.R); p.M = (float*)(ws + L.M); p.q = (float*)(ws + L.q);
  p.r = (float*)(ws + L.r); p.K = (float*)(ws + L.K); p.k = (float*)(ws + L.k); p.dX = (float*)(ws + L.dX);
  p.dU = (float*)(ws + L.dU); p.lam = (float*)(ws + L.lam); p.Pscr = (float*)(ws + L.Pscr);
  p.kbits = (unsigned*)(ws + L.kbits);

  mpxg_lq_eq_io lq{};
  lq.batch = B; lq.N = N; lq.n = d.nx; lq.m = d.nj; lq.n_eq = 0;
  lq.A = p.A; lq.Bm = p.Bm; lq.c = p.c; lq.Q = p.Q; lq.R = p.R; lq.M = p.M; lq.q = p.q; lq.r = p.r;
  lq.x0 = p.x0s; lq.K = p.K; lq.k = p.k; lq.X = p.dX; lq.U = p.dU; lq.lam = p.lam;

  cudaStream_t st = (cudaStream_t)stream;
  const size_t rsmem = (size_t)RLay<kNX, kNU, kNZ>::FLOATS * sizeof(float);
  cudaError_t e = cudaFuncSetAttribute(wb_riccati_kernel<kNX, kNU, kNZ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)rsmem);
  if (e != cudaSuccess) return lib_cuda_fail(e, "mpxg_wb_sqp: riccati attribute");
  int dev = 0, sms = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess ||
      (e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
    return lib_cuda_fail(e, "mpxg_wb_sqp: device");
  const auto per_block = [&](long long steps) { return steps < (long long)sms * kNW ? 1 : kNW; };
  const auto blocks = [](long long items, int pb) { return (unsigned)((items + pb - 1) / pb); };
  const long long jac_items = (long long)B * N * (d.nz + d.nj);
  const long long quad_items = (long long)B * (N + 1);
  p.nom_pb = per_block((long long)B * N);
  const unsigned lin_blocks = blocks((long long)B * N, p.nom_pb) + blocks(jac_items, kNW);
  const unsigned quad_blocks = (unsigned)((quad_items + 3) / 4);
  auto linearise = [&]() -> cudaError_t {
    wb_lin_kernel<<<lin_blocks, 32 * kNW, 0, st>>>(m, p);
    wb_quad_kernel<<<quad_blocks, 128, 0, st>>>(p);
    return cudaGetLastError();
  };
  e = cudaMemsetAsync(p.fvalid, 0, (size_t)B * sizeof(int), st);  // the first linearisation computes f
  if (e != cudaSuccess) return lib_cuda_fail(e, "mpxg_wb_sqp: fvalid");
  if (io->iters == 0 && p.status) {
    e = cudaMemsetAsync(p.status, 0, (size_t)B * sizeof(int), st);
    if (e != cudaSuccess) return lib_cuda_fail(e, "mpxg_wb_sqp: status");
  }
  for (int it = 0; it < io->iters; ++it) {
    p.first = it == 0;
    if ((e = linearise()) != cudaSuccess) return lib_cuda_fail(e, "mpxg_wb_sqp: linearisation");
    wb_riccati_kernel<kNX, kNU, kNZ><<<B, lqeq::kThreads, rsmem, st>>>(lq, p.Pscr);
    wb_merit_kernel<<<B, kBlk, 0, st>>>(p);
    // the full step first; the shorter steps only for instances that reject it
    p.k_lo = 0; p.k_hi = 1; p.phase = 0;
    const long long tr0 = (long long)B * (N + 1);
    p.trial_pb = per_block(tr0);
    wb_trial_kernel<<<blocks(tr0, p.trial_pb), 32 * kNW, 0, st>>>(m, p);
    wb_accept_kernel<<<B, kBlk, 0, st>>>(p);
    if (p.KT > 1) {
      p.k_lo = 1; p.k_hi = p.KT; p.phase = 1;
      const long long tr1 = (long long)B * (p.KT - 1) * (N + 1);
      p.trial_pb = per_block(tr1);
      wb_trial_kernel<<<blocks(tr1, p.trial_pb), 32 * kNW, 0, st>>>(m, p);
      wb_accept_kernel<<<B, kBlk, 0, st>>>(p);
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return lib_cuda_fail(e, "mpxg_wb_sqp: iteration");
  }
  if (io->kkt) {
    p.first = 0;
    if ((e = linearise()) != cudaSuccess) return lib_cuda_fail(e, "mpxg_wb_sqp: linearisation");
    e = cudaMemsetAsync(p.kbits, 0, (size_t)B * 3 * sizeof(unsigned), st);
    if (e != cudaSuccess) return lib_cuda_fail(e, "mpxg_wb_sqp: kkt");
    wb_kkt_kernel<<<quad_blocks, 128, 0, st>>>(p);
    wb_kkt_finish_kernel<<<(B + 127) / 128, 128, 0, st>>>(B, p.kbits, p.kkt);
    if ((e = cudaGetLastError()) != cudaSuccess) return lib_cuda_fail(e, "mpxg_wb_sqp: kkt");
  }
  return MPXG_OK;
}

}  // extern "C"
