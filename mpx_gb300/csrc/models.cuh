// Compiled-in SRBD models (device code).  Each model is written once over the
// scalar type S (float for values, DF for one Jacobian column per lane).
//
//   ModelQuat13   mpx/utils/models.py:6-37 (dynamics), mpx/utils/objectives.py:7-75
//                 (cost, barrier, Gauss-Newton Hessian); quaternion helpers are the
//                 MuJoCo MJX math the reference imports (models.py:4), restated.
//   ModelRpy12    same rigid body, roll-pitch-yaw attitude (Euler-rate map of
//                 mpx/utils/rotation.py:26-35).
//   ModelBiped12  two rectangular foot plates carrying 6-D wrenches.
#pragma once
#include "device_math.cuh"

namespace mpxg {

// Per-handle physical constants (kernel argument).
struct ModelConst {
  float dt, mass, inv_mass, gravity, mu;
  float alpha, sigma;             // barrier weight and relaxation / switch point
  float foot_length, foot_width;
  int barrier_kind, barrier_masked;
  float barrier_hess_scale;
  float I[9], Iinv[9];
  float cone_eps2;                // smoothing of the cone's tangential norm (N^2)
};

// ------------------------------------------------------------ rigid body
template <class S>
__device__ __forceinline__ void cross3(const S* a, const S* b, S* o) {
  S x = a[1] * b[2] - a[2] * b[1];
  S y = a[2] * b[0] - a[0] * b[2];
  S z = a[0] * b[1] - a[1] * b[0];
  o[0] = x; o[1] = y; o[2] = z;
}

// v+ = v + (g + F/m) dt; w+ = w + I^-1 (R^T M - w x I w) dt; p+ = p + v+ dt
template <class S>
__device__ __forceinline__ void rigid_body_step(const ModelConst& mc, const S* p, const S* v, const S* w, const S* R,
                                                const S* F, const S* Mw, S* pn, S* vn, S* wn) {
  const float dt = mc.dt;
  vn[0] = v[0] + (F[0] * mc.inv_mass) * dt;
  vn[1] = v[1] + (F[1] * mc.inv_mass) * dt;
  vn[2] = v[2] + (F[2] * mc.inv_mass - mc.gravity) * dt;
  S Iw[3], gy[3], tb[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) Iw[i] = w[0] * mc.I[3 * i] + w[1] * mc.I[3 * i + 1] + w[2] * mc.I[3 * i + 2];
  cross3(w, Iw, gy);
#pragma unroll
  for (int i = 0; i < 3; ++i) tb[i] = R[i] * Mw[0] + R[3 + i] * Mw[1] + R[6 + i] * Mw[2] - gy[i];
#pragma unroll
  for (int i = 0; i < 3; ++i)
    wn[i] = w[i] + (tb[0] * mc.Iinv[3 * i] + tb[1] * mc.Iinv[3 * i + 1] + tb[2] * mc.Iinv[3 * i + 2]) * dt;
#pragma unroll
  for (int i = 0; i < 3; ++i) pn[i] = p[i] + vn[i] * dt;
}

// The same step as increments (dp, dv, dw) = (p+ - p, v+ - v, w+ - w), never
// adding the state itself, so that increments at two nearby points differ
// by their true difference rather than by the rounding of the state.
template <class S>
__device__ __forceinline__ void rigid_body_incr(const ModelConst& mc, const S* v, const S* w, const S* R, const S* F,
                                                const S* Mw, S* dp, S* dv, S* dw) {
  const float dt = mc.dt;
  dv[0] = (F[0] * mc.inv_mass) * dt;
  dv[1] = (F[1] * mc.inv_mass) * dt;
  dv[2] = (F[2] * mc.inv_mass - mc.gravity) * dt;
  S Iw[3], gy[3], tb[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) Iw[i] = w[0] * mc.I[3 * i] + w[1] * mc.I[3 * i + 1] + w[2] * mc.I[3 * i + 2];
  cross3(w, Iw, gy);
#pragma unroll
  for (int i = 0; i < 3; ++i) tb[i] = R[i] * Mw[0] + R[3 + i] * Mw[1] + R[6 + i] * Mw[2] - gy[i];
#pragma unroll
  for (int i = 0; i < 3; ++i) dw[i] = (tb[0] * mc.Iinv[3 * i] + tb[1] * mc.Iinv[3 * i + 1] + tb[2] * mc.Iinv[3 * i + 2]) * dt;
#pragma unroll
  for (int i = 0; i < 3; ++i) dp[i] = (v[i] + dv[i]) * dt;
}

// Net force and moment about the CoM of point forces (quadruped legs).
template <class S, int LEGS>
__device__ __forceinline__ void point_wrench(const S* p, const S* u, const float* par, S* F, S* Mw) {
  F[0] = F[1] = F[2] = s_const<S>(0.0f);
  Mw[0] = Mw[1] = Mw[2] = s_const<S>(0.0f);
#pragma unroll
  for (int i = 0; i < LEGS; ++i) {
    const float c = par[i];
    S r[3] = {par[LEGS + 3 * i] - p[0], par[LEGS + 3 * i + 1] - p[1], par[LEGS + 3 * i + 2] - p[2]};
    S f[3] = {u[3 * i] * c, u[3 * i + 1] * c, u[3 * i + 2] * c};
    S t[3];
    cross3(r, f, t);
#pragma unroll
    for (int k = 0; k < 3; ++k) { F[k] = F[k] + f[k]; Mw[k] = Mw[k] + t[k]; }
  }
}

// ------------------------------------------------------------ quaternions
template <class S>
__device__ __forceinline__ void quat_mul(const S* a, const S* b, S* o) {
  S w = a[0] * b[0] - a[1] * b[1] - a[2] * b[2] - a[3] * b[3];
  S x = a[0] * b[1] + a[1] * b[0] + a[2] * b[3] - a[3] * b[2];
  S y = a[0] * b[2] - a[1] * b[3] + a[2] * b[0] + a[3] * b[1];
  S z = a[0] * b[3] + a[1] * b[2] - a[2] * b[1] + a[3] * b[0];
  o[0] = w; o[1] = x; o[2] = y; o[3] = z;
}
// homogeneous rotation matrix of (w,x,y,z)
template <class S>
__device__ __forceinline__ void quat_to_mat(const S* q, S* R) {
  S q00 = q[0] * q[0], q11 = q[1] * q[1], q22 = q[2] * q[2], q33 = q[3] * q[3];
  S q01 = q[0] * q[1], q02 = q[0] * q[2], q03 = q[0] * q[3];
  S q12 = q[1] * q[2], q13 = q[1] * q[3], q23 = q[2] * q[3];
  R[0] = q00 + q11 - q22 - q33; R[1] = 2.0f * (q12 - q03); R[2] = 2.0f * (q13 + q02);
  R[3] = 2.0f * (q12 + q03); R[4] = q00 - q11 + q22 - q33; R[5] = 2.0f * (q23 - q01);
  R[6] = 2.0f * (q13 - q02); R[7] = 2.0f * (q23 + q01); R[8] = q00 - q11 - q22 + q33;
}
// q * exp(w dt / 2), normalised; series form for small angles so that the
// derivative at w = 0 is exact.
template <class S>
__device__ __forceinline__ void quat_integrate(const S* q, const S* w, float dt, S* out) {
  S n2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
  S h2 = n2 * (0.25f * dt * dt);
  S s, c;
  if (sval(h2) < 1e-4f) {
    s = (0.5f * dt) * (1.0f - h2 * (1.0f / 6.0f) + h2 * h2 * (1.0f / 120.0f));
    c = 1.0f - h2 * 0.5f + h2 * h2 * (1.0f / 24.0f);
  } else {
    S nrm = s_sqrt(n2);
    S half = nrm * (0.5f * dt);
    S sh, ch;
    s_sincos(half, &sh, &ch);
    s = sh / nrm;
    c = ch;
  }
  S qr[4] = {c, w[0] * s, w[1] * s, w[2] * s};
  S qn[4];
  quat_mul(q, qr, qn);
  S inv = 1.0f / s_sqrt(qn[0] * qn[0] + qn[1] * qn[1] + qn[2] * qn[2] + qn[3] * qn[3]);
#pragma unroll
  for (int i = 0; i < 4; ++i) out[i] = qn[i] * inv;
}
// rotation vector of conj(qr) * q, angle wrapped to (-pi, pi]
template <class S>
__device__ __forceinline__ void quat_sub(const S* q, const float* qr, S* out) {
  S cq[4] = {s_const<S>(qr[0]), s_const<S>(-qr[1]), s_const<S>(-qr[2]), s_const<S>(-qr[3])};
  S d[4];
  quat_mul(cq, q, d);
  S s2 = d[1] * d[1] + d[2] * d[2] + d[3] * d[3];
  S w = d[0];
  S coef;
  const float wv = sval(w);
  if (sval(s2) < 1e-4f * wv * wv) {
    S r = s2 / (w * w);
    coef = (2.0f / w) * (1.0f - r * (1.0f / 3.0f) + r * r * (1.0f / 5.0f) - r * r * r * (1.0f / 7.0f));
  } else {
    S s = s_sqrt(s2);
    S ang = 2.0f * s_atan2(s, w);
    if (sval(ang) > 3.14159265358979f) ang = ang - 6.28318530717959f;
    coef = ang / s;
  }
  out[0] = coef * d[1]; out[1] = coef * d[2]; out[2] = coef * d[3];
}

// ------------------------------------------------------------ Euler angles
template <class S>
__device__ __forceinline__ void rpy_to_mat(const S* e, S* R) {
  S sr, cr, sp, cp, sy, cy;
  s_sincos(e[0], &sr, &cr);
  s_sincos(e[1], &sp, &cp);
  s_sincos(e[2], &sy, &cy);
  R[0] = cy * cp; R[1] = cy * sp * sr - sy * cr; R[2] = cy * sp * cr + sy * sr;
  R[3] = sy * cp; R[4] = sy * sp * sr + cy * cr; R[5] = sy * sp * cr - cy * sr;
  R[6] = -sp;     R[7] = cp * sr;                R[8] = cp * cr;
}
// Euler rates from body angular velocity (closed-form inverse of the map at
// mpx/utils/rotation.py:29-34)
template <class S>
__device__ __forceinline__ void rpy_rates(const S* e, const S* w, S* rd) {
  S sr, cr, sp, cp;
  s_sincos(e[0], &sr, &cr);
  s_sincos(e[1], &sp, &cp);
  S a = w[1] * sr + w[2] * cr;
  rd[0] = w[0] + a * (sp / cp);
  rd[1] = w[1] * cr - w[2] * sr;
  rd[2] = a / cp;
}

// ------------------------------------------------------------ barrier
// kind 0: penalty() of objectives.py:7-13 (value / d / d2 as autodiff sees it)
// kind 1: C2 relaxed log barrier, a*(-log c) above delta = sigma, quadratic below
struct BarrierEval {
  float val, d1, d2;
};
__device__ __forceinline__ BarrierEval barrier_eval(const ModelConst& mc, float c) {
  const float a = mc.alpha, sg = mc.sigma;
  BarrierEval b;
  if (mc.barrier_kind == 1) {
    if (c > sg) {
      b.val = -a * logf(c); b.d1 = -a / c; b.d2 = a / (c * c);
    } else {
      float r = (c - 2.0f * sg) / sg;
      b.val = 0.5f * a * (r * r - 1.0f) - a * logf(sg);
      b.d1 = a * (c - 2.0f * sg) / (sg * sg);
      b.d2 = a / (sg * sg);
    }
    return b;
  }
  const bool in_log = (c > 1e-10f) && (c < 1e6f);
  const float cl = fminf(fmaxf(c, 1e-10f), 1e6f);
  const float logb = -a * logf(cl);
  const float r = (c - 2.0f * sg) / sg;
  const bool quad = !(c > sg);
  const float raw = quad ? 0.5f * a * (r * r - 1.0f) + logb : logb;
  const bool pass = (raw > 0.0f) && (raw < 1e8f);
  b.val = fminf(fmaxf(raw, 0.0f), 1e8f);
  b.d1 = pass ? ((quad ? a * (c - 2.0f * sg) / (sg * sg) : 0.0f) + (in_log ? -a / c : 0.0f)) : 0.0f;
  b.d2 = pass ? ((quad ? a / (sg * sg) : 0.0f) + (in_log ? a / (c * c) : 0.0f)) : 0.0f;
  return b;
}
// cost-level value, gradient factor and Hessian factor of one constraint term
// 1/2 * B(c) (objectives.py:30,33,37): kind 0 clips the value to [1e-6, 1e6]
// and the Gauss-Newton curvature to [1e-6, 1e6] (objectives.py:73), kind 1 is
// the exact second derivative of 1/2 * B.
__device__ __forceinline__ void barrier_terms(const ModelConst& mc, float c, float mask_cost, float mask_hess,
                                              float* val, float* grad, float* hgn, float* curv) {
  BarrierEval b = barrier_eval(mc, c);
  if (mc.barrier_kind == 1) {
    *val = 0.5f * b.val * mask_cost;
    *grad = 0.5f * b.d1 * mask_cost;
    *hgn = 0.5f * b.d2 * mask_hess * mc.barrier_hess_scale;
    *curv = 0.5f * b.d1 * mask_hess;  // multiplies grad^2 c
  } else {
    const bool pass = (b.val > 1e-6f) && (b.val < 1e6f);
    *val = 0.5f * fminf(fmaxf(b.val, 1e-6f), 1e6f) * mask_cost;
    *grad = pass ? 0.5f * b.d1 * mask_cost : 0.0f;
    *hgn = fminf(fmaxf(b.d2, 1e-6f), 1e6f) * mask_hess * mc.barrier_hess_scale;
    *curv = 0.0f;  // the reference's Gauss-Newton drops it
  }
}

// Friction cone c = mu fz - sqrt(fx^2 + fy^2 + eps2) (objectives.py:29,66, where
// eps2 = 1e-2): value, gradient wrt (fx, fy, fz) and Hessian of the sqrt term
// (xy block).
__device__ __forceinline__ float cone(float mu, float eps2, const float* f, float* gc, float* hxx, float* hxy,
                                      float* hyy) {
  const float s2 = f[0] * f[0] + f[1] * f[1] + eps2;
  const float s = sqrtf(s2);
  gc[0] = -f[0] / s; gc[1] = -f[1] / s; gc[2] = mu;
  const float s3 = s2 * s;
  *hxx = (s2 - f[0] * f[0]) / s3; *hxy = -f[0] * f[1] / s3; *hyy = (s2 - f[1] * f[1]) / s3;
  return mu * f[2] - s;
}

// ------------------------------------------------------------ models
struct ModelQuat13 {
  static constexpr int NX = 13, NU = 12, NREF = 17, NPAR = 16, LEGS = 4, COFF = 13;
  static constexpr bool IDENT_RES = false;
  static constexpr int QOFF = 3;  // state indices 3..6 (the quaternion) map to residual rows 3..5
  // residual row carrying the weight of state index j (j outside the quaternion)
  __device__ static int wrow(int j) { return j < 3 ? j : j - 1; }
  template <class S>
  __device__ static void dynamics(const ModelConst& mc, const S* x, const S* u, const float* par, S* xn) {
    S F[3], Mw[3], R[9];
    point_wrench<S, 4>(x, u, par, F, Mw);
    quat_to_mat(x + 3, R);
    rigid_body_step(mc, x, x + 7, x + 10, R, F, Mw, xn, xn + 7, xn + 10);
    quat_integrate(x + 3, xn + 10, mc.dt, xn + 3);
  }
  // f(x, u) - x; the quaternion rows are the plain difference of the step
  template <class S>
  __device__ static void increment(const ModelConst& mc, const S* x, const S* u, const float* par, S* d) {
    S F[3], Mw[3], R[9], wn[3], qn[4];
    point_wrench<S, 4>(x, u, par, F, Mw);
    quat_to_mat(x + 3, R);
    rigid_body_incr(mc, x + 7, x + 10, R, F, Mw, d, d + 7, d + 10);
#pragma unroll
    for (int k = 0; k < 3; ++k) wn[k] = x[10 + k] + d[10 + k];
    quat_integrate(x + 3, wn, mc.dt, qn);
#pragma unroll
    for (int k = 0; k < 4; ++k) d[3 + k] = qn[k] - x[3 + k];
  }
  // tracking residual of the state (objectives.py:41-61), 12 entries
  template <class S>
  __device__ static void state_residual(const S* x, const float* ref, S* r) {
#pragma unroll
    for (int k = 0; k < 3; ++k) r[k] = x[k] - ref[k];
    quat_sub(x + 3, ref + 3, r + 3);
#pragma unroll
    for (int k = 0; k < 3; ++k) { r[6 + k] = x[7 + k] - ref[7 + k]; r[9 + k] = x[10 + k] - ref[10 + k]; }
  }
};

struct ModelRpy12 {
  static constexpr int NX = 12, NU = 12, NREF = 16, NPAR = 16, LEGS = 4, COFF = 12;
  static constexpr bool IDENT_RES = true;
  static constexpr int QOFF = 0;
  __device__ static int wrow(int j) { return j; }
  template <class S>
  __device__ static void dynamics(const ModelConst& mc, const S* x, const S* u, const float* par, S* xn) {
    S F[3], Mw[3], R[9], rd[3];
    point_wrench<S, 4>(x, u, par, F, Mw);
    rpy_to_mat(x + 3, R);
    rigid_body_step(mc, x, x + 6, x + 9, R, F, Mw, xn, xn + 6, xn + 9);
    rpy_rates(x + 3, xn + 9, rd);
#pragma unroll
    for (int k = 0; k < 3; ++k) xn[3 + k] = x[3 + k] + rd[k] * mc.dt;
  }
  // f(x, u) - x
  template <class S>
  __device__ static void increment(const ModelConst& mc, const S* x, const S* u, const float* par, S* d) {
    S F[3], Mw[3], R[9], wn[3], rd[3];
    point_wrench<S, 4>(x, u, par, F, Mw);
    rpy_to_mat(x + 3, R);
    rigid_body_incr(mc, x + 6, x + 9, R, F, Mw, d, d + 6, d + 9);
#pragma unroll
    for (int k = 0; k < 3; ++k) wn[k] = x[9 + k] + d[9 + k];
    rpy_rates(x + 3, wn, rd);
#pragma unroll
    for (int k = 0; k < 3; ++k) d[3 + k] = rd[k] * mc.dt;
  }
  template <class S>
  __device__ static void state_residual(const S* x, const float* ref, S* r) {
#pragma unroll
    for (int k = 0; k < 12; ++k) r[k] = x[k] - ref[k];
  }
};

// Net force and moment about the CoM of the biped's two foot wrenches.
template <class S>
__device__ __forceinline__ void biped_wrench(const S* x, const S* u, const float* par, S* F, S* Mw) {
  F[0] = F[1] = F[2] = s_const<S>(0.0f);
  Mw[0] = Mw[1] = Mw[2] = s_const<S>(0.0f);
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const float c = par[i];
    S r[3] = {par[2 + 3 * i] - x[0], par[3 + 3 * i] - x[1], par[4 + 3 * i] - x[2]};
    S f[3] = {u[6 * i] * c, u[6 * i + 1] * c, u[6 * i + 2] * c};
    S t[3];
    cross3(r, f, t);
#pragma unroll
    for (int k = 0; k < 3; ++k) { F[k] = F[k] + f[k]; Mw[k] = Mw[k] + t[k] + u[6 * i + 3 + k] * c; }
  }
}

struct ModelBiped12 {
  static constexpr int NX = 12, NU = 12, NREF = 14, NPAR = 8, LEGS = 2, COFF = 12;
  static constexpr bool IDENT_RES = true;
  static constexpr int QOFF = 0;
  __device__ static int wrow(int j) { return j; }
  template <class S>
  __device__ static void dynamics(const ModelConst& mc, const S* x, const S* u, const float* par, S* xn) {
    S F[3], Mw[3], R[9], rd[3];
    biped_wrench(x, u, par, F, Mw);
    rpy_to_mat(x + 3, R);
    rigid_body_step(mc, x, x + 6, x + 9, R, F, Mw, xn, xn + 6, xn + 9);
    rpy_rates(x + 3, xn + 9, rd);
#pragma unroll
    for (int k = 0; k < 3; ++k) xn[3 + k] = x[3 + k] + rd[k] * mc.dt;
  }
  // f(x, u) - x
  template <class S>
  __device__ static void increment(const ModelConst& mc, const S* x, const S* u, const float* par, S* d) {
    S F[3], Mw[3], R[9], wn[3], rd[3];
    biped_wrench(x, u, par, F, Mw);
    rpy_to_mat(x + 3, R);
    rigid_body_incr(mc, x + 6, x + 9, R, F, Mw, d, d + 6, d + 9);
#pragma unroll
    for (int k = 0; k < 3; ++k) wn[k] = x[9 + k] + d[9 + k];
    rpy_rates(x + 3, wn, rd);
#pragma unroll
    for (int k = 0; k < 3; ++k) d[3 + k] = rd[k] * mc.dt;
  }
  template <class S>
  __device__ static void state_residual(const S* x, const float* ref, S* r) {
#pragma unroll
    for (int k = 0; k < 12; ++k) r[k] = x[k] - ref[k];
  }
};

// ------------------------------------------------------------ barrier of a model
// Sum over legs of the barrier cost (1/2 included), primal only.
template <class M>
__device__ __forceinline__ float barrier_cost(const ModelConst& mc, const float* u, const float* ref) {
  float acc = 0.0f;
  if (M::LEGS == 4) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const float cont = ref[M::COFF + i];
      const float mcost = mc.barrier_masked ? cont : 1.0f;
      float gc[3], hxx, hxy, hyy;
      const float c = cone(mc.mu, mc.cone_eps2, u + 3 * i, gc, &hxx, &hxy, &hyy);
      float v, g, h, cv;
      barrier_terms(mc, c, mcost, cont, &v, &g, &h, &cv);
      acc += v;
    }
  } else {
    const float hl = 0.5f * mc.foot_length, hw = 0.5f * mc.foot_width;
    const float mz = mc.mu * 0.5f * fminf(mc.foot_length, mc.foot_width);
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const float cont = ref[M::COFF + i];
      const float mcost = mc.barrier_masked ? cont : 1.0f;
      const float* F = u + 6 * i;
      const float* T = u + 6 * i + 3;
      float gc[3], hxx, hxy, hyy;
      float cs[7];
      cs[0] = cone(mc.mu, mc.cone_eps2, F, gc, &hxx, &hxy, &hyy);
      cs[1] = hl * F[2] - T[1]; cs[2] = hl * F[2] + T[1];
      cs[3] = hw * F[2] - T[0]; cs[4] = hw * F[2] + T[0];
      cs[5] = mz * F[2] - T[2]; cs[6] = mz * F[2] + T[2];
#pragma unroll
      for (int k = 0; k < 7; ++k) {
        float v, g, h, cv;
        barrier_terms(mc, cs[k], mcost, cont, &v, &g, &h, &cv);
        acc += v;
      }
    }
  }
  return acc;
}

// Barrier terms of leg/foot `leg`: cost value (1/2 included), gradient over
// the leg's LD controls and its LD x LD Hessian model (kind 0: the reference's
// Gauss-Newton J^T diag(clip(B'')*contact) J; kind 1: exact second derivative).
template <class M, int LD>
__device__ __forceinline__ void barrier_leg(const ModelConst& mc, int leg, const float* u, const float* ref, float* val,
                                            float* grad, float (*H)[LD]) {
  const float cont = ref[M::COFF + leg];
  const float mcost = mc.barrier_masked ? cont : 1.0f;
  float gc[3], hxx, hxy, hyy;
#pragma unroll
  for (int a = 0; a < LD; ++a) {
    grad[a] = 0.0f;
#pragma unroll
    for (int b = 0; b < LD; ++b) H[a][b] = 0.0f;
  }
  if (LD == 3) {
    const float* f = u + 3 * leg;
    const float c = cone(mc.mu, mc.cone_eps2, f, gc, &hxx, &hxy, &hyy);
    float v, g, h, cv;
    barrier_terms(mc, c, mcost, cont, &v, &g, &h, &cv);
    *val = v;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      grad[a] = g * gc[a];
#pragma unroll
      for (int b = 0; b < 3; ++b) H[a][b] = h * gc[a] * gc[b];
    }
    H[0][0] += -cv * hxx; H[0][1] += -cv * hxy; H[1][0] += -cv * hxy; H[1][1] += -cv * hyy;
  } else {
    const float* F = u + 6 * leg;
    const float* T = u + 6 * leg + 3;
    const float hl = 0.5f * mc.foot_length, hw = 0.5f * mc.foot_width;
    const float mz = mc.mu * 0.5f * fminf(mc.foot_length, mc.foot_width);
    float cs[7];
    cs[0] = cone(mc.mu, mc.cone_eps2, F, gc, &hxx, &hxy, &hyy);
    cs[1] = hl * F[2] - T[1]; cs[2] = hl * F[2] + T[1];
    cs[3] = hw * F[2] - T[0]; cs[4] = hw * F[2] + T[0];
    cs[5] = mz * F[2] - T[2]; cs[6] = mz * F[2] + T[2];
    const float G[7][6] = {{gc[0], gc[1], gc[2], 0.f, 0.f, 0.f},
                           {0.f, 0.f, hl, 0.f, -1.f, 0.f}, {0.f, 0.f, hl, 0.f, 1.f, 0.f},
                           {0.f, 0.f, hw, -1.f, 0.f, 0.f}, {0.f, 0.f, hw, 1.f, 0.f, 0.f},
                           {0.f, 0.f, mz, 0.f, 0.f, -1.f}, {0.f, 0.f, mz, 0.f, 0.f, 1.f}};
    float vs = 0.0f;
#pragma unroll
    for (int k = 0; k < 7; ++k) {
      float v, g, h, cv;
      barrier_terms(mc, cs[k], mcost, cont, &v, &g, &h, &cv);
      vs += v;
#pragma unroll
      for (int a = 0; a < LD; ++a) {
        grad[a] += g * G[k][a];
#pragma unroll
        for (int b = 0; b < LD; ++b) H[a][b] += h * G[k][a] * G[k][b];
      }
      if (k == 0) { H[0][0] += -cv * hxx; H[0][1] += -cv * hxy; H[1][0] += -cv * hxy; H[1][1] += -cv * hyy; }
    }
    *val = vs;
  }
}

// Stage cost l(x,u,t) (objectives.py:15-37) with the diagonal weights w[24].
template <class M>
__device__ __forceinline__ float stage_cost(const ModelConst& mc, const float* x, const float* u, const float* ref,
                                            const float* w, bool terminal) {
  float r[12];
  M::template state_residual<float>(x, ref, r);
  float acc = 0.0f;
#pragma unroll
  for (int a = 0; a < 12; ++a) acc += w[a] * r[a] * r[a];
  if (terminal) return 0.5f * acc;
#pragma unroll
  for (int a = 0; a < M::NU; ++a) acc += w[12 + a] * u[a] * u[a];
  return 0.5f * acc + barrier_cost<M>(mc, u, ref);
}

// ------------------------------------------------------------ cost differences
// The merit line search compares phi(alpha) with phi(0).  Near convergence the
// decrease is far below float32's resolution of phi itself, so the search
// sums per-stage differences written without cancellation instead of
// differencing two float32 merits.  In exact arithmetic each function below
// equals the plain difference of the corresponding cost term.

// Quadratic branch of the barriers: q(c) = a/2 (r^2 - 1), r = (c - 2 sigma)/sigma,
// for c <= sigma, and 0 above (q is continuous at sigma, where r = -1).
__device__ __forceinline__ float barrier_q(float a, float sg, float c) {
  return (c > sg) ? 0.0f : 0.5f * a * ((c - 3.0f * sg) / sg) * ((c - sg) / sg);
}
__device__ __forceinline__ float barrier_q_diff(float a, float sg, float c0, float c1, float dc) {
  if (c0 <= sg && c1 <= sg) return 0.5f * a * (dc / sg) * ((c0 + c1 - 4.0f * sg) / sg);
  return barrier_q(a, sg, c1) - barrier_q(a, sg, c0);
}

// 1/2 mask [B(c0 + dc) - B(c0)] of one constraint term (barrier_terms' value).
__device__ __forceinline__ float barrier_diff(const ModelConst& mc, float c0, float dc, float mask) {
  if (mask == 0.0f) return 0.0f;
  const float a = mc.alpha, sg = mc.sigma;
  const float c1 = c0 + dc;
  if (mc.barrier_kind == 1) {
    // B = -a log c above sigma, q(c) - a log sigma at or below it
    float d;
    if (c0 > sg && c1 > sg) d = -a * log1pf(dc / c0);
    else if (c0 <= sg && c1 <= sg) d = barrier_q_diff(a, sg, c0, c1, dc);
    else if (c0 > sg) d = barrier_q(a, sg, c1) + a * log1pf((c0 - sg) / sg);
    else d = -a * log1pf((c1 - sg) / sg) - barrier_q(a, sg, c0);
    return 0.5f * mask * d;
  }
  // kind 0: B = clip(clip(q(c) - a log c, 0, 1e8), 1e-6, 1e6); the closed
  // form holds while no clip is active at either end
  const BarrierEval b0 = barrier_eval(mc, c0), b1 = barrier_eval(mc, c1);
  const bool open = c0 > 1e-10f && c1 > 1e-10f && c0 < 1e6f && c1 < 1e6f && b0.val > 1e-6f && b0.val < 1e6f &&
                    b1.val > 1e-6f && b1.val < 1e6f;
  if (!open) return 0.5f * mask * (fminf(fmaxf(b1.val, 1e-6f), 1e6f) - fminf(fmaxf(b0.val, 1e-6f), 1e6f));
  return 0.5f * mask * (barrier_q_diff(a, sg, c0, c1, dc) - a * log1pf(dc / c0));
}

// Friction cone c = mu fz - s, s = sqrt(fx^2 + fy^2 + eps2): value at f and
// its change for the step df, with ds = d(s^2) / (s0 + s1).
__device__ __forceinline__ float cone_diff(float mu, float eps2, const float* f, const float* df, float* dc) {
  const float s0 = sqrtf(f[0] * f[0] + f[1] * f[1] + eps2);
  const float g0 = f[0] + df[0], g1 = f[1] + df[1];
  const float s1 = sqrtf(g0 * g0 + g1 * g1 + eps2);
  const float ds = (df[0] * (2.0f * f[0] + df[0]) + df[1] * (2.0f * f[1] + df[1])) / (s0 + s1);
  *dc = mu * df[2] - ds;
  return mu * f[2] - s0;
}

// Change of barrier_cost<M> for the control step du.
template <class M>
__device__ __forceinline__ float barrier_cost_diff(const ModelConst& mc, const float* u, const float* du,
                                                   const float* ref) {
  float acc = 0.0f;
  if (M::LEGS == 4) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const float mcost = mc.barrier_masked ? ref[M::COFF + i] : 1.0f;
      float dc;
      const float c0 = cone_diff(mc.mu, mc.cone_eps2, u + 3 * i, du + 3 * i, &dc);
      acc += barrier_diff(mc, c0, dc, mcost);
    }
  } else {
    const float hl = 0.5f * mc.foot_length, hw = 0.5f * mc.foot_width;
    const float mz = mc.mu * 0.5f * fminf(mc.foot_length, mc.foot_width);
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const float mcost = mc.barrier_masked ? ref[M::COFF + i] : 1.0f;
      const float* F = u + 6 * i;
      const float* T = u + 6 * i + 3;
      const float* dF = du + 6 * i;
      const float* dT = du + 6 * i + 3;
      float dc;
      const float c0 = cone_diff(mc.mu, mc.cone_eps2, F, dF, &dc);
      acc += barrier_diff(mc, c0, dc, mcost);
      acc += barrier_diff(mc, hl * F[2] - T[1], hl * dF[2] - dT[1], mcost);
      acc += barrier_diff(mc, hl * F[2] + T[1], hl * dF[2] + dT[1], mcost);
      acc += barrier_diff(mc, hw * F[2] - T[0], hw * dF[2] - dT[0], mcost);
      acc += barrier_diff(mc, hw * F[2] + T[0], hw * dF[2] + dT[0], mcost);
      acc += barrier_diff(mc, mz * F[2] - T[2], mz * dF[2] - dT[2], mcost);
      acc += barrier_diff(mc, mz * F[2] + T[2], mz * dF[2] + dT[2], mcost);
    }
  }
  return acc;
}

// stage_cost<M>(x + dx, u + du) - stage_cost<M>(x, u).  Tracking and effort
// terms as 1/2 w d (2 r + d); the quaternion rows of the attitude residual
// (nonlinear in x) as (r1 - r0)(r1 + r0) of the two residuals.
template <class M>
__device__ __forceinline__ float stage_cost_diff(const ModelConst& mc, const float* x, const float* dx, const float* u,
                                                 const float* du, const float* ref, const float* w, bool terminal) {
  float acc = 0.0f;
  if (M::IDENT_RES) {
#pragma unroll
    for (int a = 0; a < 12; ++a) acc += w[a] * dx[a] * (2.0f * (x[a] - ref[a]) + dx[a]);
  } else {
#pragma unroll
    for (int j = 0; j < M::NX; ++j) {
      if (j >= M::QOFF && j < M::QOFF + 4) continue;
      const int a = M::wrow(j);
      acc += w[a] * dx[j] * (2.0f * (x[j] - ref[j]) + dx[j]);
    }
    float q1[4], r0[3], r1[3];
#pragma unroll
    for (int k = 0; k < 4; ++k) q1[k] = x[M::QOFF + k] + dx[M::QOFF + k];
    quat_sub(x + M::QOFF, ref + M::QOFF, r0);
    quat_sub(q1, ref + M::QOFF, r1);
#pragma unroll
    for (int k = 0; k < 3; ++k) acc += w[M::QOFF + k] * (r1[k] - r0[k]) * (r1[k] + r0[k]);
  }
  if (terminal) return 0.5f * acc;
#pragma unroll
  for (int a = 0; a < M::NU; ++a) acc += w[12 + a] * du[a] * (2.0f * u[a] + du[a]);
  return 0.5f * acc + barrier_cost_diff<M>(mc, u, du, ref);
}

}  // namespace mpxg
