// ============================================================================
// mpx SRBD-MPC hot path: CPU ORACLE (test infrastructure, not the product).
//
// This file restates, on the CPU and templated on the scalar type (double,
// float, or the forward-mode Dual below), the arithmetic of the reference's
// primal-dual iLQR SQP path for the single-rigid-body (SRBD) models:
//
//   * SRBD dynamics ............ mpx/utils/models.py:6-37
//   * SRBD cost + barrier ...... mpx/utils/objectives.py:7-37
//   * SRBD Gauss-Newton Hessian  mpx/utils/objectives.py:39-75
//   * gait timer ............... mpx/utils/mpc_utils.py:7-14
//   * SRBD reference generator . mpx/utils/mpc_utils.py:146-270
//   * warm-start shift ......... mpx/utils/mpc_wrapper_srbd.py:134-139
//
// and, for the solver whose source is absent from the reference tree
// (mpx/primal_dual_ilqr is an empty, unpinned git submodule, .gitmodules:1-3),
// the published method: primal-dual iLQR (Sousa-Pinto & Orban), i.e. a
// multiple-shooting SQP whose Gauss-Newton KKT step is a time-varying LQR
// solved by a Riccati recursion, duals recovered as LQR costates, and an
// augmented-Lagrangian merit line search.  Call sites of that solver:
// mpx/utils/mpc_wrapper_srbd.py:68,124-132, mpx/utils/mpc_wrapper.py:74,150-158.
//
// Third-party arithmetic restated from its mathematical definition (MuJoCo MJX
// 3.3.0 math: quat_to_mat, quat_integrate, quat_sub; imported at
// mpx/utils/models.py:4 and mpx/utils/objectives.py:4).
//
// Parity status: the model, cost, timer and reference-generator restatements
// are pinned against golden vectors produced by executing the reference's own
// Python source (tests/golden/make_golden.py).  The SQP/KKT solver is
// "parity unpinned": its reference implementation is not present, so it is
// restated from the published algorithm and checked only by known-answer
// tests (dense KKT solve, finite differences, pure-LQ one-step convergence).
//
// Only tests/, __graft_entry__.smoke() and bench.py (CPU baseline / reference
// arm) may load this code; the product path never does.
// ============================================================================
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

namespace oracle {

// ---------------------------------------------------------------- scalar type
template <class T>
struct Dual {
  T v, d;
  Dual() : v(0), d(0) {}
  template <class A>
  Dual(A a) : v(T(a)), d(0) {}
  Dual(T a, T b) : v(a), d(b) {}
};
template <class T> struct is_dual { static const bool value = false; };
template <class T> struct is_dual<Dual<T>> { static const bool value = true; };

template <class T> inline double val(const T& x) { return double(x); }
template <class T> inline double val(const Dual<T>& x) { return double(x.v); }

#define ORC_DUAL_BINOP(OP, VEXPR, DEXPR)                                              \
  template <class T> inline Dual<T> operator OP(const Dual<T>& a, const Dual<T>& b) { \
    return Dual<T>(VEXPR, DEXPR);                                                     \
  }
ORC_DUAL_BINOP(+, a.v + b.v, a.d + b.d)
ORC_DUAL_BINOP(-, a.v - b.v, a.d - b.d)
ORC_DUAL_BINOP(*, a.v * b.v, a.d * b.v + a.v * b.d)
ORC_DUAL_BINOP(/, a.v / b.v, (a.d * b.v - a.v * b.d) / (b.v * b.v))
#undef ORC_DUAL_BINOP
template <class T> inline Dual<T> operator-(const Dual<T>& a) { return Dual<T>(-a.v, -a.d); }
template <class T, class A> inline Dual<T> operator+(const Dual<T>& a, A b) { return a + Dual<T>(b); }
template <class T, class A> inline Dual<T> operator+(A b, const Dual<T>& a) { return Dual<T>(b) + a; }
template <class T, class A> inline Dual<T> operator-(const Dual<T>& a, A b) { return a - Dual<T>(b); }
template <class T, class A> inline Dual<T> operator-(A b, const Dual<T>& a) { return Dual<T>(b) - a; }
template <class T, class A> inline Dual<T> operator*(const Dual<T>& a, A b) { return a * Dual<T>(b); }
template <class T, class A> inline Dual<T> operator*(A b, const Dual<T>& a) { return Dual<T>(b) * a; }
template <class T, class A> inline Dual<T> operator/(const Dual<T>& a, A b) { return a / Dual<T>(b); }
template <class T, class A> inline Dual<T> operator/(A b, const Dual<T>& a) { return Dual<T>(b) / a; }
template <class T> inline Dual<T>& operator+=(Dual<T>& a, const Dual<T>& b) { a = a + b; return a; }
template <class T> inline Dual<T>& operator-=(Dual<T>& a, const Dual<T>& b) { a = a - b; return a; }

template <class T> inline Dual<T> sqrt(const Dual<T>& a) {
  T s = std::sqrt(a.v);
  return Dual<T>(s, a.d / (T(2) * s));
}
template <class T> inline Dual<T> sin(const Dual<T>& a) { return Dual<T>(std::sin(a.v), std::cos(a.v) * a.d); }
template <class T> inline Dual<T> cos(const Dual<T>& a) { return Dual<T>(std::cos(a.v), -std::sin(a.v) * a.d); }
template <class T> inline Dual<T> tan(const Dual<T>& a) {
  T c = std::cos(a.v);
  return Dual<T>(std::tan(a.v), a.d / (c * c));
}
template <class T> inline Dual<T> log(const Dual<T>& a) { return Dual<T>(std::log(a.v), a.d / a.v); }
template <class T> inline Dual<T> atan2(const Dual<T>& y, const Dual<T>& x) {
  T den = x.v * x.v + y.v * y.v;
  return Dual<T>(std::atan2(y.v, x.v), (x.v * y.d - y.v * x.d) / den);
}
using std::atan2;
using std::cos;
using std::log;
using std::sin;
using std::sqrt;
using std::tan;

// A value that carries no derivative (used by clip() outside its open range).
template <class S> inline S constant_of(const S& x) { return x; }
template <class T> inline Dual<T> constant_of(const Dual<T>& x) { return Dual<T>(x.v, T(0)); }

// Constants are converted to the base precision of S before any arithmetic so
// that the float instantiation computes in float32 throughout.
template <class S> struct Base { typedef S type; };
template <class T> struct Base<Dual<T>> { typedef T type; };
template <class S> inline typename Base<S>::type cs(double v) { return (typename Base<S>::type)v; }

// jnp.clip(x, lo, hi): value clamped; derivative passes only strictly inside.
template <class S> inline S clip(const S& x, double lo, double hi) {
  double v = val(x);
  if (v < lo) return S(lo);
  if (v > hi) return S(hi);
  return x;
}

// ------------------------------------------------------------- model params
enum ModelId { MODEL_SRBD_QUAT13 = 1, MODEL_SRBD_RPY12 = 2, MODEL_BIPED_WRENCH12 = 3, MODEL_GENERIC_LQ = 4 };

struct ModelParams {
  int model;
  int n, m;
  int n_contact;
  double dt;
  double mass;
  double gravity;        // 9.81 (models.py:19)
  double mu;             // friction coefficient of the relaxed cone (objectives.py:28: 0.7)
  double barrier_alpha;  // 0.1 (objectives.py:7)
  double barrier_sigma;  // 5   (objectives.py:7)
  double foot_length;    // biped foot plate (x extent)
  double foot_width;     // biped foot plate (y extent)
  int barrier_kind;      // 0: penalty() of objectives.py:7-13; 1: C2 relaxed log barrier
  int barrier_masked;    // 1: cost barrier multiplied by the stage contact flag
  double barrier_hess_scale;  // GN barrier curvature factor (1.0 as objectives.py:73)
  double inertia[9];     // row-major body inertia
  double inertia_inv[9]; // its inverse (host-inverted like mpc_wrapper_srbd.py:66)
  double cone_eps2 = 1e-2;  // friction cone sqrt(fx^2 + fy^2 + cone_eps2) (objectives.py:29: 1e-2)
};

// Column counts of the per-stage reference / parameter tables.
inline int ref_cols(int model) {
  switch (model) {
    case MODEL_SRBD_QUAT13: return 17;   // [p3, quat4, dp3, omega3, contact4]  (mpc_utils.py:270)
    case MODEL_SRBD_RPY12: return 16;    // [p3, rpy3, dp3, omega3, contact4]
    case MODEL_BIPED_WRENCH12: return 14; // [p3, rpy3, dp3, omega3, contact2]
    default: return 0;
  }
}
inline int par_cols(int model) {
  switch (model) {
    case MODEL_SRBD_QUAT13: return 16;   // [contact4, foot12]  (mpc_utils.py:270)
    case MODEL_SRBD_RPY12: return 16;
    case MODEL_BIPED_WRENCH12: return 8; // [contact2, foot6]
    default: return 0;
  }
}
constexpr int NW = 24;  // residual dimension of every SRBD model (12 state + 12 control)

// ------------------------------------------------------- MJX-style quaternions
// Rotation matrix of a quaternion (w,x,y,z), homogeneous form (no unit-norm
// assumption), as MuJoCo's quat-to-matrix conversion.
template <class S> inline void quat_to_mat(const S* q, S* R) {
  S q00 = q[0] * q[0], q11 = q[1] * q[1], q22 = q[2] * q[2], q33 = q[3] * q[3];
  S q01 = q[0] * q[1], q02 = q[0] * q[2], q03 = q[0] * q[3];
  S q12 = q[1] * q[2], q13 = q[1] * q[3], q23 = q[2] * q[3];
  const auto two = cs<S>(2.0);
  R[0] = q00 + q11 - q22 - q33; R[1] = two * (q12 - q03);         R[2] = two * (q13 + q02);
  R[3] = two * (q12 + q03);     R[4] = q00 - q11 + q22 - q33;     R[5] = two * (q23 - q01);
  R[6] = two * (q13 - q02);     R[7] = two * (q23 + q01);         R[8] = q00 - q11 - q22 + q33;
}
// Hamilton product a*b.
template <class S> inline void quat_mul(const S* a, const S* b, S* o) {
  S w = a[0] * b[0] - a[1] * b[1] - a[2] * b[2] - a[3] * b[3];
  S x = a[0] * b[1] + a[1] * b[0] + a[2] * b[3] - a[3] * b[2];
  S y = a[0] * b[2] - a[1] * b[3] + a[2] * b[0] + a[3] * b[1];
  S z = a[0] * b[3] + a[1] * b[2] - a[2] * b[1] + a[3] * b[0];
  o[0] = w; o[1] = x; o[2] = y; o[3] = z;
}
// q * exp(omega*dt/2) in the body frame, then normalised.  The exponential map
// is evaluated smoothly (series for small angles) so that its derivative at
// omega = 0 is the true one.
template <class S> inline void quat_integrate(const S* q, const S* w, double dt, S* out) {
  S n2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
  S h2 = n2 * cs<S>(0.25 * dt * dt);  // (|w| dt / 2)^2
  S s, c;
  const auto one = cs<S>(1.0);
  if (val(h2) < 1e-4) {
    s = cs<S>(0.5 * dt) * (one - h2 * cs<S>(1.0 / 6.0) + h2 * h2 * cs<S>(1.0 / 120.0));
    c = one - h2 * cs<S>(0.5) + h2 * h2 * cs<S>(1.0 / 24.0);
  } else {
    S nrm = sqrt(n2);
    S half = nrm * cs<S>(0.5 * dt);
    s = sin(half) / nrm;
    c = cos(half);
  }
  S qr[4] = {c, w[0] * s, w[1] * s, w[2] * s};
  S qn[4];
  quat_mul(q, qr, qn);
  S inv = one / sqrt(qn[0] * qn[0] + qn[1] * qn[1] + qn[2] * qn[2] + qn[3] * qn[3]);
  for (int i = 0; i < 4; ++i) out[i] = qn[i] * inv;
}
// Rotation-vector difference log(conj(qr) * q), angle wrapped to (-pi, pi].
template <class S> inline void quat_sub(const S* q, const S* qr, S* out) {
  S cq[4] = {qr[0], -qr[1], -qr[2], -qr[3]};
  S d[4];
  quat_mul(cq, q, d);
  S s2 = d[1] * d[1] + d[2] * d[2] + d[3] * d[3];
  S w = d[0];
  S coef;
  double wv = val(w);
  if (val(s2) < 1e-4 * wv * wv) {
    S r = s2 / (w * w);
    coef = (cs<S>(2.0) / w) * (cs<S>(1.0) - r * cs<S>(1.0 / 3.0) + r * r * cs<S>(1.0 / 5.0) - r * r * r * cs<S>(1.0 / 7.0));
  } else {
    S s = sqrt(s2);
    S ang = cs<S>(2.0) * atan2(s, w);
    if (val(ang) > val(cs<S>(M_PI))) ang = ang - cs<S>(2.0 * M_PI);
    coef = ang / s;
  }
  out[0] = coef * d[1]; out[1] = coef * d[2]; out[2] = coef * d[3];
}

// Z-Y-X Euler (roll, pitch, yaw) -> body-to-world rotation R = Rz*Ry*Rx.
template <class S> inline void rpy_to_mat(const S* rpy, S* R) {
  S cr = cos(rpy[0]), sr = sin(rpy[0]);
  S cp = cos(rpy[1]), sp = sin(rpy[1]);
  S cy = cos(rpy[2]), sy = sin(rpy[2]);
  R[0] = cy * cp; R[1] = cy * sp * sr - sy * cr; R[2] = cy * sp * cr + sy * sr;
  R[3] = sy * cp; R[4] = sy * sp * sr + cy * cr; R[5] = sy * sp * cr - cy * sr;
  R[6] = -sp;     R[7] = cp * sr;                R[8] = cp * cr;
}
// Euler-angle rates from body angular velocity: the inverse of the map of
// mpx/utils/rotation.py:26-35, written in closed form.
template <class S> inline void rpy_rates(const S* rpy, const S* w, S* rd) {
  S cr = cos(rpy[0]), sr = sin(rpy[0]);
  S cp = cos(rpy[1]), tp = tan(rpy[1]);
  S a = w[1] * sr + w[2] * cr;
  rd[0] = w[0] + a * tp;
  rd[1] = w[1] * cr - w[2] * sr;
  rd[2] = a / cp;
}

template <class S> inline void cross3(const S* a, const S* b, S* o) {
  S x = a[1] * b[2] - a[2] * b[1];
  S y = a[2] * b[0] - a[0] * b[2];
  S z = a[0] * b[1] - a[1] * b[0];
  o[0] = x; o[1] = y; o[2] = z;
}

// Shared rigid-body step for every SRBD model: given position p, velocity v,
// body angular velocity w, body->world rotation R, net world force F (without
// gravity) and net world moment about the CoM Mw, produce v+, w+, p+.
// (models.py:19,27-31)
template <class S>
inline void rigid_body_step(const ModelParams& mp, const S* p, const S* v, const S* w, const S* R,
                            const S* F, const S* Mw, S* pn, S* vn, S* wn) {
  const auto dt = cs<S>(mp.dt);
  const auto invm = cs<S>(1.0 / mp.mass);
  S acc[3] = {F[0] * invm, F[1] * invm, cs<S>(-mp.gravity) + F[2] * invm};
  for (int i = 0; i < 3; ++i) vn[i] = v[i] + acc[i] * dt;
  // body moment R^T Mw - w x (I w)
  S Iw[3], gyro[3], tb[3];
  for (int i = 0; i < 3; ++i)
    Iw[i] = cs<S>(mp.inertia[3 * i]) * w[0] + cs<S>(mp.inertia[3 * i + 1]) * w[1] + cs<S>(mp.inertia[3 * i + 2]) * w[2];
  cross3(w, Iw, gyro);
  for (int i = 0; i < 3; ++i) tb[i] = R[i] * Mw[0] + R[3 + i] * Mw[1] + R[6 + i] * Mw[2] - gyro[i];
  for (int i = 0; i < 3; ++i)
    wn[i] = w[i] + (cs<S>(mp.inertia_inv[3 * i]) * tb[0] + cs<S>(mp.inertia_inv[3 * i + 1]) * tb[1] +
                    cs<S>(mp.inertia_inv[3 * i + 2]) * tb[2]) * dt;
  for (int i = 0; i < 3; ++i) pn[i] = p[i] + vn[i] * dt;
}

// ------------------------------------------------------------ SRBD dynamics
// x = [p3, quat4, dp3, omega3], u = 4 x f3, par = [contact4, foot12]
template <class S, class P>
inline void dyn_quat13(const ModelParams& mp, const S* x, const S* u, const P* par, S* xn) {
  const S* p = x; const S* q = x + 3; const S* v = x + 7; const S* w = x + 10;
  S F[3] = {0.0, 0.0, 0.0}, Mw[3] = {0.0, 0.0, 0.0};
  for (int i = 0; i < 4; ++i) {
    S c = S(par[i]);
    S r[3] = {S(par[4 + 3 * i]) - p[0], S(par[5 + 3 * i]) - p[1], S(par[6 + 3 * i]) - p[2]};
    S f[3] = {u[3 * i] * c, u[3 * i + 1] * c, u[3 * i + 2] * c};
    S t[3];
    cross3(r, f, t);
    for (int k = 0; k < 3; ++k) { F[k] += f[k]; Mw[k] += t[k]; }
  }
  S R[9];
  quat_to_mat(q, R);
  rigid_body_step(mp, p, v, w, R, F, Mw, xn, xn + 7, xn + 10);
  quat_integrate(q, xn + 10, mp.dt, xn + 3);
}

// x = [p3, rpy3, dp3, omega3], u = 4 x f3, par = [contact4, foot12]
template <class S, class P>
inline void dyn_rpy12(const ModelParams& mp, const S* x, const S* u, const P* par, S* xn) {
  const S* p = x; const S* e = x + 3; const S* v = x + 6; const S* w = x + 9;
  S F[3] = {0.0, 0.0, 0.0}, Mw[3] = {0.0, 0.0, 0.0};
  for (int i = 0; i < 4; ++i) {
    S c = S(par[i]);
    S r[3] = {S(par[4 + 3 * i]) - p[0], S(par[5 + 3 * i]) - p[1], S(par[6 + 3 * i]) - p[2]};
    S f[3] = {u[3 * i] * c, u[3 * i + 1] * c, u[3 * i + 2] * c};
    S t[3];
    cross3(r, f, t);
    for (int k = 0; k < 3; ++k) { F[k] += f[k]; Mw[k] += t[k]; }
  }
  S R[9];
  rpy_to_mat(e, R);
  rigid_body_step(mp, p, v, w, R, F, Mw, xn, xn + 6, xn + 9);
  S rd[3];
  rpy_rates(e, xn + 9, rd);
  for (int k = 0; k < 3; ++k) xn[3 + k] = e[k] + rd[k] * cs<S>(mp.dt);
}

// x = [p3, rpy3, dp3, omega3], u = [F_L3, tau_L3, F_R3, tau_R3], par = [contact2, foot6]
template <class S, class P>
inline void dyn_biped12(const ModelParams& mp, const S* x, const S* u, const P* par, S* xn) {
  const S* p = x; const S* e = x + 3; const S* v = x + 6; const S* w = x + 9;
  S F[3] = {0.0, 0.0, 0.0}, Mw[3] = {0.0, 0.0, 0.0};
  for (int i = 0; i < 2; ++i) {
    S c = S(par[i]);
    S r[3] = {S(par[2 + 3 * i]) - p[0], S(par[3 + 3 * i]) - p[1], S(par[4 + 3 * i]) - p[2]};
    S f[3] = {u[6 * i] * c, u[6 * i + 1] * c, u[6 * i + 2] * c};
    S t[3];
    cross3(r, f, t);
    for (int k = 0; k < 3; ++k) { F[k] += f[k]; Mw[k] += t[k] + u[6 * i + 3 + k] * c; }
  }
  S R[9];
  rpy_to_mat(e, R);
  rigid_body_step(mp, p, v, w, R, F, Mw, xn, xn + 6, xn + 9);
  S rd[3];
  rpy_rates(e, xn + 9, rd);
  for (int k = 0; k < 3; ++k) xn[3 + k] = e[k] + rd[k] * cs<S>(mp.dt);
}

template <class S, class P>
inline void dynamics(const ModelParams& mp, const S* x, const S* u, const P* par, S* xn) {
  switch (mp.model) {
    case MODEL_SRBD_QUAT13: dyn_quat13(mp, x, u, par, xn); break;
    case MODEL_SRBD_RPY12: dyn_rpy12(mp, x, u, par, xn); break;
    case MODEL_BIPED_WRENCH12: dyn_biped12(mp, x, u, par, xn); break;
    default: break;
  }
}

// ------------------------------------------------------ barrier (objectives.py:7-13)
// kind 0: the reference's penalty():
//   clip(where(c > sigma, -a log(clip(c,1e-10,1e6)), a/2(((c-2 sigma)/sigma)^2 - 1) - a log(clip(c,1e-10,1e6))), 0, 1e8)
// kind 1: the C2 relaxed log barrier with relaxation delta = sigma:
//   a (-log c) for c > delta,  a (1/2 (((c - 2 delta)/delta)^2 - 1) - log delta) otherwise.
template <class S> inline S penalty(const ModelParams& mp, const S& c) {
  const double a = mp.barrier_alpha, sg = mp.barrier_sigma;
  if (mp.barrier_kind == 1) {
    if (val(c) > sg) return cs<S>(-a) * log(c);
    S r = (c - cs<S>(2.0 * sg)) / cs<S>(sg);
    return cs<S>(a * 0.5) * (r * r - cs<S>(1.0)) - cs<S>(a * std::log(sg));
  }
  S logb = cs<S>(-a) * log(clip(c, 1e-10, 1e6));
  S r = (c - cs<S>(2.0 * sg)) / cs<S>(sg);
  S quad = cs<S>(a * 0.5) * (r * r - cs<S>(1.0));
  S raw = (val(c) > val(cs<S>(sg))) ? logb : quad + logb;
  return clip(raw, 0.0, 1e8);
}
// second derivative of penalty() (for kind 0 as jax.grad(jax.grad(penalty)) evaluates it)
inline double penalty_dd(const ModelParams& mp, double c) {
  const double a = mp.barrier_alpha, sg = mp.barrier_sigma;
  if (mp.barrier_kind == 1) return (c > sg) ? a / (c * c) : a / (sg * sg);
  double cl = std::min(std::max(c, 1e-10), 1e6);
  double logb = -a * std::log(cl);
  double r = (c - 2.0 * sg) / sg;
  double raw = (c > sg) ? logb : a * 0.5 * (r * r - 1.0) + logb;
  if (!(raw > 0.0 && raw < 1e8)) return 0.0;
  double dd = 0.0;
  if (!(c > sg)) dd += a / (sg * sg);
  if (c > 1e-10 && c < 1e6) dd += a / (c * c);
  return dd;
}

// Constraint functions c_k(u) >= 0 of one SRBD model (relaxed by the barrier).
// Quadruped: friction cone per leg (objectives.py:29,63-67).  Biped: friction
// cone, centre-of-pressure box of the rectangular plate and torsional bound per
// foot.  Returns the number of constraints; foot_of[k] is the contact index.
template <class S>
inline int constraints(const ModelParams& mp, const S* u, S* c, int* foot_of) {
  if (mp.model == MODEL_BIPED_WRENCH12) {
    const double hl = 0.5 * mp.foot_length, hw = 0.5 * mp.foot_width;
    const double mz = mp.mu * 0.5 * std::min(mp.foot_length, mp.foot_width);
    for (int i = 0; i < 2; ++i) {
      const S* F = u + 6 * i; const S* tq = u + 6 * i + 3;
      S* o = c + 7 * i;
      o[0] = cs<S>(mp.mu) * F[2] - sqrt(F[0] * F[0] + F[1] * F[1] + cs<S>(mp.cone_eps2));
      o[1] = cs<S>(hl) * F[2] - tq[1];
      o[2] = cs<S>(hl) * F[2] + tq[1];
      o[3] = cs<S>(hw) * F[2] - tq[0];
      o[4] = cs<S>(hw) * F[2] + tq[0];
      o[5] = cs<S>(mz) * F[2] - tq[2];
      o[6] = cs<S>(mz) * F[2] + tq[2];
      for (int k = 0; k < 7; ++k) foot_of[7 * i + k] = i;
    }
    return 14;
  }
  for (int i = 0; i < 4; ++i) {
    c[i] = cs<S>(mp.mu) * u[3 * i + 2] - sqrt(u[3 * i + 1] * u[3 * i + 1] + u[3 * i] * u[3 * i] + cs<S>(mp.cone_eps2));
    foot_of[i] = i;
  }
  return 4;
}

// Tracking residual rho(x) (12 entries) of the state part; the control part of
// the residual is u itself (objectives.py:41-61).
template <class S, class P>
inline void state_residual(const ModelParams& mp, const S* x, const P* ref, S* res) {
  if (mp.model == MODEL_SRBD_QUAT13) {
    for (int k = 0; k < 3; ++k) res[k] = x[k] - S(ref[k]);
    S qr[4] = {S(ref[3]), S(ref[4]), S(ref[5]), S(ref[6])};
    quat_sub(x + 3, qr, res + 3);
    for (int k = 0; k < 3; ++k) res[6 + k] = x[7 + k] - S(ref[7 + k]);
    for (int k = 0; k < 3; ++k) res[9 + k] = x[10 + k] - S(ref[10 + k]);
  } else {
    for (int k = 0; k < 12; ++k) res[k] = x[k] - S(ref[k]);
  }
}

// Stage cost l(x,u,t) (objectives.py:15-37).  W is the dense 24x24 weight; the
// cost uses only its diagonal 3x3 / 12x12 blocks, like the reference.
template <class S, class P>
inline S stage_cost(const ModelParams& mp, const S* x, const S* u, const P* ref, const P* W, bool terminal) {
  S res[12];
  state_residual(mp, x, ref, res);
  S acc = 0.0;
  for (int b = 0; b < 4; ++b) {
    for (int i = 0; i < 3; ++i) {
      S wi = 0.0;
      for (int j = 0; j < 3; ++j) wi += S(W[(3 * b + i) * NW + 3 * b + j]) * res[3 * b + j];
      acc += res[3 * b + i] * wi;
    }
  }
  if (terminal) return cs<S>(0.5) * acc;
  for (int i = 0; i < 12; ++i) {
    S wi = 0.0;
    for (int j = 0; j < 12; ++j) wi += S(W[(12 + i) * NW + 12 + j]) * u[j];
    acc += u[i] * wi;
  }
  S c[14];
  int foot_of[14];
  int nc = constraints(mp, u, c, foot_of);
  const int contact_off = (mp.model == MODEL_SRBD_QUAT13) ? 13 : 12;
  for (int k = 0; k < nc; ++k) {
    S b = (mp.barrier_kind == 1) ? penalty(mp, c[k]) : clip(penalty(mp, c[k]), 1e-6, 1e6);
    if (mp.barrier_masked) b = b * S(ref[contact_off + foot_of[k]]);
    acc += b;
  }
  return cs<S>(0.5) * acc;
}

// ----------------------------------------------------------- generic LQ data
template <class T>
struct LQData {  // one instance, stage-major
  const T *A, *B, *c, *Q, *R, *M, *q, *r;  // A[N,n,n] B[N,n,m] c[N,n] Q[N+1,n,n] R[N,m,m] M[N,n,m] q[N+1,n] r[N,m]
};

// ------------------------------------------------------------ linearisation
// Everything the SQP needs about one stage t < N at (x,u):
//   A (n x n), B (n x m) row-major, fx = f(x,u), l = cost,
//   g = grad l (n+m), H = Gauss-Newton Hessian ((n+m) x (n+m)), row-major.
template <class T>
struct StageLin {
  std::vector<T> A, B, fx, g, H;
  T l;
};

template <class T>
void linearize_stage(const ModelParams& mp, int t, bool terminal, const T* x, const T* u, const T* ref, const T* par,
                     const T* W, const LQData<T>* lq, StageLin<T>& out) {
  const int n = mp.n, m = mp.m, nz = n + m;
  out.A.assign(n * n, T(0)); out.B.assign(n * m, T(0)); out.fx.assign(n, T(0));
  out.g.assign(nz, T(0)); out.H.assign(nz * nz, T(0));
  if (mp.model == MODEL_GENERIC_LQ) {
    const T* Q = lq->Q + (size_t)t * n * n; const T* q = lq->q + (size_t)t * n;
    T l = 0;
    for (int i = 0; i < n; ++i) {
      T qx = 0;
      for (int j = 0; j < n; ++j) { qx += Q[i * n + j] * x[j]; out.H[i * nz + j] = Q[i * n + j]; }
      out.g[i] = qx + q[i];
      l += x[i] * (T(0.5) * qx + q[i]);
    }
    if (!terminal) {
      const T* A = lq->A + (size_t)t * n * n; const T* B = lq->B + (size_t)t * n * m; const T* c = lq->c + (size_t)t * n;
      const T* R = lq->R + (size_t)t * m * m; const T* M = lq->M + (size_t)t * n * m; const T* r = lq->r + (size_t)t * m;
      for (int i = 0; i < n; ++i) {
        T s = c[i];
        for (int j = 0; j < n; ++j) { s += A[i * n + j] * x[j]; out.A[i * n + j] = A[i * n + j]; }
        for (int j = 0; j < m; ++j) { s += B[i * m + j] * u[j]; out.B[i * m + j] = B[i * m + j]; }
        out.fx[i] = s;
      }
      for (int i = 0; i < n; ++i) {
        T mu_ = 0;
        for (int j = 0; j < m; ++j) { mu_ += M[i * m + j] * u[j]; out.H[i * nz + n + j] = M[i * m + j]; out.H[(n + j) * nz + i] = M[i * m + j]; }
        out.g[i] += mu_;
        l += x[i] * mu_;
      }
      for (int i = 0; i < m; ++i) {
        T ru = 0, mx = 0;
        for (int j = 0; j < m; ++j) { ru += R[i * m + j] * u[j]; out.H[(n + i) * nz + n + j] = R[i * m + j]; }
        for (int j = 0; j < n; ++j) mx += M[j * m + i] * x[j];
        out.g[n + i] = ru + mx + r[i];
        l += u[i] * (T(0.5) * ru + r[i]);
      }
    }
    out.l = l;
    return;
  }
  typedef Dual<T> D;
  std::vector<D> xd(n), ud(m), fd(n);
  // primal
  {
    std::vector<T> f(n);
    if (!terminal) dynamics(mp, x, u, par, f.data());
    for (int i = 0; i < n; ++i) out.fx[i] = terminal ? T(0) : f[i];
    out.l = stage_cost(mp, x, u, ref, W, terminal);
  }
  // residual Jacobian (12 state rows) and derivatives along every direction
  std::vector<T> Jx(12 * n, T(0));
  for (int j = 0; j < nz; ++j) {
    for (int i = 0; i < n; ++i) xd[i] = D(x[i], T(i == j ? 1 : 0));
    for (int i = 0; i < m; ++i) ud[i] = D(u[i], T(n + i == j ? 1 : 0));
    if (!terminal) {
      dynamics(mp, xd.data(), ud.data(), par, fd.data());
      for (int i = 0; i < n; ++i) {
        if (j < n) out.A[i * n + j] = fd[i].d; else out.B[i * m + (j - n)] = fd[i].d;
      }
    }
    D l = stage_cost(mp, xd.data(), ud.data(), ref, W, terminal);
    out.g[j] = l.d;
    if (j < n) {
      D res[12];
      state_residual(mp, xd.data(), ref, res);
      for (int a = 0; a < 12; ++a) Jx[a * n + j] = res[a].d;
    }
  }
  // Gauss-Newton blocks: Q = Jx^T Wxx Jx, M = Jx^T Wxu, R = Wuu + barrier GN
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      T s = 0;
      for (int a = 0; a < 12; ++a) {
        if (Jx[a * n + i] == T(0)) continue;
        for (int b = 0; b < 12; ++b) s += Jx[a * n + i] * W[a * NW + b] * Jx[b * n + j];
      }
      out.H[i * nz + j] = s;
    }
  if (terminal) { for (int j = 0; j < m; ++j) out.g[n + j] = 0; return; }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < m; ++j) {
      T s = 0;
      for (int a = 0; a < 12; ++a) s += Jx[a * n + i] * W[a * NW + 12 + j];
      out.H[i * nz + n + j] = s;
      out.H[(n + j) * nz + i] = s;
    }
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < m; ++j) out.H[(n + i) * nz + n + j] = W[(12 + i) * NW + 12 + j];
  // barrier curvature J_c^T diag(clip(pen'', 1e-6, 1e6) * contact) J_c  (objectives.py:70-74)
  {
    D cd[14];
    int foot_of[14];
    T cv[14];
    std::vector<T> Jc(14 * m, T(0));
    int nc = 0;
    for (int j = 0; j < m; ++j) {
      for (int i = 0; i < m; ++i) ud[i] = D(u[i], T(i == j ? 1 : 0));
      nc = constraints(mp, ud.data(), cd, foot_of);
      for (int k = 0; k < nc; ++k) { Jc[k * m + j] = cd[k].d; cv[k] = cd[k].v; }
    }
    const int contact_off = (mp.model == MODEL_SRBD_QUAT13) ? 13 : 12;
    for (int k = 0; k < nc; ++k) {
      const double ck = double(ref[contact_off + foot_of[k]]);
      double dd = penalty_dd(mp, double(cv[k]));
      if (mp.barrier_kind == 0) {
        dd = std::min(std::max(dd, 1e-6), 1e6);
      } else {
        dd *= 0.5;  // the cost carries the barrier with a factor 1/2
      }
      double h = mp.barrier_hess_scale * dd * ck;
      for (int i = 0; i < m; ++i)
        for (int j = 0; j < m; ++j) out.H[(n + i) * nz + n + j] += T(h) * Jc[k * m + i] * Jc[k * m + j];
    }
    if (mp.barrier_kind == 1) {
      // exact curvature of the friction cones: 1/2 a beta'(c) grad^2 c, with
      // c = mu fz - sqrt(fx^2 + fy^2 + cone_eps2) (positive semidefinite, since beta' < 0)
      const int legs = (mp.model == MODEL_BIPED_WRENCH12) ? 2 : 4;
      const int stride = (mp.model == MODEL_BIPED_WRENCH12) ? 6 : 3;
      const int cstride = (mp.model == MODEL_BIPED_WRENCH12) ? 7 : 1;
      for (int i = 0; i < legs; ++i) {
        const double ck = double(ref[contact_off + i]);
        if (ck == 0.0) continue;
        const double fx = double(u[stride * i]), fy = double(u[stride * i + 1]);
        const double c = double(cv[cstride * i]);
        const double dpen = (c > mp.barrier_sigma) ? -mp.barrier_alpha / c
                                                   : mp.barrier_alpha * (c - 2.0 * mp.barrier_sigma) / (mp.barrier_sigma * mp.barrier_sigma);
        const double s2 = fx * fx + fy * fy + mp.cone_eps2, s = std::sqrt(s2), s3 = s2 * s;
        const double hxx = (s2 - fx * fx) / s3, hxy = -fx * fy / s3, hyy = (s2 - fy * fy) / s3;
        const double w = -0.5 * dpen * ck;  // grad^2 c = -grad^2 s
        const int a = n + stride * i;
        out.H[a * nz + a] += T(w * hxx); out.H[a * nz + a + 1] += T(w * hxy);
        out.H[(a + 1) * nz + a] += T(w * hxy); out.H[(a + 1) * nz + a + 1] += T(w * hyy);
      }
    }
  }
}

// Dynamics + cost only (line-search trial points).
template <class T>
void eval_stage(const ModelParams& mp, int t, bool terminal, const T* x, const T* u, const T* ref, const T* par,
                const T* W, const LQData<T>* lq, T* fx, T* l) {
  const int n = mp.n, m = mp.m;
  if (mp.model == MODEL_GENERIC_LQ) {
    const T* Q = lq->Q + (size_t)t * n * n; const T* q = lq->q + (size_t)t * n;
    T s = 0;
    for (int i = 0; i < n; ++i) {
      T qx = 0;
      for (int j = 0; j < n; ++j) qx += Q[i * n + j] * x[j];
      s += x[i] * (T(0.5) * qx + q[i]);
    }
    if (!terminal) {
      const T* A = lq->A + (size_t)t * n * n; const T* B = lq->B + (size_t)t * n * m; const T* c = lq->c + (size_t)t * n;
      const T* R = lq->R + (size_t)t * m * m; const T* M = lq->M + (size_t)t * n * m; const T* r = lq->r + (size_t)t * m;
      for (int i = 0; i < n; ++i) {
        T a = c[i];
        for (int j = 0; j < n; ++j) a += A[i * n + j] * x[j];
        for (int j = 0; j < m; ++j) a += B[i * m + j] * u[j];
        fx[i] = a;
        T mu_ = 0;
        for (int j = 0; j < m; ++j) mu_ += M[i * m + j] * u[j];
        s += x[i] * mu_;
      }
      for (int i = 0; i < m; ++i) {
        T ru = 0;
        for (int j = 0; j < m; ++j) ru += R[i * m + j] * u[j];
        s += u[i] * (T(0.5) * ru + r[i]);
      }
    }
    *l = s;
    return;
  }
  if (!terminal) dynamics(mp, x, u, par, fx);
  *l = stage_cost(mp, x, u, ref, W, terminal);
}

// ------------------------------------------------------------ small LA
template <class T>
bool cholesky(std::vector<T>& A, int m) {  // in place, lower; returns false if a pivot <= 0
  bool ok = true;
  for (int j = 0; j < m; ++j) {
    T s = A[j * m + j];
    for (int k = 0; k < j; ++k) s -= A[j * m + k] * A[j * m + k];
    if (!(s > T(0))) { ok = false; s = std::max(std::fabs(s), T(1e-12)); }
    T d = std::sqrt(s);
    A[j * m + j] = d;
    for (int i = j + 1; i < m; ++i) {
      T t = A[i * m + j];
      for (int k = 0; k < j; ++k) t -= A[i * m + k] * A[j * m + k];
      A[i * m + j] = t / d;
    }
    for (int i = 0; i < j; ++i) A[i * m + j] = 0;
  }
  return ok;
}
template <class T>
void chol_solve(const std::vector<T>& L, int m, T* b, int nrhs, int ld) {  // b is m x nrhs (row stride ld)
  for (int c = 0; c < nrhs; ++c) {
    for (int i = 0; i < m; ++i) {
      T s = b[i * ld + c];
      for (int k = 0; k < i; ++k) s -= L[i * m + k] * b[k * ld + c];
      b[i * ld + c] = s / L[i * m + i];
    }
    for (int i = m - 1; i >= 0; --i) {
      T s = b[i * ld + c];
      for (int k = i + 1; k < m; ++k) s -= L[k * m + i] * b[k * ld + c];
      b[i * ld + c] = s / L[i * m + i];
    }
  }
}

// ------------------------------------------------------------ options / status
struct Opts {
  int sqp_iters;
  int ls_max_trials;
  double ls_beta;
  double ls_eta;
  double reg;
  double rho0;
  double ls_skip_tol;
};
enum Status { ST_NAN = 1, ST_NON_PD = 2, ST_LS_FAIL = 4 };

// ------------------------------------------------------------ LQR (Riccati)
// Solves min sum_t 1/2 [dx;du]^T H_t [dx;du] + g_t^T [dx;du] + 1/2 dx_N^T H_N dx_N + g_N^T dx_N
// s.t. dx_0 = c_0, dx_{t+1} = A_t dx_t + B_t du_t + c_{t+1}; returns gains K_t (m x n), k_t, the
// value function P_t, p_t, the trajectory dx, du and the costates lam_t = P_t dx_t + p_t.
template <class T>
struct LQRSol {
  std::vector<T> K, k, P, p, dx, du, lam;
  int status = 0;
};
template <class T>
void riccati_solve(int N, int n, int m, const std::vector<StageLin<T>>& lin, const std::vector<T>& c /* (N+1) x n */,
                   T reg, LQRSol<T>& s) {
  const int nz = n + m;
  s.K.assign((size_t)N * m * n, 0); s.k.assign((size_t)N * m, 0);
  s.P.assign((size_t)(N + 1) * n * n, 0); s.p.assign((size_t)(N + 1) * n, 0);
  s.dx.assign((size_t)(N + 1) * n, 0); s.du.assign((size_t)N * m, 0); s.lam.assign((size_t)(N + 1) * n, 0);
  s.status = 0;
  std::vector<T> P(n * n), p(n);
  const StageLin<T>& LN = lin[N];
  for (int i = 0; i < n; ++i) { p[i] = LN.g[i]; for (int j = 0; j < n; ++j) P[i * n + j] = LN.H[i * nz + j]; }
  std::copy(P.begin(), P.end(), s.P.begin() + (size_t)N * n * n);
  std::copy(p.begin(), p.end(), s.p.begin() + (size_t)N * n);
  std::vector<T> PA(n * n), PB(n * m), Qxx(n * n), Quu(m * m), Qux(m * n), pc(n), qx(n), qu(m), KK(m * (n + 1));
  for (int t = N - 1; t >= 0; --t) {
    const StageLin<T>& L = lin[t];
    const T* ct = &c[(size_t)(t + 1) * n];
    for (int i = 0; i < n; ++i) {
      for (int j = 0; j < n; ++j) { T a = 0; for (int k = 0; k < n; ++k) a += P[i * n + k] * L.A[k * n + j]; PA[i * n + j] = a; }
      for (int j = 0; j < m; ++j) { T a = 0; for (int k = 0; k < n; ++k) a += P[i * n + k] * L.B[k * m + j]; PB[i * m + j] = a; }
      T a = p[i];
      for (int k = 0; k < n; ++k) a += P[i * n + k] * ct[k];
      pc[i] = a;
    }
    for (int i = 0; i < n; ++i) {
      for (int j = 0; j < n; ++j) { T a = L.H[i * nz + j]; for (int k = 0; k < n; ++k) a += L.A[k * n + i] * PA[k * n + j]; Qxx[i * n + j] = a; }
      T a = L.g[i];
      for (int k = 0; k < n; ++k) a += L.A[k * n + i] * pc[k];
      qx[i] = a;
    }
    for (int i = 0; i < m; ++i) {
      for (int j = 0; j < m; ++j) { T a = L.H[(n + i) * nz + n + j]; for (int k = 0; k < n; ++k) a += L.B[k * m + i] * PB[k * m + j]; Quu[i * m + j] = a; }
      Quu[i * m + i] += reg;
      for (int j = 0; j < n; ++j) { T a = L.H[(n + i) * nz + j]; for (int k = 0; k < n; ++k) a += L.B[k * m + i] * PA[k * n + j]; Qux[i * n + j] = a; }
      T a = L.g[n + i];
      for (int k = 0; k < n; ++k) a += L.B[k * m + i] * pc[k];
      qu[i] = a;
    }
    if (!cholesky(Quu, m)) s.status |= ST_NON_PD;
    for (int i = 0; i < m; ++i) { for (int j = 0; j < n; ++j) KK[i * (n + 1) + j] = -Qux[i * n + j]; KK[i * (n + 1) + n] = -qu[i]; }
    chol_solve(Quu, m, KK.data(), n + 1, n + 1);
    T* K = &s.K[(size_t)t * m * n]; T* k = &s.k[(size_t)t * m];
    for (int i = 0; i < m; ++i) { for (int j = 0; j < n; ++j) K[i * n + j] = KK[i * (n + 1) + j]; k[i] = KK[i * (n + 1) + n]; }
    for (int i = 0; i < n; ++i) {
      for (int j = 0; j < n; ++j) { T a = Qxx[i * n + j]; for (int k2 = 0; k2 < m; ++k2) a += Qux[k2 * n + i] * K[k2 * n + j]; P[i * n + j] = a; }
      T a = qx[i];
      for (int k2 = 0; k2 < m; ++k2) a += Qux[k2 * n + i] * k[k2];
      p[i] = a;
    }
    for (int i = 0; i < n; ++i)
      for (int j = i + 1; j < n; ++j) { T a = T(0.5) * (P[i * n + j] + P[j * n + i]); P[i * n + j] = a; P[j * n + i] = a; }
    std::copy(P.begin(), P.end(), s.P.begin() + (size_t)t * n * n);
    std::copy(p.begin(), p.end(), s.p.begin() + (size_t)t * n);
  }
  for (int i = 0; i < n; ++i) s.dx[i] = c[i];
  for (int t = 0; t <= N; ++t) {
    const T* dx = &s.dx[(size_t)t * n];
    const T* Pt = &s.P[(size_t)t * n * n]; const T* pt = &s.p[(size_t)t * n];
    for (int i = 0; i < n; ++i) { T a = pt[i]; for (int j = 0; j < n; ++j) a += Pt[i * n + j] * dx[j]; s.lam[(size_t)t * n + i] = a; }
    if (t == N) break;
    const T* K = &s.K[(size_t)t * m * n]; const T* k = &s.k[(size_t)t * m];
    T* du = &s.du[(size_t)t * m];
    for (int i = 0; i < m; ++i) { T a = k[i]; for (int j = 0; j < n; ++j) a += K[i * n + j] * dx[j]; du[i] = a; }
    const StageLin<T>& L = lin[t];
    T* dxn = &s.dx[(size_t)(t + 1) * n];
    for (int i = 0; i < n; ++i) {
      T a = c[(size_t)(t + 1) * n + i];
      for (int j = 0; j < n; ++j) a += L.A[i * n + j] * dx[j];
      for (int j = 0; j < m; ++j) a += L.B[i * m + j] * du[j];
      dxn[i] = a;
    }
  }
}

// ------------------------------------------------------------ SQP (one instance)
// Arrays: X (N+1) x n, U N x m, V (N+1) x n, ref/par (N+1) x cols, W NW x NW.
template <class T>
struct Instance {
  int N;
  const T* x0;
  const T* ref;
  const T* par;
  const T* W;
  const LQData<T>* lq;
};

template <class T>
T merit_at(const ModelParams& mp, const Instance<T>& in, const T* X, const T* U, const T* V, T rho, T* cmax_out) {
  const int n = mp.n, m = mp.m, N = in.N;
  const int rc = ref_cols(mp.model), pc = par_cols(mp.model);
  std::vector<T> fx(n);
  T J = 0, VC = 0, CS = 0, cmax = 0;
  for (int i = 0; i < n; ++i) {
    T c = in.x0[i] - X[i];
    VC += V[i] * c; CS += c * c; cmax = std::max(cmax, (T)std::fabs(c));
  }
  std::vector<T> uz(m, T(0));
  for (int t = 0; t <= N; ++t) {
    bool term = (t == N);
    T l;
    eval_stage(mp, t, term, &X[(size_t)t * n], term ? uz.data() : &U[(size_t)t * m], in.ref + (size_t)t * rc,
               in.par + (size_t)t * pc, in.W, in.lq, fx.data(), &l);
    J += l;
    if (!term) {
      for (int i = 0; i < n; ++i) {
        T c = fx[i] - X[(size_t)(t + 1) * n + i];
        VC += V[(size_t)(t + 1) * n + i] * c; CS += c * c; cmax = std::max(cmax, (T)std::fabs(c));
      }
    }
  }
  if (cmax_out) *cmax_out = cmax;
  return J + VC + T(0.5) * rho * CS;
}

template <class T>
int sqp_solve(const ModelParams& mp, const Opts& op, const Instance<T>& in, T* X, T* U, T* V, T* K_out, T* k_out) {
  const int n = mp.n, m = mp.m, N = in.N, nz = n + m;
  const int rc = ref_cols(mp.model), pc = par_cols(mp.model);
  int status = 0;
  std::vector<StageLin<T>> lin(N + 1);
  std::vector<T> c((size_t)(N + 1) * n);
  std::vector<T> uz(m, T(0));
  LQRSol<T> sol;
  std::vector<T> Xt((size_t)(N + 1) * n), Ut((size_t)N * m), Vt((size_t)(N + 1) * n);
  T rho = T(op.rho0);
  for (int it = 0; it < op.sqp_iters; ++it) {
    T J0 = 0;
    for (int t = 0; t <= N; ++t) {
      bool term = (t == N);
      linearize_stage(mp, t, term, &X[(size_t)t * n], term ? uz.data() : &U[(size_t)t * m], in.ref + (size_t)t * rc,
                      in.par + (size_t)t * pc, in.W, in.lq, lin[t]);
      J0 += lin[t].l;
    }
    for (int i = 0; i < n; ++i) c[i] = in.x0[i] - X[i];
    for (int t = 0; t < N; ++t)
      for (int i = 0; i < n; ++i) c[(size_t)(t + 1) * n + i] = lin[t].fx[i] - X[(size_t)(t + 1) * n + i];
    riccati_solve(N, n, m, lin, c, T(op.reg), sol);
    status |= sol.status;
    // merit slope
    T gd = 0, lc = 0, vc = 0, cs = 0;
    for (int t = 0; t <= N; ++t) {
      for (int i = 0; i < n; ++i) gd += lin[t].g[i] * sol.dx[(size_t)t * n + i];
      if (t < N) for (int i = 0; i < m; ++i) gd += lin[t].g[n + i] * sol.du[(size_t)t * m + i];
      for (int i = 0; i < n; ++i) {
        T ci = c[(size_t)t * n + i];
        lc += (sol.lam[(size_t)t * n + i] - T(2) * V[(size_t)t * n + i]) * ci;
        vc += V[(size_t)t * n + i] * ci;
        cs += ci * ci;
      }
    }
    T G = gd + lc;
    if (cs > T(0) && G > T(0)) rho = std::min(std::max(rho, T(2) * G / cs), T(1e12));
    T dphi = G - rho * cs;
    T phi0 = J0 + vc + T(0.5) * rho * cs;
    T alpha = 1;
    bool accepted = false;
    if (!(dphi < -T(op.ls_skip_tol) * (T(1) + std::fabs(phi0)))) {
      accepted = true;  // predicted change below the arithmetic's resolution: full step
    } else {
      for (int tr = 0; tr < op.ls_max_trials; ++tr) {
        for (size_t i = 0; i < Xt.size(); ++i) Xt[i] = X[i] + alpha * sol.dx[i];
        for (size_t i = 0; i < Ut.size(); ++i) Ut[i] = U[i] + alpha * sol.du[i];
        for (size_t i = 0; i < Vt.size(); ++i) Vt[i] = V[i] + alpha * (sol.lam[i] - V[i]);
        T phi = merit_at(mp, in, Xt.data(), Ut.data(), Vt.data(), rho, (T*)nullptr);
        if (phi <= phi0 + T(op.ls_eta) * alpha * dphi) { accepted = true; break; }
        if (tr + 1 < op.ls_max_trials) alpha *= T(op.ls_beta);
      }
    }
    if (!accepted) status |= ST_LS_FAIL;
    for (size_t i = 0; i < Xt.size(); ++i) X[i] = X[i] + alpha * sol.dx[i];
    for (size_t i = 0; i < Ut.size(); ++i) U[i] = U[i] + alpha * sol.du[i];
    for (size_t i = 0; i < Vt.size(); ++i) V[i] = V[i] + alpha * (sol.lam[i] - V[i]);
    (void)nz;
  }
  if (K_out) std::copy(sol.K.begin(), sol.K.end(), K_out);
  if (k_out) std::copy(sol.k.begin(), sol.k.end(), k_out);
  for (size_t i = 0; i < (size_t)(N + 1) * n; ++i) if (!std::isfinite(val(X[i])) || !std::isfinite(val(V[i]))) status |= ST_NAN;
  for (size_t i = 0; i < (size_t)N * m; ++i) if (!std::isfinite(val(U[i]))) status |= ST_NAN;
  return status;
}

// KKT residual at (X, U, V), evaluated in T:
//   r_prim = max_t |c_t|_inf,
//   r_dual = max |grad_{x,u} L|_inf / (1 + max |grad l|_inf),
// with L = sum l + V_0.(x0 - X_0) + sum V_{t+1}.(f(x_t,u_t) - x_{t+1}).
template <class T>
void kkt_residual(const ModelParams& mp, const Instance<T>& in, const T* X, const T* U, const T* V, T* out3) {
  const int n = mp.n, m = mp.m, N = in.N;
  const int rc = ref_cols(mp.model), pc = par_cols(mp.model);
  std::vector<T> uz(m, T(0));
  StageLin<T> L;
  T rp = 0, rd = 0, gm = 0;
  for (int i = 0; i < n; ++i) rp = std::max(rp, (T)std::fabs(in.x0[i] - X[i]));
  for (int t = 0; t <= N; ++t) {
    bool term = (t == N);
    linearize_stage(mp, t, term, &X[(size_t)t * n], term ? uz.data() : &U[(size_t)t * m], in.ref + (size_t)t * rc,
                    in.par + (size_t)t * pc, in.W, in.lq, L);
    const T* Vt = &V[(size_t)t * n];
    for (int j = 0; j < n + (term ? 0 : m); ++j) gm = std::max(gm, (T)std::fabs(L.g[j]));
    if (term) {
      for (int i = 0; i < n; ++i) rd = std::max(rd, (T)std::fabs(L.g[i] - Vt[i]));
      break;
    }
    const T* Vn = &V[(size_t)(t + 1) * n];
    for (int i = 0; i < n; ++i) rp = std::max(rp, (T)std::fabs(L.fx[i] - X[(size_t)(t + 1) * n + i]));
    for (int j = 0; j < n; ++j) {
      T a = L.g[j] - Vt[j];
      for (int i = 0; i < n; ++i) a += L.A[i * n + j] * Vn[i];
      rd = std::max(rd, (T)std::fabs(a));
    }
    for (int j = 0; j < m; ++j) {
      T a = L.g[n + j];
      for (int i = 0; i < n; ++i) a += L.B[i * m + j] * Vn[i];
      rd = std::max(rd, (T)std::fabs(a));
    }
  }
  out3[0] = rp;
  out3[1] = rd / (T(1) + gm);
  out3[2] = std::max(out3[0], out3[1]);
}

// ------------------------------------------------------------ gait + reference
// mpc_utils.py:7-14, FP32, as XLA evaluates it without contraction:
//   leg_time = leg_time + dt*step_freq; wrap once if > 1; contact = leg_time < duty
inline void timer_run_f32(float duty, float step_freq, float* leg_time, float dt, int n_legs, int* contact) {
  volatile float inc = dt * step_freq;  // rounded product (no fused multiply-add)
  for (int i = 0; i < n_legs; ++i) {
    volatile float t = leg_time[i] + inc;
    float tt = t;
    if (tt > 1.0f) { volatile float w = tt - 1.0f; tt = w; }
    leg_time[i] = tt;
    contact[i] = (tt < duty) ? 1 : 0;
  }
}

}  // namespace oracle
