// ============================================================================
// Model-FLOP count of one SQP stage (measurement infrastructure, not the
// product).  The roofline's algorithmic work per stage and SQP iteration is
// the work-efficient Riccati count plus the model work of the stage: its
// linearisation (dynamics value and Jacobian [A B], tracking residual and its
// Jacobian, friction-cone constraints and their Jacobian, stage cost, the
// Gauss-Newton blocks, the gradient and the barrier curvature) and one
// line-search trial (dynamics and cost at the trial point).
//
// The count runs the oracle's own model functions (oracle.hpp: dynamics,
// state_residual, constraints, stage_cost, which restate mpx/utils/models.py:
// 6-37 and mpx/utils/objectives.py:7-75) on a counting scalar.  The scalar
// is a forward-mode value with up to 32 tangents that tracks which tangents
// are structurally nonzero, so one evaluation yields a Jacobian at the cost of
// sparse forward mode: a tangent operation is counted only where an operand's
// tangent can be nonzero, and operations with an exact 0 or 1 constant are
// free.  Each add, subtract, multiply, divide and each elementary function
// (sqrt, sin, cos, tan, log, atan2) counts one FLOP; negation is free.
// ============================================================================
#pragma once

#include <cstdint>
#include <type_traits>

#include "oracle.hpp"

namespace oracle {
namespace flopcount {

inline double& counter() {
  static thread_local double n = 0.0;
  return n;
}
inline int pop(uint32_t m) { return __builtin_popcount(m); }

struct Flop {
  double v;
  uint32_t m;  // directions whose tangent can be nonzero
  bool var;    // depends on a variable (x or u); otherwise a constant
  Flop() : v(0.0), m(0), var(false) {}
  Flop(double a) : v(a), m(0), var(false) {}
  Flop(double a, uint32_t mask, bool variable) : v(a), m(mask), var(variable) {}
  explicit operator double() const { return v; }
};

// Only constants are exempt: a variable that happens to be 0 still costs.
inline bool is_const(const Flop& a, double c) { return !a.var && a.v == c; }
inline Flop result(double v, const Flop& a, const Flop& b) { return Flop(v, a.m | b.m, a.var || b.var); }

inline Flop operator-(const Flop& a) { return Flop(-a.v, a.m, a.var); }
inline Flop operator+(const Flop& a, const Flop& b) {
  if (is_const(a, 0.0)) return b;
  if (is_const(b, 0.0)) return a;
  counter() += 1 + pop(a.m & b.m);
  return result(a.v + b.v, a, b);
}
inline Flop operator-(const Flop& a, const Flop& b) {
  if (is_const(b, 0.0)) return a;
  if (is_const(a, 0.0)) return -b;
  counter() += 1 + pop(a.m & b.m);
  return result(a.v - b.v, a, b);
}
inline Flop operator*(const Flop& a, const Flop& b) {
  if (is_const(a, 0.0) || is_const(b, 0.0)) return Flop(0.0);
  if (is_const(a, 1.0)) return b;
  if (is_const(b, 1.0)) return a;
  // (ab)' = a' b + a b': one multiply where one side varies, three where both do
  counter() += 1 + pop(a.m & ~b.m) + pop(b.m & ~a.m) + 3 * pop(a.m & b.m);
  return result(a.v * b.v, a, b);
}
inline Flop operator/(const Flop& a, const Flop& b) {
  if (is_const(a, 0.0)) return Flop(0.0);
  if (is_const(b, 1.0)) return a;
  if (b.m == 0) {
    counter() += 1 + pop(a.m);  // a' / b
  } else {
    // q = a / b, r = 1 / b; (a/b)' = (a' - q b') r
    counter() += 2 + pop(a.m & ~b.m) + 2 * pop(b.m & ~a.m) + 3 * pop(a.m & b.m);
  }
  return result(a.v / b.v, a, b);
}
template <class A, class = typename std::enable_if<std::is_arithmetic<A>::value>::type>
inline Flop operator+(const Flop& a, A b) { return a + Flop(double(b)); }
template <class A, class = typename std::enable_if<std::is_arithmetic<A>::value>::type>
inline Flop operator+(A b, const Flop& a) { return Flop(double(b)) + a; }
template <class A, class = typename std::enable_if<std::is_arithmetic<A>::value>::type>
inline Flop operator-(const Flop& a, A b) { return a - Flop(double(b)); }
template <class A, class = typename std::enable_if<std::is_arithmetic<A>::value>::type>
inline Flop operator-(A b, const Flop& a) { return Flop(double(b)) - a; }
template <class A, class = typename std::enable_if<std::is_arithmetic<A>::value>::type>
inline Flop operator*(const Flop& a, A b) { return a * Flop(double(b)); }
template <class A, class = typename std::enable_if<std::is_arithmetic<A>::value>::type>
inline Flop operator*(A b, const Flop& a) { return Flop(double(b)) * a; }
template <class A, class = typename std::enable_if<std::is_arithmetic<A>::value>::type>
inline Flop operator/(const Flop& a, A b) { return a / Flop(double(b)); }
template <class A, class = typename std::enable_if<std::is_arithmetic<A>::value>::type>
inline Flop operator/(A b, const Flop& a) { return Flop(double(b)) / a; }
inline Flop& operator+=(Flop& a, const Flop& b) { a = a + b; return a; }
inline Flop& operator-=(Flop& a, const Flop& b) { a = a - b; return a; }

// f(a) and its tangents f'(a) a': one FLOP for f, `dcost` for the scalar
// f'(a), one multiply per varying tangent.
inline Flop unary(double v, const Flop& a, int dcost) {
  counter() += 1 + (a.m ? dcost + pop(a.m) : 0);
  return Flop(v, a.m, a.var);
}
inline Flop sqrt(const Flop& a) { return unary(std::sqrt(a.v), a, 1); }   // 1/(2 s)
inline Flop sin(const Flop& a) { return unary(std::sin(a.v), a, 1); }     // cos a
inline Flop cos(const Flop& a) { return unary(std::cos(a.v), a, 1); }     // -sin a
inline Flop tan(const Flop& a) { return unary(std::tan(a.v), a, 2); }     // 1 + tan^2 a
inline Flop log(const Flop& a) { return unary(std::log(a.v), a, 1); }     // 1 / a
inline Flop atan2(const Flop& y, const Flop& x) {
  const uint32_t m = x.m | y.m;
  // r = 1/(x^2 + y^2); (x y' - y x') r
  counter() += 1 + (m ? 4 + 2 * pop(y.m & ~x.m) + 2 * pop(x.m & ~y.m) + 4 * pop(x.m & y.m) : 0);
  return Flop(std::atan2(y.v, x.v), m, x.var || y.var);
}

// Seeds of a variable vector: entry i varies along direction first + i (no
// tangents when first < 0).
inline void seed(const double* v, int cnt, int first, Flop* out) {
  for (int i = 0; i < cnt; ++i) out[i] = Flop(v[i], first >= 0 ? (1u << (first + i)) : 0u, true);
}

struct StageCount {
  double dyn_value;      // f(x, u)
  double dyn_jacobian;   // f and [A B] in one sparse forward-mode pass
  double cost_value;     // l(x, u)
  double linearisation;  // everything the Riccati pass needs about the stage
  double trial;          // one line-search trial: f and l at the trial point
};

// Counts of one non-terminal stage of an SRBD model at (x, u) with the
// parameter row `par` (contact flags, foot positions), reference row `ref`
// and the dense 24 x 24 weight W (only its diagonal is used by the models).
inline StageCount count_stage(const ModelParams& mp, const double* x, const double* u, const double* ref,
                              const double* par, const double* W) {
  const int n = mp.n, m = mp.m;
  double& c = counter();
  StageCount out;
  Flop xs[16], us[16], fx[16];
  // f alone
  seed(x, n, -1, xs); seed(u, m, -1, us);
  c = 0; dynamics(mp, xs, us, par, fx); out.dyn_value = c;
  // f and its Jacobian
  seed(x, n, 0, xs); seed(u, m, n, us);
  c = 0; dynamics(mp, xs, us, par, fx); out.dyn_jacobian = c;
  // l alone
  seed(x, n, -1, xs); seed(u, m, -1, us);
  c = 0; stage_cost(mp, xs, us, ref, W, false); out.cost_value = c;

  // ---- linearisation
  double lin = out.dyn_jacobian + out.cost_value;
  // defect f(x, u) - x_{t+1}
  lin += n;
  // residual r(x) and its Jacobian Jx (12 x n)
  Flop r[12], cu[14];
  int foot_of[14];
  seed(x, n, 0, xs);
  c = 0; state_residual(mp, xs, ref, r); lin += c;
  // constraints c(u) and their Jacobian Jc (nc x m)
  seed(u, m, 0, us);
  c = 0;
  const int nc = constraints(mp, us, cu, foot_of);
  lin += c;
  // Gauss-Newton blocks and gradient, on the structural patterns of Jx and Jc
  // with the diagonal weights: Q = Jx' W Jx (upper triangle), R = W_u + the
  // barrier's curvature, M = Jx' W_xu = 0; g_x = Jx' (W r), g_u = W_u u + the
  // barrier's gradient.
  auto var = [](double v) { return Flop(v, 0u, true); };  // a value that depends on (x, u)
  auto Jx = [&](int a, int j) { return (r[a].m >> j) & 1u ? var(1.5) : Flop(0.0); };
  auto Jc = [&](int k, int j) { return (cu[k].m >> j) & 1u ? var(1.5) : Flop(0.0); };
  const int contact_off = (mp.model == MODEL_SRBD_QUAT13) ? 13 : 12;
  c = 0;
  for (int i = 0; i < n; ++i)
    for (int j = i; j < n; ++j) {
      Flop s = 0.0;
      for (int a = 0; a < 12; ++a) s += Jx(a, i) * Flop(W[a * NW + a]) * Jx(a, j);
    }
  Flop wr[12];
  for (int a = 0; a < 12; ++a) wr[a] = Flop(W[a * NW + a]) * var(r[a].v);
  for (int i = 0; i < n; ++i) {
    Flop s = 0.0;
    for (int a = 0; a < 12; ++a) s += Jx(a, i) * wr[a];
  }
  Flop gu[16];
  for (int j = 0; j < m; ++j) gu[j] = Flop(W[(12 + j) * NW + 12 + j]) * var(u[j]);
  for (int k = 0; k < nc; ++k) {
    const double ck = ref[contact_off + foot_of[k]];
    if (mp.barrier_masked && ck == 0.0) continue;
    const Flop ckf(ck), cv = var(cu[k].v);
    // beta'(c) and beta''(c) of the relaxed log barrier (-a/c, a/c^2 above
    // sigma; affine and constant below), weighted by the contact flag
    const Flop d1 = (cv.v > mp.barrier_sigma ? Flop(-mp.barrier_alpha) / cv
                                             : Flop(mp.barrier_alpha / (mp.barrier_sigma * mp.barrier_sigma)) *
                                                   (cv - Flop(2.0 * mp.barrier_sigma))) * ckf;
    const Flop d2 = (cv.v > mp.barrier_sigma ? Flop(mp.barrier_alpha) / (cv * cv)
                                             : Flop(mp.barrier_alpha / (mp.barrier_sigma * mp.barrier_sigma))) * ckf;
    for (int j = 0; j < m; ++j) gu[j] += d1 * Jc(k, j);
    for (int i = 0; i < m; ++i)
      for (int j = i; j < m; ++j) {
        const Flop h = d2 * Jc(k, i) * Jc(k, j);
        if (!is_const(h, 0.0)) c += 1;  // added into R
      }
  }
  if (mp.barrier_kind == 1) {
    // exact curvature of the cones, 1/2 a beta'(c) grad^2 c, per leg in stance
    const int legs = (mp.model == MODEL_BIPED_WRENCH12) ? 2 : 4;
    const int stride = (mp.model == MODEL_BIPED_WRENCH12) ? 6 : 3;
    const int cstride = (mp.model == MODEL_BIPED_WRENCH12) ? 7 : 1;
    for (int i = 0; i < legs; ++i) {
      if (ref[contact_off + i] == 0.0) continue;
      const Flop fx_ = var(u[stride * i]), fy_ = var(u[stride * i + 1]), cv = var(cu[cstride * i].v);
      const Flop s2 = fx_ * fx_ + fy_ * fy_ + Flop(mp.cone_eps2), s = sqrt(s2), s3 = s2 * s;
      const Flop dpen = cv.v > mp.barrier_sigma ? Flop(-mp.barrier_alpha) / cv
                                                : Flop(mp.barrier_alpha / (mp.barrier_sigma * mp.barrier_sigma)) *
                                                      (cv - Flop(2.0 * mp.barrier_sigma));
      const Flop w = Flop(-0.5) * dpen;
      const Flop hxx = w * ((s2 - fx_ * fx_) / s3), hxy = w * (Flop(-1.0) * fx_ * fy_ / s3),
                 hyy = w * ((s2 - fy_ * fy_) / s3);
      c += 3;  // added into the three distinct entries of the 2 x 2 block
      (void)hxx; (void)hxy; (void)hyy;
    }
  }
  lin += c;
  out.linearisation = lin;
  out.trial = out.dyn_value + out.cost_value + n;  // f, l and the defect at the trial point
  return out;
}

}  // namespace flopcount
}  // namespace oracle
