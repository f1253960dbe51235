// ============================================================================
// CPU ORACLE (test infrastructure): SRBD gait timer and reference generator.
//
// FP32 restatement of mpx/utils/mpc_utils.py:7-14 (timer_run) and
// mpx/utils/mpc_utils.py:146-270 (reference_generator_srbd, the path with
// use_terrain_estimator = False, which is what config_srbd.py:31 selects).
// Every expression is evaluated in float32 in the order the Python source
// writes it, without fused multiply-add (compile with -ffp-contract=off), so
// that the contact schedule is bit-exact and the float outputs agree with the
// reference's own source to float32 rounding.  Integer powers follow
// jax.lax.integer_pow's square-and-multiply order.
//
// Pinned by tests/golden (vectors produced by executing the reference's
// source under a numpy float32 stand-in for jax.numpy).
// ============================================================================
#pragma once
#include <cmath>

namespace oracle {

struct RefGenCfg {
  int N;
  float dt;
  int n_contact;  // 4
  float mass;
  float foot0[12];  // config.p_legs0
  float duty_factor, step_freq, step_height, clearence_speed;
};

static inline float f32(double v) { return (float)v; }
static inline float ipow2(float s) { volatile float r = s * s; return r; }
static inline float ipow3(float s) { float s2 = ipow2(s); volatile float r = s * s2; return r; }
static inline float ipow4(float s) { float s2 = ipow2(s); volatile float r = s2 * s2; return r; }
// The volatile temporaries below force one float32 rounding per operation.
#define R32(e) ([&]() { volatile float _r = (e); return (float)_r; }())

static inline float splineXY(float cur, float fh, float v0, float s) {
  float d = R32(fh - cur);
  float a0 = cur, a1 = v0;
  float a2 = R32(R32(3.0f * d) - R32(2.0f * v0));
  float a3 = R32(v0 - R32(2.0f * d));
  float r = R32(a0 + R32(a1 * s));
  r = R32(r + R32(a2 * ipow2(s)));
  r = R32(r + R32(a3 * ipow3(s)));
  return r;
}
static inline float splineXY_dot(float cur, float fh, float v0, float s) {
  float d = R32(fh - cur);
  float a1 = v0;
  float a2 = R32(R32(3.0f * d) - R32(2.0f * v0));
  float a3 = R32(v0 - R32(2.0f * d));
  float r = R32(R32(R32(2.0f * a2) * s) + R32(R32(3.0f * a3) * ipow2(s)));
  return R32(r + a1);
}
// cubic_splineZ(current_foot, foothold, step_height, val), initial_speed = 0.7
static inline float splineZ_coef(float cur, float fh, float sh, float* a, float* b, float* c) {
  const float two_v = f32(2 * 0.7), five_v = f32(5 * 0.7), four_v = f32(4 * 0.7);
  *a = R32(R32(R32(R32(16.0f * sh) - R32(8.0f * fh)) - R32(8.0f * cur)) - two_v);
  *b = R32(R32(R32(five_v + R32(14.0f * fh)) + R32(18.0f * cur)) - R32(32.0f * sh));
  *c = R32(R32(R32(R32(16.0f * sh) - R32(5.0f * fh)) - R32(11.0f * cur)) - four_v);
  return f32(0.7);
}
static inline float splineZ(float cur, float fh, float sh, float s) {
  float a, b, c;
  float d = splineZ_coef(cur, fh, sh, &a, &b, &c);
  float r = R32(R32(a * ipow4(s)) + R32(b * ipow3(s)));
  r = R32(r + R32(c * ipow2(s)));
  r = R32(r + R32(d * s));
  return R32(r + cur);
}
static inline float splineZ_dot(float cur, float fh, float sh, float s) {
  float a, b, c;
  float d = splineZ_coef(cur, fh, sh, &a, &b, &c);
  float r = R32(R32(R32(4.0f * a) * ipow3(s)) + R32(R32(3.0f * b) * ipow2(s)));
  r = R32(r + R32(R32(2.0f * c) * s));
  return R32(r + d);
}

// timer_run for n legs; returns contact in cont[] (1/0), updates leg_time.
static inline void timer_run(float duty, float step_freq, float dt, int n, float* leg_time, int* cont) {
  float inc = R32(dt * step_freq);
  for (int i = 0; i < n; ++i) {
    float t = R32(leg_time[i] + inc);
    if (t > 1.0f) t = R32(t - 1.0f);
    leg_time[i] = t;
    cont[i] = (t < duty) ? 1 : 0;
  }
}

// reference_generator_srbd (mpc_utils.py:146-270).  Outputs:
//   reference[(N+1) x 17] = [p_ref3, quat_ref4, dp_ref3, omega_ref3, contact4]
//   parameter[(N+1) x 16] = [contact4, foot_ref12]
//   liftoff[12] (in/out), foot_ref_dot[(N+1) x 12]
static inline void refgen_srbd(const RefGenCfg& g, const float* t_timer, const float* x, const float* foot,
                               const float* input, const float* contact, float* liftoff, float* reference,
                               float* parameter, float* foot_ref_dot) {
  const int N = g.N, nc = 4;
  const float q0 = x[3], q1 = x[4], q2 = x[5], q3 = x[6];
  float yaw = std::atan2(R32(2.0f * R32(R32(q0 * q3) + R32(q1 * q2))),
                         R32(1.0f - R32(2.0f * R32(R32(q2 * q2) + R32(q3 * q3)))));
  float cy = std::cos(yaw), sy = std::sin(yaw);
  float Ryaw[9] = {cy, -sy, 0.0f, sy, cy, 0.0f, 0.0f, 0.0f, 1.0f};
  float lz_sum = R32(R32(R32(liftoff[2] + liftoff[5]) + liftoff[8]) + liftoff[11]);
  float proprio_height = R32(input[6] + R32(lz_sum / (float)nc));
  float p[3] = {x[0], x[1], proprio_height};
  // pitch of quat_ref = [1,0,0,0] is exactly 0, so Rpitch = I and Ryaw @ Rpitch = Ryaw.
  float rlv[3];
  for (int r = 0; r < 3; ++r)
    rlv[r] = R32(R32(R32(Ryaw[3 * r] * input[0]) + R32(Ryaw[3 * r + 1] * input[1])) + R32(Ryaw[3 * r + 2] * input[2]));
  float fp[12];
  for (int i = 0; i < nc; ++i)
    for (int r = 0; r < 3; ++r) {
      float d = R32(R32(R32(g.foot0[3 * i] * Ryaw[3 * r]) + R32(g.foot0[3 * i + 1] * Ryaw[3 * r + 1])) +
                    R32(g.foot0[3 * i + 2] * Ryaw[3 * r + 2]));
      fp[3 * i + r] = R32(p[r] + d);
    }
  // early contact from one timer step (mpc_utils.py:176-177)
  float cur_t[4];
  int des[4];
  for (int i = 0; i < nc; ++i) cur_t[i] = t_timer[i];
  timer_run(g.duty_factor, g.step_freq, g.dt, nc, cur_t, des);
  float thr = R32(0.5f + R32(0.5f * g.duty_factor));
  int early[4];
  for (int i = 0; i < nc; ++i) early[i] = (des[i] == 0 && contact[i] == 1.0f && cur_t[i] > thr) ? 1 : 0;
  // initial_speed = -rlv / (norm(rlv) + 1e-6) * clearence_speed
  float nrm = std::sqrt(R32(R32(R32(rlv[0] * rlv[0]) + R32(rlv[1] * rlv[1])) + R32(rlv[2] * rlv[2])));
  float den = R32(nrm + 1e-6f);
  float ispeed[3];
  for (int r = 0; r < 3; ++r) ispeed[r] = R32(R32(-rlv[r] / den) * g.clearence_speed);
  // tables
  for (int t = 0; t <= N; ++t) {
    float tf = R32((float)t * g.dt);
    float* ref = reference + t * 17;
    ref[0] = R32(R32(tf * rlv[0]) + p[0]);
    ref[1] = R32(R32(tf * rlv[1]) + p[1]);
    ref[2] = proprio_height;
    ref[3] = 1.0f; ref[4] = 0.0f; ref[5] = 0.0f; ref[6] = 0.0f;
    for (int r = 0; r < 3; ++r) { ref[7 + r] = rlv[r]; ref[10 + r] = input[3 + r]; }
    for (int i = 0; i < 12; ++i) { parameter[t * 16 + 4 + i] = foot[i]; foot_ref_dot[t * 12 + i] = 0.0f; }
    for (int i = 0; i < 4; ++i) { ref[13 + i] = 0.0f; parameter[t * 16 + i] = 0.0f; }
  }
  float lx[4], ly[4], lz[4];
  for (int i = 0; i < nc; ++i) { lx[i] = liftoff[3 * i]; ly[i] = liftoff[3 * i + 1]; lz[i] = liftoff[3 * i + 2]; }
  float new_t[4];
  for (int i = 0; i < nc; ++i) new_t[i] = t_timer[i];
  const float sq = std::sqrt(R32(input[6] / 9.81f));
  float fh[2][4];
  for (int d = 0; d < 2; ++d)
    for (int i = 0; i < nc; ++i) {
      float f1 = R32(R32(R32(0.5f * rlv[d]) * g.duty_factor) / g.step_freq);
      float f2 = R32(sq * R32(x[7 + d] - rlv[d]));
      fh[d][i] = R32(R32(f1 + f2) + fp[3 * i + d]);
    }
  const float one_m_duty = R32(1.0f - g.duty_factor);
  for (int t = 0; t <= N; ++t) {
    const int tp = (t == 0) ? N : t - 1;  // python index t-1 wraps to the last row
    float* foot_prev = parameter + tp * 16 + 4;
    float prev_x[4], prev_y[4], prev_z[4];
    for (int i = 0; i < nc; ++i) { prev_x[i] = foot_prev[3 * i]; prev_y[i] = foot_prev[3 * i + 1]; prev_z[i] = foot_prev[3 * i + 2]; }
    int cs[4];
    timer_run(g.duty_factor, g.step_freq, g.dt, nc, new_t, cs);
    for (int i = 0; i < nc; ++i) { reference[t * 17 + 13 + i] = (float)cs[i]; parameter[t * 16 + i] = (float)cs[i]; }
    for (int i = 0; i < nc; ++i) {
      bool prev_c = parameter[tp * 16 + i] != 0.0f;
      if (!(cs[i] != 0) && prev_c) { lx[i] = prev_x[i]; ly[i] = prev_y[i]; lz[i] = prev_z[i]; }
    }
    float* foot_t = parameter + t * 16 + 4;
    float* fdot = foot_ref_dot + t * 12;
    for (int i = 0; i < nc; ++i) {
      float s = R32(R32(new_t[i] - g.duty_factor) / one_m_duty);
      bool stance = (cs[i] > 0) || (early[i] == 1);
      float sh = R32(lz[i] + g.step_height);
      if (stance) {
        foot_t[3 * i] = prev_x[i]; foot_t[3 * i + 1] = prev_y[i]; foot_t[3 * i + 2] = prev_z[i];
        fdot[3 * i] = 0.0f; fdot[3 * i + 1] = 0.0f; fdot[3 * i + 2] = 0.0f;
      } else {
        foot_t[3 * i] = splineXY(lx[i], fh[0][i], ispeed[0], s);
        foot_t[3 * i + 1] = splineXY(ly[i], fh[1][i], ispeed[1], s);
        foot_t[3 * i + 2] = splineZ(lz[i], lz[i], sh, s);
        fdot[3 * i] = splineXY_dot(lx[i], fh[0][i], ispeed[0], s);
        fdot[3 * i + 1] = splineXY_dot(ly[i], fh[1][i], ispeed[1], s);
        fdot[3 * i + 2] = splineZ_dot(lz[i], lz[i], sh, s);
      }
    }
  }
  for (int i = 0; i < nc; ++i) { liftoff[3 * i] = lx[i]; liftoff[3 * i + 1] = ly[i]; liftoff[3 * i + 2] = lz[i]; }
}
// terrain_orientation (mpc_utils.py:15-37): the frame [front-back vector of
// the liftoff points, Ryaw e_y, their normal], columns normalised, to a unit
// quaternion (w, x, y, z) by the pivot on the largest of the diagonal and the
// trace (jax.scipy.spatial.transform.Rotation.from_matrix), then rolled.
static inline void terrain_orientation(const float* lo, const float* Ryaw, float* q) {
  float fb[3], lr[3], nr[3];
  for (int i = 0; i < 3; ++i) fb[i] = R32(R32(R32(R32(lo[i] + lo[3 + i]) - lo[6 + i]) - lo[9 + i]) / 2.0f);
  for (int i = 0; i < 3; ++i) lr[i] = Ryaw[3 * i + 1];
  nr[0] = R32(R32(fb[1] * lr[2]) - R32(fb[2] * lr[1]));
  nr[1] = R32(R32(fb[2] * lr[0]) - R32(fb[0] * lr[2]));
  nr[2] = R32(R32(fb[0] * lr[1]) - R32(fb[1] * lr[0]));
  float* v[3] = {fb, lr, nr};
  for (int k = 0; k < 3; ++k) {
    float n = std::sqrt(R32(R32(R32(v[k][0] * v[k][0]) + R32(v[k][1] * v[k][1])) + R32(v[k][2] * v[k][2])));
    for (int i = 0; i < 3; ++i) v[k][i] = R32(v[k][i] / n);
  }
  float m[3][3];
  for (int r = 0; r < 3; ++r) { m[r][0] = fb[r]; m[r][1] = lr[r]; m[r][2] = nr[r]; }
  float tr = R32(R32(m[0][0] + m[1][1]) + m[2][2]);
  float dec[4] = {m[0][0], m[1][1], m[2][2], tr};
  int c = 0;
  for (int i = 1; i < 4; ++i)
    if (dec[i] > dec[c]) c = i;
  float xyzw[4];
  if (c != 3) {
    int i = c, j = (i + 1) % 3, k = (j + 1) % 3;
    xyzw[i] = R32(R32(1.0f - tr) + R32(2.0f * m[i][i]));
    xyzw[j] = R32(m[j][i] + m[i][j]);
    xyzw[k] = R32(m[k][i] + m[i][k]);
    xyzw[3] = R32(m[k][j] - m[j][k]);
  } else {
    xyzw[0] = R32(m[2][1] - m[1][2]);
    xyzw[1] = R32(m[0][2] - m[2][0]);
    xyzw[2] = R32(m[1][0] - m[0][1]);
    xyzw[3] = R32(1.0f + tr);
  }
  float n = std::sqrt(R32(R32(R32(R32(xyzw[0] * xyzw[0]) + R32(xyzw[1] * xyzw[1])) + R32(xyzw[2] * xyzw[2])) +
                          R32(xyzw[3] * xyzw[3])));
  q[0] = R32(xyzw[3] / n);
  q[1] = R32(xyzw[0] / n);
  q[2] = R32(xyzw[1] / n);
  q[3] = R32(xyzw[2] / n);
}

// reference_generator (mpc_utils.py:39-145), the whole-body generator, for 4
// contact points and nj joints.  x is the whole-body state (base velocity at
// x[7 + nj]).  Outputs:
//   reference[(N+1) x (13 + nj + 28)] = [p_ref3, quat_ref4, q0 (nj), dp_ref3,
//       omega_ref3, foot_ref12, contact4, grf_ref12]
//   parameter[(N+1) x 4] = contact sequence;  liftoff[12] (in/out).
static inline void refgen_wb(const RefGenCfg& g, int nj, const float* q0v, int terrain, const float* t_timer,
                             const float* x, const float* foot, const float* input, const float* contact,
                             float* liftoff, float* reference, float* parameter) {
  const int N = g.N, nc = 4, C = 13 + nj + 28, cf = 13 + nj, cc = cf + 12, cg = cc + 4;
  const float q0 = x[3], q1 = x[4], q2 = x[5], q3 = x[6];
  float yaw = std::atan2(R32(2.0f * R32(R32(q0 * q3) + R32(q1 * q2))),
                         R32(1.0f - R32(2.0f * R32(R32(q2 * q2) + R32(q3 * q3)))));
  float cy = std::cos(yaw), sy = std::sin(yaw);
  float Ryaw[9] = {cy, -sy, 0.0f, sy, cy, 0.0f, 0.0f, 0.0f, 1.0f};
  float lz_sum = R32(R32(R32(liftoff[2] + liftoff[5]) + liftoff[8]) + liftoff[11]);
  float proprio_height = R32(input[6] + R32(lz_sum / (float)nc));
  float p[3] = {x[0], x[1], proprio_height};
  float qr[4] = {1.0f, 0.0f, 0.0f, 0.0f};
  if (terrain) terrain_orientation(liftoff, Ryaw, qr);
  float pitch = std::asin(R32(2.0f * R32(R32(qr[0] * qr[2]) - R32(qr[3] * qr[1]))));
  float cp = std::cos(pitch), sp = std::sin(pitch);
  float Rp[9] = {cp, 0.0f, sp, 0.0f, 1.0f, 0.0f, -sp, 0.0f, cp};
  float M[9];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c)
      M[3 * r + c] = R32(R32(R32(Ryaw[3 * r] * Rp[c]) + R32(Ryaw[3 * r + 1] * Rp[3 + c])) + R32(Ryaw[3 * r + 2] * Rp[6 + c]));
  float rlv[3];
  for (int r = 0; r < 3; ++r)
    rlv[r] = R32(R32(R32(M[3 * r] * input[0]) + R32(M[3 * r + 1] * input[1])) + R32(M[3 * r + 2] * input[2]));
  float fp[12];
  for (int i = 0; i < nc; ++i)
    for (int r = 0; r < 3; ++r) {
      float d = R32(R32(R32(g.foot0[3 * i] * Ryaw[3 * r]) + R32(g.foot0[3 * i + 1] * Ryaw[3 * r + 1])) +
                    R32(g.foot0[3 * i + 2] * Ryaw[3 * r + 2]));
      fp[3 * i + r] = R32(p[r] + d);
    }
  float cur_t[4];
  int des[4];
  for (int i = 0; i < nc; ++i) cur_t[i] = t_timer[i];
  timer_run(g.duty_factor, g.step_freq, g.dt, nc, cur_t, des);
  float thr = R32(0.5f + R32(0.5f * g.duty_factor));
  int early[4];
  for (int i = 0; i < nc; ++i) early[i] = (des[i] == 0 && contact[i] == 1.0f && cur_t[i] > thr) ? 1 : 0;
  float nrm = std::sqrt(R32(R32(R32(rlv[0] * rlv[0]) + R32(rlv[1] * rlv[1])) + R32(rlv[2] * rlv[2])));
  float den = R32(nrm + 1e-6f);
  float ispeed[3];
  for (int r = 0; r < 3; ++r) ispeed[r] = R32(R32(-rlv[r] / den) * g.clearence_speed);
  for (int t = 0; t <= N; ++t) {
    float tf = R32((float)t * g.dt);
    float* ref = reference + t * C;
    ref[0] = R32(R32(tf * rlv[0]) + p[0]);
    ref[1] = R32(R32(tf * rlv[1]) + p[1]);
    ref[2] = proprio_height;
    for (int i = 0; i < 4; ++i) ref[3 + i] = qr[i];
    for (int j = 0; j < nj; ++j) ref[7 + j] = q0v[j];
    for (int r = 0; r < 3; ++r) { ref[7 + nj + r] = rlv[r]; ref[10 + nj + r] = input[3 + r]; }
    for (int i = 0; i < 12; ++i) { ref[cf + i] = foot[i]; ref[cg + i] = 0.0f; }
    for (int i = 0; i < 4; ++i) { ref[cc + i] = 0.0f; parameter[t * 4 + i] = 0.0f; }
  }
  float lx[4], ly[4], lz[4];
  for (int i = 0; i < nc; ++i) { lx[i] = liftoff[3 * i]; ly[i] = liftoff[3 * i + 1]; lz[i] = liftoff[3 * i + 2]; }
  float new_t[4];
  for (int i = 0; i < nc; ++i) new_t[i] = t_timer[i];
  const float sq = std::sqrt(R32(input[6] / 9.81f));
  const float* dp = x + 7 + nj;
  float fh[2][4];
  for (int d = 0; d < 2; ++d)
    for (int i = 0; i < nc; ++i) {
      float f1 = R32(R32(R32(0.5f * rlv[d]) * g.duty_factor) / g.step_freq);
      float f2 = R32(sq * R32(dp[d] - rlv[d]));
      fh[d][i] = R32(R32(f1 + f2) + fp[3 * i + d]);
    }
  const float one_m_duty = R32(1.0f - g.duty_factor);
  for (int t = 0; t <= N; ++t) {
    const int tp = (t == 0) ? N : t - 1;
    const float* foot_prev = reference + tp * C + cf;
    float prev_x[4], prev_y[4], prev_z[4];
    for (int i = 0; i < nc; ++i) { prev_x[i] = foot_prev[3 * i]; prev_y[i] = foot_prev[3 * i + 1]; prev_z[i] = foot_prev[3 * i + 2]; }
    int cs[4];
    timer_run(g.duty_factor, g.step_freq, g.dt, nc, new_t, cs);
    float* ref = reference + t * C;
    for (int i = 0; i < nc; ++i) {
      bool prev_c = parameter[tp * 4 + i] != 0.0f;
      ref[cc + i] = (float)cs[i];
      parameter[t * 4 + i] = (float)cs[i];
      if (!(cs[i] != 0) && prev_c) { lx[i] = prev_x[i]; ly[i] = prev_y[i]; lz[i] = prev_z[i]; }
    }
    for (int i = 0; i < nc; ++i) {
      float s = R32(R32(new_t[i] - g.duty_factor) / one_m_duty);
      bool stance = (cs[i] > 0) || (early[i] == 1);
      float sh = R32(lz[i] + g.step_height);
      float* ft = ref + cf + 3 * i;
      if (stance) {
        ft[0] = prev_x[i]; ft[1] = prev_y[i]; ft[2] = prev_z[i];
      } else {
        ft[0] = splineXY(lx[i], fh[0][i], ispeed[0], s);
        ft[1] = splineXY(ly[i], fh[1][i], ispeed[1], s);
        ft[2] = splineZ(lz[i], lz[i], sh, s);
      }
    }
    float csum = R32(R32(R32((float)cs[0] + (float)cs[1]) + (float)cs[2]) + (float)cs[3]);
    float dn = R32(csum + 1e-5f);
    for (int i = 0; i < nc; ++i) ref[cg + 3 * i + 2] = R32(R32(R32((float)cs[i] * g.mass) * 9.81f) / dn);
  }
  for (int i = 0; i < nc; ++i) { liftoff[3 * i] = lx[i]; liftoff[3 * i + 1] = ly[i]; liftoff[3 * i + 2] = lz[i]; }
}
#undef R32

}  // namespace oracle
