// Small per-tick kernels around the solve: warm-start shift, gait timer and
// the SRBD reference generator (one thread per instance).
#pragma once
#include <cuda_runtime.h>

#include "../../include/mpxg.h"

namespace mpxg {

// mpx/utils/mpc_wrapper_srbd.py:135-137 per instance horizon: rows [shift..N]
// move to [0..N-shift], the last row is repeated into the freed tail.
__global__ void shift_kernel(int batch, const int* slot, int n_max, int nx, int nu, const int* horizon, int shift,
                             const float* X, const float* U, const float* V, float* Xo, float* Uo, float* Vo) {
  if ((int)blockIdx.x >= batch) return;
  const int b = slot ? slot[blockIdx.x] : (int)blockIdx.x;
  const int N = horizon ? horizon[b] : n_max;
  if (N < 1 || N > n_max) return;
  const size_t xo = (size_t)b * (n_max + 1) * nx, uo = (size_t)b * n_max * nu;
  // read everything first when shifting in place: one block owns one instance
  extern __shared__ float buf[];
  float* bx = buf;
  float* bv = bx + (size_t)(N + 1) * nx;
  float* bu = bv + (size_t)(N + 1) * nx;
  for (int e = threadIdx.x; e < (N + 1) * nx; e += blockDim.x) { bx[e] = X[xo + e]; bv[e] = V[xo + e]; }
  for (int e = threadIdx.x; e < N * nu; e += blockDim.x) bu[e] = U[uo + e];
  __syncthreads();
  for (int e = threadIdx.x; e < (N + 1) * nx; e += blockDim.x) {
    const int t = e / nx, i = e - t * nx;
    const int src = min(t + shift, N);
    Xo[xo + e] = bx[src * nx + i];
    Vo[xo + e] = bv[src * nx + i];
  }
  for (int e = threadIdx.x; e < N * nu; e += blockDim.x) {
    const int t = e / nu, i = e - t * nu;
    const int src = min(t + shift, N - 1);
    Uo[uo + e] = bu[src * nu + i];
  }
}

// mpx/utils/mpc_utils.py:7-14 with explicit round-to-nearest operations (no
// fused multiply-add), so that the schedule is bit-identical to float32 CPU
// arithmetic.
__device__ __forceinline__ void timer_step(float duty, float inc, float& t, int& contact) {
  t = __fadd_rn(t, inc);
  if (t > 1.0f) t = __fadd_rn(t, -1.0f);
  contact = (t < duty) ? 1 : 0;
}

__global__ void timer_kernel(int n, int n_legs, float duty, float step_freq, float dt, float* leg_time, int* contact) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const float inc = __fmul_rn(dt, step_freq);
  float t = leg_time[e];
  int c;
  timer_step(duty, inc, t, c);
  leg_time[e] = t;
  contact[e] = c;
  (void)n_legs;
}

// ------------------------------------------------------------ reference generator
// mpx/utils/mpc_utils.py:146-270 (use_terrain_estimator = False), one thread
// per instance, float32 with one rounding per operation as the Python source
// writes it (integer powers as square-and-multiply).
struct RefGenArgs {
  int batch, N, n_max;
  float dt;
  float foot0[12];
  float duty, step_freq, step_height, clearence;
  const float *t_timer, *x, *foot, *input, *contact;
  float *liftoff, *reference, *parameter, *foot_ref_dot;
};

__device__ __forceinline__ float sq_(float s) { return __fmul_rn(s, s); }
__device__ __forceinline__ float cu_(float s) { return __fmul_rn(s, sq_(s)); }
__device__ __forceinline__ float qu_(float s) { const float s2 = sq_(s); return __fmul_rn(s2, s2); }
#define ADD __fadd_rn
#define SUB __fsub_rn
#define MUL __fmul_rn
#define DIV __fdiv_rn

__device__ __forceinline__ float splineXY(float cur, float fh, float v0, float s) {
  const float d = SUB(fh, cur);
  const float a2 = SUB(MUL(3.0f, d), MUL(2.0f, v0));
  const float a3 = SUB(v0, MUL(2.0f, d));
  float r = ADD(cur, MUL(v0, s));
  r = ADD(r, MUL(a2, sq_(s)));
  return ADD(r, MUL(a3, cu_(s)));
}
__device__ __forceinline__ float splineXY_dot(float cur, float fh, float v0, float s) {
  const float d = SUB(fh, cur);
  const float a2 = SUB(MUL(3.0f, d), MUL(2.0f, v0));
  const float a3 = SUB(v0, MUL(2.0f, d));
  const float r = ADD(MUL(MUL(2.0f, a2), s), MUL(MUL(3.0f, a3), sq_(s)));
  return ADD(r, v0);
}
__device__ __forceinline__ void splineZ_coef(float cur, float fh, float sh, float* a, float* b, float* c) {
  const float two_v = 1.4f, five_v = 3.5f, four_v = 2.8f;  // 2*0.7, 5*0.7, 4*0.7 rounded to float
  *a = SUB(SUB(SUB(MUL(16.0f, sh), MUL(8.0f, fh)), MUL(8.0f, cur)), two_v);
  *b = SUB(ADD(ADD(five_v, MUL(14.0f, fh)), MUL(18.0f, cur)), MUL(32.0f, sh));
  *c = SUB(SUB(SUB(MUL(16.0f, sh), MUL(5.0f, fh)), MUL(11.0f, cur)), four_v);
}
__device__ __forceinline__ float splineZ(float cur, float fh, float sh, float s) {
  float a, b, c;
  splineZ_coef(cur, fh, sh, &a, &b, &c);
  float r = ADD(MUL(a, qu_(s)), MUL(b, cu_(s)));
  r = ADD(r, MUL(c, sq_(s)));
  r = ADD(r, MUL(0.7f, s));
  return ADD(r, cur);
}
__device__ __forceinline__ float splineZ_dot(float cur, float fh, float sh, float s) {
  float a, b, c;
  splineZ_coef(cur, fh, sh, &a, &b, &c);
  float r = ADD(MUL(MUL(4.0f, a), cu_(s)), MUL(MUL(3.0f, b), sq_(s)));
  r = ADD(r, MUL(MUL(2.0f, c), s));
  return ADD(r, 0.7f);
}

__global__ void refgen_srbd_kernel(RefGenArgs g) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= g.batch) return;
  const int N = g.N, S = g.n_max + 1;
  const float* x = g.x + b * 13;
  const float* input = g.input + b * 7;
  const float* foot = g.foot + b * 12;
  float* lo = g.liftoff + b * 12;
  float* ref = g.reference + (size_t)b * S * 17;
  float* par = g.parameter + (size_t)b * S * 16;
  float* frd = g.foot_ref_dot + (size_t)b * S * 12;
  const float q0 = x[3], q1 = x[4], q2 = x[5], q3 = x[6];
  const float yaw = atan2f(MUL(2.0f, ADD(MUL(q0, q3), MUL(q1, q2))), SUB(1.0f, MUL(2.0f, ADD(MUL(q2, q2), MUL(q3, q3)))));
  float sy, cy;
  sincosf(yaw, &sy, &cy);
  const float Ry[9] = {cy, -sy, 0.0f, sy, cy, 0.0f, 0.0f, 0.0f, 1.0f};
  const float lzs = ADD(ADD(ADD(lo[2], lo[5]), lo[8]), lo[11]);
  const float ph = ADD(input[6], DIV(lzs, 4.0f));
  const float p[3] = {x[0], x[1], ph};
  float rlv[3];
#pragma unroll
  for (int r = 0; r < 3; ++r)
    rlv[r] = ADD(ADD(MUL(Ry[3 * r], input[0]), MUL(Ry[3 * r + 1], input[1])), MUL(Ry[3 * r + 2], input[2]));
  float fp[12];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      const float d = ADD(ADD(MUL(g.foot0[3 * i], Ry[3 * r]), MUL(g.foot0[3 * i + 1], Ry[3 * r + 1])),
                          MUL(g.foot0[3 * i + 2], Ry[3 * r + 2]));
      fp[3 * i + r] = ADD(p[r], d);
    }
  const float inc = MUL(g.dt, g.step_freq);
  float cur_t[4];
  int des[4], early[4];
  const float thr = ADD(0.5f, MUL(0.5f, g.duty));
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    cur_t[i] = g.t_timer[b * 4 + i];
    timer_step(g.duty, inc, cur_t[i], des[i]);
    early[i] = (des[i] == 0 && g.contact[b * 4 + i] == 1.0f && cur_t[i] > thr) ? 1 : 0;
  }
  const float nrm = sqrtf(ADD(ADD(MUL(rlv[0], rlv[0]), MUL(rlv[1], rlv[1])), MUL(rlv[2], rlv[2])));
  const float den = ADD(nrm, 1e-6f);
  float isp[3];
#pragma unroll
  for (int r = 0; r < 3; ++r) isp[r] = MUL(DIV(-rlv[r], den), g.clearence);
  for (int t = 0; t <= N; ++t) {
    const float tf = MUL((float)t, g.dt);
    float* rr = ref + t * 17;
    rr[0] = ADD(MUL(tf, rlv[0]), p[0]);
    rr[1] = ADD(MUL(tf, rlv[1]), p[1]);
    rr[2] = ph;
    rr[3] = 1.0f; rr[4] = 0.0f; rr[5] = 0.0f; rr[6] = 0.0f;
#pragma unroll
    for (int r = 0; r < 3; ++r) { rr[7 + r] = rlv[r]; rr[10 + r] = input[3 + r]; }
#pragma unroll
    for (int i = 0; i < 12; ++i) { par[t * 16 + 4 + i] = foot[i]; frd[t * 12 + i] = 0.0f; }
#pragma unroll
    for (int i = 0; i < 4; ++i) { rr[13 + i] = 0.0f; par[t * 16 + i] = 0.0f; }
  }
  float lx[4], ly[4], lz[4], nt[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    lx[i] = lo[3 * i]; ly[i] = lo[3 * i + 1]; lz[i] = lo[3 * i + 2];
    nt[i] = g.t_timer[b * 4 + i];
  }
  const float sqh = sqrtf(DIV(input[6], 9.81f));
  float fh[2][4];
#pragma unroll
  for (int d = 0; d < 2; ++d)
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const float f1 = DIV(MUL(MUL(0.5f, rlv[d]), g.duty), g.step_freq);
      const float f2 = MUL(sqh, SUB(x[7 + d], rlv[d]));
      fh[d][i] = ADD(ADD(f1, f2), fp[3 * i + d]);
    }
  const float omd = SUB(1.0f, g.duty);
  for (int t = 0; t <= N; ++t) {
    const int tp = (t == 0) ? N : t - 1;  // Python index t-1 wraps to the last row
    const float* fprev = par + tp * 16 + 4;
    float px[4], py[4], pz[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) { px[i] = fprev[3 * i]; py[i] = fprev[3 * i + 1]; pz[i] = fprev[3 * i + 2]; }
    int cs[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) timer_step(g.duty, inc, nt[i], cs[i]);
    float prev_c[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) prev_c[i] = par[tp * 16 + i];
#pragma unroll
    for (int i = 0; i < 4; ++i) { ref[t * 17 + 13 + i] = (float)cs[i]; par[t * 16 + i] = (float)cs[i]; }
#pragma unroll
    for (int i = 0; i < 4; ++i)
      if (cs[i] == 0 && prev_c[i] != 0.0f) { lx[i] = px[i]; ly[i] = py[i]; lz[i] = pz[i]; }
    float* ft = par + t * 16 + 4;
    float* fd = frd + t * 12;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const float s = DIV(SUB(nt[i], g.duty), omd);
      const bool stance = (cs[i] > 0) || (early[i] == 1);
      const float sh = ADD(lz[i], g.step_height);
      if (stance) {
        ft[3 * i] = px[i]; ft[3 * i + 1] = py[i]; ft[3 * i + 2] = pz[i];
        fd[3 * i] = 0.0f; fd[3 * i + 1] = 0.0f; fd[3 * i + 2] = 0.0f;
      } else {
        ft[3 * i] = splineXY(lx[i], fh[0][i], isp[0], s);
        ft[3 * i + 1] = splineXY(ly[i], fh[1][i], isp[1], s);
        ft[3 * i + 2] = splineZ(lz[i], lz[i], sh, s);
        fd[3 * i] = splineXY_dot(lx[i], fh[0][i], isp[0], s);
        fd[3 * i + 1] = splineXY_dot(ly[i], fh[1][i], isp[1], s);
        fd[3 * i + 2] = splineZ_dot(lz[i], lz[i], sh, s);
      }
    }
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) { lo[3 * i] = lx[i]; lo[3 * i + 1] = ly[i]; lo[3 * i + 2] = lz[i]; }
}

// Whole-body reference generator (mpx/utils/mpc_utils.py:39-145,
// reference_generator) for a batch, one thread per instance: the SRBD
// generator's schedule, feet and base rows above in the whole-body row layout
// [p, quat, q0, dp, omega, feet (12), contact (4), forces (12)], plus
//  - the base velocity read at x[7 + nj] (the whole-body state),
//  - q_ref = q0 and the contact forces m g / (legs in contact) on stance legs,
//  - with terrain != 0, quat_ref from terrain_orientation (mpc_utils.py:15-37):
//    the frame [front-back vector of the liftoff points, yaw-rotated y axis,
//    their normal], each normalised, to a quaternion by the method that picks
//    the largest of the trace and the diagonal (Shepperd's), normalised;
//    its pitch rotates the commanded velocity (ref_lin_vel = Ryaw Rpitch v).
// parameter [B,N+1,4] is the contact sequence.  With terrain = 0 every float
// step matches the reference's float32 arithmetic.
struct RefGenWbArgs {
  int batch, N, nj, nx, terrain;
  float dt, mass;
  float foot0[12], q0[MPXG_WB_MAX_DOF];
  float duty, step_freq, step_height, clearence;
  const float *t_timer, *x, *foot, *input, *contact;
  float *liftoff, *reference, *parameter;
};

__device__ void terrain_quat(const float* lo, const float* Ry, float* q) {
  float fb[3], lr[3], nr[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) fb[i] = DIV(SUB(SUB(ADD(lo[i], lo[3 + i]), lo[6 + i]), lo[9 + i]), 2.0f);
#pragma unroll
  for (int i = 0; i < 3; ++i) lr[i] = Ry[3 * i + 1];
  nr[0] = SUB(MUL(fb[1], lr[2]), MUL(fb[2], lr[1]));
  nr[1] = SUB(MUL(fb[2], lr[0]), MUL(fb[0], lr[2]));
  nr[2] = SUB(MUL(fb[0], lr[1]), MUL(fb[1], lr[0]));
  float* v[3] = {fb, lr, nr};
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float n = sqrtf(ADD(ADD(MUL(v[k][0], v[k][0]), MUL(v[k][1], v[k][1])), MUL(v[k][2], v[k][2])));
#pragma unroll
    for (int i = 0; i < 3; ++i) v[k][i] = DIV(v[k][i], n);
  }
  // m(r, c): column c is fb, lr, nr
  float m[3][3];
#pragma unroll
  for (int r = 0; r < 3; ++r) { m[r][0] = fb[r]; m[r][1] = lr[r]; m[r][2] = nr[r]; }
  const float tr = ADD(ADD(m[0][0], m[1][1]), m[2][2]);
  const float dec[4] = {m[0][0], m[1][1], m[2][2], tr};
  int c = 0;
#pragma unroll
  for (int i = 1; i < 4; ++i)
    if (dec[i] > dec[c]) c = i;
  float xyzw[4];
  if (c != 3) {
    const int i = c, j = (i + 1) % 3, k = (j + 1) % 3;
    xyzw[i] = ADD(SUB(1.0f, tr), MUL(2.0f, m[i][i]));
    xyzw[j] = ADD(m[j][i], m[i][j]);
    xyzw[k] = ADD(m[k][i], m[i][k]);
    xyzw[3] = SUB(m[k][j], m[j][k]);
  } else {
    xyzw[0] = SUB(m[2][1], m[1][2]);
    xyzw[1] = SUB(m[0][2], m[2][0]);
    xyzw[2] = SUB(m[1][0], m[0][1]);
    xyzw[3] = ADD(1.0f, tr);
  }
  const float n = sqrtf(ADD(ADD(ADD(MUL(xyzw[0], xyzw[0]), MUL(xyzw[1], xyzw[1])), MUL(xyzw[2], xyzw[2])),
                            MUL(xyzw[3], xyzw[3])));
  q[0] = DIV(xyzw[3], n);
  q[1] = DIV(xyzw[0], n);
  q[2] = DIV(xyzw[1], n);
  q[3] = DIV(xyzw[2], n);
}

__global__ void refgen_wb_kernel(RefGenWbArgs g) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= g.batch) return;
  const int N = g.N, nj = g.nj, C = 13 + nj + 28;
  const int cf = 13 + nj, cc = cf + 12, cg = cc + 4;  // feet, contact, forces columns
  const float* x = g.x + (size_t)b * g.nx;
  const float* input = g.input + b * 7;
  const float* foot = g.foot + b * 12;
  float* lo = g.liftoff + b * 12;
  float* ref = g.reference + (size_t)b * (N + 1) * C;
  float* par = g.parameter + (size_t)b * (N + 1) * 4;
  const float q0 = x[3], q1 = x[4], q2 = x[5], q3 = x[6];
  const float yaw = atan2f(MUL(2.0f, ADD(MUL(q0, q3), MUL(q1, q2))), SUB(1.0f, MUL(2.0f, ADD(MUL(q2, q2), MUL(q3, q3)))));
  float sy, cy;
  sincosf(yaw, &sy, &cy);
  const float Ry[9] = {cy, -sy, 0.0f, sy, cy, 0.0f, 0.0f, 0.0f, 1.0f};
  const float lzs = ADD(ADD(ADD(lo[2], lo[5]), lo[8]), lo[11]);
  const float ph = ADD(input[6], DIV(lzs, 4.0f));
  const float p[3] = {x[0], x[1], ph};
  float qr[4] = {1.0f, 0.0f, 0.0f, 0.0f};
  if (g.terrain) terrain_quat(lo, Ry, qr);
  const float pitch = asinf(MUL(2.0f, SUB(MUL(qr[0], qr[2]), MUL(qr[3], qr[1]))));
  float sp, cp;
  sincosf(pitch, &sp, &cp);
  const float Rp[9] = {cp, 0.0f, sp, 0.0f, 1.0f, 0.0f, -sp, 0.0f, cp};
  float M[9];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c)
      M[3 * r + c] = ADD(ADD(MUL(Ry[3 * r], Rp[c]), MUL(Ry[3 * r + 1], Rp[3 + c])), MUL(Ry[3 * r + 2], Rp[6 + c]));
  float rlv[3];
#pragma unroll
  for (int r = 0; r < 3; ++r)
    rlv[r] = ADD(ADD(MUL(M[3 * r], input[0]), MUL(M[3 * r + 1], input[1])), MUL(M[3 * r + 2], input[2]));
  float fp[12];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      const float d = ADD(ADD(MUL(g.foot0[3 * i], Ry[3 * r]), MUL(g.foot0[3 * i + 1], Ry[3 * r + 1])),
                          MUL(g.foot0[3 * i + 2], Ry[3 * r + 2]));
      fp[3 * i + r] = ADD(p[r], d);
    }
  const float inc = MUL(g.dt, g.step_freq);
  float cur_t[4];
  int des[4], early[4];
  const float thr = ADD(0.5f, MUL(0.5f, g.duty));
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    cur_t[i] = g.t_timer[b * 4 + i];
    timer_step(g.duty, inc, cur_t[i], des[i]);
    early[i] = (des[i] == 0 && g.contact[b * 4 + i] == 1.0f && cur_t[i] > thr) ? 1 : 0;
  }
  const float nrm = sqrtf(ADD(ADD(MUL(rlv[0], rlv[0]), MUL(rlv[1], rlv[1])), MUL(rlv[2], rlv[2])));
  const float den = ADD(nrm, 1e-6f);
  float isp[3];
#pragma unroll
  for (int r = 0; r < 3; ++r) isp[r] = MUL(DIV(-rlv[r], den), g.clearence);
  for (int t = 0; t <= N; ++t) {
    const float tf = MUL((float)t, g.dt);
    float* rr = ref + (size_t)t * C;
    rr[0] = ADD(MUL(tf, rlv[0]), p[0]);
    rr[1] = ADD(MUL(tf, rlv[1]), p[1]);
    rr[2] = ph;
#pragma unroll
    for (int i = 0; i < 4; ++i) rr[3 + i] = qr[i];
    for (int j = 0; j < nj; ++j) rr[7 + j] = g.q0[j];
#pragma unroll
    for (int r = 0; r < 3; ++r) { rr[7 + nj + r] = rlv[r]; rr[10 + nj + r] = input[3 + r]; }
#pragma unroll
    for (int i = 0; i < 12; ++i) { rr[cf + i] = foot[i]; rr[cg + i] = 0.0f; }
#pragma unroll
    for (int i = 0; i < 4; ++i) { rr[cc + i] = 0.0f; par[t * 4 + i] = 0.0f; }
  }
  float lx[4], ly[4], lz[4], nt[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    lx[i] = lo[3 * i]; ly[i] = lo[3 * i + 1]; lz[i] = lo[3 * i + 2];
    nt[i] = g.t_timer[b * 4 + i];
  }
  const float sqh = sqrtf(DIV(input[6], 9.81f));
  const float* dp = x + 7 + nj;
  float fh[2][4];
#pragma unroll
  for (int d = 0; d < 2; ++d)
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const float f1 = DIV(MUL(MUL(0.5f, rlv[d]), g.duty), g.step_freq);
      const float f2 = MUL(sqh, SUB(dp[d], rlv[d]));
      fh[d][i] = ADD(ADD(f1, f2), fp[3 * i + d]);
    }
  const float omd = SUB(1.0f, g.duty);
  for (int t = 0; t <= N; ++t) {
    const int tp = (t == 0) ? N : t - 1;  // Python index t-1 wraps to the last row
    const float* fprev = ref + (size_t)tp * C + cf;
    float px[4], py[4], pz[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) { px[i] = fprev[3 * i]; py[i] = fprev[3 * i + 1]; pz[i] = fprev[3 * i + 2]; }
    int cs[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) timer_step(g.duty, inc, nt[i], cs[i]);
    float prev_c[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) prev_c[i] = par[tp * 4 + i];
    float* rr = ref + (size_t)t * C;
#pragma unroll
    for (int i = 0; i < 4; ++i) { rr[cc + i] = (float)cs[i]; par[t * 4 + i] = (float)cs[i]; }
#pragma unroll
    for (int i = 0; i < 4; ++i)
      if (cs[i] == 0 && prev_c[i] != 0.0f) { lx[i] = px[i]; ly[i] = py[i]; lz[i] = pz[i]; }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const float s = DIV(SUB(nt[i], g.duty), omd);
      const bool stance = (cs[i] > 0) || (early[i] == 1);
      const float sh = ADD(lz[i], g.step_height);
      float* ft = rr + cf + 3 * i;
      if (stance) {
        ft[0] = px[i]; ft[1] = py[i]; ft[2] = pz[i];
      } else {
        ft[0] = splineXY(lx[i], fh[0][i], isp[0], s);
        ft[1] = splineXY(ly[i], fh[1][i], isp[1], s);
        ft[2] = splineZ(lz[i], lz[i], sh, s);
      }
    }
    const float csum = ADD(ADD(ADD((float)cs[0], (float)cs[1]), (float)cs[2]), (float)cs[3]);
    const float dn = ADD(csum, 1e-5f);
#pragma unroll
    for (int i = 0; i < 4; ++i) rr[cg + 3 * i + 2] = DIV(MUL(MUL((float)cs[i], g.mass), 9.81f), dn);
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) { lo[3 * i] = lx[i]; lo[3 * i + 1] = ly[i]; lo[3 * i + 2] = lz[i]; }
}
#undef ADD
#undef SUB
#undef MUL
#undef DIV

// ------------------------------------------------------------ gait tables
// (see mpxg_gait_tables in include/mpxg.h)
__device__ __forceinline__ unsigned int hash_u32(unsigned int x) {
  // integer finaliser (xor-shift-multiply), a bijection of 32-bit words
  x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
  return x;
}
__device__ __forceinline__ float hash_normal(unsigned int seed, unsigned int row, unsigned int i) {
  const unsigned int a = hash_u32(seed * 0x9e3779b9U ^ hash_u32(row * 64u + i));
  const unsigned int b = hash_u32(a ^ 0x68bc21ebU);
  const float u1 = ((a >> 8) + 1.0f) * (1.0f / 16777217.0f);  // (0, 1]
  const float u2 = (b >> 8) * (1.0f / 16777216.0f);
  return sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);         // Box-Muller
}

// One warp per batch entry, a lane per stage.  A lane reaches its stage's
// gait timers by replaying the timer steps from the entry's timers, so every
// stage sees the same float sequence as a sequential sweep.
__global__ void gait_tables_kernel(mpxg_gait_args g, int nx, int nu, int legs, int ref_cols, int par_cols,
                                   int contact_col) {
  const int bi = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (bi >= g.batch) return;
  const int b = g.slot ? g.slot[bi] : bi;
  const int N = g.horizon ? g.horizon[b] : g.n_max;
  if (N < 1 || N > g.n_max) return;
  const size_t xo = (size_t)b * (g.n_max + 1) * nx;
  float* x0 = g.x0 + (size_t)b * nx;
  // state of this tick: mode 1 takes the shifted warm start plus drift
  float px0, py0, x0l = 0.0f;
  if (g.mode == 1) {
    const bool dr = g.drift_std > 0.0f;
    px0 = g.X[xo + 0] + (dr ? g.drift_std * hash_normal(g.seed, (unsigned)b, 0u) : 0.0f);
    py0 = g.X[xo + 1] + (dr ? g.drift_std * hash_normal(g.seed, (unsigned)b, 1u) : 0.0f);
    if (lane < nx) x0l = g.X[xo + lane] + (dr ? g.drift_std * hash_normal(g.seed, (unsigned)b, (unsigned)lane) : 0.0f);
  } else {
    px0 = x0[0];
    py0 = x0[1];
    if (lane < nx) x0l = x0[lane];
  }
  __syncwarp();
  if (g.mode == 1 && lane < nx) x0[lane] = x0l;
  const float inc = __fmul_rn(g.dt, g.step_freq);
  float lt0[4];
  for (int i = 0; i < legs; ++i) {
    lt0[i] = g.leg_time[b * legs + i];
    if (g.mode != 0) { int c; timer_step(g.duty_factor, inc, lt0[i], c); }
  }
  __syncwarp();
  if (g.mode != 0 && lane < legs) g.leg_time[b * legs + lane] = lt0[lane < legs ? lane : 0];
  const float v = g.v_ref[b];
  float* ref = g.reference + (size_t)b * (g.n_max + 1) * ref_cols;
  float* par = g.parameter + (size_t)b * (g.n_max + 1) * par_cols;
  const int per = nu / legs;
  // timers at stage `lane` (t = lane + 1 steps from lt0); later stages advance by 32
  float lt[4];
  int cs[4];
  for (int i = 0; i < legs; ++i) {
    lt[i] = lt0[i];
    for (int k = 0; k <= lane; ++k) timer_step(g.duty_factor, inc, lt[i], cs[i]);
  }
  for (int t = lane; t <= N; t += 32) {
    if (t != lane)
      for (int i = 0; i < legs; ++i)
        for (int k = 0; k < 32; ++k) timer_step(g.duty_factor, inc, lt[i], cs[i]);
    float* rr = ref + (size_t)t * ref_cols;
    float* pp = par + (size_t)t * par_cols;
    for (int k = 0; k < ref_cols; ++k) rr[k] = 0.0f;
    const float px = px0 + __fmul_rn(__fmul_rn((float)t, g.dt), v);
    rr[0] = px; rr[1] = py0; rr[2] = g.height;
    if (nx == 13) { rr[3] = 1.0f; rr[7] = v; } else { rr[6] = v; }
    int ns = 0;
    for (int i = 0; i < legs; ++i) {
      ns += cs[i];
      rr[contact_col + i] = (float)cs[i];
      pp[i] = (float)cs[i];
      pp[legs + 3 * i] = px + g.offsets[3 * i];
      pp[legs + 3 * i + 1] = py0 + g.offsets[3 * i + 1];
      pp[legs + 3 * i + 2] = g.height + g.offsets[3 * i + 2];
    }
    if (g.mode == 0) {  // cold start of the warm start
      for (int i = 0; i < nx; ++i) { g.X[xo + (size_t)t * nx + i] = x0[i]; g.V[xo + (size_t)t * nx + i] = 0.0f; }
      if (t < N) {
        float* u = g.U + ((size_t)b * g.n_max + t) * nu;
        const float fz = g.weight / (float)(ns > 0 ? ns : 1);
        for (int a = 0; a < nu; ++a) u[a] = 0.0f;
        for (int i = 0; i < legs; ++i) u[per * i + 2] = cs[i] ? fz : 0.0f;
      }
    }
  }
}

// ------------------------------------------------------------ queue order
// Counting sort of the batch entries by horizon, longest first, into order[]
// (one block).  Entries with an invalid horizon go last.  Serving the
// persistent grid's queue longest-first shortens the tail of a batch whose
// horizons differ (list scheduling, longest processing time first).
//
// n_long (optional) receives the number of entries with a horizon of at least
// split_h: the queue prefix the time-parallel team kernel takes.
//
// A second batch (batch2 entries, slot2 / horizon2) may be ordered together
// with the first: its entry i is queue code batch + i (the mixed-model
// launch).
__global__ void __launch_bounds__(1024) order_by_horizon_kernel(int batch, int n_max, const int* __restrict__ slot,
                                                                const int* __restrict__ horizon, int* __restrict__ order,
                                                                int split_h = 0, int* __restrict__ n_long = nullptr,
                                                                int batch2 = 0, const int* __restrict__ slot2 = nullptr,
                                                                const int* __restrict__ horizon2 = nullptr) {
  extern __shared__ int bins[];       // n_max + 1 bins: bin j holds horizon n_max - j; bin n_max: invalid
  __shared__ int warp_tot[32];
  const int nb = n_max + 1;
  const int total = batch + batch2;
  auto hor = [&](int i) {
    return i < batch ? horizon[slot ? slot[i] : i] : horizon2[slot2 ? slot2[i - batch] : i - batch];
  };
  for (int j = threadIdx.x; j < nb; j += blockDim.x) bins[j] = 0;
  __syncthreads();
  for (int i = threadIdx.x; i < total; i += blockDim.x) {
    const int h = hor(i);
    atomicAdd(&bins[(h >= 1 && h <= n_max) ? n_max - h : n_max], 1);
  }
  __syncthreads();
  // exclusive scan of bins: each thread scans a contiguous chunk
  const int chunk = (nb + blockDim.x - 1) / blockDim.x;
  const int lo = threadIdx.x * chunk, hi = min(lo + chunk, nb);
  int local = 0;
  for (int j = lo; j < hi; ++j) local += bins[j];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int incl = local;
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) warp_tot[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    int t = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += v;
    }
    warp_tot[lane] = t;  // inclusive over warps
  }
  __syncthreads();
  int run = (wid > 0 ? warp_tot[wid - 1] : 0) + incl - local;
  for (int j = lo; j < hi; ++j) { const int c = bins[j]; bins[j] = run; run += c; }
  __syncthreads();
  if (n_long && threadIdx.x == 0)  // bins now hold start offsets; horizon h sits in bin n_max - h
    *n_long = (split_h < 1) ? total : (split_h > n_max ? 0 : bins[n_max - split_h + 1]);
  __syncthreads();
  for (int i = threadIdx.x; i < total; i += blockDim.x) {
    const int h = hor(i);
    order[atomicAdd(&bins[(h >= 1 && h <= n_max) ? n_max - h : n_max], 1)] = i;
  }
}

}  // namespace mpxg
