// Time-parallel LQR (mpxg_lqr_solve method 1): the backward value-function
// recursion as an associative scan over the horizon, after Sarkka and
// Garcia-Fernandez, "Temporal parallelization of dynamic programming and
// linear quadratic control", IEEE TAC 2023.
//
// Same problem as the sequential Riccati kernel (lqr_kernels.cuh).  After the
// cross term is eliminated (u = v - R^-1 (M'x + r)), stage t is the element
//   e_t = (A_t, b_t, C_t, eta_t, J_t) = (A - B R^-1 M', c - B R^-1 r,
//                                        B R^-1 B', M R^-1 r - q, Q - M R^-1 M')
// of the semigroup whose product e_i (x) e_j (i before j) is
//   Z = I + C_i J_j
//   A_ij = A_j Z^-1 A_i            b_ij = A_j Z^-1 (b_i + C_i eta_j) + b_j
//   C_ij = A_j Z^-1 C_i A_j' + C_j
//   eta_ij = (Z^-1 A_i)' (eta_j - J_j b_i) + eta_i
//   J_ij = (Z^-1 A_i)' J_j A_i + J_i,
// and the value function V_t(x) = 1/2 x'J x - eta'x of stage t is the (J, eta)
// part of e_t (x) e_{t+1} (x) ... (x) e_N, e_N = (0, 0, 0, -q_N, Q_N).
//
// GB300 mapping: one block of 8 warps per problem.  The horizon is split into
// 8 chunks; warp c owns chunk c.
//   1. Each warp folds its chunk into one element, prepending one stage at a
//      time.  A single stage has C = B R^-1 B' of rank m, so the prepend
//      needs only the m x m inverse (R + B'J B)^-1 (push-through identity);
//      ~3n^3 + 5n^2 m multiply-adds per stage.
//   2. Warp 0 runs the scan across the chunk elements backward from the
//      terminal value function: the value at the start of chunk c is
//      E_c (x) V (pivoted Gauss-Jordan solve with Z = I + C_c J_V).
//   3. With its boundary value function known, each warp runs the plain
//      Riccati recursion over its chunk (gains K, k and value functions).
//   4. Warp 0 rolls the closed loop forward (X, U, costates).
// Matrices live in shared memory column-major; a lane per output column keeps
// its column of one operand in registers while the other operand is read as
// broadcast float4.
#pragma once
#include <cuda_runtime.h>

#include "../../include/mpxg.h"

namespace mpxg {
namespace lqscan {

constexpr int kWarps = 8;

// out(r, c) = alpha * sum_l X(r, l) Y(l, c) [+ Add(r, c)] for r < ROWS, c < COLS.
// X(r,l) = TX ? X[r*ldx + l] : X[l*ldx + r];  Y(l,c) = TY ? Y[l*ldy + c] : Y[c*ldy + l];
// Add(r,c) = TA ? Add[r*lda + c] : Add[c*lda + r].  One lane per output column:
// the lane's column of Y is held in registers and X is read as broadcast
// float4 (leading dimensions and buffer offsets are multiples of 4).  `out`
// may alias Y (not transposed) or Add (not transposed), never X.
template <int ROWS, int INNER, int COLS, bool TX, bool TY, bool TA>
__device__ __forceinline__ void mm(float* out, int ldo, const float* X, int ldx, const float* Y, int ldy,
                                   float alpha, const float* Add, int lda) {
  const int lane = threadIdx.x & 31;
  for (int c = lane; c < COLS; c += 32) {
    float y[INNER];
    if (TY) {
#pragma unroll
      for (int l = 0; l < INNER; ++l) y[l] = Y[l * ldy + c];
    } else {
#pragma unroll
      for (int l4 = 0; l4 < INNER / 4; ++l4) {
        const float4 v = *reinterpret_cast<const float4*>(Y + c * ldy + 4 * l4);
        y[4 * l4] = v.x; y[4 * l4 + 1] = v.y; y[4 * l4 + 2] = v.z; y[4 * l4 + 3] = v.w;
      }
#pragma unroll
      for (int l = INNER / 4 * 4; l < INNER; ++l) y[l] = Y[c * ldy + l];
    }
    float acc[ROWS];
    if (!TX) {
#pragma unroll
      for (int r = 0; r < ROWS; ++r) acc[r] = 0.0f;
#pragma unroll
      for (int l = 0; l < INNER; ++l) {
        const float* xc = X + l * ldx;
#pragma unroll
        for (int r4 = 0; r4 < ROWS / 4; ++r4) {
          const float4 x = *reinterpret_cast<const float4*>(xc + 4 * r4);
          acc[4 * r4] += x.x * y[l]; acc[4 * r4 + 1] += x.y * y[l];
          acc[4 * r4 + 2] += x.z * y[l]; acc[4 * r4 + 3] += x.w * y[l];
        }
#pragma unroll
        for (int r = ROWS / 4 * 4; r < ROWS; ++r) acc[r] += xc[r] * y[l];
      }
    } else {
#pragma unroll
      for (int r = 0; r < ROWS; ++r) {
        const float* xr = X + r * ldx;
        float a = 0.0f;
#pragma unroll
        for (int l4 = 0; l4 < INNER / 4; ++l4) {
          const float4 x = *reinterpret_cast<const float4*>(xr + 4 * l4);
          a += x.x * y[4 * l4] + x.y * y[4 * l4 + 1] + x.z * y[4 * l4 + 2] + x.w * y[4 * l4 + 3];
        }
#pragma unroll
        for (int l = INNER / 4 * 4; l < INNER; ++l) a += xr[l] * y[l];
        acc[r] = a;
      }
    }
#pragma unroll
    for (int r = 0; r < ROWS; ++r) {
      float v = alpha * acc[r];
      if (Add) v += TA ? Add[r * lda + c] : Add[c * lda + r];
      out[c * ldo + r] = v;
    }
  }
  __syncwarp();
}

// out[r] = alpha * sum_l X(r, l) v[l] + add[r] (add may be null; out may alias add).
template <int ROWS, int INNER, bool TX>
__device__ __forceinline__ void mv(float* out, const float* X, int ldx, const float* v, float alpha, const float* add) {
  const int lane = threadIdx.x & 31;
  for (int r = lane; r < ROWS; r += 32) {
    float acc = 0.0f;
    if (TX) {
      const float* xr = X + r * ldx;
#pragma unroll
      for (int l4 = 0; l4 < INNER / 4; ++l4) {
        const float4 x = *reinterpret_cast<const float4*>(xr + 4 * l4);
        acc += x.x * v[4 * l4] + x.y * v[4 * l4 + 1] + x.z * v[4 * l4 + 2] + x.w * v[4 * l4 + 3];
      }
#pragma unroll
      for (int l = INNER / 4 * 4; l < INNER; ++l) acc += xr[l] * v[l];
    } else {
      float a4[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
      for (int l = 0; l < INNER; ++l) a4[l & 3] += X[l * ldx + r] * v[l];
      acc = (a4[0] + a4[1]) + (a4[2] + a4[3]);
    }
    out[r] = alpha * acc + (add ? add[r] : 0.0f);
  }
  __syncwarp();
}

// Inverse of a symmetric positive definite M x M matrix (2M <= 32):
// Gauss-Jordan on [S | I] with one column per lane held in registers.
template <int M>
__device__ __forceinline__ void spd_inverse(const float* S, int lds, float* out, int ldo) {
  static_assert(2 * M <= 32, "spd_inverse: 2M columns must fit one warp");
  const int lane = threadIdx.x & 31;
  float col[M];
#pragma unroll
  for (int r = 0; r < M; ++r) col[r] = lane < M ? S[lane * lds + r] : (lane - M == r ? 1.0f : 0.0f);
#pragma unroll
  for (int p = 0; p < M; ++p) {
    float pc[M];
#pragma unroll
    for (int r = 0; r < M; ++r) pc[r] = __shfl_sync(0xffffffffu, col[r], p);
    float d = pc[p];
    if (!(d > 0.0f)) d = fmaxf(fabsf(d), 1e-30f);
    const float v = col[p] / d;
#pragma unroll
    for (int r = 0; r < M; ++r) col[r] = (r == p) ? v : col[r] - pc[r] * v;
  }
  if (lane >= M && lane < 2 * M) {
#pragma unroll
    for (int r = 0; r < M; ++r) out[(lane - M) * ldo + r] = col[r];
  }
  __syncwarp();
}

// T = Z^-1 Ain for a general N x N Z (Gauss-Jordan with partial pivoting on
// [Z | Ain], two columns per lane in registers, rows never moved: the pivot
// of column p is recorded and the solution row p read from it at the end).
template <int N>
__device__ __forceinline__ void pivoted_solve(const float* Z, int ldz, const float* Ain, int lda, float* T, int ldt) {
  static_assert(2 * N <= 64, "pivoted_solve: 2N columns must fit two per lane");
  const int lane = threadIdx.x & 31;
  float c0[N], c1[N];  // columns lane and lane + 32 of [Z | Ain]
  const int j0 = lane, j1 = lane + 32;
#pragma unroll
  for (int r = 0; r < N; ++r) {
    c0[r] = j0 < N ? Z[j0 * ldz + r] : (j0 < 2 * N ? Ain[(j0 - N) * lda + r] : 0.0f);
    c1[r] = j1 < N ? Z[j1 * ldz + r] : (j1 < 2 * N ? Ain[(j1 - N) * lda + r] : 0.0f);
  }
  unsigned long long used = 0ull;
  int piv_of[N];
#pragma unroll
  for (int p = 0; p < N; ++p) {
    float pc[N];
    const int owner = p & 31;
#pragma unroll
    for (int r = 0; r < N; ++r) {
      const float a = __shfl_sync(0xffffffffu, c0[r], owner);
      const float b = __shfl_sync(0xffffffffu, c1[r], owner);
      pc[r] = p < 32 ? a : b;
    }
    int piv = 0;
    float best = -1.0f;
#pragma unroll
    for (int r = 0; r < N; ++r) {
      const float m = fabsf(pc[r]);
      if (!((used >> r) & 1ull) && m > best) { best = m; piv = r; }
    }
    used |= 1ull << piv;
    piv_of[p] = piv;
    float d = 0.0f, v0 = 0.0f, v1 = 0.0f;
#pragma unroll
    for (int r = 0; r < N; ++r)
      if (r == piv) { d = pc[r]; v0 = c0[r]; v1 = c1[r]; }
    if (fabsf(d) < 1e-30f) d = d < 0.0f ? -1e-30f : 1e-30f;
    v0 /= d;
    v1 /= d;
#pragma unroll
    for (int r = 0; r < N; ++r) {
      c0[r] = (r == piv) ? v0 : c0[r] - pc[r] * v0;
      c1[r] = (r == piv) ? v1 : c1[r] - pc[r] * v1;
    }
  }
  // solution row p sits in row piv_of[p] of the right half
#pragma unroll
  for (int p = 0; p < N; ++p) {
    const int pr = piv_of[p];
    float v0 = 0.0f, v1 = 0.0f;
#pragma unroll
    for (int r = 0; r < N; ++r)
      if (r == pr) { v0 = c0[r]; v1 = c1[r]; }
    if (j0 >= N && j0 < 2 * N) T[(j0 - N) * ldt + p] = v0;
    if (j1 >= N && j1 < 2 * N) T[(j1 - N) * ldt + p] = v1;
  }
  __syncwarp();
}

// In-place symmetrisation of an N x N column-major matrix (lane c owns the
// pairs (r, c), r < c).
template <int N>
__device__ __forceinline__ void symmetrize(float* S, int ld) {
  const int lane = threadIdx.x & 31;
  for (int c = lane; c < N; c += 32) {
    float lo[N], hi[N];
#pragma unroll
    for (int r = 0; r < N; ++r) {
      lo[r] = S[c * ld + r];
      hi[r] = S[r * ld + c];
    }
#pragma unroll
    for (int r = 0; r < N; ++r)
      if (r < c) {
        const float v = 0.5f * (lo[r] + hi[r]);
        S[c * ld + r] = v;
        S[r * ld + c] = v;
      }
  }
  __syncwarp();
}

// Copy a row-major [ROWS x COLS] global block into column-major shared
// memory: every lane issues all its loads before its first store, so the
// block's loads are in flight together.
template <int ROWS, int COLS>
__device__ __forceinline__ void load_cm(float* dst, int ld, const float* __restrict__ src) {
  constexpr int E = ROWS * COLS, PER = (E + 31) / 32;
  const int lane = threadIdx.x & 31;
  float v[PER];
#pragma unroll
  for (int i = 0; i < PER; ++i) {
    const int e = lane + 32 * i;
    v[i] = (e < E) ? __ldg(src + e) : 0.0f;
  }
#pragma unroll
  for (int i = 0; i < PER; ++i) {
    const int e = lane + 32 * i;
    if (e < E) dst[(e % COLS) * ld + e / COLS] = v[i];
  }
}
template <int N>
__device__ __forceinline__ void load_vec(float* dst, const float* __restrict__ src, float scale) {
  const int lane = threadIdx.x & 31;
  if (lane < N) dst[lane] = scale * __ldg(src + lane);
  if (N > 32 && lane + 32 < N) dst[lane + 32] = scale * __ldg(src + lane + 32);
}

// Leading dimension: a multiple of 4 (float4 access) whose quarter is odd, so
// that eight lanes reading 16 bytes at stride ld hit eight distinct bank groups.
constexpr int lead_dim(int n) { return ((n + 3) / 4 % 2 == 1) ? (n + 3) / 4 * 4 : (n + 3) / 4 * 4 + 4; }

template <int NX, int NU>
struct Layout {
  static constexpr int LD = lead_dim(NX);   // rows of n-row matrices
  static constexpr int LM = lead_dim(NU);   // rows of m-row matrices
  static constexpr int NN = NX * LD, NM = NU * LD, MN = NX * LM, MM = NU * LM;
  // aggregate element
  static constexpr int EA = 0, EA2 = EA + NN, EC = EA2 + NN, EJ = EC + NN, EB = EJ + NN, EE = EB + LD;
  // stage data
  static constexpr int SA = EE + LD, SB = SA + NN, SC = SB + NM, SQ = SC + LD, SQV = SQ + NN, SR = SQV + LD,
                       SM = SR + MM, SRV = SM + NM;
  // temporaries
  static constexpr int TJB = SRV + LM, TS = TJB + NM, TG = TS + MM, TJF = TG + MM, TBJ = TJF + NN, TK = TBJ + (MN > NM ? MN : NM),
                       TY = TK + MN, TT = TY + LD, TV1 = TT + LD, TV2 = TV1 + LM;
  static constexpr int FLOATS = (TV2 + LM + 3) / 4 * 4;
};

template <int NX, int NU>
constexpr size_t scan_smem_bytes() { return (size_t)kWarps * Layout<NX, NU>::FLOATS * sizeof(float); }

template <int NX, int NU>
struct Stage {
  const float *A, *B, *c, *Q, *R, *M, *q, *r;
};

template <int NX, int NU>
__device__ __forceinline__ Stage<NX, NU> stage_ptrs(const mpxg_lq_io& io, int b, int t) {
  const int N = io.N;
  Stage<NX, NU> s;
  s.A = io.A + ((size_t)b * N + t) * NX * NX;
  s.B = io.Bm + ((size_t)b * N + t) * NX * NU;
  s.c = io.c + ((size_t)b * N + t) * NX;
  s.Q = io.Q + ((size_t)b * (N + 1) + t) * NX * NX;
  s.R = io.R + ((size_t)b * N + t) * NU * NU;
  s.M = io.M + ((size_t)b * N + t) * NX * NU;
  s.q = io.q + ((size_t)b * (N + 1) + t) * NX;
  s.r = io.r + ((size_t)b * N + t) * NU;
  return s;
}

// Load stage t's data into the warp's stage buffers.
template <int NX, int NU>
__device__ __forceinline__ void load_stage(float* w, const Stage<NX, NU>& s) {
  typedef Layout<NX, NU> L;
  load_cm<NX, NX>(w + L::SA, L::LD, s.A);
  load_cm<NX, NU>(w + L::SB, L::LD, s.B);
  load_vec<NX>(w + L::SC, s.c, 1.0f);
  load_cm<NX, NX>(w + L::SQ, L::LD, s.Q);
  load_vec<NX>(w + L::SQV, s.q, 1.0f);
  load_cm<NU, NU>(w + L::SR, L::LM, s.R);
  load_cm<NX, NU>(w + L::SM, L::LD, s.M);
  load_vec<NU>(w + L::SRV, s.r, 1.0f);
  __syncwarp();
}

// Turn the loaded stage into its element: SA <- F = A - B R^-1 M',
// SC <- c - B R^-1 r, SQ <- J = Q - M R^-1 M', SQV <- eta = M R^-1 r - q.
template <int NX, int NU>
__device__ __forceinline__ void stage_element(float* w) {
  typedef Layout<NX, NU> L;
  spd_inverse<NU>(w + L::SR, L::LM, w + L::TG, L::LM);                                        // R^-1
  mm<NU, NU, NX, false, true, false>(w + L::TBJ, L::LM, w + L::TG, L::LM, w + L::SM, L::LD,    // X1 = R^-1 M'
                                     1.0f, nullptr, 0);
  mv<NU, NU, false>(w + L::TV1, w + L::TG, L::LM, w + L::SRV, 1.0f, nullptr);                  // x2 = R^-1 r
  mm<NX, NU, NX, false, false, false>(w + L::SA, L::LD, w + L::SB, L::LD, w + L::TBJ, L::LM,   // F
                                      -1.0f, w + L::SA, L::LD);
  mm<NX, NU, NX, false, false, false>(w + L::SQ, L::LD, w + L::SM, L::LD, w + L::TBJ, L::LM,   // J
                                      -1.0f, w + L::SQ, L::LD);
  mv<NX, NU, false>(w + L::SC, w + L::SB, L::LD, w + L::TV1, -1.0f, w + L::SC);                // c - B x2
  mv<NX, NU, false>(w + L::TY, w + L::SM, L::LD, w + L::TV1, 1.0f, nullptr);                   // M x2
  const int lane = threadIdx.x & 31;
  if (lane < NX) w[L::SQV + lane] = w[L::TY + lane] - w[L::SQV + lane];
  __syncwarp();
  symmetrize<NX>(w + L::SQ, L::LD);
}

// Aggregate <- (stage element) (x) aggregate.  The stage's C = B R^-1 B' has
// rank m, so Z^-1 = I - B G B' J with G = (R + B'J B)^-1 (m x m).
template <int NX, int NU>
__device__ __forceinline__ void prepend(float* w, float*& EA, float*& EA2) {
  typedef Layout<NX, NU> L;
  constexpr int LD = L::LD, LM = L::LM;
  float *EC = w + L::EC, *EJ = w + L::EJ, *Eb = w + L::EB, *Ee = w + L::EE;
  float *F = w + L::SA, *B = w + L::SB, *ct = w + L::SC, *Ji = w + L::SQ, *ei = w + L::SQV, *R = w + L::SR;
  float *JB = w + L::TJB, *S = w + L::TS, *G = w + L::TG, *JF = w + L::TJF, *BJF = w + L::TBJ;
  float *y = w + L::TY, *t2 = w + L::TT, *v1 = w + L::TV1, *v2 = w + L::TV2;
  mm<NX, NX, NU, false, false, false>(JB, LD, EJ, LD, B, LD, 1.0f, nullptr, 0);          // J B
  mm<NU, NX, NU, true, false, false>(S, LM, B, LD, JB, LD, 1.0f, R, LM);                 // R + B'J B
  spd_inverse<NU>(S, LM, G, LM);                                                         // G
  mm<NX, NX, NX, false, false, false>(JF, LD, EJ, LD, F, LD, 1.0f, nullptr, 0);          // J F
  mm<NU, NX, NX, true, false, false>(BJF, LM, JB, LD, F, LD, 1.0f, nullptr, 0);          // B'J F
  mm<NU, NU, NX, false, false, false>(BJF, LM, G, LM, BJF, LM, 1.0f, nullptr, 0);        // W = G B'J F
  mv<NX, NX, false>(y, EJ, LD, ct, -1.0f, Ee);                                           // y = eta_j - J c
  mm<NX, NU, NX, false, false, false>(F, LD, B, LD, BJF, LM, -1.0f, F, LD);              // T1 = F - B W
  mv<NU, NX, true>(v1, B, LD, y, 1.0f, nullptr);                                         // B'y
  mv<NU, NU, false>(v2, G, LM, v1, 1.0f, nullptr);                                       // G B'y
  mv<NX, NU, false>(t2, B, LD, v2, 1.0f, ct);                                            // t2 = c + B G B'y
  mm<NX, NX, NX, true, false, false>(EJ, LD, F, LD, JF, LD, 1.0f, Ji, LD);               // J_new = T1'JF + J_i
  mv<NX, NX, true>(Ee, F, LD, y, 1.0f, ei);                                              // eta_new = T1'y + eta_i
  mm<NX, NX, NX, false, false, false>(EA2, LD, EA, LD, F, LD, 1.0f, nullptr, 0);         // A_new = A_j T1
  mv<NX, NX, false>(Eb, EA, LD, t2, 1.0f, Eb);                                           // b_new = A_j t2 + b_j
  mm<NX, NX, NU, false, false, false>(JB, LD, EA, LD, B, LD, 1.0f, nullptr, 0);          // AB = A_j B
  mm<NX, NU, NU, false, false, false>(BJF, LD, JB, LD, G, LM, 1.0f, nullptr, 0);         // V1 = AB G
  mm<NX, NU, NX, false, true, false>(EC, LD, BJF, LD, JB, LD, 1.0f, EC, LD);             // C_new = V1 AB' + C_j
  float* t = EA; EA = EA2; EA2 = t;
  symmetrize<NX>(EJ, LD);
  symmetrize<NX>(EC, LD);
}

// One Riccati step: value function (P in EJ, p = -eta in EE) of stage t+1 to
// stage t; writes K_t, k_t and the augmented value function of stage t.
template <int NX, int NU>
__device__ __forceinline__ void riccati_step(float* w, const mpxg_lq_io& io, int b, int t, float* Pt) {
  typedef Layout<NX, NU> L;
  constexpr int LD = L::LD, LM = L::LM, NP = NX + 1;
  float *P = w + L::EJ, *pe = w + L::EE;  // pe holds -p
  float *A = w + L::SA, *B = w + L::SB, *c = w + L::SC, *Q = w + L::SQ, *q = w + L::SQV, *R = w + L::SR;
  float *M = w + L::SM, *r = w + L::SRV;
  float *PA = w + L::TJF, *PB = w + L::TJB, *Quu = w + L::TS, *G = w + L::TG, *Qux = w + L::TBJ, *K = w + L::TK;
  float *wv = w + L::TY, *qu = w + L::TV1, *kk = w + L::TV2, *pn = w + L::TT;
  const int lane = threadIdx.x & 31;
  mm<NX, NX, NX, false, false, false>(PA, LD, P, LD, A, LD, 1.0f, nullptr, 0);           // P A
  mm<NX, NX, NU, false, false, false>(PB, LD, P, LD, B, LD, 1.0f, nullptr, 0);           // P B
  mm<NU, NX, NU, true, false, false>(Quu, LM, B, LD, PB, LD, 1.0f, R, LM);               // R + B'P B
  mm<NU, NX, NX, true, false, true>(Qux, LM, B, LD, PA, LD, 1.0f, M, LD);                // M' + B'P A
  mv<NX, NX, false>(wv, P, LD, c, 1.0f, nullptr);                                        // P c
  if (lane < NX) wv[lane] -= pe[lane];                                                   // + p
  __syncwarp();
  mv<NU, NX, true>(qu, B, LD, wv, 1.0f, r);                                              // r + B'(P c + p)
  spd_inverse<NU>(Quu, LM, G, LM);
  mm<NU, NU, NX, false, false, false>(K, LM, G, LM, Qux, LM, -1.0f, nullptr, 0);         // K = -G Qux
  mv<NU, NU, false>(kk, G, LM, qu, -1.0f, nullptr);                                      // k = -G qu
  float* Ko = io.K + ((size_t)b * io.N + t) * NU * NX;
  float* ko = io.k + ((size_t)b * io.N + t) * NU;
  for (int e = lane; e < NU * NX; e += 32) {
    const int a = e / NX, i = e - a * NX;
    Ko[e] = K[i * LM + a];
  }
  if (lane < NU) ko[lane] = kk[lane];
  // p_new = q + A'(P c + p) + Qux' k
  mv<NX, NX, true>(pn, A, LD, wv, 1.0f, q);
  mv<NX, NU, true>(pn, Qux, LM, kk, 1.0f, pn);
  // P_new = Q + A'P A + Qux' K
  mm<NX, NX, NX, true, false, false>(P, LD, A, LD, PA, LD, 1.0f, Q, LD);
  mm<NX, NU, NX, true, false, false>(P, LD, Qux, LM, K, LM, 1.0f, P, LD);
  symmetrize<NX>(P, LD);
  if (lane < NX) pe[lane] = -pn[lane];
  __syncwarp();
  for (int e = lane; e < NP * NP; e += 32) {
    const int j = e / NP, i = e - j * NP;
    Pt[e] = (i < NX && j < NX) ? P[j * LD + i] : (i == NX && j == NX ? 0.0f : pn[i < NX ? i : j]);
  }
  __syncwarp();
}

// One stage's rows for the forward sweep, held by lane i: row i of A_t and
// B_t and c_t[i] (i < n); row i of K_t and k_t[i] (i < m).
template <int NX, int NU>
struct FwdRow {
  float a[NX], bq[NU], kr[NX], c, k;
  __device__ __forceinline__ void load(const mpxg_lq_io& io, int b, int t, int lane) {
    const size_t st = (size_t)b * io.N + t;
    const bool xr = lane < NX, ur = lane < NU;
    const float* A = io.A + st * NX * NX + (size_t)(xr ? lane : 0) * NX;
    const float* Bm = io.Bm + st * NX * NU + (size_t)(xr ? lane : 0) * NU;
    const float* K = io.K + st * NU * NX + (size_t)(ur ? lane : 0) * NX;
#pragma unroll
    for (int k = 0; k < NX; ++k) { a[k] = xr ? __ldg(A + k) : 0.0f; kr[k] = ur ? K[k] : 0.0f; }
#pragma unroll
    for (int q = 0; q < NU; ++q) bq[q] = xr ? __ldg(Bm + q) : 0.0f;
    c = xr ? __ldg(io.c + st * NX + lane) : 0.0f;
    k = ur ? io.k[st * NU + lane] : 0.0f;
  }
};

template <int NX, int NU>
__global__ void __launch_bounds__(kWarps * 32, 1) lqr_scan_kernel(mpxg_lq_io io, float* Pscr) {
  typedef Layout<NX, NU> L;
  constexpr int LD = L::LD, NP = NX + 1;
  extern __shared__ float4 smem4[];
  float* smem = reinterpret_cast<float*>(smem4);
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float* w = smem + (size_t)wid * L::FLOATS;
  const int b = blockIdx.x, N = io.N;
  const int chunk = (N + kWarps - 1) / kWarps;
  const int s0 = wid * chunk, s1 = min(N, s0 + chunk);
  float* Ps = Pscr + (size_t)b * (N + 1) * NP * NP;

  // ---- 1. fold chunk wid (wid >= 1) into one element, starting from the identity
  float* EA = w + L::EA;
  float* EA2 = w + L::EA2;
  if (wid >= 1) {
    for (int e = lane; e < NX * LD; e += 32) {
      const int c = e / LD, r = e - c * LD;
      EA[e] = (r == c) ? 1.0f : 0.0f;
      w[L::EC + e] = 0.0f;
      w[L::EJ + e] = 0.0f;
    }
    if (lane < LD) { w[L::EB + lane] = 0.0f; w[L::EE + lane] = 0.0f; }
    __syncwarp();
    for (int t = s1 - 1; t >= s0; --t) {
      load_stage<NX, NU>(w, stage_ptrs<NX, NU>(io, b, t));
      stage_element<NX, NU>(w);
      prepend<NX, NU>(w, EA, EA2);
    }
  }
  // the aggregate's A may sit in either buffer: publish its offset
  __shared__ int ea_off[kWarps];
  if (lane == 0) ea_off[wid] = (int)(EA - w);
  // terminal value function into the last warp's boundary slot (SQ = J, SQV = eta)
  if (wid == kWarps - 1) {
    load_cm<NX, NX>(w + L::SQ, LD, io.Q + ((size_t)b * (N + 1) + N) * NX * NX);
    load_vec<NX>(w + L::SQV, io.q + ((size_t)b * (N + 1) + N) * NX, -1.0f);
  }
  __syncthreads();

  // ---- 2. scan across the chunks (warp 0): V_start(c) = E_c (x) V_end(c)
  if (wid == 0) {
    for (int c = kWarps - 1; c >= 1; --c) {
      float* wc = smem + (size_t)c * L::FLOATS;
      float* wd = smem + (size_t)(c - 1) * L::FLOATS;  // receives V_end(c-1) = V_start(c)
      const float *Ac = wc + ea_off[c], *Cc = wc + L::EC, *Jc = wc + L::EJ, *bc = wc + L::EB, *ec = wc + L::EE;
      const float *JV = wc + L::SQ, *eV = wc + L::SQV;
      float *Z = w + L::TJF, *T1 = w + L::SA, *JA = w + L::SQ, *y = w + L::TY;
      mm<NX, NX, NX, false, false, false>(Z, LD, Cc, LD, JV, LD, 1.0f, nullptr, 0);       // C_c J_V
      for (int e = lane; e < NX; e += 32) Z[e * LD + e] += 1.0f;                          // + I
      __syncwarp();
      pivoted_solve<NX>(Z, LD, Ac, LD, T1, LD);                                           // T1 = Z^-1 A_c
      mm<NX, NX, NX, false, false, false>(JA, LD, JV, LD, Ac, LD, 1.0f, nullptr, 0);      // J_V A_c
      mv<NX, NX, false>(y, JV, LD, bc, -1.0f, eV);                                        // eta_V - J_V b_c
      mm<NX, NX, NX, true, false, false>(wd + L::SQ, LD, T1, LD, JA, LD, 1.0f, Jc, LD);   // J
      mv<NX, NX, true>(wd + L::SQV, T1, LD, y, 1.0f, ec);                                 // eta
      symmetrize<NX>(wd + L::SQ, LD);
    }
  }
  __syncthreads();

  // ---- 3. Riccati over the own chunk from its boundary value function
  {
    // P <- J_V, EE <- eta_V (= -p)
    for (int e = lane; e < NX * LD; e += 32) w[L::EJ + e] = w[L::SQ + e];
    if (lane < NX) w[L::EE + lane] = w[L::SQV + lane];
    __syncwarp();
    if (wid == kWarps - 1) {  // the terminal value function itself
      float* PN = Ps + (size_t)N * NP * NP;
      for (int e = lane; e < NP * NP; e += 32) {
        const int j = e / NP, i = e - j * NP;
        PN[e] = (i < NX && j < NX) ? w[L::EJ + j * LD + i]
                                   : (i == NX && j == NX ? 0.0f : -w[L::EE + (i < NX ? i : j)]);
      }
    }
    for (int t = s1 - 1; t >= s0; --t) {
      load_stage<NX, NU>(w, stage_ptrs<NX, NU>(io, b, t));
      riccati_step<NX, NU>(w, io, b, t, Ps + (size_t)t * NP * NP);
    }
  }
  __syncthreads();

  // ---- 4. forward pass (warp 0): u = K x + k, x+ = A x + B u + c; the rows of
  // stage t+1 are loaded while stage t is computed
  if (wid == 0) {
    float x = lane < NX ? io.x0[(size_t)b * NX + lane] : 0.0f;
    float* X = io.X + (size_t)b * (N + 1) * NX;
    float* U = io.U + (size_t)b * N * NU;
    FwdRow<NX, NU> cur, nxt;
    cur.load(io, b, 0, lane);
    for (int t = 0; t < N; ++t) {
      if (t + 1 < N) nxt.load(io, b, t + 1, lane);
      float xs[NX];
#pragma unroll
      for (int k = 0; k < NX; ++k) xs[k] = __shfl_sync(0xffffffffu, x, k);
      if (lane < NX) X[t * NX + lane] = x;
      float u = cur.k;
#pragma unroll
      for (int k = 0; k < NX; ++k) u += cur.kr[k] * xs[k];
      if (lane < NU) U[t * NU + lane] = u;
      float xn = cur.c;
#pragma unroll
      for (int k = 0; k < NX; ++k) xn += cur.a[k] * xs[k];
#pragma unroll
      for (int a = 0; a < NU; ++a) xn += cur.bq[a] * __shfl_sync(0xffffffffu, u, a);
      x = xn;
      cur = nxt;
    }
    if (lane < NX) X[N * NX + lane] = x;
  }
  __syncthreads();
  // ---- 5. costates lam_t = P_t x_t + p_t, stage-parallel over the warps
  {
    const float* X = io.X + (size_t)b * (N + 1) * NX;
    float* Lm = io.lam + (size_t)b * (N + 1) * NX;
    for (int t = wid; t <= N; t += kWarps) {
      const float* Pt = Ps + (size_t)t * NP * NP;
      const float xl = lane < NX ? X[t * NX + lane] : 0.0f;
      float xs[NX];
#pragma unroll
      for (int k = 0; k < NX; ++k) xs[k] = __shfl_sync(0xffffffffu, xl, k);
      if (lane < NX) {
        float lam = Pt[NX * NP + lane];
#pragma unroll
        for (int k = 0; k < NX; ++k) lam += Pt[k * NP + lane] * xs[k];
        Lm[t * NX + lane] = lam;
      }
    }
  }
}

}  // namespace lqscan
}  // namespace mpxg
