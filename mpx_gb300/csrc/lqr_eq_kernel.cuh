// Equality-constrained time-varying LQR (mpxg_lqr_eq_solve): the LQ/KKT
// step for large linearised problems (n = 72, m = 30, 12 equality rows per
// stage), in absolute coordinates:
//   x_{t+1} = A x + B u + c,   C x + D u = e,
//   l_t = 1/2 x'Q x + x'M u + 1/2 u'R u + q'x + r'u,  l_N = 1/2 x'Q_N x + q_N'x.
// Stagewise Riccati with the control QP of each stage solved by a Schur
// complement:
//   Q_xx = Q + A'P A, Q_ux = M' + B'P A, Q_uu = R + B'P B,
//   q_x = q + A'(P c + p), q_u = r + B'(P c + p),
//   Z = Q_uu^-1 Q_ux, g = Q_uu^-1 q_u, W = Q_uu^-1 D', S = D W,
//   K_nu = S^-1 (C - D Z), k_nu = -S^-1 (D g + e), K = -(Z + W K_nu), k = -(g + W k_nu),
//   P <- Q_xx + Q_ux'K + C'K_nu,  p <- q_x + Q_ux'k + C'k_nu   (D K = -C).
// GB300 mapping (the CUDA-core kernel, method 1 of mpxg_lqr_eq_solve_method;
// lqr_eq_tc.cuh puts the stage products on the tensor cores): one 256-thread
// block per problem; all stage matrices live in shared memory column-major
// with odd leading dimensions (~152 KB for n = 72); products are 16 x
// 16-thread register-tiled block products; the eliminations with Q_uu and S
// are column-parallel block Gauss-Jordan solves (4 x 4 Cholesky pivots, a
// thread per right-hand side), shared with the tensor-core kernel, as are the
// forward sweep and the costates below.
#pragma once
#include <cuda_runtime.h>

#include "../../include/mpxg.h"

namespace mpxg {
namespace lqeq {

constexpr int kThreads = 256;

// out(r,c) = alpha * sum_l X(r,l) Y(l,c) [+ Add(r,c)]  (column-major; see the
// transposition flags in the scan kernel's mm).  16 x 16 threads, each a
// ceil(ROWS/16) x ceil(COLS/16) tile of strided rows and columns.  `out` may
// alias Add (same element per thread), never X or Y.  Ends with a barrier.
template <int ROWS, int INNER, int COLS, bool TX, bool TY, bool TA>
__device__ __forceinline__ void bmm(float* out, int ldo, const float* X, int ldx, const float* Y, int ldy, float alpha,
                                    const float* Add, int lda) {
  constexpr int TR = (ROWS + 15) / 16, TC = (COLS + 15) / 16;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  float acc[TR][TC];
#pragma unroll
  for (int i = 0; i < TR; ++i)
#pragma unroll
    for (int j = 0; j < TC; ++j) acc[i][j] = 0.0f;
#pragma unroll 2
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
  // out never aliases X or Y (and Add only element by element), so the
  // results are written without a barrier; the one below orders them before
  // their readers
#pragma unroll
  for (int i = 0; i < TR; ++i)
#pragma unroll
    for (int j = 0; j < TC; ++j) {
      const int r = ty + 16 * i, c = tx + 16 * j;
      if (r < ROWS && c < COLS) {
        float v = alpha * acc[i][j];
        if (Add) v += TA ? Add[r * lda + c] : Add[c * lda + r];
        out[c * ldo + r] = v;
      }
    }
  __syncthreads();
}

// out[r] = alpha * sum_l X(r,l) v[l] + add[r]; out may alias add.
template <int ROWS, int INNER, bool TX>
__device__ __forceinline__ void bmv(float* out, const float* X, int ldx, const float* v, float alpha, const float* add) {
  for (int r = threadIdx.x; r < ROWS; r += kThreads) {
    float a = 0.0f;
#pragma unroll 4
    for (int l = 0; l < INNER; ++l) a += (TX ? X[r * ldx + l] : X[l * ldx + r]) * v[l];
    out[r] = alpha * a + (add ? add[r] : 0.0f);
  }
  __syncthreads();
}

// Solve S X = Y for a symmetric positive definite S (R x R) by block
// Gauss-Jordan over the augmented [S | Y] (NCOL columns), one thread per
// column, the column in registers.  Pivots are taken BS at a time (BS a
// multiple of 4): the owners of the block's columns publish them
// (double-buffered panel, one barrier per block), and every later column
// solves the BS x BS pivot block D y = v[block] by Cholesky, then
// v[i] -= panel[i] . y off the block and v[block] = y.  load(j, v) fills
// column j; store(j, v) receives the solution columns j >= R.  panel:
// 2 x 32 x BS floats of shared memory, 16-byte aligned (row i's BS
// pivot-column entries contiguous, read as 16-byte broadcasts).
template <int R, int NCOL, int BS = 4, class Load, class Store>
__device__ __forceinline__ void gj_solve(float* panel, Load load, Store store) {
  static_assert(R <= 32 && NCOL <= kThreads, "pivots within 32 rows, one thread per column");
  static_assert(BS % 4 == 0, "pivot blocks of a multiple of 4");
  const int j = threadIdx.x;
  float v[R];
  if (j < NCOL) load(j, v);
#pragma unroll
  for (int b0 = 0; b0 < R; b0 += BS) {
    const int bs = (R - b0) < BS ? (R - b0) : BS;
    float* pb = panel + ((b0 / BS) & 1) * BS * 32;
    if (j >= b0 && j < b0 + bs) {
#pragma unroll
      for (int i = 0; i < R; ++i) pb[i * BS + (j - b0)] = v[i];
    }
    __syncthreads();
    if (j >= b0 + bs && j < NCOL) {
      // pivot block D(r, k) = pb[(b0 + r) * BS + k]; Cholesky D = L L'
      float Lm[BS][BS], il[BS], y[BS];
#pragma unroll
      for (int r = 0; r < BS; ++r) {
        if (r >= bs) continue;
        float drv[BS];
#pragma unroll
        for (int q4 = 0; q4 < BS / 4; ++q4) {
          const float4 dr = *reinterpret_cast<const float4*>(pb + (b0 + r) * BS + 4 * q4);
          drv[4 * q4] = dr.x; drv[4 * q4 + 1] = dr.y; drv[4 * q4 + 2] = dr.z; drv[4 * q4 + 3] = dr.w;
        }
#pragma unroll
        for (int k = 0; k <= r; ++k) {
          float a = drv[k];
#pragma unroll
          for (int q = 0; q < k; ++q) a -= Lm[r][q] * Lm[k][q];
          if (k == r) {
            if (!(a > 0.0f)) a = fmaxf(fabsf(a), 1e-30f);
            il[r] = rsqrtf(a);
            Lm[r][r] = a * il[r];
          } else {
            Lm[r][k] = a * il[k];
          }
        }
      }
      // y = D^-1 v[block]: L z = v, L' y = z
#pragma unroll
      for (int r = 0; r < BS; ++r) {
        if (r >= bs) continue;
        float a = v[b0 + r];
#pragma unroll
        for (int q = 0; q < r; ++q) a -= Lm[r][q] * y[q];
        y[r] = a * il[r];
      }
#pragma unroll
      for (int r = BS - 1; r >= 0; --r) {
        if (r >= bs) continue;
        float a = y[r];
#pragma unroll
        for (int q = r + 1; q < BS; ++q)
          if (q < bs) a -= Lm[q][r] * y[q];
        y[r] = a * il[r];
      }
#pragma unroll
      for (int i = 0; i < R; ++i) {
        if (i >= b0 && i < b0 + bs) continue;
        float a = v[i];
#pragma unroll
        for (int q4 = 0; q4 < BS / 4; ++q4) {
          const float4 pr = *reinterpret_cast<const float4*>(pb + i * BS + 4 * q4);
          const float prv[4] = {pr.x, pr.y, pr.z, pr.w};
#pragma unroll
          for (int k = 0; k < 4; ++k)
            if (4 * q4 + k < bs) a -= prv[k] * y[4 * q4 + k];
        }
        v[i] = a;
      }
#pragma unroll
      for (int r = 0; r < BS; ++r)
        if (r < bs) v[b0 + r] = y[r];
    }
  }
  if (j >= R && j < NCOL) store(j, v);
  __syncthreads();
}

// Row-major [ROWS x COLS] global block -> column-major shared memory.
template <int ROWS, int COLS>
__device__ __forceinline__ void load_cm(float* dst, int ld, const float* __restrict__ src, float scale = 1.0f) {
  constexpr int E = ROWS * COLS, PER = (E + kThreads - 1) / kThreads;
  float v[PER];
#pragma unroll
  for (int i = 0; i < PER; ++i) {
    const int e = threadIdx.x + kThreads * i;
    v[i] = (e < E) ? __ldg(src + e) : 0.0f;
  }
#pragma unroll
  for (int i = 0; i < PER; ++i) {
    const int e = threadIdx.x + kThreads * i;
    if (e < E) dst[(e % COLS) * ld + e / COLS] = scale * v[i];
  }
}
template <int N>
__device__ __forceinline__ void load_vec(float* dst, const float* __restrict__ src) {
  for (int i = threadIdx.x; i < N; i += kThreads) dst[i] = __ldg(src + i);
}

// pivot-block size of the Q_uu elimination (NU up to 30 columns of pivots)
constexpr int kGjBlock = 8;

template <int NX, int NU, int NE>
struct Lay {
  static constexpr int LX = NX + (NX % 2 == 0 ? 1 : 2), LU = NU + (NU % 2 == 0 ? 1 : 2),
                       LE = NE + (NE % 2 == 0 ? 1 : 2);
  // ZW: the solution [Z | g | W] of Q_uu [Z | g | W] = [Q_ux | q_u | D'];
  // TS: D [Z | g | W]; KK: [K_nu | k_nu]; PAN: the Gauss-Jordan pivot panel
  static constexpr int NZW = NX + 1 + NE;
  static constexpr int P = 0, A = P + NX * LX, PA = A + NX * LX, Q = PA + NX * LX, B = Q + NX * LX, PB = B + NU * LX,
                       M = PB + NU * LX, QUU = M + NU * LX, QUX = QUU + NU * LU, ZW = QUX + NX * LU,
                       C = ZW + NZW * LU, D = C + NX * LE, TS = D + NU * LE, KK = TS + NZW * LE,
                       PAN = (KK + (NX + 1) * LE + 3) / 4 * 4, V = PAN + 2 * kGjBlock * 32;
  // vectors, NX + 4 floats each
  static constexpr int VL = NX + 4;
  static constexpr int vc = V, vq = vc + VL, vr = vq + VL, ve = vr + VL, vw = ve + VL, vp = vw + VL, vqx = vp + VL,
                       vqu = vqx + VL, vkn = vqu + VL, vk = vkn + VL, vx = vk + VL,
                       vu = vx + VL, FLOATS = vu + VL;
};

// Forward sweep from x0: u_t = K_t x_t + k_t, x_{t+1} = A_t x_t + B_t u_t + c_t.
// Each stage's A, B, K (with c, k) is staged in shared memory transposed, with
// odd leading dimensions, so one thread per output row reads consecutive
// words and the transposing stores are conflict-free; stage t+1 is loaded
// into registers while stage t computes (two buffers of FwdLay::STG floats).
template <int NX, int NU>
struct FwdLay {
  static constexpr int LA = NX % 2 ? NX : NX + 1, LK = NU % 2 ? NU : NU + 1;
  static constexpr int OA = 0, OB = NX * LA, OK = OB + NU * LA, OC = OK + NX * LK, OKK = OC + NX, STG = OKK + NU;
  static constexpr int SA = NX * NX, SB = NX * NU, SK = NU * NX, SRC = SA + SB + SK + NX + NU;
  // staged slot of source element e of A | B | K | c | k (each row-major)
  __device__ static int slot(int e) {
    if (e < SA) return OA + (e % NX) * LA + e / NX;
    e -= SA;
    if (e < SB) return OB + (e % NU) * LA + e / NU;
    e -= SB;
    if (e < SK) return OK + (e % NX) * LK + e / NX;
    e -= SK;
    return e < NX ? OC + e : OKK + (e - NX);
  }
};

template <int NX, int NU>
__device__ __forceinline__ void forward_sweep(const mpxg_lq_eq_io& io, int b, float* stg0, float* stg1, float* vx,
                                              float* vu, float* vt) {
  typedef FwdLay<NX, NU> F;
  static_assert(NX <= kThreads && NU <= kThreads, "one thread per output row");
  const int N = io.N, tid = threadIdx.x;
  const size_t sn = (size_t)b * N, sn1 = (size_t)b * (N + 1);
  auto src = [&](int t, int e) -> float {
    if (e < F::SA) return __ldg(io.A + (sn + t) * F::SA + e);
    e -= F::SA;
    if (e < F::SB) return __ldg(io.Bm + (sn + t) * F::SB + e);
    e -= F::SB;
    if (e < F::SK) return io.K[(sn + t) * F::SK + e];  // written by this kernel
    e -= F::SK;
    return e < NX ? __ldg(io.c + (sn + t) * NX + e) : io.k[(sn + t) * NU + e - NX];
  };
  constexpr int PF = (F::SRC + kThreads - 1) / kThreads;
  float* stg[2] = {stg0, stg1};
  float* X = io.X + sn1 * NX;
  float* U = io.U + sn * NU;
  for (int i = tid; i < NX; i += kThreads) vx[i] = io.x0[(size_t)b * NX + i];
  for (int e = tid; e < F::SRC; e += kThreads) stg[0][F::slot(e)] = src(0, e);
  __syncthreads();
  for (int t = 0; t < N; ++t) {
    const float* cur = stg[t & 1];
    float pre[PF];
    if (t + 1 < N) {
#pragma unroll
      for (int q = 0; q < PF; ++q) {
        const int e = tid + kThreads * q;
        pre[q] = e < F::SRC ? src(t + 1, e) : 0.0f;
      }
    }
    for (int i = tid; i < NX; i += kThreads) X[t * NX + i] = vx[i];
    if (tid < NU) {  // u = K x + k
      const int a = tid;
      float s0 = cur[F::OKK + a], s1 = 0.0f;
#pragma unroll 4
      for (int j = 0; j + 1 < NX; j += 2) {
        s0 += cur[F::OK + j * F::LK + a] * vx[j];
        s1 += cur[F::OK + (j + 1) * F::LK + a] * vx[j + 1];
      }
      if (NX & 1) s0 += cur[F::OK + (NX - 1) * F::LK + a] * vx[NX - 1];
      const float u = s0 + s1;
      vu[a] = u;
      U[t * NU + a] = u;
    }
    __syncthreads();
    if (tid < NX) {  // x+ = A x + B u + c
      const int i = tid;
      float s0 = cur[F::OC + i], s1 = 0.0f;
#pragma unroll 4
      for (int j = 0; j + 1 < NX; j += 2) {
        s0 += cur[F::OA + j * F::LA + i] * vx[j];
        s1 += cur[F::OA + (j + 1) * F::LA + i] * vx[j + 1];
      }
      if (NX & 1) s0 += cur[F::OA + (NX - 1) * F::LA + i] * vx[NX - 1];
#pragma unroll 2
      for (int a = 0; a < NU; ++a) s1 += cur[F::OB + a * F::LA + i] * vu[a];
      vt[i] = s0 + s1;
    }
    if (t + 1 < N) {
      float* nxt = stg[(t + 1) & 1];
#pragma unroll
      for (int q = 0; q < PF; ++q) {
        const int e = tid + kThreads * q;
        if (e < F::SRC) nxt[F::slot(e)] = pre[q];
      }
    }
    __syncthreads();
    for (int i = tid; i < NX; i += kThreads) vx[i] = vt[i];
    __syncthreads();
  }
  for (int i = tid; i < NX; i += kThreads) X[N * NX + i] = vx[i];
}

// Costates lam_t = P_t x_t + p_t and multipliers nu_t = K_nu,t x_t + k_nu,t,
// a warp per stage.  P_t (workspace, exactly symmetric) is read by columns:
// lane r accumulates lam[r] = sum_j P[j][r] x[j] with coalesced loads and no
// reductions; nu by shuffle reductions over its p rows.  xs: (threads / 32)
// x NX floats of shared memory.
template <int NX, int NE>
__device__ __forceinline__ void costates(const mpxg_lq_eq_io& io, int b, const float* Ps, float* xs) {
  constexpr int NP = NX + 1, Q = (NX + 31) / 32;
  const int N = io.N, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const size_t sn = (size_t)b * N, sn1 = (size_t)b * (N + 1);
  const float* X = io.X + sn1 * NX;
  float* xw = xs + warp * NX;
  for (int t = warp; t <= N; t += kThreads / 32) {
    const float* Pt = Ps + (size_t)t * NP * NX;
#pragma unroll
    for (int q = 0; q < Q; ++q)
      if (lane + 32 * q < NX) xw[lane + 32 * q] = X[(size_t)t * NX + lane + 32 * q];
    __syncwarp();
    float acc[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) acc[q] = 0.0f;
#pragma unroll 4
    for (int j = 0; j < NX; ++j) {
      const float xj = xw[j];
#pragma unroll
      for (int q = 0; q < Q; ++q)
        if (lane + 32 * q < NX) acc[q] += Pt[(size_t)j * NX + lane + 32 * q] * xj;
    }
#pragma unroll
    for (int q = 0; q < Q; ++q)
      if (lane + 32 * q < NX) io.lam[(sn1 + t) * NX + lane + 32 * q] = acc[q] + Pt[NX * NX + lane + 32 * q];
    if (t < N) {
      const float* Knt = io.Knu + (sn + t) * NE * NX;
      for (int jr = 0; jr < NE; ++jr) {
        float a = 0.0f;
#pragma unroll
        for (int q = 0; q < Q; ++q)
          if (lane + 32 * q < NX) a += Knt[(size_t)jr * NX + lane + 32 * q] * xw[lane + 32 * q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        if (lane == 0) io.nu[(sn + t) * NE + jr] = a + io.knu[(sn + t) * NE + jr];
      }
    }
    __syncwarp();
  }
}

template <int NX, int NU, int NE>
constexpr size_t smem_bytes() { return (size_t)Lay<NX, NU, NE>::FLOATS * sizeof(float); }

template <int NX, int NU, int NE>
__global__ void __launch_bounds__(kThreads, 1) lqr_eq_kernel(mpxg_lq_eq_io io, float* Pscr) {
  typedef Lay<NX, NU, NE> L;
  constexpr int LX = L::LX, LU = L::LU, LE = L::LE;
  extern __shared__ float4 smem4[];
  float* s = reinterpret_cast<float*>(smem4);
  float *P = s + L::P, *sA = s + L::A, *PA = s + L::PA, *sQ = s + L::Q, *sB = s + L::B, *PB = s + L::PB;
  float *sM = s + L::M, *Quu = s + L::QUU, *Qux = s + L::QUX, *ZW = s + L::ZW, *sC = s + L::C;
  float *sD = s + L::D, *TS = s + L::TS, *KK = s + L::KK, *pan = s + L::PAN;
  float *vc = s + L::vc, *vq = s + L::vq, *vr = s + L::vr, *ve = s + L::ve, *vw = s + L::vw, *vp = s + L::vp;
  float *vqx = s + L::vqx, *vqu = s + L::vqu, *vkn = s + L::vkn, *vk = s + L::vk;
  float *vx = s + L::vx, *vu = s + L::vu;
  const int b = blockIdx.x, N = io.N, tid = threadIdx.x;
  constexpr int NP = NX + 1;  // workspace rows per stage: P (NX x NX) then p
  float* Ps = Pscr + (size_t)b * (N + 1) * NP * NX;
  const size_t sn = (size_t)b * N, sn1 = (size_t)b * (N + 1);

  // ---- terminal value function
  load_cm<NX, NX>(P, LX, io.Q + (sn1 + N) * NX * NX);
  load_vec<NX>(vp, io.q + (sn1 + N) * NX);
  __syncthreads();
  for (int e = tid; e < NX * NX; e += kThreads) Ps[(size_t)N * NP * NX + e] = P[(e / NX) * LX + e % NX];
  for (int i = tid; i < NX; i += kThreads) Ps[(size_t)N * NP * NX + NX * NX + i] = vp[i];

  for (int t = N - 1; t >= 0; --t) {
    // ---- stage data
    load_cm<NX, NX>(sA, LX, io.A + (sn + t) * NX * NX);
    load_cm<NX, NU>(sB, LX, io.Bm + (sn + t) * NX * NU);
    load_cm<NX, NX>(sQ, LX, io.Q + (sn1 + t) * NX * NX);
    load_cm<NX, NU>(sM, LX, io.M + (sn + t) * NX * NU);
    load_cm<NU, NU>(Quu, LU, io.R + (sn + t) * NU * NU);
    load_cm<NE, NX>(sC, LE, io.C + (sn + t) * NE * NX);
    load_cm<NE, NU>(sD, LE, io.D + (sn + t) * NE * NU);
    load_vec<NX>(vc, io.c + (sn + t) * NX);
    load_vec<NX>(vq, io.q + (sn1 + t) * NX);
    load_vec<NU>(vr, io.r + (sn + t) * NU);
    load_vec<NE>(ve, io.e + (sn + t) * NE);
    __syncthreads();
    // ---- P A, P B, w = P c + p
    bmm<NX, NX, NX, false, false, false>(PA, LX, P, LX, sA, LX, 1.0f, nullptr, 0);
    bmm<NX, NX, NU, false, false, false>(PB, LX, P, LX, sB, LX, 1.0f, nullptr, 0);
    bmv<NX, NX, false>(vw, P, LX, vc, 1.0f, vp);
    // ---- Q-function blocks
    bmm<NX, NX, NX, true, false, false>(sQ, LX, sA, LX, PA, LX, 1.0f, sQ, LX);        // Q_xx
    bmm<NU, NX, NX, true, false, true>(Qux, LU, sB, LX, PA, LX, 1.0f, sM, LX);        // Q_ux = M' + B'PA
    bmm<NU, NX, NU, true, false, false>(Quu, LU, sB, LX, PB, LX, 1.0f, Quu, LU);      // Q_uu = R + B'PB
    bmv<NX, NX, true>(vqx, sA, LX, vw, 1.0f, vq);                                     // q_x
    bmv<NU, NX, true>(vqu, sB, LX, vw, 1.0f, vr);                                     // q_u
    // ---- elimination, two column-parallel block Gauss-Jordan solves:
    //   Q_uu [Z | g | W] = [Q_ux | q_u | D'];
    //   [S | T | h] = [D W | C - D Z | D g + e],  S [K_nu | -k_nu] = [T | h];
    //   Z += W K_nu (K = -Z), g += W k_nu (k = -g)
    gj_solve<NU, NU + L::NZW, kGjBlock>(pan, [&](int j, float* v) {
#pragma unroll
      for (int i = 0; i < NU; ++i)
        v[i] = j < NU ? Quu[j * LU + i]
                      : (j < NU + NX ? Qux[(j - NU) * LU + i]
                                     : (j == NU + NX ? vqu[i] : sD[i * LE + (j - NU - NX - 1)]));
    }, [&](int j, const float* v) {
#pragma unroll
      for (int i = 0; i < NU; ++i) ZW[(j - NU) * LU + i] = v[i];
    });
    bmm<NE, NU, L::NZW, false, false, false>(TS, LE, sD, LE, ZW, LU, 1.0f, nullptr, 0);
    gj_solve<NE, NE + NX + 1>(pan, [&](int j, float* v) {
#pragma unroll
      for (int i = 0; i < NE; ++i)
        v[i] = j < NE ? TS[(NX + 1 + j) * LE + i]
                      : (j < NE + NX ? sC[(j - NE) * LE + i] - TS[(j - NE) * LE + i] : TS[NX * LE + i] + ve[i]);
    }, [&](int j, const float* v) {
      const float sg = (j == NE + NX) ? -1.0f : 1.0f;
#pragma unroll
      for (int i = 0; i < NE; ++i) KK[(j - NE) * LE + i] = sg * v[i];
    });
    bmm<NU, NE, NX + 1, false, false, false>(ZW, LU, ZW + (NX + 1) * LU, LU, KK, LE, 1.0f, ZW, LU);
    // ---- gains out
    {
      float* Ko = io.K + (sn + t) * NU * NX;
      float* ko = io.k + (sn + t) * NU;
      float* Kno = io.Knu + (sn + t) * NE * NX;
      float* kno = io.knu + (sn + t) * NE;
      for (int e = tid; e < NU * NX; e += kThreads) Ko[e] = -ZW[(e % NX) * LU + e / NX];
      for (int e = tid; e < NE * NX; e += kThreads) Kno[e] = KK[(e % NX) * LE + e / NX];
      for (int a = tid; a < NU; a += kThreads) { vk[a] = -ZW[NX * LU + a]; ko[a] = -ZW[NX * LU + a]; }
      for (int j = tid; j < NE; j += kThreads) { vkn[j] = KK[NX * LE + j]; kno[j] = KK[NX * LE + j]; }
    }
    __syncthreads();
    // ---- P <- Q_xx - Q_ux' Z + C' K_nu,  p <- q_x + Q_ux' k + C' k_nu
    bmm<NX, NU, NX, true, false, false>(P, LX, Qux, LU, ZW, LU, -1.0f, sQ, LX);
    bmm<NX, NE, NX, true, false, false>(P, LX, sC, LE, KK, LE, 1.0f, P, LX);
    bmv<NX, NU, true>(vp, Qux, LU, vk, 1.0f, vqx);
    bmv<NX, NE, true>(vp, sC, LE, vkn, 1.0f, vp);
    for (int e = tid; e < NX * NX; e += kThreads) {  // symmetrise into PA, copy back
      const int c = e / NX, r = e % NX;
      PA[c * LX + r] = 0.5f * (P[c * LX + r] + P[r * LX + c]);
    }
    __syncthreads();
    float* Pt = Ps + (size_t)t * NP * NX;
    for (int e = tid; e < NX * NX; e += kThreads) {
      const int c = e / NX, r = e % NX;
      const float v = PA[c * LX + r];
      P[c * LX + r] = v;
      Pt[e] = v;  // symmetric: row-major = column-major
    }
    for (int i = tid; i < NX; i += kThreads) Pt[NX * NX + i] = vp[i];
    __syncthreads();
  }

  // ---- forward sweep (staging over the matrix buffers, below the vectors)
  // and the costates
  static_assert(2 * FwdLay<NX, NU>::STG <= L::V, "forward staging must fit the matrix buffers (below the vectors)");
  forward_sweep<NX, NU>(io, b, s, s + FwdLay<NX, NU>::STG, vx, vu, vq);
  __syncthreads();
  costates<NX, NE>(io, b, Ps, s);
}

inline size_t lqr_eq_scratch_bytes(int batch, int N, int n) { return (size_t)batch * (N + 1) * (n + 1) * n * 4; }

template <int NX, int NU, int NE>
inline cudaError_t launch_lqr_eq(cudaStream_t st, const mpxg_lq_eq_io& io) {
  const size_t smem = smem_bytes<NX, NU, NE>();
  cudaError_t e = cudaFuncSetAttribute(lqr_eq_kernel<NX, NU, NE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  lqr_eq_kernel<NX, NU, NE><<<io.batch, kThreads, smem, st>>>(io, io.workspace);
  return cudaGetLastError();
}

}  // namespace lqeq
}  // namespace mpxg
