// Fused primal-dual SQP solve, one MPC instance per warp.
//
// Each SQP iteration (the Newton-KKT step of the reference's multiple-shooting
// SQP; call sites mpx/utils/mpc_wrapper_srbd.py:124-132, solver module absent
// from the reference tree) runs four phases inside one warp:
//
//  1. linearise   lane = stage (32 stages at a time): dynamics Jacobian [A|B]
//                 by forward-mode dual numbers with several tangents per pass
//                 on the increment form f = x + d(x, u), defect
//                 c = f(x,u) - x+, stage cost, gradient, barrier blocks.
//                 Results go to the warp's scratch (L2-resident).
//  2. backward    lane = column of the augmented stage matrix
//                     H = G + F^T P F,   F = [A B c; 0 0 1]
//                 built from the scratch, then the m control pivots are
//                 eliminated by 4x4 block Gauss-Jordan: what remains is the new
//                 value function (P, p) and the gains (K, k).  The closed-loop
//                 map (A + BK, Bk + c) is stored for phase 3.
//  3. forward     dx+ = (A+BK) dx + (Bk+c), du = K dx + k and the costates
//                 lam = P dx + p (the new duals); column partials are reduced
//                 through shared memory.
//  4. merit       stage-parallel augmented-Lagrangian merit
//                 phi = J + V.c + rho/2 |c|^2 with backtracking, then the step.
//                 The Armijo test sums per-stage differences phi(alpha) - phi(0)
//                 written without cancellation (dynamics increments kept from
//                 phase 1), so that decreases far below float32's resolution
//                 of phi itself are still resolved.
#pragma once
#include "models.cuh"

namespace mpxg {

enum { ST_NAN = 1, ST_NON_PD = 2, ST_LS_FAIL = 4, ST_BAD_HORIZON = 8 };

struct SqpParams {
  int sqp_iters, ls_max_trials;
  float ls_beta, ls_eta, reg, rho0, ls_skip_tol;
  int compute_kkt;
  int team_exact_last;  // team kernel: the last iteration's KKT step as one sequential sweep
};

struct BatchPtrs {
  int batch, n_max;
  const int* slot;   // pool row of each batch entry (null: identity)
  const int* horizon;
  const float *x0, *X_in, *U_in, *V_in, *ref, *par, *w;
  float *X, *U, *V, *K, *k, *kkt;
  int* status;
  float* first;              // optional per-batch-entry result rows [batch, NU+4]
  int* counter;              // work-queue head (zeroed before each launch)
  float* scratch;            // per-warp scratch
  long long scratch_stride;  // floats per warp
  int single_instance;       // >= 0: solve only this instance with warp 0 (plain path)
  // Scratch slots claimed per warp from a bitmap shared by every launch of one
  // handle (null: the warp's grid index is its slot).  n_slots is the most
  // warps of this kernel that can be resident on the device at once, so a
  // resident warp always finds a free slot.
  unsigned int* slot_bits = nullptr;
  int n_slots = 0;
  int* error = nullptr;      // bit 0: a warp gave up claiming a slot
  // Optional processing order of the batch entries (longest horizon first):
  // the i-th instance taken from the work queue is batch entry order[i].
  const int* order = nullptr;
  // Queue split between the time-parallel team kernel (sqp_team.cuh), which
  // takes queue entries [0, *split), and this kernel, which then takes
  // [*split, batch) (null: this kernel takes the whole queue).
  const int* split = nullptr;
  // Vector-Jacobian product mode (sqp_vjp_kernel): cotangents gX, gU of the
  // converged X, U in; adjoint solution wX, wU, wL and the gradients with
  // respect to x0 and to the state reference out.
  const float *gX = nullptr, *gU = nullptr;
  float *wX = nullptr, *wU = nullptr, *wL = nullptr, *gx0 = nullptr, *gref = nullptr;
};

// Bounded claim of a free scratch slot (lane 0 only); -1 after the limit.
__device__ inline int claim_scratch_slot(unsigned int* bits, int n_slots, int pref) {
  const int nwords = (n_slots + 31) >> 5;
  int wi = pref >> 5;
  for (int it = 0; it < (1 << 16); ++it) {
    const unsigned int w = atomicAdd(&bits[wi], 0u);
    unsigned int avail = ~w;
    if (wi == nwords - 1 && (n_slots & 31)) avail &= (1u << (n_slots & 31)) - 1u;
    if (avail) {
      const int want = pref & 31;
      const int bit = (it == 0 && wi == (pref >> 5) && ((avail >> want) & 1u)) ? want : __ffs(avail) - 1;
      const unsigned int old = atomicOr(&bits[wi], 1u << bit);
      if (!(old & (1u << bit))) return wi * 32 + bit;
    } else {
      wi = wi + 1 == nwords ? 0 : wi + 1;
    }
  }
  return -1;
}

// Arguments of the mixed-model launch (sqp_mixed.cuh): two models' batches
// served from one queue.  Queue entry i is code order[i] (identity if null):
// codes below bp[0].batch are model 0's batch entries, the others model 1's
// entry code - bp[0].batch.
struct MixedArgs {
  ModelConst mc[2];
  SqpParams sp[2];
  BatchPtrs bp[2];
  const int* order;
  int total;
  int* counter;
  float* scratch;
  long long scratch_stride;
  unsigned int* slot_bits;
  int n_slots;
  int* error;
};

constexpr int rup4(int v) { return (v + 3) / 4 * 4; }

// n floats from a 16-byte aligned address into registers (float4 where possible)
template <int N>
__device__ __forceinline__ void ld_vec(const float* __restrict__ src, float* dst) {
#pragma unroll
  for (int q = 0; q < N / 4; ++q) {
    const float4 v = *reinterpret_cast<const float4*>(src + 4 * q);
    dst[4 * q] = v.x; dst[4 * q + 1] = v.y; dst[4 * q + 2] = v.z; dst[4 * q + 3] = v.w;
  }
#pragma unroll
  for (int r = (N / 4) * 4; r < N; ++r) dst[r] = src[r];
}
template <int N>
__device__ __forceinline__ void st_vec(float* __restrict__ dst, const float* src) {
#pragma unroll
  for (int q = 0; q < N / 4; ++q)
    *reinterpret_cast<float4*>(dst + 4 * q) = make_float4(src[4 * q], src[4 * q + 1], src[4 * q + 2], src[4 * q + 3]);
#pragma unroll
  for (int r = (N / 4) * 4; r < N; ++r) dst[r] = src[r];
}

// 16-byte asynchronous global -> shared copies (L2 only), in commit groups
__device__ __forceinline__ void cp_async16(float* smem, const float* gmem) {
  const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int PENDING>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(PENDING) : "memory");
}
// FLOATS floats (a multiple of 4, both ends 16-byte aligned) spread over the warp's lanes
template <int FLOATS>
__device__ __forceinline__ void cp_async_block(float* dst, const float* src, int lane) {
#pragma unroll
  for (int q = lane; q < FLOATS / 4; q += 32) cp_async16(dst + 4 * q, src + 4 * q);
}

template <class M>
struct Dims {
  static constexpr int NX = M::NX, NU = M::NU;
  static constexpr int NZ = NX + NU + 1;      // augmented columns: x, u, affine
  static constexpr int JA = NX + NU;          // affine column / lane
  static constexpr int NP = NX + 1;           // value-function rows: x, affine
  static constexpr int LDP = rup4(NP);        // shared / scratch column stride of P
  static constexpr int FS = rup4(NX);         // scratch column stride of F
  static constexpr int FTS = rup4(NZ);        // shared row stride of F's rows (WarpSmem::FT)
  static constexpr int LD = (M::LEGS == 4) ? 3 : 6;  // controls per leg / foot
  static constexpr int QB = M::IDENT_RES ? 0 : 4;    // quaternion Gauss-Newton block
  // per-stage cost data: gradient (NX+NU), barrier blocks, quaternion block, cost value
  static constexpr int G_GRAD = 0, G_HB = NX + NU, G_QQ = G_HB + M::LEGS * LD * LD, G_L = G_QQ + QB * QB;
  static constexpr int GS = rup4(G_L + 1);
  static constexpr int RS = rup4(NU + NX);    // forward-sweep partial row
  // staged stage blocks (WarpSmem::stg): the backward sweep stages F at 0 and
  // G at NZ * FS; the forward sweep stages P, K, F and G at SP, SK, SF, SG
  static constexpr int SP = 0, SK = NP * LDP, SF = SK + NP * NU, SG = SF + NZ * FS, STG = SG + GS;
  static constexpr int TANG = 2;              // tangents per dual-number pass
};

template <class M>
struct __align__(16) WarpSmem {
  typedef Dims<M> D;
  float w[24];
  float P[D::NP * D::LDP];     // value function of stage t+1, column-major
  float Praw[D::NP * D::LDP];  // unsymmetrised new value function
  float FT[D::NX * D::FTS];    // rows 0..n-1 of stage t's F (the backward sweep's F'T products)
  float CT[D::NZ * 4];         // pivot block columns, row-interleaved
  float red[(D::NX + 1) * D::RS];
  float dx[16];
  float stg[2][D::STG];        // stage blocks copied in by cp.async, double-buffered
};

template <class M>
__host__ __device__ inline long long scratch_floats(int n_max) {
  typedef Dims<M> D;
  long long f = 0;
  f += (long long)n_max * D::NZ * D::FS;           // F columns (later A+BK, Bk+c) and defects
  f += (long long)(n_max + 1) * D::GS;             // cost data
  f += (long long)n_max * D::NP * M::NU;           // [K | k] column-major
  f += (long long)(n_max + 1) * D::NP * D::LDP;    // value functions
  f += (long long)n_max * D::FS;                   // dynamics increments f - x at the iterate
  f += (long long)(n_max + 1) * D::NX * 2;         // dX, lam
  f += (long long)n_max * M::NU;                   // dU
  return (f + 31) / 32 * 32;
}

template <class M>
struct Scratch {
  typedef Dims<M> D;
  float *F, *G, *K, *P, *D0, *dX, *L, *dU;
  __device__ Scratch(float* base, int n_max) {
    F = base;
    G = F + (size_t)n_max * D::NZ * D::FS;
    K = G + (size_t)(n_max + 1) * D::GS;
    P = K + (size_t)n_max * D::NP * M::NU;
    D0 = P + (size_t)(n_max + 1) * D::NP * D::LDP;
    dX = D0 + (size_t)n_max * D::FS;
    L = dX + (size_t)(n_max + 1) * D::NX;
    dU = L + (size_t)(n_max + 1) * D::NX;
  }
};

// ----------------------------------------------------------------- phase 1
// Stage t (0..N) on one lane.  STORE (KKT = false): write the stage's F
// columns and cost data to the scratch.  KKT = true: accumulate the primal /
// dual KKT residuals of the current iterate instead.
template <class M, bool KKT>
__device__ __forceinline__ void lin_stage(const ModelConst& mc, int t, int N, const float* x0, const float* X,
                                          const float* U, const float* V, const float* ref, const float* par,
                                          const float* w, const Scratch<M>& s, float* lsum, float* rp, float* rd,
                                          float* gm) {
  typedef Dims<M> D;
  constexpr int NX = D::NX, NU = D::NU, JA = D::JA, FS = D::FS, LD = D::LD, TK = D::TANG;
  const bool term = (t == N);
  const float* rr = ref + t * M::NREF;
  float x[NX], u[NU], xn[NX];
#pragma unroll
  for (int i = 0; i < NX; ++i) x[i] = X[t * NX + i];
#pragma unroll
  for (int a = 0; a < NU; ++a) u[a] = term ? 0.0f : U[t * NU + a];
#pragma unroll
  for (int i = 0; i < NX; ++i) xn[i] = term ? 0.0f : X[(t + 1) * NX + i];
  float vn[NX];
#pragma unroll
  for (int i = 0; i < NX; ++i) vn[i] = 0.0f;
  if (KKT) {
    if (!term) {
#pragma unroll
      for (int i = 0; i < NX; ++i) vn[i] = V[(t + 1) * NX + i];
    }
    if (t == 0) {
#pragma unroll
      for (int i = 0; i < NX; ++i) *rp = fmaxf(*rp, fabsf(x0[i] - x[i]));
    }
  }
  // ---- cost: tracking residual, gradient, Gauss-Newton blocks, barrier
  float g[NX + NU];
  float r[12];
  M::template state_residual<float>(x, rr, r);
  float l = 0.0f;
#pragma unroll
  for (int a = 0; a < 12; ++a) l += w[a] * r[a] * r[a];
  float Qq[4][4];
  if (M::IDENT_RES) {
#pragma unroll
    for (int i = 0; i < NX; ++i) g[i] = w[i] * r[i];
  } else {
    // quaternion rows of the residual Jacobian by one 4-tangent pass
    DK<4> qd[4], rq[3];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      qd[k].v = x[M::QOFF + k];
#pragma unroll
      for (int e = 0; e < 4; ++e) qd[k].d[e] = (e == k) ? 1.0f : 0.0f;
    }
    quat_sub(qd, rr + 3, rq);
#pragma unroll
    for (int i = 0; i < NX; ++i) {
      if (i >= M::QOFF && i < M::QOFF + 4) {
        const int k = i - M::QOFF;
        g[i] = w[3] * r[3] * rq[0].d[k] + w[4] * r[4] * rq[1].d[k] + w[5] * r[5] * rq[2].d[k];
      } else {
        const int a = M::wrow(i);
        g[i] = w[a] * r[a];
      }
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int k = 0; k < 4; ++k)
        Qq[i][k] = w[3] * rq[0].d[i] * rq[0].d[k] + w[4] * rq[1].d[i] * rq[1].d[k] + w[5] * rq[2].d[i] * rq[2].d[k];
  }
  float Hb[M::LEGS][LD][LD];
  if (!term) {
#pragma unroll
    for (int a = 0; a < NU; ++a) { g[NX + a] = w[12 + a] * u[a]; l += w[12 + a] * u[a] * u[a]; }
    l *= 0.5f;
#pragma unroll
    for (int leg = 0; leg < M::LEGS; ++leg) {
      float v, gb[LD];
      barrier_leg<M, LD>(mc, leg, u, rr, &v, gb, Hb[leg]);
      l += v;
#pragma unroll
      for (int a = 0; a < LD; ++a) g[NX + LD * leg + a] += gb[a];
    }
  } else {
    l *= 0.5f;
#pragma unroll
    for (int a = 0; a < NU; ++a) g[NX + a] = 0.0f;
#pragma unroll
    for (int leg = 0; leg < M::LEGS; ++leg)
#pragma unroll
      for (int a = 0; a < LD; ++a)
#pragma unroll
        for (int b = 0; b < LD; ++b) Hb[leg][a][b] = 0.0f;
  }
  *lsum += l;
  if (!KKT) {
    float gv[D::GS];
#pragma unroll
    for (int i = 0; i < D::GS; ++i) gv[i] = 0.0f;
#pragma unroll
    for (int i = 0; i < NX + NU; ++i) gv[D::G_GRAD + i] = g[i];
#pragma unroll
    for (int leg = 0; leg < M::LEGS; ++leg)
#pragma unroll
      for (int a = 0; a < LD; ++a)
#pragma unroll
        for (int b = 0; b < LD; ++b) gv[D::G_HB + (leg * LD + a) * LD + b] = Hb[leg][a][b];
    if (D::QB) {
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int k = 0; k < 4; ++k) gv[D::G_QQ + i * 4 + k] = Qq[i][k];
    }
    gv[D::G_L] = l;
    st_vec<D::GS>(s.G + (size_t)t * D::GS, gv);
  } else if (term) {
#pragma unroll
    for (int i = 0; i < NX; ++i) {
      *rd = fmaxf(*rd, fabsf(g[i] - V[t * NX + i]));
      *gm = fmaxf(*gm, fabsf(g[i]));
    }
  }
  if (term) return;
  // ---- dynamics in increment form f = x + d(x, u): defect, Jacobian columns
  // (identity + dd/dz) and, for the merit line search, d itself
  const float* pp = par + t * M::NPAR;
  float* Ft = s.F + (size_t)t * D::NZ * FS;
#pragma unroll 1
  for (int p0 = 0; p0 < NX + NU; p0 += TK) {
    DK<TK> xd[NX], ud[NU], fd[NX];
#pragma unroll
    for (int i = 0; i < NX; ++i) {
      xd[i].v = x[i];
#pragma unroll
      for (int k = 0; k < TK; ++k) xd[i].d[k] = (i == p0 + k) ? 1.0f : 0.0f;
    }
#pragma unroll
    for (int a = 0; a < NU; ++a) {
      ud[a].v = u[a];
#pragma unroll
      for (int k = 0; k < TK; ++k) ud[a].d[k] = (NX + a == p0 + k) ? 1.0f : 0.0f;
    }
    M::template increment<DK<TK>>(mc, xd, ud, pp, fd);
    if (!KKT) {
      if (p0 == 0) {
        float cv[FS], dv[FS];
#pragma unroll
        for (int i = 0; i < FS; ++i) {
          const int ii = i < NX ? i : 0;
          cv[i] = (i < NX) ? (x[ii] + fd[ii].v) - xn[ii] : 0.0f;
          dv[i] = (i < NX) ? fd[ii].v : 0.0f;
        }
        st_vec<FS>(Ft + JA * FS, cv);
        st_vec<FS>(s.D0 + (size_t)t * FS, dv);
      }
#pragma unroll
      for (int k = 0; k < TK; ++k) {
        const int dir = p0 + k;
        if (dir < NX + NU) {
          float cv[FS];
#pragma unroll
          for (int i = 0; i < FS; ++i) cv[i] = (i < NX) ? fd[i < NX ? i : 0].d[k] + (i == dir ? 1.0f : 0.0f) : 0.0f;
          st_vec<FS>(Ft + dir * FS, cv);
        }
      }
    } else {
      if (p0 == 0) {
#pragma unroll
        for (int i = 0; i < NX; ++i) *rp = fmaxf(*rp, fabsf((x[i] + fd[i].v) - xn[i]));
      }
#pragma unroll
      for (int k = 0; k < TK; ++k) {
        const int dir = p0 + k;
        if (dir < NX + NU) {
          float acc = 0.0f, gd = 0.0f, vt = 0.0f;
#pragma unroll
          for (int i = 0; i < NX; ++i) acc += (fd[i].d[k] + (i == dir ? 1.0f : 0.0f)) * vn[i];
#pragma unroll
          for (int i = 0; i < NX + NU; ++i) gd = (i == dir) ? g[i] : gd;
          if (dir < NX) vt = V[t * NX + dir];
          *rd = fmaxf(*rd, fabsf(gd + acc - vt));
          *gm = fmaxf(*gm, fabsf(gd));
        }
      }
    }
  }
}

// ----------------------------------------------------------------- merit
// Stage t's share of phi(alpha) - phi(0), the merit change along the step
// (dX, dU, L - V) scaled by alpha, written without cancellation: cost terms by
// stage_cost_diff, and the defect change from the dynamics increments,
//   dc_t = alpha dx_{t-1} + [d(x_{t-1} + alpha dx_{t-1}, .) - d(x_{t-1}, .)] - alpha dx_t,
// d = f - x, so that
//   d(V.c) = dV.(c0 + dc) + V.dc,  d(|c|^2 / 2) = dc.(2 c0 + dc) / 2.
template <class M>
__device__ __forceinline__ float merit_diff_stage(const ModelConst& mc, int t, int N, float alpha, float rho,
                                                  const float* x0, const float* X, const float* U, const float* V,
                                                  const Scratch<M>& s, const float* ref, const float* par,
                                                  const float* w) {
  constexpr int NX = M::NX, NU = M::NU;
  float xt[NX], dxt[NX], c0[NX], dc[NX];
#pragma unroll
  for (int i = 0; i < NX; ++i) { xt[i] = X[t * NX + i]; dxt[i] = alpha * s.dX[t * NX + i]; }
  float dl;
  {
    float ut[NU], dut[NU];
#pragma unroll
    for (int a = 0; a < NU; ++a) {
      ut[a] = (t < N) ? U[t * NU + a] : 0.0f;
      dut[a] = (t < N) ? alpha * s.dU[t * NU + a] : 0.0f;
    }
    dl = stage_cost_diff<M>(mc, xt, dxt, ut, dut, ref + t * M::NREF, w, t == N);
  }
  if (t == 0) {
#pragma unroll
    for (int i = 0; i < NX; ++i) { c0[i] = x0[i] - xt[i]; dc[i] = -dxt[i]; }
  } else {
    float xp[NX], up[NU], d0[NX], d1[NX];
#pragma unroll
    for (int i = 0; i < NX; ++i) xp[i] = X[(t - 1) * NX + i];
#pragma unroll
    for (int a = 0; a < NU; ++a) up[a] = U[(t - 1) * NU + a];
    const float* pt = par + (t - 1) * M::NPAR;
    ld_vec<NX>(s.D0 + (size_t)(t - 1) * Dims<M>::FS, d0);  // d(x, u) of phase 1
#pragma unroll
    for (int i = 0; i < NX; ++i) {
      c0[i] = (xp[i] + d0[i]) - xt[i];
      dc[i] = alpha * s.dX[(t - 1) * NX + i] - dxt[i];
      xp[i] += alpha * s.dX[(t - 1) * NX + i];
    }
#pragma unroll
    for (int a = 0; a < NU; ++a) up[a] += alpha * s.dU[(t - 1) * NU + a];
    M::template increment<float>(mc, xp, up, pt, d1);
#pragma unroll
    for (int i = 0; i < NX; ++i) dc[i] += d1[i] - d0[i];
  }
  float acc = 0.0f;
#pragma unroll
  for (int i = 0; i < NX; ++i) {
    const float vt = V[t * NX + i];
    const float dv = alpha * (s.L[t * NX + i] - vt);
    acc += dv * (c0[i] + dc[i]) + vt * dc[i] + 0.5f * rho * dc[i] * (2.0f * c0[i] + dc[i]);
  }
  return dl + acc;
}

// ----------------------------------------------------------------- block Gauss-Jordan
// Eliminate the pivot block S = {s0..s0+3} from the column this lane holds (h):
// rows S <- D^-1 h[S], other rows h[i] -= H[i,S] D^-1 h[S], with D = H[S,S]
// (SPD) factored by Cholesky on every lane.
//
// EXTRA: the lane also carries a second column v of which only the control
// rows [U0, U0 + NU) are eliminated (after all pivot blocks they hold
// Quu^-1 v; the other rows are not needed by the caller).
template <int NZ, bool EXTRA = false, int U0 = 0, int NU = 0>
__device__ __forceinline__ void gj_block4(float* h, int s0, int lane, float* CT, int* status, float* v = nullptr) {
  __syncwarp();
  if (lane >= s0 && lane < s0 + 4) {
    const int k = lane - s0;
#pragma unroll
    for (int i = 0; i < NZ; ++i) CT[i * 4 + k] = h[i];
  }
  __syncwarp();
  float Dm[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const float4 rowa = *reinterpret_cast<const float4*>(CT + (s0 + a) * 4);
    Dm[a][0] = rowa.x; Dm[a][1] = rowa.y; Dm[a][2] = rowa.z; Dm[a][3] = rowa.w;
  }
  float L[4][4], il[4];
  bool bad = false;
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    float dsum = Dm[a][a];
#pragma unroll
    for (int k = 0; k < a; ++k) dsum -= L[a][k] * L[a][k];
    if (!(dsum > 0.0f)) { bad = true; dsum = fmaxf(fabsf(dsum), 1e-20f); }
    il[a] = rsqrtf(dsum);
#pragma unroll
    for (int b = a + 1; b < 4; ++b) {
      float v = Dm[b][a];
#pragma unroll
      for (int k = 0; k < a; ++k) v -= L[b][k] * L[a][k];
      L[b][a] = v * il[a];
    }
  }
  if (bad) *status |= ST_NON_PD;
  float y[4];
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    float v = 0.0f;
#pragma unroll
    for (int i = 0; i < NZ; ++i) v = (i == s0 + a) ? h[i] : v;
#pragma unroll
    for (int k = 0; k < a; ++k) v -= L[a][k] * y[k];
    y[a] = v * il[a];
  }
#pragma unroll
  for (int a = 3; a >= 0; --a) {
    float v = y[a];
#pragma unroll
    for (int k = a + 1; k < 4; ++k) v -= L[k][a] * y[k];
    y[a] = v * il[a];
  }
  if (EXTRA) {
    float yv[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      float vv = 0.0f;
#pragma unroll
      for (int i = U0; i < U0 + NU; ++i) vv = (i == s0 + a) ? v[i] : vv;
#pragma unroll
      for (int k = 0; k < a; ++k) vv -= L[a][k] * yv[k];
      yv[a] = vv * il[a];
    }
#pragma unroll
    for (int a = 3; a >= 0; --a) {
      float vv = yv[a];
#pragma unroll
      for (int k = a + 1; k < 4; ++k) vv -= L[k][a] * yv[k];
      yv[a] = vv * il[a];
    }
#pragma unroll
    for (int i = U0; i < U0 + NU; ++i) {
      const float4 hc = *reinterpret_cast<const float4*>(CT + i * 4);
      const float upd = hc.x * yv[0] + hc.y * yv[1] + hc.z * yv[2] + hc.w * yv[3];
      float yi = 0.0f;
#pragma unroll
      for (int a = 0; a < 4; ++a) yi = (i == s0 + a) ? yv[a] : yi;
      v[i] = (i >= s0 && i < s0 + 4) ? yi : v[i] - upd;
    }
  }
#pragma unroll
  for (int i = 0; i < NZ; ++i) {
    const float4 hc = *reinterpret_cast<const float4*>(CT + i * 4);
    const float upd = hc.x * y[0] + hc.y * y[1] + hc.z * y[2] + hc.w * y[3];
    float yi = 0.0f;
#pragma unroll
    for (int a = 0; a < 4; ++a) yi = (i == s0 + a) ? y[a] : yi;
    h[i] = (i >= s0 && i < s0 + 4) ? yi : h[i] - upd;
  }
}

// ----------------------------------------------------------------- chunk elements
// Accumulators of a time-parallel chunk's element while its Riccati sweep
// runs from a zero terminal cost (see riccati_sweep, ELEM = 2): the
// closed-loop affine map x_e = Phi x_t + phi from stage t to the chunk end and
// the Gramian G = sum Phi_{t+1->e} B Quu^-1 B' Phi_{t+1->e}'.  Column-major,
// column stride FS.  Also the outputs of the chunk combination (sqp_team.cuh).
template <class M>
struct __align__(16) ElemSmem {
  typedef Dims<M> D;
  float Phi[2][D::NX * D::FS];      // Phi_{t+1->e}, double-buffered
  float PB[D::NU * D::FS];          // Phi_{t+1->e} B_t
  float G[D::NX * D::FS];           // Gramian
  float phi[D::FS];                 // affine part of the map
  float Z[(D::NX + 1) * D::FS];     // [Z_Phi | z]: the chunk's end state as a map of its start state
  float Pin[D::NP * D::LDP];        // true value function at the chunk's start (WarpSmem::P layout)
  int cur;                          // buffer of Phi holding the map after the sweep
};


// ----------------------------------------------------------------- phase 2
// Terminal value function (P_N, p_N): the terminal cost's Gauss-Newton block
// and gradient, into the warp's shared P (and the scratch when STORE).
template <class M, bool STORE>
__device__ __forceinline__ void riccati_terminal(int N, WarpSmem<M>& sm, const Scratch<M>& s, int lane) {
  typedef Dims<M> D;
  constexpr int NX = D::NX, NP = D::NP, LDP = D::LDP;
  const int j = lane;
  const float* GN = s.G + (size_t)N * D::GS;
  if (j < NX) {
    float col[NP];
#pragma unroll
    for (int i = 0; i < NX; ++i) col[i] = 0.0f;
    if (D::QB && j >= M::QOFF && j < M::QOFF + 4) {
#pragma unroll
      for (int k = 0; k < 4; ++k) col[M::QOFF + k] = GN[D::G_QQ + (j - M::QOFF) * 4 + k];
    } else {
      const float wj = sm.w[M::wrow(j)];
#pragma unroll
      for (int i = 0; i < NX; ++i) col[i] = (i == j) ? wj : col[i];
    }
    const float gj = GN[D::G_GRAD + j];
    col[NX] = gj;
    float* Pn = s.P + (size_t)N * NP * LDP;
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      sm.P[j * LDP + i] = col[i];
      if (STORE) Pn[j * LDP + i] = col[i];
    }
    sm.P[NX * LDP + j] = gj;
    if (STORE) Pn[NX * LDP + j] = gj;
  }
  if (j == 0) {
    sm.P[NX * LDP + NX] = 0.0f;
    if (STORE) s.P[(size_t)N * NP * LDP + NX * LDP + NX] = 0.0f;
  }
  __syncwarp();
}

// Backward Riccati sweep over stages hi-1 .. lo from the value function in
// the warp's shared P (the value at stage hi).  Lane j owns column j of the
// augmented stage matrix H = G + F' P F, F = [A B c; 0 0 1]; the control
// pivots are eliminated by 4x4 block Gauss-Jordan, which leaves the value
// function of stage t (into the shared P) and the gains.
//   STORE: write gains K = [K | k], the closed loop (A + BK, Bk + c) over F's
//          first columns, and P to the scratch (the forward sweep reads them).
//   ELEM:  1: accumulate the closed-loop affine map x_hi = Phi x_t + phi of
//          this sweep's policy in es (ElemSmem); 2: also the Gramian G of the
//          chunk element.  On entry the caller has set es->Phi[0] = I; on
//          return es->Phi[es->cur], es->phi (and es->G) hold the result.
template <class M, bool STORE, int ELEM>
__device__ __forceinline__ void riccati_sweep(const SqpParams& sp, int lo, int hi, WarpSmem<M>& sm, const Scratch<M>& s,
                                              ElemSmem<M>* es, int* status, int lane) {
  typedef Dims<M> D;
  constexpr int NX = D::NX, NU = D::NU, NZ = D::NZ, JA = D::JA, NP = D::NP, LDP = D::LDP, FS = D::FS;
  constexpr int LD = D::LD;
  const int j = lane;
  if (hi <= lo) return;
  int cur = 0;
  float gcol[FS];  // ELEM 2: column j of G (state lanes); ELEM >= 1: phi (lane JA)
#pragma unroll
  for (int i = 0; i < FS; ++i) gcol[i] = 0.0f;
  // stage t's F and cost data G are copied into sm.stg[buf] by cp.async one
  // stage ahead (the copy of t - 1 runs while stage t is eliminated)
  auto stage_in = [&](int t, int b) {
    cp_async_block<NZ * FS>(sm.stg[b], s.F + (size_t)t * NZ * FS, lane);
    cp_async_block<D::GS>(sm.stg[b] + NZ * FS, s.G + (size_t)t * D::GS, lane);
  };
  stage_in(hi - 1, 0);
  cp_async_commit();
  int buf = 0;
  for (int t = hi - 1; t >= lo; --t) {
    if (t > lo) stage_in(t - 1, buf ^ 1);
    cp_async_commit();
    cp_async_wait<1>();  // stage t's copies (all but the newest group) have landed
    __syncwarp();
    const float* Fr = sm.stg[buf];
    const float* Gt = Fr + NZ * FS;
    // ---- column j of F and of the cost model G
    float fcol[NP], h[NZ];
#pragma unroll
    for (int i = 0; i < NP; ++i) fcol[i] = 0.0f;
#pragma unroll
    for (int i = 0; i < NZ; ++i) h[i] = 0.0f;
    if (j < NZ) {
#pragma unroll
      for (int q = 0; q < FS / 4; ++q) {
        const float4 v = *reinterpret_cast<const float4*>(Fr + j * FS + 4 * q);
        if (4 * q < NX) fcol[4 * q] = v.x;
        if (4 * q + 1 < NX) fcol[4 * q + 1] = v.y;
        if (4 * q + 2 < NX) fcol[4 * q + 2] = v.z;
        if (4 * q + 3 < NX) fcol[4 * q + 3] = v.w;
      }
      // F's rows for the F'T products: lane j writes column j of them
#pragma unroll
      for (int r = 0; r < NX; ++r) sm.FT[r * D::FTS + j] = fcol[r];
    }
    fcol[NX] = (j == JA) ? 1.0f : 0.0f;
    if (j < NX) {
      if (D::QB && j >= M::QOFF && j < M::QOFF + 4) {
#pragma unroll
        for (int k = 0; k < 4; ++k) h[M::QOFF + k] = Gt[D::G_QQ + (j - M::QOFF) * 4 + k];
      } else {
        const float wj = sm.w[M::wrow(j)];
#pragma unroll
        for (int i = 0; i < NX; ++i) h[i] = (i == j) ? wj : h[i];
      }
      h[JA] = Gt[D::G_GRAD + j];
    } else if (j < JA) {
      const int a = j - NX, leg = a / LD, c = a - LD * leg;
      float hb[LD];
#pragma unroll
      for (int r2 = 0; r2 < LD; ++r2) hb[r2] = Gt[D::G_HB + (leg * LD + c) * LD + r2];
      const float wa = sm.w[12 + a];
#pragma unroll
      for (int bb = 0; bb < NU; ++bb) {
        float v = (bb == a) ? wa : 0.0f;
#pragma unroll
        for (int r2 = 0; r2 < LD; ++r2) v += (bb == LD * leg + r2) ? hb[r2] : 0.0f;
        h[NX + bb] = v;
      }
      h[JA] = Gt[D::G_GRAD + j];
    } else if (j == JA) {
#pragma unroll
      for (int i = 0; i < JA; ++i) h[i] = Gt[D::G_GRAD + i];
    }
    __syncwarp();
    // ---- T = P F[:, j];  H[:, j] = G[:, j] + F^T T
    // T over the NP rows of P (fcol[NX] is 1 on the affine lane, else 0); then
    // F^T T as NX rank-1 updates with the rows of F, each advancing NZ
    // independent sums, and F's last row (1 in the affine column) adds T[NX]
    // to H[JA, j].
    float tv[NP];
#pragma unroll
    for (int i = 0; i < NP; ++i) tv[i] = 0.0f;
#pragma unroll
    for (int k = 0; k < NP; ++k) {
      const float fk = fcol[k];
      const float* pk = sm.P + k * LDP;
#pragma unroll
      for (int q = 0; q < NP / 4; ++q) {
        const float4 pv = *reinterpret_cast<const float4*>(pk + 4 * q);
        tv[4 * q] += pv.x * fk; tv[4 * q + 1] += pv.y * fk; tv[4 * q + 2] += pv.z * fk; tv[4 * q + 3] += pv.w * fk;
      }
#pragma unroll
      for (int r = (NP / 4) * 4; r < NP; ++r) tv[r] += pk[r] * fk;
    }
#pragma unroll
    for (int r = 0; r < NX; ++r) {
      const float tr = tv[r];
      const float* fr = sm.FT + r * D::FTS;
#pragma unroll
      for (int q = 0; q < D::FTS / 4; ++q) {
        const float4 fv = *reinterpret_cast<const float4*>(fr + 4 * q);
        if (4 * q < NZ) h[4 * q] += fv.x * tr;
        if (4 * q + 1 < NZ) h[4 * q + 1] += fv.y * tr;
        if (4 * q + 2 < NZ) h[4 * q + 2] += fv.z * tr;
        if (4 * q + 3 < NZ) h[4 * q + 3] += fv.w * tr;
      }
    }
    h[JA] += tv[NX];
#pragma unroll
    for (int a = NX; a < JA; ++a)
      if (a == j) h[a] += sp.reg;
    // ---- chunk element: Phi B_t, and row j of it as an extra right-hand side of the elimination
    float v[NZ];
    if (ELEM == 2) {
      const float* Phc = es->Phi[cur];
      if (j >= NX && j < JA) {
        float pb[FS];
#pragma unroll
        for (int i = 0; i < FS; ++i) pb[i] = 0.0f;
#pragma unroll
        for (int k = 0; k < NX; ++k) {
          const float fk = fcol[k];
#pragma unroll
          for (int q = 0; q < FS / 4; ++q) {
            const float4 pv = *reinterpret_cast<const float4*>(Phc + k * FS + 4 * q);
            pb[4 * q] += pv.x * fk; pb[4 * q + 1] += pv.y * fk; pb[4 * q + 2] += pv.z * fk; pb[4 * q + 3] += pv.w * fk;
          }
        }
        st_vec<FS>(es->PB + (j - NX) * FS, pb);
      }
      __syncwarp();
#pragma unroll
      for (int i = 0; i < NZ; ++i) v[i] = (i >= NX && i < JA && j < NX) ? es->PB[(i >= NX && i < JA ? i - NX : 0) * FS + (j < NX ? j : 0)] : 0.0f;
    }
    // ---- block Gauss-Jordan elimination of the control pivots
#pragma unroll
    for (int s0 = NX; s0 < JA; s0 += 4) gj_block4<NZ, ELEM == 2, NX, NU>(h, s0, lane, sm.CT, status, v);
    // ---- gains, closed loop, new value function
    float* Kt = s.K + (size_t)t * NP * NU;
    float* Fo = s.F + (size_t)t * NZ * FS;
    if (j < NX || j == JA) {
      const int col = (j == JA) ? NX : j;
      float kc[NU];
#pragma unroll
      for (int a = 0; a < NU; ++a) kc[a] = -h[NX + a];
      if (STORE) st_vec<NU>(Kt + col * NU, kc);
      // closed loop: (A + B K)[:, j] for state lanes, B k + c for the affine lane
      float cl[FS];
#pragma unroll
      for (int i = 0; i < FS; ++i) cl[i] = (i < NX) ? fcol[i < NX ? i : 0] : 0.0f;
#pragma unroll
      for (int a = 0; a < NU; ++a)
#pragma unroll
        for (int q = 0; q < FS / 4; ++q) {
          const float4 bv = *reinterpret_cast<const float4*>(Fr + (NX + a) * FS + 4 * q);
          cl[4 * q] += bv.x * kc[a]; cl[4 * q + 1] += bv.y * kc[a];
          cl[4 * q + 2] += bv.z * kc[a]; cl[4 * q + 3] += bv.w * kc[a];
        }
#pragma unroll
      for (int i = NX; i < FS; ++i) cl[i] = 0.0f;
      const int slot = (j == JA) ? NX : j;  // A+BK overwrites A, Bk+c goes to the first B slot
      if (STORE) st_vec<FS>(Fo + slot * FS, cl);
#pragma unroll
      for (int i = 0; i < NX; ++i) sm.Praw[col * LDP + i] = h[i];
      if (ELEM >= 1) {  // Phi <- Phi (A + B K), phi <- phi + Phi (B k + c), G <- G + (Phi B) Quu^-1 (Phi B)'
        const float* Phc = es->Phi[cur];
        float pn[FS];
#pragma unroll
        for (int i = 0; i < FS; ++i) pn[i] = 0.0f;
#pragma unroll
        for (int k = 0; k < NX; ++k) {
          const float ck = cl[k];
#pragma unroll
          for (int q = 0; q < FS / 4; ++q) {
            const float4 pv = *reinterpret_cast<const float4*>(Phc + k * FS + 4 * q);
            pn[4 * q] += pv.x * ck; pn[4 * q + 1] += pv.y * ck; pn[4 * q + 2] += pv.z * ck; pn[4 * q + 3] += pv.w * ck;
          }
        }
        if (j < NX) {
          st_vec<FS>(es->Phi[cur ^ 1] + j * FS, pn);
#pragma unroll
          for (int a = 0; a < (ELEM == 2 ? NU : 0); ++a) {
            const float ya = v[NX + a];
#pragma unroll
            for (int q = 0; q < FS / 4; ++q) {
              const float4 bv = *reinterpret_cast<const float4*>(es->PB + a * FS + 4 * q);
              gcol[4 * q] += bv.x * ya; gcol[4 * q + 1] += bv.y * ya; gcol[4 * q + 2] += bv.z * ya;
              gcol[4 * q + 3] += bv.w * ya;
            }
          }
        } else {
#pragma unroll
          for (int i = 0; i < FS; ++i) gcol[i] += pn[i];  // lane JA carries phi in gcol
        }
      }
    }
    if (ELEM >= 1) cur ^= 1;
    __syncwarp();
    {
      float* Pt = s.P + (size_t)t * NP * LDP;
      if (j < NX) {
        float pc[LDP];
#pragma unroll
        for (int i = 0; i < LDP; ++i) pc[i] = 0.0f;
#pragma unroll
        for (int i = 0; i < NX; ++i) pc[i] = 0.5f * (h[i] + sm.Praw[i * LDP + j]);
        pc[NX] = 0.5f * (h[JA] + sm.Praw[NX * LDP + j]);
#pragma unroll
        for (int i = 0; i < NP; ++i) sm.P[j * LDP + i] = pc[i];
        sm.P[NX * LDP + j] = pc[NX];
        if (STORE) {
          st_vec<LDP>(Pt + j * LDP, pc);
          Pt[NX * LDP + j] = pc[NX];
        }
      } else if (j < LDP) {
        if (STORE) Pt[NX * LDP + j] = 0.0f;  // [NX][NX] and the padding rows of column NX
        if (j == NX) sm.P[NX * LDP + NX] = 0.0f;
      }
    }
    __syncwarp();
    buf ^= 1;
  }
  cp_async_wait<0>();
  if (ELEM >= 1) {
    if (ELEM == 2 && j < NX) st_vec<FS>(es->G + j * FS, gcol);
    if (j == JA) st_vec<FS>(es->phi, gcol);
    if (j == 0) es->cur = cur;
    __syncwarp();
  }
  (void)LD;
}

// ----------------------------------------------------------------- phase 3
// Forward sweep over stages lo .. hi from the state step in sm.dx (set by
// the caller): dx_{t+1} = (A+BK) dx_t + (Bk+c), du_t = K dx_t + k and the
// costates lam_t = P_t dx_t + p_t into the scratch, plus the merit sums.
// c_init is the defect paired with V at stage lo (lane i < n holds row i).
// last: the sweep also writes the costate of stage hi (the horizon's end);
// otherwise stage hi belongs to the next chunk.
template <class M>
__device__ __forceinline__ void forward_sweep(int lo, int hi, bool last, float c_init, const float* V, WarpSmem<M>& sm,
                                              const Scratch<M>& s, int lane, double* a_gd, double* a_lc,
                                              double* a_vc, double* a_cs) {
  typedef Dims<M> D;
  constexpr int NX = D::NX, NU = D::NU, NZ = D::NZ, JA = D::JA, NP = D::NP, LDP = D::LDP, FS = D::FS;
  constexpr int RS = D::RS;
  float c_cur = c_init;
  // stage t's blocks are copied into sm.stg[buf] by cp.async one stage ahead,
  // only what this sweep reads: P's columns 0..n-1, the gradient rows of G
  // and, for t < hi, the gains K and F's closed-loop columns 0..n and its
  // defect column
  constexpr int GG = (NX + NU + 3) / 4 * 4;
  static_assert(D::G_GRAD == 0 && GG <= D::GS, "gradient rows lead the cost data");
  auto stage_in = [&](int t, int b, bool kf) {
    float* d = sm.stg[b];
    cp_async_block<NX * LDP>(d + D::SP, s.P + (size_t)t * NP * LDP, lane);
    cp_async_block<GG>(d + D::SG, s.G + (size_t)t * D::GS, lane);
    if (kf) {
      cp_async_block<NP * NU>(d + D::SK, s.K + (size_t)t * NP * NU, lane);
      cp_async_block<(NX + 1) * FS>(d + D::SF, s.F + (size_t)t * NZ * FS, lane);
      cp_async_block<FS>(d + D::SF + JA * FS, s.F + (size_t)t * NZ * FS + JA * FS, lane);
    }
  };
  const int tend = last ? hi : hi - 1;  // last stage whose costate this sweep writes
  stage_in(lo, 0, lo < hi);
  cp_async_commit();
  int buf = 0;
  float vnext = (lane < NX) ? V[lo * NX + lane] : 0.0f;  // V of the next stage, loaded a stage ahead
  for (int t = lo; t <= tend; ++t) {
    const float vt = vnext;
    if (lane < NX && t + 1 <= tend) vnext = V[(t + 1) * NX + lane];
    if (t + 1 <= tend) stage_in(t + 1, buf ^ 1, t + 1 < hi);
    cp_async_commit();
    cp_async_wait<1>();  // stage t's copies have landed
    __syncwarp();
    const float* Pr = sm.stg[buf] + D::SP;
    const float* Kr = sm.stg[buf] + D::SK;
    const float* Fr = sm.stg[buf] + D::SF;
    const float* Gr = sm.stg[buf] + D::SG;
    if (lane < NX) {
      const float dxi = sm.dx[lane];
      float lam = Pr[lane * LDP + NX];
#pragma unroll
      for (int k = 0; k < NX; ++k) lam += Pr[lane * LDP + k] * sm.dx[k];
      *a_lc += (double)((lam - 2.0f * vt) * c_cur);
      *a_vc += (double)(vt * c_cur);
      *a_cs += (double)(c_cur * c_cur);
      *a_gd += (double)(Gr[D::G_GRAD + lane] * dxi);
      s.L[t * NX + lane] = lam;
      s.dX[t * NX + lane] = dxi;
    }
    if (t == hi) break;
    if (lane < NX || lane == JA) {
      const int col = (lane == JA) ? NX : lane;
      const float sc = (lane == JA) ? 1.0f : sm.dx[col];
      float* rw = sm.red + col * RS;
#pragma unroll
      for (int a = 0; a < NU; ++a) rw[a] = Kr[col * NU + a] * sc;
#pragma unroll
      for (int i = 0; i < NX; ++i) rw[NU + i] = Fr[col * FS + i] * sc;
    }
    __syncwarp();
    float sum = 0.0f;
    if (lane < NU) {
#pragma unroll
      for (int r2 = 0; r2 <= NX; ++r2) sum += sm.red[r2 * RS + lane];
      s.dU[t * NU + lane] = sum;
      *a_gd += (double)(Gr[D::G_GRAD + NX + lane] * sum);
    } else if (lane >= 16 && lane < 16 + NX) {
#pragma unroll
      for (int r2 = 0; r2 <= NX; ++r2) sum += sm.red[r2 * RS + NU + (lane - 16)];
    }
    if (lane < NX) c_cur = Fr[JA * FS + lane];  // defect of stage t pairs with V_{t+1}
    __syncwarp();
    if (lane >= 16 && lane < 16 + NX) sm.dx[lane - 16] = sum;
    __syncwarp();
    buf ^= 1;
  }
  cp_async_wait<0>();
  __syncwarp();
}

// ----------------------------------------------------------------- one instance
// VJP = true: one Gauss-Newton KKT solve at the given (converged) X, U with
// the gradient replaced by -(cotangents), zero defects and dx_0 = 0 -- the
// adjoint system of the implicit-function theorem -- instead of the SQP loop.
template <class M, bool VJP = false>
__device__ void solve_instance(const ModelConst& mc, const SqpParams& sp, const BatchPtrs& bp, int bidx,
                               WarpSmem<M>& sm, float* scr) {
  const int b = bp.slot ? bp.slot[bidx] : bidx;  // pool row of this batch entry
  typedef Dims<M> D;
  constexpr int NX = D::NX, NU = D::NU, NZ = D::NZ, JA = D::JA, NP = D::NP, LDP = D::LDP, FS = D::FS;
  constexpr int LD = D::LD, RS = D::RS;
  static_assert(NU % 4 == 0, "block elimination assumes m divisible by 4");
  static_assert(NX <= 16, "forward reduction assumes n <= 16");
  const int lane = threadIdx.x & 31;
  const int j = lane;
  const int n_max = bp.n_max;
  const int N = bp.horizon ? bp.horizon[b] : n_max;
  if (N < 1 || N > n_max) {  // invalid horizon: report, touch nothing else
    if (bp.status && lane == 0) bp.status[b] = ST_BAD_HORIZON;
    if (bp.first && lane == 0) bp.first[(size_t)bidx * (M::NU + 4) + M::NU + 3] = (float)ST_BAD_HORIZON;
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

  if (!VJP && bp.X_in != bp.X)
    for (int e = lane; e < (N + 1) * NX; e += 32) X[e] = bp.X_in[xo + e];
  if (!VJP && bp.V_in != bp.V)
    for (int e = lane; e < (N + 1) * NX; e += 32) V[e] = bp.V_in[xo + e];
  if (!VJP && bp.U_in != bp.U)
    for (int e = lane; e < N * NU; e += 32) U[e] = bp.U_in[uo + e];
  if (lane < 24) sm.w[lane] = bp.w[(size_t)b * 24 + lane];
  // zero padding rows of the shared P / F columns (read by the float4 products)
  for (int e = lane; e < NP * LDP; e += 32) { sm.P[e] = 0.0f; sm.Praw[e] = 0.0f; }
  for (int e = lane; e < NX * D::FTS; e += 32) sm.FT[e] = 0.0f;
  __syncwarp();

  float rho = sp.rho0;
  int status = 0;

  for (int it = 0; it < (VJP ? 1 : sp.sqp_iters); ++it) {
    // ================================================ phase 1: linearise all stages
    float lsum = 0.0f, dummy = 0.0f;
    for (int t = lane; t <= N; t += 32)
      lin_stage<M, false>(mc, t, N, x0, X, U, V, ref, par, sm.w, s, &lsum, &dummy, &dummy, &dummy);
    const double Jc = warp_sum((double)lsum);
    __syncwarp();
    if (VJP) {  // adjoint right-hand side: gradient <- -cotangent, defects <- 0
      const float* gx = bp.gX + xo;
      const float* gu = bp.gU + uo;
      for (int t = lane; t <= N; t += 32) {
        float* Gt = s.G + (size_t)t * D::GS;
#pragma unroll
        for (int i = 0; i < NX; ++i) Gt[D::G_GRAD + i] = -gx[t * NX + i];
        if (t < N) {
#pragma unroll
          for (int a = 0; a < NU; ++a) Gt[D::G_GRAD + NX + a] = -gu[t * NU + a];
          float* Fa = s.F + (size_t)t * NZ * FS + JA * FS;
#pragma unroll
          for (int i = 0; i < FS; ++i) Fa[i] = 0.0f;
        }
      }
      __syncwarp();
    }
    // ================================================ phase 2: backward Riccati
    riccati_terminal<M, true>(N, sm, s, lane);
    // whole-warp fence: phase-1 stores are complete before the block loads
    __threadfence_block();
    __syncwarp();
    riccati_sweep<M, true, 0>(sp, 0, N, sm, s, nullptr, &status, lane);
    // ================================================ phase 3: forward sweep
    __threadfence_block();
    __syncwarp();
    double a_gd = 0.0, a_lc = 0.0, a_vc = 0.0, a_cs = 0.0;
    if (lane < NX) sm.dx[lane] = VJP ? 0.0f : x0[lane] - X[lane];
    forward_sweep<M>(0, N, true, VJP ? 0.0f : (lane < NX ? x0[lane] - X[lane] : 0.0f), V, sm, s, lane, &a_gd, &a_lc,
                     &a_vc, &a_cs);
    const double gd = warp_sum(a_gd), lc = warp_sum(a_lc), vc = warp_sum(a_vc), cs = warp_sum(a_cs);
    if (VJP) {  // adjoint solution and gradients out; no step is taken
      __threadfence_block();
      __syncwarp();
      float* wx = bp.wX ? bp.wX + xo : nullptr;
      float* wl = bp.wL ? bp.wL + xo : nullptr;
      for (int e = lane; e < (N + 1) * NX; e += 32) {
        if (wx) wx[e] = s.dX[e];
        if (wl) wl[e] = s.L[e];
      }
      if (bp.wU)
        for (int e = lane; e < N * NU; e += 32) bp.wU[uo + e] = s.dU[e];
      if (bp.gx0 && lane < NX) bp.gx0[(size_t)b * NX + lane] = -s.L[lane];  // mu_0 = -lambda_0
      if (bp.gref && M::IDENT_RES) {  // tracking rows: d(grad l)/d(ref) = -W, so g_ref = W w_x
        float* gr = bp.gref + (size_t)b * (n_max + 1) * 12;
        for (int e = lane; e < (N + 1) * 12; e += 32) {
          const int t = e / 12, a = e - 12 * t;
          gr[e] = sm.w[a] * s.dX[t * NX + a];
        }
      }
      break;
    }
    // ================================================ phase 4: merit line search
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
        for (int t = lane; t <= N; t += 32)
          acc += (double)merit_diff_stage<M>(mc, t, N, alpha, rho, x0, X, U, V, s, ref, par, sm.w);
        const double dphi_alpha = warp_sum(acc);  // phi(alpha) - phi(0)
        if (dphi_alpha <= (double)sp.ls_eta * alpha * dphi) { accepted = true; break; }
        if (tr + 1 < sp.ls_max_trials) alpha *= sp.ls_beta;
      }
    }
    if (!accepted) status |= ST_LS_FAIL;
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
      const int t = e / (NU * NX), r2 = e - t * NU * NX, a = r2 / NX, jj = r2 - a * NX;
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
    float rp = 0.0f, rd = 0.0f, gm = 0.0f, lsum = 0.0f;
    for (int t = lane; t <= N; t += 32)
      lin_stage<M, true>(mc, t, N, x0, X, U, V, ref, par, sm.w, s, &lsum, &rp, &rd, &gm);
    rp = warp_max(rp);
    rd = warp_max(rd);
    gm = warp_max(gm);
    if (lane == 0) {
      float* o = bp.kkt + (size_t)b * 3;
      o[0] = rp;
      o[1] = rd / (1.0f + gm);
      o[2] = fmaxf(o[0], o[1]);
      if (bp.first) {
        float* f = bp.first + (size_t)bidx * (NU + 4) + NU;
        f[0] = o[0]; f[1] = o[1]; f[2] = o[2];
      }
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
  if (bp.first) {
    float* f = bp.first + (size_t)bidx * (NU + 4);
    if (lane < NU) f[lane] = U[lane];
    if (lane == 0 && !(bp.kkt && sp.compute_kkt)) { f[NU] = 0.0f; f[NU + 1] = 0.0f; f[NU + 2] = 0.0f; }
    __syncwarp();
    if (lane == 0) {
      // the row's other entries, then its status word: a reader of a row in
      // mapped host memory takes a written status word as the row's arrival
      __threadfence_system();
      *(volatile float*)(f + NU + 3) = (float)status;
    }
  }
  (void)LD;
}

// Two register budgets of the same kernel.  The latency variant (168
// registers, 3 blocks = 12 warps per SM) runs a warp fastest and serves
// batches that fit the grid in one wave and the plain path; the throughput
// variant (per model, 4 blocks = 16 warps per SM for the roll-pitch-yaw
// quadruped: 128 registers) hides more latency across warps and serves
// larger batches: 4-7 % faster there, ~20 % slower per lone warp (spills).
#ifndef MPXG_SQP_MIN_BLOCKS
#define MPXG_SQP_MIN_BLOCKS 3
#endif
template <class M>
struct SqpMinBlocks { static constexpr int value = MPXG_SQP_MIN_BLOCKS; };
#ifndef MPXG_SQP_TPUT_BLOCKS
#define MPXG_SQP_TPUT_BLOCKS 4
#endif
template <>
struct SqpMinBlocks<ModelRpy12> { static constexpr int value = MPXG_SQP_TPUT_BLOCKS; };

template <class M, bool VJP = false>
__device__ __forceinline__ void sqp_body(const ModelConst& mc, const SqpParams& sp, const BatchPtrs& bp) {
  extern __shared__ float4 smem_raw[];
  WarpSmem<M>* sms = reinterpret_cast<WarpSmem<M>*>(smem_raw);
  const int wib = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int gw = blockIdx.x * (blockDim.x >> 5) + wib;
  WarpSmem<M>& sm = sms[wib];
  if (bp.single_instance >= 0 && gw != 0) return;
  int slot = gw;
  if (bp.slot_bits) {
    int s = 0;
    if (lane == 0) s = claim_scratch_slot(bp.slot_bits, bp.n_slots, gw % bp.n_slots);
    slot = __shfl_sync(0xffffffffu, s, 0);
    if (slot < 0) {  // leaves its share of the queue to the other warps
      if (lane == 0 && bp.error) atomicOr(bp.error, 1);
      return;
    }
  }
  float* scr = bp.scratch + (size_t)slot * bp.scratch_stride;
  const int q0 = bp.split ? *bp.split : 0;
  for (int done = 0; !done;) {
    int b = bp.single_instance;
    if (b < 0) {
      if (lane == 0) {
        const int i = q0 + atomicAdd(bp.counter, 1);
        b = (i < bp.batch) ? (bp.order ? bp.order[i] : i) : bp.batch;
      }
      b = __shfl_sync(0xffffffffu, b, 0);
      if (b >= bp.batch) break;
    } else {
      done = 1;
    }
    solve_instance<M, VJP>(mc, sp, bp, b, sm, scr);
  }
  if (bp.slot_bits) {  // release the slot once every lane's scratch writes are visible
    __threadfence();
    __syncwarp();
    if (lane == 0) atomicAnd(&bp.slot_bits[slot >> 5], ~(1u << (slot & 31)));
  }
}

template <class M>
__global__ void __launch_bounds__(128, MPXG_SQP_MIN_BLOCKS) sqp_kernel(ModelConst mc, SqpParams sp, BatchPtrs bp) {
  sqp_body<M>(mc, sp, bp);
}
template <class M>
__global__ void __launch_bounds__(128, SqpMinBlocks<M>::value) sqp_kernel_tput(ModelConst mc, SqpParams sp,
                                                                              BatchPtrs bp) {
  sqp_body<M>(mc, sp, bp);
}
// Vector-Jacobian product of converged solutions (mpxg_solve_vjp).
template <class M>
__global__ void __launch_bounds__(128, MPXG_SQP_MIN_BLOCKS) sqp_vjp_kernel(ModelConst mc, SqpParams sp, BatchPtrs bp) {
  sqp_body<M, true>(mc, sp, bp);
}

}  // namespace mpxg
