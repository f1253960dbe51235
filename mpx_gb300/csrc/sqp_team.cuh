// Time-parallel SQP solve: one block of W warps per MPC instance.
//
// For long horizons a lone warp's solve is a chain of N dependent Riccati and
// forward steps (62 % and 20 % of its time at N = 200).  Here the horizon is
// split into W chunks, one per warp, and the KKT step of every SQP iteration
// is solved by the temporal parallelisation of LQR (Saerkkae and
// Garcia-Fernandez, IEEE TAC 2023; the reference claims the same design for
// its absent solver module, README.md:23-24,29):
//
//  2a. every warp but the last runs its chunk's Riccati sweep from a zero
//      terminal cost and accumulates the chunk's element (closed-loop map Phi,
//      phi and the Gramian G of the map's controllability; riccati_sweep with
//      ELEM); the last warp runs its chunk from the true terminal cost;
//  2m. warp 0 combines the elements from the last chunk backwards: the true
//      value function at each chunk start,
//          Z = (I + G P_e)^-1 [Phi | phi - G p_e],
//          P_s = J + Phi' P_e Z_Phi,  p_s = eta + Phi' (P_e z + p_e);
//  2b. every warp but the last re-runs its chunk's sweep from the true value
//      at its end (gains, closed loop and value functions to the scratch) and
//      composes the chunk's true closed-loop affine map x_e = Phi x_s + phi;
//  2f. warp 0 composes those maps from dx_0 = c_0: the state steps at the
//      chunk starts (the forward pass as composed affine maps, consistent
//      with each chunk's own forward sweep);
//  3.  every warp runs its chunk's forward sweep from its boundary state.
//
// The linearisation (phase 1) and the merit line search (phase 4) are
// stage-parallel over all W x 32 lanes.  oracle/chunked_lqr.py restates the
// same algebra in float64; it equals the sequential Riccati recursion.
#pragma once
#include "sqp_kernel.cuh"

namespace mpxg {

template <class M, int W>
struct __align__(16) TeamSmem {
  WarpSmem<M> ws[W];
  ElemSmem<M> el[W];
  float xb[W + 1][16];  // state steps at the chunk starts
  double red[W][4];     // per-warp partial sums
  int bounds[W + 1];    // chunk c covers stages [bounds[c], bounds[c+1])
};

// Sum of one double per thread over the block (the same value on every
// thread: the per-warp partials are added in warp order).
template <int W>
__device__ __forceinline__ double block_sum(double v, double (*red)[4], int k) {
  const int warp = threadIdx.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[warp][k] = v;
  __syncthreads();
  double t = 0.0;
#pragma unroll
  for (int w = 0; w < W; ++w) t += red[w][k];
  return t;
}

// Chunk bounds: the last chunk (solved once, from the true terminal cost)
// is 1.4 times as long as the others (solved twice, the first time with
// the element accumulation, ~1.4 times a plain sweep).
template <int W>
__device__ __forceinline__ void team_bounds(int N, int* bounds) {
  const float unit = (float)N / ((float)(W - 1) + 1.4f);
  bounds[0] = 0;
  for (int c = 1; c < W; ++c) {
    int b = (int)(unit * (float)c + 0.5f);
    b = max(b, bounds[c - 1] + 1);
    b = min(b, N - (W - c));
    bounds[c] = b;
  }
  bounds[W] = N;
}

// Warp 0: combine the chunk elements from the last chunk backwards (true
// value at every chunk start into el[c].Pin; el[c].Z is [Z_Phi | z]).
template <class M, int W>
__device__ __forceinline__ void team_combine(TeamSmem<M, W>& ts, int lane) {
  typedef Dims<M> D;
  constexpr int NX = D::NX, LDP = D::LDP, FS = D::FS;
  static_assert(2 * NX + 1 <= 32, "one lane per column of [S | Phi | phi - G p]");
  float* tmp = ts.ws[0].Praw;  // raw P_s before symmetrisation (warp 0's Riccati scratch, idle here)
  for (int c = W - 2; c >= 0; --c) {
    ElemSmem<M>& el = ts.el[c];
    const float* Pe = ts.el[c + 1].Pin;  // true value at the chunk's end: P_e[i][k] = Pe[k * LDP + i]
    const float* Phi = el.Phi[el.cur];
    // ---- column `lane` of [S | Phi | phi - G p_e], S = I + G P_e (rows NX..FS-1: zero padding)
    float col[FS];
#pragma unroll
    for (int i = NX; i < FS; ++i) col[i] = 0.0f;
    if (lane < NX) {
#pragma unroll
      for (int i = 0; i < NX; ++i) col[i] = (i == lane) ? 1.0f : 0.0f;
#pragma unroll
      for (int k = 0; k < NX; ++k) {
        const float pk = Pe[lane * LDP + k];
#pragma unroll
        for (int i = 0; i < NX; ++i) col[i] += el.G[k * FS + i] * pk;
      }
    } else if (lane < 2 * NX) {
#pragma unroll
      for (int i = 0; i < NX; ++i) col[i] = Phi[(lane - NX) * FS + i];
    } else if (lane == 2 * NX) {
#pragma unroll
      for (int i = 0; i < NX; ++i) col[i] = el.phi[i];
#pragma unroll
      for (int k = 0; k < NX; ++k) {
        const float pk = Pe[NX * LDP + k];
#pragma unroll
        for (int i = 0; i < NX; ++i) col[i] -= el.G[k * FS + i] * pk;
      }
    } else {
#pragma unroll
      for (int i = 0; i < NX; ++i) col[i] = 0.0f;
    }
    // ---- Gauss-Jordan with partial pivoting (S's eigenvalues are real and >= 1)
    float* pcol = el.PB;  // pivot column broadcast (the element's Phi B buffer, no longer needed)
#pragma unroll
    for (int k = 0; k < NX; ++k) {
      int r = k;
      float best = 0.0f;
      if (lane == k) {
        best = fabsf(col[k]);
#pragma unroll
        for (int i = k + 1; i < NX; ++i)
          if (fabsf(col[i]) > best) { best = fabsf(col[i]); r = i; }
      }
      r = __shfl_sync(0xffffffffu, r, k);
      // swap rows k and r in every column
      float ck = 0.0f, cr = 0.0f;
#pragma unroll
      for (int i = 0; i < NX; ++i) { ck = (i == k) ? col[i] : ck; cr = (i == r) ? col[i] : cr; }
#pragma unroll
      for (int i = 0; i < NX; ++i) col[i] = (i == k) ? cr : ((i == r) ? ck : col[i]);
      __syncwarp();
      if (lane == k) {
#pragma unroll
        for (int i = 0; i < NX; ++i) pcol[i] = col[i];
      }
      __syncwarp();
      const float d = pcol[k];
      const float y = col[k] / d;
#pragma unroll
      for (int i = 0; i < NX; ++i) col[i] = (i == k) ? y : col[i] - pcol[i] * y;
    }
    __syncwarp();
    if (lane >= NX && lane <= 2 * NX) st_vec<FS>(el.Z + (lane - NX) * FS, col);
    __syncwarp();
    // ---- P_s = J + Phi' P_e Z_Phi (lane j < NX: column j), p_s = eta + Phi' (P_e z + p_e) (lane NX)
    const float* Js = ts.ws[c].P;  // the chunk's zero-terminal value (J, eta) in the P layout
    if (lane <= NX) {
      float w[NX];
#pragma unroll
      for (int i = 0; i < NX; ++i) w[i] = (lane == NX) ? Pe[NX * LDP + i] : 0.0f;
#pragma unroll
      for (int k = 0; k < NX; ++k) {
        const float zk = el.Z[lane * FS + k];
#pragma unroll
        for (int i = 0; i < NX; ++i) w[i] += Pe[k * LDP + i] * zk;
      }
#pragma unroll
      for (int r2 = 0; r2 < NX; ++r2) {
        float a = Js[lane * LDP + r2];
#pragma unroll
        for (int i = 0; i < NX; ++i) a += Phi[r2 * FS + i] * w[i];
        tmp[lane * LDP + r2] = a;
      }
    }
    __syncwarp();
    float* Pin = el.Pin;
    if (lane < NX) {
#pragma unroll
      for (int i = 0; i < NX; ++i) Pin[lane * LDP + i] = 0.5f * (tmp[lane * LDP + i] + tmp[i * LDP + lane]);
      Pin[lane * LDP + NX] = tmp[NX * LDP + lane];
      Pin[NX * LDP + lane] = tmp[NX * LDP + lane];
#pragma unroll
      for (int i = NX + 1; i < LDP; ++i) Pin[lane * LDP + i] = 0.0f;  // padding rows read by float4 products
    } else if (lane < LDP) {
      Pin[NX * LDP + lane] = 0.0f;  // [NX][NX] and padding rows of column NX
    }
    __syncwarp();
  }
}

// Warp 0: the state steps at the chunk starts, xb[c+1] = Phi_c xb[c] + phi_c
// over the chunks' true closed-loop maps (xb[0] = c_0 given).
template <class M, int W>
__device__ __forceinline__ void team_boundary_states(TeamSmem<M, W>& ts, int lane) {
  typedef Dims<M> D;
  constexpr int NX = D::NX, FS = D::FS;
  for (int c = 0; c + 1 < W; ++c) {
    const ElemSmem<M>& el = ts.el[c];
    const float* Phi = el.Phi[el.cur];
    if (lane < NX) {
      float a = el.phi[lane];
#pragma unroll
      for (int k = 0; k < NX; ++k) a += Phi[k * FS + lane] * ts.xb[c][k];
      ts.xb[c + 1][lane] = a;
    }
    __syncwarp();
  }
}

template <class M, int W>
__device__ void solve_instance_team(const ModelConst& mc, const SqpParams& sp, const BatchPtrs& bp, int bidx,
                                    TeamSmem<M, W>& ts, float* scr) {
  const int b = bp.slot ? bp.slot[bidx] : bidx;
  typedef Dims<M> D;
  constexpr int NX = D::NX, NU = D::NU, NZ = D::NZ, JA = D::JA, NP = D::NP, LDP = D::LDP, FS = D::FS;
  constexpr int NT = 32 * W;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  WarpSmem<M>& sm = ts.ws[warp];
  ElemSmem<M>& el = ts.el[warp];
  const int n_max = bp.n_max;
  const int N = bp.horizon ? bp.horizon[b] : n_max;
  if (N < 1 || N > n_max) {
    if (tid == 0) {
      if (bp.status) bp.status[b] = ST_BAD_HORIZON;
      if (bp.first) bp.first[(size_t)bidx * (NU + 4) + NU + 3] = (float)ST_BAD_HORIZON;
    }
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

  if (bp.X_in != bp.X)
    for (int e = tid; e < (N + 1) * NX; e += NT) X[e] = bp.X_in[xo + e];
  if (bp.V_in != bp.V)
    for (int e = tid; e < (N + 1) * NX; e += NT) V[e] = bp.V_in[xo + e];
  if (bp.U_in != bp.U)
    for (int e = tid; e < N * NU; e += NT) U[e] = bp.U_in[uo + e];
  if (lane < 24) sm.w[lane] = bp.w[(size_t)b * 24 + lane];
  for (int e = lane; e < NP * LDP; e += 32) { sm.P[e] = 0.0f; sm.Praw[e] = 0.0f; }
  for (int e = lane; e < NX * D::FTS; e += 32) sm.FT[e] = 0.0f;
  if (tid == 0) team_bounds<W>(N, ts.bounds);
  __syncthreads();
  const int lo = ts.bounds[warp], hi = ts.bounds[warp + 1];
  const bool last = (warp == W - 1);

  float rho = sp.rho0;
  int status = 0;
  for (int it = 0; it < sp.sqp_iters; ++it) {
    // team_exact_last: the last iteration's KKT step as one sequential sweep
    // over the whole horizon by the last warp (the others idle through it)
    const bool seq = sp.team_exact_last && it + 1 == sp.sqp_iters;
    const int lo_i = seq ? 0 : lo, hi_i = seq ? (last ? N : 0) : hi;
    // ================================================ phase 1: linearise all stages
    float lsum = 0.0f, dummy = 0.0f;
    for (int t = tid; t <= N; t += NT)
      lin_stage<M, false>(mc, t, N, x0, X, U, V, ref, par, sm.w, s, &lsum, &dummy, &dummy, &dummy);
    __threadfence_block();
    const double Jc = block_sum<W>((double)lsum, ts.red, 0);
    // ================================================ phase 2a: chunk elements; the last chunk exactly
    if (last) {
      riccati_terminal<M, true>(N, sm, s, lane);
      riccati_sweep<M, true, 0>(sp, lo_i, hi_i, sm, s, nullptr, &status, lane);
      for (int e = lane; e < NP * LDP; e += 32) el.Pin[e] = sm.P[e];
    } else if (!seq) {
      for (int e = lane; e < NP * LDP; e += 32) sm.P[e] = 0.0f;
      for (int e = lane; e < NX * FS; e += 32) {
        const int cc = e / FS, rr = e - cc * FS;
        el.Phi[0][e] = (rr == cc) ? 1.0f : 0.0f;
      }
      __syncwarp();
      riccati_sweep<M, false, 2>(sp, lo, hi, sm, s, &el, &status, lane);
    }
    if (warp == 0 && lane < NX) ts.xb[0][lane] = x0[lane] - X[lane];
    __syncthreads();
    // ================================================ phase 2m: combine the chunks
    if (warp == 0 && !seq) team_combine<M, W>(ts, lane);
    __syncthreads();
    // ================================================ phase 2b: chunk sweeps from the true values
    if (!last && !seq) {
      const float* Pe = ts.el[warp + 1].Pin;
      for (int e = lane; e < NP * LDP; e += 32) sm.P[e] = Pe[e];
      for (int e = lane; e < NX * FS; e += 32) {
        const int cc = e / FS, rr = e - cc * FS;
        el.Phi[0][e] = (rr == cc) ? 1.0f : 0.0f;
      }
      __syncwarp();
      riccati_sweep<M, true, 1>(sp, lo, hi, sm, s, &el, &status, lane);
    }
    __threadfence_block();
    __syncthreads();
    // ================================================ phase 2f: chunk-boundary states
    if (warp == 0 && !seq) team_boundary_states<M, W>(ts, lane);
    __syncthreads();
    // ================================================ phase 3: chunk forward sweeps
    double a_gd = 0.0, a_lc = 0.0, a_vc = 0.0, a_cs = 0.0;
    if (!seq || last) {
      float c_init = 0.0f;
      if (lane < NX) {
        sm.dx[lane] = ts.xb[seq ? 0 : warp][lane];
        c_init = (lo_i == 0) ? x0[lane] - X[lane] : s.F[(size_t)(lo_i - 1) * NZ * FS + JA * FS + lane];
      }
      forward_sweep<M>(lo_i, hi_i, last, c_init, V, sm, s, lane, &a_gd, &a_lc, &a_vc, &a_cs);
    }
    __threadfence_block();
    const double gd = block_sum<W>(a_gd, ts.red, 0), lc = block_sum<W>(a_lc, ts.red, 1);
    const double vc = block_sum<W>(a_vc, ts.red, 2), cs = block_sum<W>(a_cs, ts.red, 3);
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
        for (int t = tid; t <= N; t += NT)
          acc += (double)merit_diff_stage<M>(mc, t, N, alpha, rho, x0, X, U, V, s, ref, par, sm.w);
        const double dphi_alpha = block_sum<W>(acc, ts.red, 0);
        if (dphi_alpha <= (double)sp.ls_eta * alpha * dphi) { accepted = true; break; }
        if (tr + 1 < sp.ls_max_trials) alpha *= sp.ls_beta;
      }
    }
    if (!accepted) status |= ST_LS_FAIL;
    for (int e = tid; e < (N + 1) * NX; e += NT) {
      X[e] += alpha * s.dX[e];
      V[e] += alpha * (s.L[e] - V[e]);
    }
    for (int e = tid; e < N * NU; e += NT) U[e] += alpha * s.dU[e];
    __threadfence_block();
    __syncthreads();
  }

  // ================================================ gains of the last step
  if (bp.K) {
    float* Ko = bp.K + (size_t)b * n_max * NU * NX;
    for (int e = tid; e < N * NU * NX; e += NT) {
      const int t = e / (NU * NX), r2 = e - t * NU * NX, a = r2 / NX, jj = r2 - a * NX;
      Ko[e] = s.K[(size_t)t * NP * NU + jj * NU + a];
    }
  }
  if (bp.k) {
    float* ko = bp.k + (size_t)b * n_max * NU;
    for (int e = tid; e < N * NU; e += NT) {
      const int t = e / NU, a = e - t * NU;
      ko[e] = s.K[(size_t)t * NP * NU + NX * NU + a];
    }
  }
  // ================================================ KKT residual of the result
  float kk[3] = {0.0f, 0.0f, 0.0f};
  if (bp.kkt && sp.compute_kkt) {
    float rp = 0.0f, rd = 0.0f, gm = 0.0f, lsum = 0.0f;
    for (int t = tid; t <= N; t += NT)
      lin_stage<M, true>(mc, t, N, x0, X, U, V, ref, par, sm.w, s, &lsum, &rp, &rd, &gm);
    rp = warp_max(rp);
    rd = warp_max(rd);
    gm = warp_max(gm);
    __syncthreads();
    if (lane == 0) { ts.red[warp][0] = rp; ts.red[warp][1] = rd; ts.red[warp][2] = gm; }
    __syncthreads();
    for (int w = 0; w < W; ++w) {
      rp = fmaxf(rp, (float)ts.red[w][0]);
      rd = fmaxf(rd, (float)ts.red[w][1]);
      gm = fmaxf(gm, (float)ts.red[w][2]);
    }
    kk[0] = rp;
    kk[1] = rd / (1.0f + gm);
    kk[2] = fmaxf(kk[0], kk[1]);
    if (tid == 0) {
      float* o = bp.kkt + (size_t)b * 3;
      o[0] = kk[0]; o[1] = kk[1]; o[2] = kk[2];
    }
  }
  // ================================================ status
  int bad = 0;
  for (int e = tid; e < (N + 1) * NX; e += NT)
    if (!isfinite(X[e]) || !isfinite(V[e])) bad = 1;
  for (int e = tid; e < N * NU; e += NT)
    if (!isfinite(U[e])) bad = 1;
  // bitwise OR of the status words over the block (__syncthreads_or would give a 0/1 predicate)
  int st = warp_or(status | (bad ? ST_NAN : 0));
  __syncthreads();
  if (lane == 0) ts.red[warp][0] = (double)st;
  __syncthreads();
  st = 0;
  for (int w = 0; w < W; ++w) st |= (int)ts.red[w][0];
  if (bp.status && tid == 0) bp.status[b] = st;
  if (bp.first && warp == 0) {
    float* f = bp.first + (size_t)bidx * (NU + 4);
    if (lane < NU) f[lane] = U[lane];
    if (lane == 0) {
      f[NU] = kk[0]; f[NU + 1] = kk[1]; f[NU + 2] = kk[2];
    }
    __syncwarp();
    if (lane == 0) {  // the status word last (see sqp_kernel.cuh)
      __threadfence_system();
      *(volatile float*)(f + NU + 3) = (float)st;
    }
  }
  __syncthreads();  // the block's shared memory is reused by its next instance
}

// Persistent team launch: each block takes the next instance of the queue
// range [0, *split) (longest horizons first, from order_by_horizon_kernel),
// or [0, batch) when split is null.
template <class M, int W>
__global__ void __launch_bounds__(32 * W, 1) sqp_team_kernel(ModelConst mc, SqpParams sp, BatchPtrs bp) {
  extern __shared__ float4 smem_raw[];
  TeamSmem<M, W>& ts = *reinterpret_cast<TeamSmem<M, W>*>(smem_raw);
  __shared__ int next;
  const int end = bp.split ? *bp.split : bp.batch;
  int slot = blockIdx.x;
  if (bp.slot_bits) {
    if (threadIdx.x == 0) next = claim_scratch_slot(bp.slot_bits, bp.n_slots, blockIdx.x % bp.n_slots);
    __syncthreads();
    slot = next;
    __syncthreads();
    if (slot < 0) {
      if (threadIdx.x == 0 && bp.error) atomicOr(bp.error, 1);
      return;
    }
  }
  float* scr = bp.scratch + (size_t)slot * bp.scratch_stride;
  for (;;) {
    if (threadIdx.x == 0) {
      int i = atomicAdd(bp.counter + 1, 1);
      next = (i < end) ? (bp.order ? bp.order[i] : i) : -1;
    }
    __syncthreads();
    const int b = next;
    __syncthreads();
    if (b < 0) break;
    solve_instance_team<M, W>(mc, sp, bp, b, ts, scr);
  }
  if (bp.slot_bits) {
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) atomicAnd(&bp.slot_bits[slot >> 5], ~(1u << (slot & 31)));
  }
}

}  // namespace mpxg
