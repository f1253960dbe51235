// Time-varying LQR in absolute coordinates (the KKT system of one SQP step
// when the problem is already linear-quadratic):
//   x_{t+1} = A_t x_t + B_t u_t + c_t,
//   l_t = 1/2 x'Q x + x'M u + 1/2 u'R u + q'x + r'u,  l_N = 1/2 x'Q_N x + q_N'x.
// One thread block per instance; thread j owns column j of the augmented
// stage matrix H = G + F^T P F (F = [A B c; 0 0 1]) and the m control pivots
// are eliminated by Gauss-Jordan, which leaves the next value function and the
// gains in place (one Riccati step per stage).
#pragma once
#include <cuda_runtime.h>

#include <string>

#include "../../include/mpxg.h"
#include "lqr_scan.cuh"

namespace mpxg {

template <int NX, int NU>
struct LqDims {
  static constexpr int NZ = NX + NU + 1, JA = NX + NU, NP = NX + 1;
  static constexpr int LDP = (NP + 3) / 4 * 4;
  static constexpr int NT = (NZ + 31) / 32 * 32;
};

template <int NX, int NU>
__global__ void lqr_riccati_kernel(mpxg_lq_io io, float* Pscr) {
  typedef LqDims<NX, NU> D;
  constexpr int NZ = D::NZ, JA = D::JA, NP = D::NP, LDP = D::LDP;
  __shared__ __align__(16) float sP[NP * LDP];
  __shared__ __align__(16) float sF[NZ * LDP];
  __shared__ float sCT[NZ * 4];  // the pivot block's columns, row-major [NZ][BS]
  __shared__ float sx[NP + 3], su[NU + 3];
  const int b = blockIdx.x;
  const int j = threadIdx.x;
  const int N = io.N;
  const float* A = io.A + (size_t)b * N * NX * NX;
  const float* Bm = io.Bm + (size_t)b * N * NX * NU;
  const float* c = io.c + (size_t)b * N * NX;
  const float* Q = io.Q + (size_t)b * (N + 1) * NX * NX;
  const float* R = io.R + (size_t)b * N * NU * NU;
  const float* M = io.M + (size_t)b * N * NX * NU;
  const float* q = io.q + (size_t)b * (N + 1) * NX;
  const float* r = io.r + (size_t)b * N * NU;
  float* Ps = Pscr + (size_t)b * (N + 1) * NP * NP;
  // ---- terminal value function
  if (j < NX) {
    const float* QN = Q + (size_t)N * NX * NX;
    for (int i = 0; i < NX; ++i) sP[j * LDP + i] = QN[i * NX + j];
    const float qj = q[(size_t)N * NX + j];
    sP[j * LDP + NX] = qj;
    sP[NX * LDP + j] = qj;
  }
  if (j == 0) sP[NX * LDP + NX] = 0.0f;
  __syncthreads();
  if (j < NP)
    for (int i = 0; i < NP; ++i) Ps[(size_t)N * NP * NP + j * NP + i] = sP[j * LDP + i];
  for (int t = N - 1; t >= 0; --t) {
    // ---- column j of F and G
    float f[NP], g[NZ];
#pragma unroll
    for (int i = 0; i < NP; ++i) f[i] = 0.0f;
#pragma unroll
    for (int i = 0; i < NZ; ++i) g[i] = 0.0f;
    const float* At = A + (size_t)t * NX * NX;
    const float* Bt = Bm + (size_t)t * NX * NU;
    const float* Qt = Q + (size_t)t * NX * NX;
    const float* Rt = R + (size_t)t * NU * NU;
    const float* Mt = M + (size_t)t * NX * NU;
    if (j < NX) {
#pragma unroll
      for (int i = 0; i < NX; ++i) { f[i] = At[i * NX + j]; g[i] = Qt[i * NX + j]; }
#pragma unroll
      for (int a = 0; a < NU; ++a) g[NX + a] = Mt[j * NU + a];
      g[JA] = q[(size_t)t * NX + j];
    } else if (j < JA) {
      const int a = j - NX;
#pragma unroll
      for (int i = 0; i < NX; ++i) { f[i] = Bt[i * NU + a]; g[i] = Mt[i * NU + a]; }
#pragma unroll
      for (int e = 0; e < NU; ++e) g[NX + e] = Rt[e * NU + a];
      g[JA] = r[(size_t)t * NU + a];
    } else if (j == JA) {
#pragma unroll
      for (int i = 0; i < NX; ++i) { f[i] = c[(size_t)t * NX + i]; g[i] = q[(size_t)t * NX + i]; }
#pragma unroll
      for (int a = 0; a < NU; ++a) g[NX + a] = r[(size_t)t * NU + a];
      f[NX] = 1.0f;
    }
    if (j < NZ) {
#pragma unroll
      for (int i = 0; i < NP; ++i) sF[j * LDP + i] = f[i];
    }
    __syncthreads();
    // ---- H[:, j] = G[:, j] + F^T (P F[:, j])
    float tv[NP];
#pragma unroll
    for (int i = 0; i < NP; ++i) tv[i] = 0.0f;
#pragma unroll
    for (int k = 0; k < NP; ++k) {
      const float fk = f[k];
#pragma unroll
      for (int i = 0; i < NP; ++i) tv[i] += sP[k * LDP + i] * fk;
    }
    float h[NZ];
#pragma unroll
    for (int i = 0; i < NZ; ++i) {
      float a = g[i];
#pragma unroll
      for (int k = 0; k < NP; ++k) a += sF[i * LDP + k] * tv[k];
      h[i] = a;
    }
    // ---- Gauss-Jordan on the control pivots, BS at a time: the BS pivot
    // columns are shared once, every thread factors the BS x BS pivot block
    // (Cholesky) and eliminates it from its own column (two barriers per
    // block instead of two per pivot)
    constexpr int BS = (NU % 4 == 0) ? 4 : ((NU % 2 == 0) ? 2 : 1);
#pragma unroll
    for (int s0 = NX; s0 < JA; s0 += BS) {
      __syncthreads();  // every thread is done with the previous block's columns
      if (j >= s0 && j < s0 + BS) {
#pragma unroll
        for (int i = 0; i < NZ; ++i) sCT[i * BS + (j - s0)] = h[i];
      }
      __syncthreads();
      float Lc[BS][BS], il[BS];  // Cholesky factor; il = 1 / diagonal
#pragma unroll
      for (int a = 0; a < BS; ++a) {
        float dsum = sCT[(s0 + a) * BS + a];
#pragma unroll
        for (int k = 0; k < a; ++k) dsum -= Lc[a][k] * Lc[a][k];
        if (!(dsum > 0.0f)) dsum = fmaxf(fabsf(dsum), 1e-20f);
        il[a] = rsqrtf(dsum);
#pragma unroll
        for (int c = a + 1; c < BS; ++c) {
          float v = sCT[(s0 + c) * BS + a];
#pragma unroll
          for (int k = 0; k < a; ++k) v -= Lc[c][k] * Lc[a][k];
          Lc[c][a] = v * il[a];
        }
      }
      float y[BS];
#pragma unroll
      for (int a = 0; a < BS; ++a) {
        float v = h[s0 + a];
#pragma unroll
        for (int k = 0; k < a; ++k) v -= Lc[a][k] * y[k];
        y[a] = v * il[a];
      }
#pragma unroll
      for (int a = BS - 1; a >= 0; --a) {
        float v = y[a];
#pragma unroll
        for (int k = a + 1; k < BS; ++k) v -= Lc[k][a] * y[k];
        y[a] = v * il[a];
      }
#pragma unroll
      for (int i = 0; i < NZ; ++i) {
        if (i >= s0 && i < s0 + BS) {
          h[i] = y[i - s0];
        } else {
          float upd = 0.0f;
#pragma unroll
          for (int a = 0; a < BS; ++a) upd += sCT[i * BS + a] * y[a];
          h[i] -= upd;
        }
      }
    }
    // ---- gains and new value function
    if (j < NX) {
      float* Kt = io.K + ((size_t)b * N + t) * NU * NX;
#pragma unroll
      for (int a = 0; a < NU; ++a) Kt[a * NX + j] = -h[NX + a];
    } else if (j == JA) {
      float* kt = io.k + ((size_t)b * N + t) * NU;
#pragma unroll
      for (int a = 0; a < NU; ++a) kt[a] = -h[NX + a];
    }
    __syncthreads();  // everyone is done reading sP / sF of this stage
    if (j < NX) {
#pragma unroll
      for (int i = 0; i < NX; ++i) sF[j * LDP + i] = h[i];  // reuse sF as the raw (unsymmetrised) P
    } else if (j == JA) {
#pragma unroll
      for (int i = 0; i < NX; ++i) sF[NX * LDP + i] = h[i];
    }
    __syncthreads();
    if (j < NX) {
      float* Pt = Ps + (size_t)t * NP * NP;
#pragma unroll
      for (int i = 0; i < NX; ++i) {
        const float v = 0.5f * (h[i] + sF[i * LDP + j]);
        sP[j * LDP + i] = v;
        Pt[j * NP + i] = v;
      }
      const float pj = 0.5f * (h[JA] + sF[NX * LDP + j]);
      sP[j * LDP + NX] = pj;
      sP[NX * LDP + j] = pj;
      Pt[j * NP + NX] = pj;
      Pt[NX * NP + j] = pj;
    }
    if (j == 0) {
      sP[NX * LDP + NX] = 0.0f;
      Ps[(size_t)t * NP * NP + NX * NP + NX] = 0.0f;
    }
    __syncthreads();
  }
  // ---- forward pass: u = K x + k, lam = P x + p, x+ = A x + B u + c
  if (j < NX) sx[j] = io.x0[(size_t)b * NX + j];
  __syncthreads();
  float* X = io.X + (size_t)b * (N + 1) * NX;
  float* U = io.U + (size_t)b * N * NU;
  float* L = io.lam + (size_t)b * (N + 1) * NX;
  for (int t = 0; t <= N; ++t) {
    const float* Pt = Ps + (size_t)t * NP * NP;
    if (j < NX) {
      float lam = Pt[NX * NP + j];
      for (int k = 0; k < NX; ++k) lam += Pt[k * NP + j] * sx[k];
      L[t * NX + j] = lam;
      X[t * NX + j] = sx[j];
    }
    if (t == N) break;
    if (j < NU) {
      const float* Kt = io.K + ((size_t)b * N + t) * NU * NX;
      float u = io.k[((size_t)b * N + t) * NU + j];
      for (int k = 0; k < NX; ++k) u += Kt[j * NX + k] * sx[k];
      su[j] = u;
      U[t * NU + j] = u;
    }
    __syncthreads();
    float xn = 0.0f;
    if (j < NX) {
      const float* At = A + (size_t)t * NX * NX;
      const float* Bt = Bm + (size_t)t * NX * NU;
      xn = c[(size_t)t * NX + j];
      for (int k = 0; k < NX; ++k) xn += At[j * NX + k] * sx[k];
      for (int a = 0; a < NU; ++a) xn += Bt[j * NU + a] * su[a];
    }
    __syncthreads();
    if (j < NX) sx[j] = xn;
    __syncthreads();
  }
}

// Scratch bytes of the LQR path (value functions for the costate recovery).
inline size_t lqr_scratch_bytes(int batch, int N, int n) { return (size_t)batch * (N + 1) * (n + 1) * (n + 1) * 4; }

template <int NX, int NU>
inline cudaError_t launch_lqr(cudaStream_t st, const mpxg_lq_io& io, float* scr, int method) {
  if (method == 1) {
    const size_t smem = lqscan::scan_smem_bytes<NX, NU>();
    cudaError_t e = cudaFuncSetAttribute(lqscan::lqr_scan_kernel<NX, NU>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    lqscan::lqr_scan_kernel<NX, NU><<<io.batch, lqscan::kWarps * 32, smem, st>>>(io, scr);
  } else {
    lqr_riccati_kernel<NX, NU><<<io.batch, LqDims<NX, NU>::NT, 0, st>>>(io, scr);
  }
  return cudaGetLastError();
}

// Host side of mpxg_lqr_solve (allocates nothing: the value functions used
// for the costates live in the caller's workspace).
inline mpxg_status lqr_solve_host(void* stream, const mpxg_lq_io* io, int method, std::string* err) {
  if (!io || io->batch < 0 || io->N < 1 || !io->A || !io->Bm || !io->c || !io->Q || !io->R || !io->M || !io->q ||
      !io->r || !io->x0 || !io->K || !io->k || !io->X || !io->U || !io->lam || !io->workspace) {
    *err = "mpxg_lqr_solve: bad arguments";
    return MPXG_ERR_INVALID_ARG;
  }
  if (method != 0 && method != 1) {
    *err = "mpxg_lqr_solve: method must be 0 (sequential Riccati) or 1 (associative scan)";
    return MPXG_ERR_UNSUPPORTED;
  }
  if (io->batch == 0) return MPXG_OK;
  float* scr = io->workspace;
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e;
  if (io->n == 24 && io->m == 12) e = launch_lqr<24, 12>(st, *io, scr, method);
  else if (io->n == 12 && io->m == 12) e = launch_lqr<12, 12>(st, *io, scr, method);
  else if (io->n == 8 && io->m == 4) e = launch_lqr<8, 4>(st, *io, scr, method);
  else if (io->n == 4 && io->m == 2) e = launch_lqr<4, 2>(st, *io, scr, method);
  else {
    *err = "mpxg_lqr_solve: (n, m) not instantiated; built sizes: (24,12) (12,12) (8,4) (4,2)";
    return MPXG_ERR_UNSUPPORTED;
  }
  if (e != cudaSuccess) {
    *err = std::string("lqr kernel launch: ") + cudaGetErrorString(e);
    return MPXG_ERR_CUDA;
  }
  return MPXG_OK;
}

}  // namespace mpxg
