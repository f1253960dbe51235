// Equality-constrained LQ solve of the large linearised problems
// (mpxg_lqr_eq_solve): tensor cores (lqr_eq_tc.cuh) and CUDA cores
// (lqr_eq_kernel.cuh); SQP iterations on top of it (mpxg_lqr_eq_sqp):
// step-problem data and KKT residuals by lqeq_eval_kernel, the full step by
// lqeq_update_kernel.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <string>

#include "../../include/mpxg.h"
#include "internal.h"
#include "lqr_eq_tc.cuh"

using namespace mpxg;

namespace {

constexpr int kEvalThreads = 256;
constexpr int kEvalMaxN = 72, kEvalMaxM = 32, kEvalMaxE = 16;

bool eq_size_built(int n, int m, int ne) {
  return (n == 72 && m == 30 && ne == 12) || (n == 16 && m == 8 && ne == 4) || (n == 8 && m == 5 && ne == 2);
}

const char* eq_io_problem(const mpxg_lq_eq_io* io) {
  if (!io || io->batch < 0 || io->N < 1 || !io->A || !io->Bm || !io->c || !io->Q || !io->R || !io->M || !io->q ||
      !io->r || !io->C || !io->D || !io->e || !io->x0 || !io->K || !io->k || !io->Knu || !io->knu || !io->X ||
      !io->U || !io->lam || !io->nu || !io->workspace)
    return "bad arguments";
  return nullptr;
}

// Step workspace of mpxg_lqr_eq_sqp, offsets in floats, each array on a
// 16-byte boundary: step data c' [B,N,n], q' [B,N+1,n], r' [B,N,m],
// e' [B,N,ne], x0' [B,n]; the step dX [B,N+1,n], dU [B,N,m]; the KKT maxima
// [B,3] (float bits).
struct SqpLayout {
  size_t cs, qs, rs, es, x0s, dX, dU, bits, floats;
};

SqpLayout sqp_layout(int B, int N, int n, int m, int ne) {
  auto pad = [](size_t v) { return (v + 3) & ~size_t(3); };
  SqpLayout L{};
  size_t o = 0;
  L.cs = o;   o += pad((size_t)B * N * n);
  L.qs = o;   o += pad((size_t)B * (N + 1) * n);
  L.rs = o;   o += pad((size_t)B * N * m);
  L.es = o;   o += pad((size_t)B * N * ne);
  L.x0s = o;  o += pad((size_t)B * n);
  L.dX = o;   o += pad((size_t)B * (N + 1) * n);
  L.dU = o;   o += pad((size_t)B * N * m);
  L.bits = o; o += pad((size_t)B * 3);
  L.floats = o;
  return L;
}

struct EqEval {
  int N, n, m, ne;
  const float *A, *Bm, *c, *Q, *R, *M, *q, *r, *C, *D, *e, *x0;
  const float *X, *U, *lam, *nu;
  float *cs, *qs, *rs, *es, *x0s;  // step data (step-data mode)
  unsigned* bits;                   // [B][3] maxima of |primal|, |dual|, |gradient| (KKT mode)
};

// max that keeps a NaN (fmaxf drops it): a non-finite residual must show
__device__ __forceinline__ float nan_max(float a, float b) { return (a > b || a != a) ? a : b; }

__device__ __forceinline__ float warp_sum_f(float v) {
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ float warp_max_f(float v) {
  for (int o = 16; o; o >>= 1) v = nan_max(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// One block per (instance b = blockIdx.x, stage t = blockIdx.y in 0..N).
// Rows (one warp each, lanes along the row): the cost gradient
// g_x = Q x + M u + q, the defect A x + B u + c - x+, the constraint
// residual e - C x - D u.  Columns (one thread each): g_u = M'x + R u + r
// and, for the KKT, the dual residuals g_x + A'lam+ + C'nu - lam (t >= 1;
// lam_0 is the multiplier of x_0 = x0) and g_u + B'lam+ + D'nu.
// KKT = false writes the step problem's data; KKT = true folds the
// residuals' maxima into bits[b] with atomicMax on the float bits (all
// values are >= 0, and a NaN's bits sort above +inf).
template <bool KKT>
__global__ void __launch_bounds__(kEvalThreads) lqeq_eval_kernel(EqEval p) {
  const int b = blockIdx.x, t = blockIdx.y, n = p.n, m = p.m, ne = p.ne, N = p.N;
  const bool mid = t < N;
  __shared__ float x[kEvalMaxN], xn[kEvalMaxN], lx[kEvalMaxN], ln[kEvalMaxN], u[kEvalMaxM], nu[kEvalMaxE];
  __shared__ float red[3][kEvalThreads / 32];
  const size_t s0 = (size_t)b * N + t;        // stage of a [B,N,...] array
  const size_t s1 = (size_t)b * (N + 1) + t;  // stage of a [B,N+1,...] array
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    x[i] = p.X[s1 * n + i];
    if (mid) xn[i] = p.X[(s1 + 1) * n + i];
    if (KKT && mid) ln[i] = p.lam[(s1 + 1) * n + i];
  }
  if (mid)
    for (int i = threadIdx.x; i < m; i += blockDim.x) u[i] = p.U[s0 * m + i];
  if (KKT && mid)
    for (int i = threadIdx.x; i < ne; i += blockDim.x) nu[i] = p.nu[s0 * ne + i];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  float pr = 0.f, du = 0.f, gr = 0.f;
  const int rows = mid ? 2 * n + ne : n;
  for (int row = warp; row < rows; row += nwarps) {
    const float *a, *bm;
    int i;
    if (row < n) {
      i = row;
      a = p.Q + (s1 * n + i) * n;
      bm = mid ? p.M + (s0 * n + i) * m : nullptr;
    } else if (row < 2 * n) {
      i = row - n;
      a = p.A + (s0 * n + i) * n;
      bm = p.Bm + (s0 * n + i) * m;
    } else {
      i = row - 2 * n;
      a = p.C + (s0 * ne + i) * n;
      bm = p.D + (s0 * ne + i) * m;
    }
    float acc = 0.f;
    for (int j = lane; j < n; j += 32) acc = fmaf(a[j], x[j], acc);
    if (bm)
      for (int j = lane; j < m; j += 32) acc = fmaf(bm[j], u[j], acc);
    acc = warp_sum_f(acc);
    if (lane == 0) {
      if (row < n) {
        const float g = acc + p.q[s1 * n + i];
        if (KKT) {
          lx[i] = g;
          gr = nan_max(gr, fabsf(g));
        } else {
          p.qs[s1 * n + i] = g;
        }
      } else if (row < 2 * n) {
        const float d = acc + p.c[s0 * n + i] - xn[i];
        if (KKT) pr = nan_max(pr, fabsf(d));
        else p.cs[s0 * n + i] = d;
      } else {
        const float r = p.e[s0 * ne + i] - acc;
        if (KKT) pr = nan_max(pr, fabsf(r));
        else p.es[s0 * ne + i] = r;
      }
    }
  }
  if (t == 0)
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const float d = p.x0[(size_t)b * n + i] - x[i];
      if (KKT) pr = nan_max(pr, fabsf(d));
      else p.x0s[(size_t)b * n + i] = d;
    }
  if (KKT) __syncthreads();  // lx complete
  const int tid = threadIdx.x;
  if (mid && tid < m) {  // control columns
    const int i = tid;
    float g = p.r[s0 * m + i];
    const float* Mc = p.M + s0 * n * m + i;
    for (int j = 0; j < n; ++j) g = fmaf(Mc[(size_t)j * m], x[j], g);
    const float* Rr = p.R + (s0 * m + i) * m;
    for (int j = 0; j < m; ++j) g = fmaf(Rr[j], u[j], g);
    if (KKT) {
      gr = nan_max(gr, fabsf(g));
      float d = g;
      const float* Bc = p.Bm + s0 * n * m + i;
      for (int j = 0; j < n; ++j) d = fmaf(Bc[(size_t)j * m], ln[j], d);
      const float* Dc = p.D + s0 * ne * m + i;
      for (int k = 0; k < ne; ++k) d = fmaf(Dc[(size_t)k * m], nu[k], d);
      du = nan_max(du, fabsf(d));
    } else {
      p.rs[s0 * m + i] = g;
    }
  }
  if (KKT && t >= 1 && tid >= kEvalMaxM && tid - kEvalMaxM < n) {  // state columns
    const int i = tid - kEvalMaxM;
    float d = lx[i] - p.lam[s1 * n + i];
    if (mid) {
      const float* Ac = p.A + s0 * n * n + i;
      for (int j = 0; j < n; ++j) d = fmaf(Ac[(size_t)j * n], ln[j], d);
      const float* Cc = p.C + s0 * ne * n + i;
      for (int k = 0; k < ne; ++k) d = fmaf(Cc[(size_t)k * n], nu[k], d);
    }
    du = nan_max(du, fabsf(d));
  }
  if (KKT) {
    pr = warp_max_f(pr);
    du = warp_max_f(du);
    gr = warp_max_f(gr);
    if (lane == 0) {
      red[0][warp] = pr;
      red[1][warp] = du;
      red[2][warp] = gr;
    }
    __syncthreads();
    if (tid < 3) {
      float v = 0.f;
      for (int w = 0; w < nwarps; ++w) v = nan_max(v, red[tid][w]);
      atomicMax(p.bits + (size_t)b * 3 + tid, __float_as_uint(v));
    }
  }
}

// kkt[b] = (primal, dual / (1 + max |gradient|), the larger of the two)
__global__ void lqeq_kkt_finish_kernel(int B, const unsigned* bits, float* kkt) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const float pr = __uint_as_float(bits[3 * b]), du = __uint_as_float(bits[3 * b + 1]);
  const float gr = __uint_as_float(bits[3 * b + 2]);
  const float d = du / (1.f + gr);
  kkt[3 * b] = pr;
  kkt[3 * b + 1] = d;
  kkt[3 * b + 2] = nan_max(pr, d);
}

// the full step: X += dX, U += dU
__global__ void lqeq_update_kernel(size_t nx, size_t nu, float* X, const float* dX, float* U, const float* dU) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < nx + nu; i += stride) {
    if (i < nx) X[i] += dX[i];
    else U[i - nx] += dU[i - nx];
  }
}

cudaError_t launch_eq_solve(cudaStream_t st, const mpxg_lq_eq_io& io, bool tcores) {
  if (io.n == 72) return tcores ? lqeq::launch_lqr_eq_tc<72, 30, 12>(st, io) : lqeq::launch_lqr_eq<72, 30, 12>(st, io);
  if (io.n == 16) return tcores ? lqeq::launch_lqr_eq_tc<16, 8, 4>(st, io) : lqeq::launch_lqr_eq<16, 8, 4>(st, io);
  return tcores ? lqeq::launch_lqr_eq_tc<8, 5, 2>(st, io) : lqeq::launch_lqr_eq<8, 5, 2>(st, io);
}

}  // namespace

extern "C" {

size_t mpxg_lqr_eq_workspace_bytes(int batch, int N, int n) {
  if (batch < 0 || N < 1 || n < 1) return 0;
  return lqeq::lqr_eq_scratch_bytes(batch, N, n);
}

mpxg_status mpxg_lqr_eq_solve_method(void* stream, const mpxg_lq_eq_io* io, int method) {
  if (eq_io_problem(io)) return lib_fail(MPXG_ERR_INVALID_ARG, "mpxg_lqr_eq_solve: bad arguments");
  if (method != 0 && method != 1) return lib_fail(MPXG_ERR_INVALID_ARG, "mpxg_lqr_eq_solve: method is 0 or 1");
  if (method == 0 && (reinterpret_cast<uintptr_t>(io->workspace) & 15u) != 0)
    return lib_fail(MPXG_ERR_INVALID_ARG, "mpxg_lqr_eq_solve: workspace must be 16-byte aligned");
  if (!eq_size_built(io->n, io->m, io->n_eq))
    return lib_fail(MPXG_ERR_UNSUPPORTED, "mpxg_lqr_eq_solve: (n, m, n_eq) not built: (72,30,12) (16,8,4) (8,5,2)");
  if (io->batch == 0) return MPXG_OK;
  const cudaError_t e = launch_eq_solve((cudaStream_t)stream, *io, method == 0);
  return e == cudaSuccess ? MPXG_OK : lib_cuda_fail(e, "lqr_eq kernel launch");
}

mpxg_status mpxg_lqr_eq_solve(void* stream, const mpxg_lq_eq_io* io) { return mpxg_lqr_eq_solve_method(stream, io, 0); }

size_t mpxg_lqr_eq_sqp_workspace_bytes(int batch, int N, int n, int m, int n_eq) {
  if (batch < 0 || N < 1 || n < 1 || m < 1 || n_eq < 1) return 0;
  return sqp_layout(batch, N, n, m, n_eq).floats * sizeof(float);
}

mpxg_status mpxg_lqr_eq_sqp(void* stream, const mpxg_lq_eq_sqp_io* io) {
  if (!io || eq_io_problem(&io->lq)) return lib_fail(MPXG_ERR_INVALID_ARG, "mpxg_lqr_eq_sqp: bad arguments");
  const mpxg_lq_eq_io& lq = io->lq;
  if (io->method != 0 && io->method != 1) return lib_fail(MPXG_ERR_INVALID_ARG, "mpxg_lqr_eq_sqp: method is 0 or 1");
  if (io->iters < 0 || io->iters > 100) return lib_fail(MPXG_ERR_INVALID_ARG, "mpxg_lqr_eq_sqp: iters in 0..100");
  if (io->iters == 0 && !io->kkt) return lib_fail(MPXG_ERR_INVALID_ARG, "mpxg_lqr_eq_sqp: iters = 0 needs kkt");
  if (!io->step || (reinterpret_cast<uintptr_t>(io->step) & 15u) != 0 ||
      (io->method == 0 && (reinterpret_cast<uintptr_t>(lq.workspace) & 15u) != 0))
    return lib_fail(MPXG_ERR_INVALID_ARG, "mpxg_lqr_eq_sqp: step and workspace must be 16-byte aligned");
  if (!eq_size_built(lq.n, lq.m, lq.n_eq))
    return lib_fail(MPXG_ERR_UNSUPPORTED, "mpxg_lqr_eq_sqp: (n, m, n_eq) not built: (72,30,12) (16,8,4) (8,5,2)");
  if (lq.N + 1 > 65535) return lib_fail(MPXG_ERR_INVALID_ARG, "mpxg_lqr_eq_sqp: N + 1 > 65535");
  if (lq.batch == 0) return MPXG_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const int B = lq.batch, N = lq.N, n = lq.n, m = lq.m, ne = lq.n_eq;
  const SqpLayout L = sqp_layout(B, N, n, m, ne);
  EqEval ev{N, n, m, ne, lq.A, lq.Bm, lq.c, lq.Q, lq.R, lq.M, lq.q, lq.r, lq.C, lq.D, lq.e, lq.x0,
            lq.X, lq.U, lq.lam, lq.nu,
            io->step + L.cs, io->step + L.qs, io->step + L.rs, io->step + L.es, io->step + L.x0s,
            reinterpret_cast<unsigned*>(io->step + L.bits)};
  // the step problem: the caller's matrices, the step data, the step as the trajectory
  mpxg_lq_eq_io sub = lq;
  sub.c = ev.cs;
  sub.q = ev.qs;
  sub.r = ev.rs;
  sub.e = ev.es;
  sub.x0 = ev.x0s;
  sub.X = io->step + L.dX;
  sub.U = io->step + L.dU;
  const dim3 grid(B, N + 1);
  const size_t nx = (size_t)B * (N + 1) * n, nuu = (size_t)B * N * m;
  const int ublocks = (int)std::min<size_t>((nx + nuu + 255) / 256, 152 * 16);
  cudaError_t e = cudaSuccess;
  for (int it = 0; it < io->iters && e == cudaSuccess; ++it) {
    lqeq_eval_kernel<false><<<grid, kEvalThreads, 0, st>>>(ev);
    if ((e = cudaGetLastError()) != cudaSuccess) break;
    if ((e = launch_eq_solve(st, sub, io->method == 0)) != cudaSuccess) break;
    lqeq_update_kernel<<<ublocks, 256, 0, st>>>(nx, nuu, lq.X, sub.X, lq.U, sub.U);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && io->kkt) {
    e = cudaMemsetAsync(ev.bits, 0, (size_t)B * 3 * sizeof(unsigned), st);
    if (e == cudaSuccess) {
      lqeq_eval_kernel<true><<<grid, kEvalThreads, 0, st>>>(ev);
      lqeq_kkt_finish_kernel<<<(B + 127) / 128, 128, 0, st>>>(B, ev.bits, io->kkt);
      e = cudaGetLastError();
    }
  }
  return e == cudaSuccess ? MPXG_OK : lib_cuda_fail(e, "mpxg_lqr_eq_sqp launch");
}

}  // extern "C"
