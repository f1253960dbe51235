// The launchers of one model's SQP, vector-Jacobian-product and evaluation
// kernels (the SqpOps table of internal.h).  Included by one small unit per
// model, which instantiates them with MPXG_DEFINE_SQP_OPS.
#pragma once
#include "evaluate_kernel.cuh"
#include "internal.h"
#include "sqp_kernel.cuh"
#include "sqp_queue.cuh"
#include "sqp_team.cuh"

namespace mpxg {

template <class M>
struct SqpLaunch {
  // Models whose two register budgets coincide use one kernel for both.
  static void (*kernel(bool tput))(ModelConst, SqpParams, BatchPtrs) {
    if constexpr (SqpMinBlocks<M>::value != MPXG_SQP_MIN_BLOCKS) {
      if (tput) return sqp_kernel_tput<M>;
    }
    return sqp_kernel<M>;
  }
  static long long scratch(int n_max) { return scratch_floats<M>(n_max); }
  static int resident_blocks(int wpb, bool tput) {
    int nb = 0;
    const size_t smem = sizeof(WarpSmem<M>) * (size_t)wpb;
    auto fn = kernel(tput);
    if (smem > 48 * 1024) cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, wpb * 32, smem) != cudaSuccess) {
      cudaGetLastError();
      return 1;
    }
    return nb > 0 ? nb : 1;
  }
  static cudaError_t launch(const ModelConst& mc, const SqpParams& sp, const BatchPtrs& bp, int blocks, int wpb,
                            bool tput, cudaStream_t st) {
    const size_t smem = sizeof(WarpSmem<M>) * (size_t)wpb;
    auto fn = kernel(tput);
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
    }
    fn<<<blocks, wpb * 32, smem, st>>>(mc, sp, bp);
    return cudaGetLastError();
  }
  static cudaError_t launch_vjp(const ModelConst& mc, const SqpParams& sp, const BatchPtrs& bp, int blocks, int wpb,
                                cudaStream_t st) {
    const size_t smem = sizeof(WarpSmem<M>) * (size_t)wpb;
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(sqp_vjp_kernel<M>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
    }
    sqp_vjp_kernel<M><<<blocks, wpb * 32, smem, st>>>(mc, sp, bp);
    return cudaGetLastError();
  }
  // Team kernels of 8 and 4 warps per instance (the horizon in 8 or 4 chunks).
  template <int W>
  static int team_blocks_w() {
    int nb = 0;
    const size_t smem = sizeof(TeamSmem<M, W>);
    auto fn = sqp_team_kernel<M, W>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, 32 * W, smem) != cudaSuccess) {
      cudaGetLastError();
      return 1;
    }
    return nb > 0 ? nb : 1;
  }
  static int team_resident_blocks(int warps) { return warps == 4 ? team_blocks_w<4>() : team_blocks_w<8>(); }
  template <int W>
  static cudaError_t launch_team_w(const ModelConst& mc, const SqpParams& sp, const BatchPtrs& bp, int blocks,
                                   cudaStream_t st) {
    const size_t smem = sizeof(TeamSmem<M, W>);
    auto fn = sqp_team_kernel<M, W>;
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
    }
    fn<<<blocks, 32 * W, smem, st>>>(mc, sp, bp);
    return cudaGetLastError();
  }
  static cudaError_t launch_team(const ModelConst& mc, const SqpParams& sp, const BatchPtrs& bp, int blocks,
                                 int warps, cudaStream_t st) {
    return warps == 4 ? launch_team_w<4>(mc, sp, bp, blocks, st) : launch_team_w<8>(mc, sp, bp, blocks, st);
  }
  static cudaError_t launch_evaluate(const ModelConst& mc, int batch, int n_max, const int* horizon, const float* x0,
                                     const float* X, const float* U, const float* reference, const float* parameter,
                                     const float* w, float* g, float* c, cudaStream_t st) {
    const long long n = (long long)batch * (n_max + 1);
    const int threads = 128;
    const unsigned blocks = (unsigned)((n + threads - 1) / threads);
    evaluate_kernel<M><<<blocks, threads, 0, st>>>(mc, batch, n_max, horizon, x0, X, U, reference, parameter, w, g,
                                                   c);
    return cudaGetLastError();
  }
  static cudaError_t launch_queue(const ModelConst& mc, const SqpParams& sp, const BatchPtrs& bp, const QueueArgs& q,
                                  int blocks, int wpb, cudaStream_t st) {
    const size_t smem = sizeof(WarpSmem<M>) * (size_t)wpb;
    auto fn = sqp_queue_kernel<M>;
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
    }
    fn<<<blocks, wpb * 32, smem, st>>>(mc, sp, bp, q);
    return cudaGetLastError();
  }
  static const SqpOps& ops() {
    static const SqpOps o = {sizeof(WarpSmem<M>), &scratch, &resident_blocks, &launch, &launch_vjp,
                             &team_resident_blocks, &launch_team, &launch_evaluate, &launch_queue};
    return o;
  }
};

}  // namespace mpxg

#define MPXG_DEFINE_SQP_OPS(MODEL, NAME) \
  namespace mpxg {                       \
  const SqpOps& sqp_ops_##NAME() { return SqpLaunch<MODEL>::ops(); } \
  }
