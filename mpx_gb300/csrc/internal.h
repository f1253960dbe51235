// Declarations shared by the translation units of libmpxg.so (host code
// only; never installed).  Each model's SQP kernels are compiled in a unit
// of their own (sqp_<model>.cu) and reached through a table of launchers,
// so that the units compile in parallel.
#pragma once
#include <cuda_runtime.h>

#include <string>

#include "../../include/mpxg.h"

namespace mpxg {

struct ModelConst;
struct SqpParams;
struct BatchPtrs;
struct QueueArgs;

// Launchers of one compiled model's kernels.
struct SqpOps {
  size_t smem_per_warp;                         // dynamic shared memory per warp of the SQP kernels
  long long (*scratch_floats)(int n_max);       // per-warp scratch of one solve
  int (*resident_blocks)(int wpb, bool tput);   // blocks per SM of the latency / throughput variant
  // persistent SQP launch (latency variant, or the throughput variant if tput)
  cudaError_t (*launch)(const ModelConst& mc, const SqpParams& sp, const BatchPtrs& bp, int blocks, int wpb,
                        bool tput, cudaStream_t st);
  cudaError_t (*launch_vjp)(const ModelConst& mc, const SqpParams& sp, const BatchPtrs& bp, int blocks, int wpb,
                            cudaStream_t st);
  // time-parallel team kernel, `warps` (4 or 8) warps per instance; occupancy of it
  int (*team_resident_blocks)(int warps);
  cudaError_t (*launch_team)(const ModelConst& mc, const SqpParams& sp, const BatchPtrs& bp, int blocks, int warps,
                             cudaStream_t st);
  cudaError_t (*launch_evaluate)(const ModelConst& mc, int batch, int n_max, const int* horizon, const float* x0,
                                 const float* X, const float* U, const float* reference, const float* parameter,
                                 const float* w, float* g, float* c, cudaStream_t st);
  // persistent kernel draining a device work queue (sqp_queue.cuh)
  cudaError_t (*launch_queue)(const ModelConst& mc, const SqpParams& sp, const BatchPtrs& bp, const QueueArgs& q,
                              int blocks, int wpb, cudaStream_t st);
};

// Launchers of the mixed-model kernel of one model pair (sqp_mixed.cu).
struct MixedArgs;
struct MixedOps {
  size_t smem_per_warp;                    // dynamic shared memory per warp (the larger model's)
  long long (*scratch_floats)(int n_max);  // per-warp scratch (the larger model's)
  int (*resident_blocks)(int wpb);
  cudaError_t (*launch)(const MixedArgs& p, int blocks, int wpb, cudaStream_t st);
};
// The pair's table (null: the pair (model_a, model_b) is not built).
const MixedOps* mixed_ops(int model_a, int model_b);

const SqpOps& sqp_ops_quat13();
const SqpOps& sqp_ops_rpy12();
const SqpOps& sqp_ops_biped12();

// The table of a model id (null for an unknown id).
inline const SqpOps* sqp_ops(int model) {
  switch (model) {
    case MPXG_MODEL_SRBD_QUAT13: return &sqp_ops_quat13();
    case MPXG_MODEL_SRBD_RPY12: return &sqp_ops_rpy12();
    case MPXG_MODEL_BIPED_WRENCH12: return &sqp_ops_biped12();
    default: return nullptr;
  }
}

// Host checks of a whole-body model (wb.cu): null when the whole-body
// kernels can index its shared arrays by the model's fields, else why not.
const char* wb_model_check(const mpxg_wb_model* m);

// The library's last error of this host thread (mpxg_last_error(NULL)).
std::string& lib_error();
inline mpxg_status lib_fail(mpxg_status st, const std::string& msg) {
  lib_error() = msg;
  return st;
}
inline mpxg_status lib_cuda_fail(cudaError_t e, const char* where) {
  return lib_fail(MPXG_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

}  // namespace mpxg
