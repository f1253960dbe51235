// Mixed-model persistent SQP launch: one grid serves the batches of two
// models (a quadruped and a biped pool of the served stream) from one
// longest-horizon-first queue.  Each warp takes queue entries one at a time
// and solves the entry with its own model's solve_instance -- the same
// device code, in the same order of operations, as that model's one-warp
// kernel -- so an instance's result does not depend on the mix it is solved
// in.  The warp's shared memory and scratch are sized for the larger model.
#pragma once
#include "internal.h"
#include "sqp_kernel.cuh"

namespace mpxg {

template <class MA, class MB>
struct MixedDims {
  static constexpr size_t a = sizeof(WarpSmem<MA>), b = sizeof(WarpSmem<MB>);
  static constexpr size_t smem_per_warp = ((a > b ? a : b) + 15) / 16 * 16;
};

template <class MA, class MB>
__global__ void __launch_bounds__(128, MPXG_SQP_MIN_BLOCKS) sqp_mixed_kernel(const __grid_constant__ MixedArgs p) {
  extern __shared__ float4 smem_raw[];
  constexpr size_t WS = MixedDims<MA, MB>::smem_per_warp;
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gw = blockIdx.x * (blockDim.x >> 5) + wib;
  char* wsm = reinterpret_cast<char*>(smem_raw) + (size_t)wib * WS;
  int slot = 0;
  if (lane == 0) slot = claim_scratch_slot(p.slot_bits, p.n_slots, gw % p.n_slots);
  slot = __shfl_sync(0xffffffffu, slot, 0);
  if (slot < 0) {  // leaves its share of the queue to the other warps
    if (lane == 0 && p.error) atomicOr(p.error, 1);
    return;
  }
  float* scr = p.scratch + (size_t)slot * p.scratch_stride;
  const int na = p.bp[0].batch;
  for (;;) {
    int code = -1;
    if (lane == 0) {
      const int i = atomicAdd(p.counter, 1);
      code = i < p.total ? (p.order ? p.order[i] : i) : -1;
    }
    code = __shfl_sync(0xffffffffu, code, 0);
    if (code < 0) break;
    if (code < na)
      solve_instance<MA>(p.mc[0], p.sp[0], p.bp[0], code, *reinterpret_cast<WarpSmem<MA>*>(wsm), scr);
    else
      solve_instance<MB>(p.mc[1], p.sp[1], p.bp[1], code - na, *reinterpret_cast<WarpSmem<MB>*>(wsm), scr);
    __syncwarp();
  }
  __threadfence();  // release the slot once every lane's scratch writes are visible
  __syncwarp();
  if (lane == 0) atomicAnd(&p.slot_bits[slot >> 5], ~(1u << (slot & 31)));
}

template <class MA, class MB>
struct MixedLaunch {
  static long long scratch(int n_max) {
    const long long a = scratch_floats<MA>(n_max), b = scratch_floats<MB>(n_max);
    return a > b ? a : b;
  }
  static int resident_blocks(int wpb) {
    int nb = 0;
    const size_t smem = MixedDims<MA, MB>::smem_per_warp * (size_t)wpb;
    auto fn = sqp_mixed_kernel<MA, MB>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, wpb * 32, smem) != cudaSuccess) {
      cudaGetLastError();
      return 1;
    }
    return nb > 0 ? nb : 1;
  }
  static cudaError_t launch(const MixedArgs& p, int blocks, int wpb, cudaStream_t st) {
    const size_t smem = MixedDims<MA, MB>::smem_per_warp * (size_t)wpb;
    auto fn = sqp_mixed_kernel<MA, MB>;
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
    }
    fn<<<blocks, wpb * 32, smem, st>>>(p);
    return cudaGetLastError();
  }
  static const MixedOps& ops() {
    static const MixedOps o = {MixedDims<MA, MB>::smem_per_warp, &scratch, &resident_blocks, &launch};
    return o;
  }
};

}  // namespace mpxg
