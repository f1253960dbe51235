// Device work queue drained by a persistent SQP kernel (mpxg_queue_*): the
// host publishes pool rows into a ring in mapped host memory while the
// kernel runs; each warp claims the next ring entry, waits until the host
// has published it, solves it with solve_instance (the one-warp kernels'
// device code, so the result has the bits mpxg_solve gives) and flags it
// done in mapped host memory.  Every wait is bounded: a warp that waits for
// an entry longer than the queue's idle timeout (%globaltimer) or an
// iteration cap sets QUEUE_TIMEOUT in the status word and returns -- no
// trap, the context stays usable.
#pragma once
#include "sqp_kernel.cuh"

namespace mpxg {

enum { QUEUE_TIMEOUT = 1, QUEUE_NO_SLOT = 2 };

struct QueueArgs {
  const int* entries;   // mapped host ring [capacity]: pool row of ticket i at i % capacity
  const int* tail;      // mapped host: tickets published so far
  const int* stop;      // mapped host: nonzero = exit once no published entry is left
  int* done;            // mapped host ring [capacity]: ticket + 1 once ticket's result is written
  int* status;          // mapped host: QUEUE_* bits
  int* head;            // device: next ticket to claim
  int capacity;
  long long timeout_ns;
};

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ int ld_acquire_sys(const int* p) {
  int v;
  asm volatile("ld.acquire.sys.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_sys(int* p, int v) {
  asm volatile("st.release.sys.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Lane 0: claim the next ticket and wait (bounded) until the host publishes
// it.  Returns its pool row, or -1 (stop requested with nothing left, or the
// wait timed out: QUEUE_TIMEOUT set).
__device__ inline int queue_next(const QueueArgs& q, int* ticket) {
  const int i = atomicAdd(q.head, 1);
  *ticket = i;
  const unsigned long long t0 = global_ns();
  unsigned ns = 256;
  for (int spin = 0; spin < (1 << 24); ++spin) {
    if (ld_acquire_sys(q.tail) > i) return ld_acquire_sys(q.entries + (i % q.capacity));
    if (ld_acquire_sys(q.stop)) return -1;
    if ((long long)(global_ns() - t0) > q.timeout_ns) break;
    __nanosleep(ns);  // back off to 32 us: keeps the idle warps' polls of host memory rare
    ns = ns < 32768 ? 2 * ns : 32768;
  }
  atomicOr(q.status, QUEUE_TIMEOUT);
  return -1;
}

template <class M>
__global__ void __launch_bounds__(128, MPXG_SQP_MIN_BLOCKS) sqp_queue_kernel(ModelConst mc, SqpParams sp, BatchPtrs bp,
                                                                            QueueArgs q) {
  extern __shared__ float4 smem_raw[];
  WarpSmem<M>* sms = reinterpret_cast<WarpSmem<M>*>(smem_raw);
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gw = blockIdx.x * (blockDim.x >> 5) + wib;
  WarpSmem<M>& sm = sms[wib];
  int slot = 0;
  if (lane == 0) slot = claim_scratch_slot(bp.slot_bits, bp.n_slots, gw % bp.n_slots);
  slot = __shfl_sync(0xffffffffu, slot, 0);
  if (slot < 0) {
    if (lane == 0) atomicOr(q.status, QUEUE_NO_SLOT);
    return;
  }
  float* scr = bp.scratch + (size_t)slot * bp.scratch_stride;
  for (;;) {
    int row = -1, ticket = 0;
    if (lane == 0) row = queue_next(q, &ticket);
    row = __shfl_sync(0xffffffffu, row, 0);
    ticket = __shfl_sync(0xffffffffu, ticket, 0);
    if (row < 0 || row >= bp.batch) break;  // (a row outside the pool was refused by the host)
    solve_instance<M>(mc, sp, bp, row, sm, scr);
    __syncwarp();
    if (lane == 0) {
      __threadfence_system();  // the result rows before the done flag
      st_release_sys(q.done + (ticket % q.capacity), ticket + 1);
    }
  }
  __threadfence();
  __syncwarp();
  if (lane == 0) atomicAnd(&bp.slot_bits[slot >> 5], ~(1u << (slot & 31)));
}

}  // namespace mpxg
