// C ABI of libmpxg.so (declared in include/mpxg.h): handle management, the
// host side of the SQP launches (kernels in sqp_<model>.cu), the per-tick
// auxiliary kernels, the allocation-free solve, the XLA targets and the
// serving runtime.  The LQ solves are in lqr.cu and lqr_eq.cu, the
// whole-body kernels in wb.cu.  No torch types cross this boundary.
#include <cuda_runtime.h>

#include <dlfcn.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/mpxg.h"
#include "aux_kernels.cuh"
#include "internal.h"
#include "sqp_kernel.cuh"  // the structs the launchers take; the kernels are compiled in sqp_<model>.cu
#include "sqp_queue.cuh"

using namespace mpxg;

struct mpxg_handle {
  mpxg_problem_desc desc;
  mpxg_solver_opts opts;
  int device = 0;
  int num_sms = 0;
  int warps_per_block = 0, blocks_per_sm = 0, total_warps = 0;  // throughput variant (large batches)
  int blocks_per_sm_lat = 0;                                     // latency variant
  int team_blocks = 0;                 // team kernel: resident blocks (0: no team path)
  int team_warps = 0;                  // warps (horizon chunks) per team instance: 4 or 8
  int team_min_horizon = 0;
  long long scratch_stride = 0;
  int n_slots = 0;                     // scratch slots: most warps resident at once
  float* scratch = nullptr;
  unsigned int* slot_bits = nullptr;   // claimed scratch slots
  int* error = nullptr;                // device error word
  // Work counters, one per solve in flight: kRing for eager solves (reuse
  // waits on the event of the solve that last used the entry) and kRing for
  // solves captured into CUDA graphs.
  static constexpr int kRing = 64, kCounterStride = 32;
  int* counters = nullptr;
  int* orders = nullptr;               // per ring entry: batch_max queue-order entries
  cudaEvent_t ring_ev[kRing] = {};
  bool ring_used[kRing] = {};
  int ring_next = 0, capture_next = 0;
  // With the team path: the team kernel of a solve runs on a side stream,
  // forked from the solve's stream after the ordering kernel and joined
  // before the solve's end, so that it overlaps the one-warp kernel (ring
  // entry r forks and joins with its own events; side stream r % kSide).
  static constexpr int kSide = 32;
  cudaStream_t side[kSide] = {};
  cudaEvent_t fork_ev[2 * kRing] = {}, join_ev[2 * kRing] = {};
  ModelConst mc;
  SqpParams sp;
  std::string err;
};

static thread_local std::string g_lib_err;
std::string& mpxg::lib_error() { return g_lib_err; }

static mpxg_status fail(mpxg_handle* h, mpxg_status st, const std::string& msg) {
  if (h) h->err = msg; else g_lib_err = msg;
  return st;
}
static mpxg_status cuda_fail(mpxg_handle* h, cudaError_t e, const char* where) {
  return fail(h, MPXG_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

static bool model_dims(int model, int* nx, int* nu) {
  switch (model) {
    case MPXG_MODEL_SRBD_QUAT13: *nx = 13; *nu = 12; return true;
    case MPXG_MODEL_SRBD_RPY12: *nx = 12; *nu = 12; return true;
    case MPXG_MODEL_BIPED_WRENCH12: *nx = 12; *nu = 12; return true;
    default: return false;
  }
}

// Scratch slots of a handle: the most warps of its kernel resident at once.
static int scratch_slots(int model, int wpb, int num_sms) {
  const SqpOps* ops = sqp_ops(model);
  if (!ops) return 0;
  const int rb = std::max(ops->resident_blocks(wpb, true), ops->resident_blocks(wpb, false));
  return num_sms * rb * wpb;
}

static long long scratch_stride_for(int model, int n_max) {
  const SqpOps* ops = sqp_ops(model);
  return ops ? ops->scratch_floats(n_max) : 0;
}

// Kernel constants of a model description.
static ModelConst model_const(const mpxg_problem_desc* d) {
  ModelConst mc;
  mc.dt = d->dt; mc.mass = d->mass; mc.inv_mass = 1.0f / d->mass; mc.gravity = d->gravity; mc.mu = d->mu;
  mc.alpha = d->barrier_alpha; mc.sigma = d->barrier_sigma;
  mc.foot_length = d->foot_length; mc.foot_width = d->foot_width;
  mc.barrier_kind = d->barrier_kind; mc.barrier_masked = d->barrier_masked;
  mc.barrier_hess_scale = d->barrier_hess_scale;
  for (int i = 0; i < 9; ++i) { mc.I[i] = d->inertia[i]; mc.Iinv[i] = d->inertia_inv[i]; }
  mc.cone_eps2 = d->cone_eps2 > 0.0f ? d->cone_eps2 : 1e-2f;
  return mc;
}

// Persistent grid: warps_per_block warps per block and as many blocks per SM
// as stay resident (one instance per warp at a time), for the throughput
// variant (*bps) and the latency variant (*bps_lat).
static void launch_geometry(const mpxg_problem_desc* d, const mpxg_solver_opts* o, int* wpb, int* bps,
                            int* bps_lat = nullptr) {
  *wpb = (o && o->warps_per_block > 0) ? o->warps_per_block : 4;
  int t = 1, l = 1;
  if (const SqpOps* ops = sqp_ops(d->model)) {
    t = ops->resident_blocks(*wpb, true);
    l = ops->resident_blocks(*wpb, false);
  }
  if (o && o->blocks_per_sm > 0) t = l = o->blocks_per_sm;
  *bps = t;
  if (bps_lat) *bps_lat = l;
}

extern "C" {

int mpxg_version(void) { return 100; }

const char* mpxg_status_string(int st) {
  switch (st) {
    case MPXG_OK: return "ok";
    case MPXG_ERR_INVALID_ARG: return "invalid argument";
    case MPXG_ERR_OUT_OF_MEMORY: return "out of device memory";
    case MPXG_ERR_BUDGET: return "device-memory budget exhausted";
    case MPXG_ERR_CUDA: return "CUDA error";
    case MPXG_ERR_TIMEOUT: return "timeout";
    case MPXG_ERR_NUMERICAL: return "numerical failure";
    case MPXG_ERR_NOT_READY: return "not ready";
    case MPXG_ERR_UNSUPPORTED: return "unsupported";
    default: return "unknown status";
  }
}

const char* mpxg_last_error(const mpxg_handle* h) { return h ? h->err.c_str() : g_lib_err.c_str(); }

size_t mpxg_workspace_bytes(const mpxg_problem_desc* d, const mpxg_solver_opts* o) {
  if (!d) return 0;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  int wpb, bps;
  launch_geometry(d, o, &wpb, &bps);
  const long long stride = scratch_stride_for(d->model, d->n_max);
  const size_t slots = (size_t)scratch_slots(d->model, wpb, sms);
  return (size_t)stride * sizeof(float) * slots + (slots + 31) / 32 * 4 + 256 +
         (size_t)2 * mpxg_handle::kRing * (mpxg_handle::kCounterStride + (size_t)d->batch_max) * sizeof(int);
}

mpxg_status mpxg_create(const mpxg_problem_desc* d, const mpxg_solver_opts* o, mpxg_handle** out) {
  if (!d || !o || !out) return fail(nullptr, MPXG_ERR_INVALID_ARG, "mpxg_create: null argument");
  *out = nullptr;
  int nx, nu;
  if (!model_dims(d->model, &nx, &nu)) return fail(nullptr, MPXG_ERR_UNSUPPORTED, "mpxg_create: unknown model id");
  if (d->n != nx || d->m != nu) return fail(nullptr, MPXG_ERR_INVALID_ARG, "mpxg_create: n/m do not match the model");
  if (d->n_max < 1 || d->n_max > 4096) return fail(nullptr, MPXG_ERR_INVALID_ARG, "mpxg_create: n_max out of range");
  if (d->batch_max < 1) return fail(nullptr, MPXG_ERR_INVALID_ARG, "mpxg_create: batch_max < 1");
  if (o->sqp_iters < 0 || o->ls_max_trials < 1) return fail(nullptr, MPXG_ERR_INVALID_ARG, "mpxg_create: bad options");
  if (o->warps_per_block < 0 || o->warps_per_block > 4 || o->blocks_per_sm < 0)
    return fail(nullptr, MPXG_ERR_INVALID_ARG, "mpxg_create: warps_per_block must be 0..4 (128-thread blocks)");
  if (!(o->team_warps == 0 || o->team_warps == 1 || o->team_warps == 4 || o->team_warps == 8) ||
      o->team_min_horizon < 0)
    return fail(nullptr, MPXG_ERR_INVALID_ARG,
                "mpxg_create: team_warps must be 0, 1, 4 or 8 and team_min_horizon >= 0");
  if (!(d->dt > 0.0f) || !(d->mass > 0.0f)) return fail(nullptr, MPXG_ERR_INVALID_ARG, "mpxg_create: dt and mass must be > 0");
  mpxg_handle* h = new mpxg_handle();
  h->desc = *d;
  h->opts = *o;
  cudaError_t e = cudaGetDevice(&h->device);
  if (e != cudaSuccess) { delete h; return cuda_fail(nullptr, e, "cudaGetDevice"); }
  e = cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, h->device);
  if (e != cudaSuccess) { delete h; return cuda_fail(nullptr, e, "cudaDeviceGetAttribute"); }
  launch_geometry(d, o, &h->warps_per_block, &h->blocks_per_sm, &h->blocks_per_sm_lat);
  h->total_warps = h->num_sms * h->blocks_per_sm * h->warps_per_block;
  if (o->team_warps == 4 || o->team_warps == 8) {
    // the team kernel needs at least one stage per warp
    h->team_warps = o->team_warps;
    h->team_min_horizon = std::max(o->team_min_horizon, o->team_warps);
    h->team_blocks = h->num_sms * sqp_ops(d->model)->team_resident_blocks(o->team_warps);
  }
  h->scratch_stride = scratch_stride_for(d->model, d->n_max);
  h->n_slots = scratch_slots(d->model, h->warps_per_block, h->num_sms);
  const size_t bytes = (size_t)h->scratch_stride * sizeof(float) * (size_t)h->n_slots;
  const size_t nwords = ((size_t)h->n_slots + 31) / 32;
  const size_t ctr_bytes = (size_t)2 * mpxg_handle::kRing * mpxg_handle::kCounterStride * sizeof(int);
  const size_t order_bytes = (size_t)2 * mpxg_handle::kRing * (size_t)d->batch_max * sizeof(int);
  if (cudaMalloc(&h->scratch, bytes) != cudaSuccess || cudaMalloc(&h->slot_bits, nwords * 4 + 256) != cudaSuccess ||
      cudaMalloc(&h->counters, ctr_bytes) != cudaSuccess || cudaMalloc(&h->orders, order_bytes) != cudaSuccess) {
    cudaGetLastError();
    mpxg_destroy(h);
    return fail(nullptr, MPXG_ERR_OUT_OF_MEMORY, "mpxg_create: scratch allocation failed");
  }
  h->error = reinterpret_cast<int*>(h->slot_bits + nwords);
  for (int i = 0; i < mpxg_handle::kRing; ++i) {
    if (cudaEventCreateWithFlags(&h->ring_ev[i], cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      mpxg_destroy(h);
      return fail(nullptr, MPXG_ERR_CUDA, "mpxg_create: cudaEventCreate failed");
    }
  }
  if (h->team_blocks > 0) {
    bool ok = true;
    for (int i = 0; i < mpxg_handle::kSide && ok; ++i)
      ok = cudaStreamCreateWithFlags(&h->side[i], cudaStreamNonBlocking) == cudaSuccess;
    for (int i = 0; i < 2 * mpxg_handle::kRing && ok; ++i)
      ok = cudaEventCreateWithFlags(&h->fork_ev[i], cudaEventDisableTiming) == cudaSuccess &&
           cudaEventCreateWithFlags(&h->join_ev[i], cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
      cudaGetLastError();
      mpxg_destroy(h);
      return fail(nullptr, MPXG_ERR_CUDA, "mpxg_create: side stream or event creation failed");
    }
  }
  e = cudaMemset(h->slot_bits, 0, nwords * 4 + 256);
  if (e == cudaSuccess) e = cudaMemset(h->counters, 0, ctr_bytes);
  if (e != cudaSuccess) { mpxg_destroy(h); return cuda_fail(nullptr, e, "mpxg_create: cudaMemset"); }
  h->mc = model_const(d);
  SqpParams& sp = h->sp;
  sp.sqp_iters = o->sqp_iters; sp.ls_max_trials = o->ls_max_trials; sp.ls_beta = o->ls_beta; sp.ls_eta = o->ls_eta;
  sp.reg = o->reg; sp.rho0 = o->rho0; sp.ls_skip_tol = o->ls_skip_tol; sp.compute_kkt = o->compute_kkt;
  sp.team_exact_last = o->team_exact_last;
  *out = h;
  return MPXG_OK;
}

/* Launch geometry chosen for a handle: warps per block, blocks per SM, SMs. */
mpxg_status mpxg_query_geometry(const mpxg_handle* h, int* warps_per_block, int* blocks_per_sm, int* num_sms) {
  if (!h || !warps_per_block || !blocks_per_sm || !num_sms) return MPXG_ERR_INVALID_ARG;
  *warps_per_block = h->warps_per_block;
  *blocks_per_sm = h->blocks_per_sm;
  *num_sms = h->num_sms;
  return MPXG_OK;
}

void mpxg_destroy(mpxg_handle* h) {
  if (!h) return;
  if (h->scratch) cudaFree(h->scratch);
  if (h->slot_bits) cudaFree(h->slot_bits);
  if (h->counters) cudaFree(h->counters);
  if (h->orders) cudaFree(h->orders);
  for (int i = 0; i < mpxg_handle::kRing; ++i)
    if (h->ring_ev[i]) cudaEventDestroy(h->ring_ev[i]);
  for (int i = 0; i < 2 * mpxg_handle::kRing; ++i) {
    if (h->fork_ev[i]) cudaEventDestroy(h->fork_ev[i]);
    if (h->join_ev[i]) cudaEventDestroy(h->join_ev[i]);
  }
  for (int i = 0; i < mpxg_handle::kSide; ++i)
    if (h->side[i]) cudaStreamDestroy(h->side[i]);
  delete h;
}

}  // extern "C"

static mpxg_status dispatch(mpxg_handle* h, cudaStream_t st, const BatchPtrs& bp, int blocks, int wpb,
                            bool tput = false) {
  const SqpOps* ops = sqp_ops(h->desc.model);
  if (!ops) return fail(h, MPXG_ERR_UNSUPPORTED, "model");
  const cudaError_t e = ops->launch(h->mc, h->sp, bp, blocks, wpb, tput, st);
  return e == cudaSuccess ? MPXG_OK : cuda_fail(h, e, "sqp_kernel launch");
}

static mpxg_status check_io(mpxg_handle* h, const mpxg_batch_io* io) {
  if (!h) return fail(nullptr, MPXG_ERR_INVALID_ARG, "null handle");
  if (!io) return fail(h, MPXG_ERR_INVALID_ARG, "null io");
  if (io->batch < 0 || io->batch > h->desc.batch_max) return fail(h, MPXG_ERR_INVALID_ARG, "batch exceeds batch_max");
  if (io->batch > 0 && (!io->x0 || !io->X_in || !io->U_in || !io->V_in || !io->reference || !io->parameter ||
                        !io->w || !io->X || !io->U || !io->V))
    return fail(h, MPXG_ERR_INVALID_ARG, "required pointer is null");
  return MPXG_OK;
}

static BatchPtrs make_ptrs(mpxg_handle* h, const mpxg_batch_io* io) {
  BatchPtrs bp;
  bp.batch = io->batch; bp.n_max = h->desc.n_max; bp.slot = io->slot; bp.horizon = io->horizon;
  bp.x0 = io->x0; bp.X_in = io->X_in; bp.U_in = io->U_in; bp.V_in = io->V_in;
  bp.ref = io->reference; bp.par = io->parameter; bp.w = io->w;
  bp.X = io->X; bp.U = io->U; bp.V = io->V; bp.K = io->K; bp.k = io->k; bp.kkt = io->kkt; bp.status = io->status;
  bp.first = io->first;
  bp.counter = nullptr; bp.scratch = h->scratch; bp.scratch_stride = h->scratch_stride;
  bp.single_instance = -1;
  bp.slot_bits = h->slot_bits; bp.n_slots = h->n_slots; bp.error = h->error;
  return bp;
}

extern "C" {

mpxg_status mpxg_solve(mpxg_handle* h, void* stream, const mpxg_batch_io* io) {
  mpxg_status s = check_io(h, io);
  if (s != MPXG_OK) return s;
  if (io->batch == 0) return MPXG_OK;
  cudaStream_t st = (cudaStream_t)stream;
  BatchPtrs bp = make_ptrs(h, io);
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cap) != cudaSuccess) {
    cudaGetLastError();
    return fail(h, MPXG_ERR_CUDA, "mpxg_solve: cudaStreamIsCapturing failed");
  }
  const bool eager = cap == cudaStreamCaptureStatusNone;
  int r;
  if (eager) {
    r = h->ring_next;
    h->ring_next = (r + 1) % mpxg_handle::kRing;
    if (h->ring_used[r]) {  // the solve that last used this counter has finished
      cudaError_t e = cudaStreamWaitEvent(st, h->ring_ev[r], 0);
      if (e != cudaSuccess) return cuda_fail(h, e, "cudaStreamWaitEvent");
    }
  } else {
    r = mpxg_handle::kRing + h->capture_next;
    h->capture_next = (h->capture_next + 1) % mpxg_handle::kRing;
  }
  bp.counter = h->counters + (size_t)r * mpxg_handle::kCounterStride;
  cudaError_t e = cudaMemsetAsync(bp.counter, 0, 3 * sizeof(int), st);  // warp queue, team queue, split
  if (e != cudaSuccess) return cuda_fail(h, e, "cudaMemsetAsync");
  // time-parallel team path for the long horizons (by horizon alone)
  const bool team = h->team_blocks > 0 && h->team_min_horizon <= h->desc.n_max;
  if (io->horizon && (io->batch > h->total_warps || team)) {  // longest horizons first (and the team's share)
    int* order = h->orders + (size_t)r * h->desc.batch_max;
    order_by_horizon_kernel<<<1, 1024, (size_t)(h->desc.n_max + 1) * sizeof(int), st>>>(
        io->batch, h->desc.n_max, io->slot, io->horizon, order, team ? h->team_min_horizon : 0,
        team ? bp.counter + 2 : nullptr);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(h, e, "order_by_horizon_kernel launch");
    bp.order = order;
  }
  bool joined = true;
  if (team) {
    BatchPtrs tb = bp;
    tb.split = io->horizon ? bp.counter + 2 : nullptr;  // no horizons: every instance has n_max >= the minimum
    const int blocks = std::min(io->batch, h->team_blocks);
    cudaStream_t ts = st;
    if (io->horizon) {  // both kernels may have work: the team kernel on a side stream, overlapping
      ts = h->side[r % mpxg_handle::kSide];
      e = cudaEventRecord(h->fork_ev[r], st);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(ts, h->fork_ev[r], 0);
      if (e != cudaSuccess) return cuda_fail(h, e, "mpxg_solve: fork");
      joined = false;
    }
    e = sqp_ops(h->desc.model)->launch_team(h->mc, h->sp, tb, blocks, h->team_warps, ts);
    if (e != cudaSuccess) return cuda_fail(h, e, "sqp_team_kernel launch");
    if (!joined) {
      e = cudaEventRecord(h->join_ev[r], ts);
      if (e != cudaSuccess) return cuda_fail(h, e, "mpxg_solve: join");
    }
    if (!io->horizon) {  // every instance went to the team kernel
      if (!eager) return MPXG_OK;
      e = cudaEventRecord(h->ring_ev[r], st);
      if (e != cudaSuccess) return cuda_fail(h, e, "cudaEventRecord");
      h->ring_used[r] = true;
      return MPXG_OK;
    }
    bp.split = bp.counter + 2;
  }
  const int wpb = h->warps_per_block;
  // more instances than the latency variant's resident warps: throughput variant
  const bool tput = io->batch > h->num_sms * h->blocks_per_sm_lat * wpb;
  int blocks = h->num_sms * (tput ? h->blocks_per_sm : h->blocks_per_sm_lat);
  const int need = (io->batch + wpb - 1) / wpb;
  if (need < blocks) blocks = need;
  mpxg_status s2 = dispatch(h, st, bp, blocks, wpb, tput);
  if (!joined) {  // the solve ends when both kernels have
    e = cudaStreamWaitEvent(st, h->join_ev[r], 0);
    if (e != cudaSuccess) return cuda_fail(h, e, "mpxg_solve: join wait");
  }
  if (s2 != MPXG_OK || !eager) return s2;
  e = cudaEventRecord(h->ring_ev[r], st);
  if (e != cudaSuccess) return cuda_fail(h, e, "cudaEventRecord");
  h->ring_used[r] = true;
  return MPXG_OK;
}

mpxg_status mpxg_solve_plain(mpxg_handle* h, void* stream, const mpxg_batch_io* io) {
  mpxg_status s = check_io(h, io);
  if (s != MPXG_OK) return s;
  cudaStream_t st = (cudaStream_t)stream;
  BatchPtrs bp = make_ptrs(h, io);
  for (int b = 0; b < io->batch; ++b) {
    bp.single_instance = b;
    s = dispatch(h, st, bp, 1, 1);
    if (s != MPXG_OK) return s;
  }
  return MPXG_OK;
}

}  // extern "C"

// A mixed-model launcher: the scratch, slot bitmap and work counters of the
// pair's kernel (the handles keep their own for their single-model solves).
struct mpxg_mixed {
  mpxg_handle* h[2] = {nullptr, nullptr};
  const MixedOps* ops = nullptr;
  int num_sms = 0, wpb = 4, blocks_per_sm = 0, n_slots = 0;
  long long scratch_stride = 0;
  float* scratch = nullptr;
  unsigned int* slot_bits = nullptr;
  int* error = nullptr;
  static constexpr int kRing = 64, kCounterStride = 32;
  int* counters = nullptr;  // 2 kRing entries: eager solves, then captured ones
  int* orders = nullptr;    // per entry: batch_max(a) + batch_max(b) queue codes
  int order_stride = 0;
  cudaEvent_t ring_ev[kRing] = {};
  bool ring_used[kRing] = {};
  int ring_next = 0, capture_next = 0;
};

extern "C" {

void mpxg_mixed_destroy(mpxg_mixed* mx) {
  if (!mx) return;
  if (mx->scratch) cudaFree(mx->scratch);
  if (mx->slot_bits) cudaFree(mx->slot_bits);
  if (mx->counters) cudaFree(mx->counters);
  if (mx->orders) cudaFree(mx->orders);
  for (int i = 0; i < mpxg_mixed::kRing; ++i)
    if (mx->ring_ev[i]) cudaEventDestroy(mx->ring_ev[i]);
  delete mx;
}

mpxg_status mpxg_mixed_create(mpxg_handle* a, mpxg_handle* b, mpxg_mixed** out) {
  if (!a || !b || !out) return fail(nullptr, MPXG_ERR_INVALID_ARG, "mpxg_mixed_create: null argument");
  *out = nullptr;
  const MixedOps* ops = mixed_ops(a->desc.model, b->desc.model);
  if (!ops)
    return fail(nullptr, MPXG_ERR_UNSUPPORTED,
                "mpxg_mixed_create: model pair not built (SRBD_RPY12 or SRBD_QUAT13 with BIPED_WRENCH12)");
  if (a->desc.n_max != b->desc.n_max || a->device != b->device)
    return fail(nullptr, MPXG_ERR_INVALID_ARG, "mpxg_mixed_create: the handles must share n_max and the device");
  mpxg_mixed* mx = new mpxg_mixed();
  mx->h[0] = a;
  mx->h[1] = b;
  mx->ops = ops;
  mx->num_sms = a->num_sms;
  mx->blocks_per_sm = ops->resident_blocks(mx->wpb);
  mx->n_slots = mx->num_sms * mx->blocks_per_sm * mx->wpb;
  mx->scratch_stride = ops->scratch_floats(a->desc.n_max);
  mx->order_stride = a->desc.batch_max + b->desc.batch_max;
  const size_t nwords = ((size_t)mx->n_slots + 31) / 32;
  const size_t ctr_bytes = (size_t)2 * mpxg_mixed::kRing * mpxg_mixed::kCounterStride * sizeof(int);
  const size_t order_bytes = (size_t)2 * mpxg_mixed::kRing * (size_t)mx->order_stride * sizeof(int);
  if (cudaMalloc(&mx->scratch, (size_t)mx->scratch_stride * sizeof(float) * (size_t)mx->n_slots) != cudaSuccess ||
      cudaMalloc(&mx->slot_bits, nwords * 4 + 256) != cudaSuccess ||
      cudaMalloc(&mx->counters, ctr_bytes) != cudaSuccess || cudaMalloc(&mx->orders, order_bytes) != cudaSuccess) {
    cudaGetLastError();
    mpxg_mixed_destroy(mx);
    return fail(nullptr, MPXG_ERR_OUT_OF_MEMORY, "mpxg_mixed_create: scratch allocation failed");
  }
  mx->error = reinterpret_cast<int*>(mx->slot_bits + nwords);
  for (int i = 0; i < mpxg_mixed::kRing; ++i)
    if (cudaEventCreateWithFlags(&mx->ring_ev[i], cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      mpxg_mixed_destroy(mx);
      return fail(nullptr, MPXG_ERR_CUDA, "mpxg_mixed_create: cudaEventCreate failed");
    }
  cudaError_t e = cudaMemset(mx->slot_bits, 0, nwords * 4 + 256);
  if (e == cudaSuccess) e = cudaMemset(mx->counters, 0, ctr_bytes);
  if (e != cudaSuccess) {
    mpxg_mixed_destroy(mx);
    return cuda_fail(nullptr, e, "mpxg_mixed_create: cudaMemset");
  }
  *out = mx;
  return MPXG_OK;
}

mpxg_status mpxg_solve_mixed(mpxg_mixed* mx, void* stream, const mpxg_batch_io* io_a, const mpxg_batch_io* io_b) {
  if (!mx) return fail(nullptr, MPXG_ERR_INVALID_ARG, "mpxg_solve_mixed: null handle");
  mpxg_handle* ha = mx->h[0];
  mpxg_handle* hb = mx->h[1];
  mpxg_status s = check_io(ha, io_a);
  if (s != MPXG_OK) return fail(nullptr, s, std::string("mpxg_solve_mixed: first batch: ") + ha->err);
  s = check_io(hb, io_b);
  if (s != MPXG_OK) return fail(nullptr, s, std::string("mpxg_solve_mixed: second batch: ") + hb->err);
  const int total = io_a->batch + io_b->batch;
  if (total == 0) return MPXG_OK;
  cudaStream_t st = (cudaStream_t)stream;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cap) != cudaSuccess) {
    cudaGetLastError();
    return fail(nullptr, MPXG_ERR_CUDA, "mpxg_solve_mixed: cudaStreamIsCapturing failed");
  }
  const bool eager = cap == cudaStreamCaptureStatusNone;
  int r;
  if (eager) {
    r = mx->ring_next;
    mx->ring_next = (r + 1) % mpxg_mixed::kRing;
    if (mx->ring_used[r]) {  // the solve that last used this entry has finished
      cudaError_t e = cudaStreamWaitEvent(st, mx->ring_ev[r], 0);
      if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaStreamWaitEvent");
    }
  } else {
    r = mpxg_mixed::kRing + mx->capture_next;
    mx->capture_next = (mx->capture_next + 1) % mpxg_mixed::kRing;
  }
  MixedArgs p;
  p.mc[0] = ha->mc; p.mc[1] = hb->mc;
  p.sp[0] = ha->sp; p.sp[1] = hb->sp;
  p.bp[0] = make_ptrs(ha, io_a);
  p.bp[1] = make_ptrs(hb, io_b);
  p.total = total;
  p.counter = mx->counters + (size_t)r * mpxg_mixed::kCounterStride;
  p.scratch = mx->scratch;
  p.scratch_stride = mx->scratch_stride;
  p.slot_bits = mx->slot_bits;
  p.n_slots = mx->n_slots;
  p.error = mx->error;
  p.order = nullptr;
  cudaError_t e = cudaMemsetAsync(p.counter, 0, sizeof(int), st);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaMemsetAsync");
  if ((io_a->batch == 0 || io_a->horizon) && (io_b->batch == 0 || io_b->horizon)) {  // longest first, both batches
    int* order = mx->orders + (size_t)r * mx->order_stride;
    const int n_max = ha->desc.n_max;
    order_by_horizon_kernel<<<1, 1024, (size_t)(n_max + 1) * sizeof(int), st>>>(
        io_a->batch, n_max, io_a->slot, io_a->horizon, order, 0, nullptr, io_b->batch, io_b->slot, io_b->horizon);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "order_by_horizon_kernel launch");
    p.order = order;
  }
  int blocks = mx->num_sms * mx->blocks_per_sm;
  const int need = (total + mx->wpb - 1) / mx->wpb;
  if (need < blocks) blocks = need;
  e = mx->ops->launch(p, blocks, mx->wpb, st);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "sqp_mixed_kernel launch");
  if (!eager) return MPXG_OK;
  e = cudaEventRecord(mx->ring_ev[r], st);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaEventRecord");
  mx->ring_used[r] = true;
  return MPXG_OK;
}

}  // extern "C"

// A running device work queue: the ring, flags and result rows live in one
// block of mapped pinned host memory (the kernel reads and writes them in
// place); the claim counter lives on the device.
struct mpxg_queue {
  mpxg_handle* h = nullptr;
  cudaStream_t stream = nullptr;
  int capacity = 0, rows = 0, row_len = 0;
  int* host = nullptr;        // [entries cap | done cap | tail | stop | status | pad] then result rows
  int* dev = nullptr;         // the same block seen from the device
  int* head = nullptr;        // device claim counter
  long long next_ticket = 0;
  std::vector<int> ring_row;  // pool row of the ticket at each ring entry
  int* entries() { return host; }
  int* done() { return host + capacity; }
  int* tail() { return host + 2 * capacity; }
  int* stop() { return host + 2 * capacity + 1; }
  int* status() { return host + 2 * capacity + 2; }
  size_t rows_offset() const { return ((size_t)2 * capacity + 4 + 3) / 4 * 4; }  // ints, 16-byte aligned
  float* result_rows() { return reinterpret_cast<float*>(host + rows_offset()); }
};

static void queue_free(mpxg_queue* q) {
  if (q->host) cudaFreeHost(q->host);
  if (q->head) cudaFree(q->head);
  delete q;
}

extern "C" {

mpxg_status mpxg_queue_start(mpxg_handle* h, void* stream, const mpxg_batch_io* pool, int capacity,
                             long long idle_timeout_ns, mpxg_queue** out) {
  if (!h || !pool || !out) return fail(nullptr, MPXG_ERR_INVALID_ARG, "mpxg_queue_start: null argument");
  *out = nullptr;
  mpxg_status s = check_io(h, pool);
  if (s != MPXG_OK) return s;
  if (pool->batch < 1 || pool->slot || capacity < 1 || capacity > (1 << 20) || idle_timeout_ns < 1000000LL ||
      idle_timeout_ns > 60000000000LL)
    return fail(h, MPXG_ERR_INVALID_ARG,
                "mpxg_queue_start: pool of >= 1 rows without a slot map, capacity 1..2^20, idle timeout 1 ms..60 s");
  mpxg_queue* q = new mpxg_queue();
  q->h = h;
  q->stream = (cudaStream_t)stream;
  q->capacity = capacity;
  q->rows = pool->batch;
  q->row_len = h->desc.m + 4;
  q->ring_row.assign(capacity, -1);
  const size_t bytes = q->rows_offset() * sizeof(int) + (size_t)q->rows * q->row_len * sizeof(float);
  if (cudaHostAlloc(reinterpret_cast<void**>(&q->host), bytes, cudaHostAllocMapped) != cudaSuccess ||
      cudaHostGetDevicePointer(reinterpret_cast<void**>(&q->dev), q->host, 0) != cudaSuccess ||
      cudaMalloc(&q->head, sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    queue_free(q);
    return fail(h, MPXG_ERR_OUT_OF_MEMORY, "mpxg_queue_start: mapped host allocation failed");
  }
  std::memset(q->host, 0, bytes);
  cudaError_t e = cudaMemsetAsync(q->head, 0, sizeof(int), q->stream);
  if (e != cudaSuccess) {
    queue_free(q);
    return cuda_fail(h, e, "mpxg_queue_start: cudaMemsetAsync");
  }
  BatchPtrs bp = make_ptrs(h, pool);
  bp.slot = nullptr;
  bp.first = reinterpret_cast<float*>(q->dev + q->rows_offset());
  QueueArgs qa;
  qa.entries = q->dev;
  qa.done = q->dev + capacity;
  qa.tail = q->dev + 2 * capacity;
  qa.stop = q->dev + 2 * capacity + 1;
  qa.status = q->dev + 2 * capacity + 2;
  qa.head = q->head;
  qa.capacity = capacity;
  qa.timeout_ns = idle_timeout_ns;
  // one block per SM: as many concurrent solves as SMs x warps per block, and
  // few idle warps polling the ring in host memory
  const int wpb = h->warps_per_block;
  const int blocks = h->num_sms;
  e = sqp_ops(h->desc.model)->launch_queue(h->mc, h->sp, bp, qa, blocks, wpb, q->stream);
  if (e != cudaSuccess) {
    queue_free(q);
    return cuda_fail(h, e, "sqp_queue_kernel launch");
  }
  *out = q;
  return MPXG_OK;
}

mpxg_status mpxg_queue_push(mpxg_queue* q, int row, long long* ticket) {
  if (!q || !ticket) return fail(nullptr, MPXG_ERR_INVALID_ARG, "mpxg_queue_push: null argument");
  if (row < 0 || row >= q->rows) return fail(q->h, MPXG_ERR_INVALID_ARG, "mpxg_queue_push: row outside the pool");
  if (__atomic_load_n(q->status(), __ATOMIC_ACQUIRE) & QUEUE_TIMEOUT)
    return fail(q->h, MPXG_ERR_TIMEOUT, "mpxg_queue_push: the queue kernel timed out waiting and has stopped");
  const long long t = q->next_ticket;
  if (t >= 0x7ffffffe) return fail(q->h, MPXG_ERR_INVALID_ARG, "mpxg_queue_push: ticket space exhausted");
  const int k = (int)(t % q->capacity);
  if (t >= q->capacity && __atomic_load_n(q->done() + k, __ATOMIC_ACQUIRE) != (int)(t - q->capacity) + 1)
    return MPXG_ERR_NOT_READY;  // the ring entry's previous ticket has not finished yet
  q->entries()[k] = row;
  q->ring_row[k] = row;
  __atomic_store_n(q->tail(), (int)(t + 1), __ATOMIC_RELEASE);
  q->next_ticket = t + 1;
  *ticket = t;
  return MPXG_OK;
}

mpxg_status mpxg_queue_result(mpxg_queue* q, long long ticket, float* row_out) {
  if (!q || !row_out) return fail(nullptr, MPXG_ERR_INVALID_ARG, "mpxg_queue_result: null argument");
  if (ticket < 0 || ticket >= q->next_ticket || ticket < q->next_ticket - q->capacity)
    return fail(q->h, MPXG_ERR_INVALID_ARG, "mpxg_queue_result: ticket not pushed or its ring entry reused");
  const int k = (int)(ticket % q->capacity);
  if (__atomic_load_n(q->done() + k, __ATOMIC_ACQUIRE) != (int)ticket + 1)
    return (__atomic_load_n(q->status(), __ATOMIC_ACQUIRE) & QUEUE_TIMEOUT) ? MPXG_ERR_TIMEOUT : MPXG_ERR_NOT_READY;
  const float* src = q->result_rows() + (size_t)q->ring_row[k] * q->row_len;
  for (int i = 0; i < q->row_len; ++i) row_out[i] = src[i];
  return MPXG_OK;
}

mpxg_status mpxg_queue_finish(mpxg_queue* q) {
  if (!q) return fail(nullptr, MPXG_ERR_INVALID_ARG, "mpxg_queue_finish: null queue");
  __atomic_store_n(q->stop(), 1, __ATOMIC_RELEASE);
  const cudaError_t e = cudaStreamSynchronize(q->stream);  // bounded: every wait of the kernel is
  const int st = __atomic_load_n(q->status(), __ATOMIC_ACQUIRE);
  mpxg_handle* h = q->h;
  queue_free(q);
  if (e != cudaSuccess) return cuda_fail(h, e, "mpxg_queue_finish: cudaStreamSynchronize");
  if (st & QUEUE_TIMEOUT) return fail(h, MPXG_ERR_TIMEOUT, "mpxg_queue_finish: a warp's wait for work timed out");
  if (st & QUEUE_NO_SLOT) return fail(h, MPXG_ERR_CUDA, "mpxg_queue_finish: a warp found no scratch slot");
  return MPXG_OK;
}

mpxg_status mpxg_shift_warm_start(mpxg_handle* h, void* stream, int batch, const int* slot, const int* horizon,
                                  int shift, const float* X, const float* U, const float* V, float* Xo, float* Uo,
                                  float* Vo) {
  if (!h) return fail(nullptr, MPXG_ERR_INVALID_ARG, "null handle");
  if (batch < 0 || shift < 0 || !X || !U || !V || !Xo || !Uo || !Vo)
    return fail(h, MPXG_ERR_INVALID_ARG, "mpxg_shift_warm_start: bad arguments");
  if (batch == 0 || shift == 0 && X == Xo && U == Uo && V == Vo) return MPXG_OK;
  const int nx = h->desc.n, nu = h->desc.m, nm = h->desc.n_max;
  const size_t smem = ((size_t)(nm + 1) * nx * 2 + (size_t)nm * nu) * sizeof(float);
  if (smem > 200 * 1024) return fail(h, MPXG_ERR_UNSUPPORTED, "mpxg_shift_warm_start: horizon too long");
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(shift_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaFuncSetAttribute");
  }
  shift_kernel<<<batch, 128, smem, (cudaStream_t)stream>>>(batch, slot, nm, nx, nu, horizon, shift, X, U, V, Xo, Uo,
                                                           Vo);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MPXG_OK : cuda_fail(h, e, "shift_kernel launch");
}

}  // extern "C"

extern "C" {

mpxg_status mpxg_solve_vjp(mpxg_handle* h, void* stream, const mpxg_vjp_io* v) {
  if (!v) return fail(h, MPXG_ERR_INVALID_ARG, "mpxg_solve_vjp: null io");
  mpxg_batch_io io = v->io;
  io.X = const_cast<float*>(io.X_in);
  io.U = const_cast<float*>(io.U_in);
  io.V = const_cast<float*>(io.V_in);
  mpxg_status s = check_io(h, &io);
  if (s != MPXG_OK) return s;
  if (!v->gX || !v->gU) return fail(h, MPXG_ERR_INVALID_ARG, "mpxg_solve_vjp: cotangents gX, gU required");
  if (io.batch == 0) return MPXG_OK;
  cudaStream_t st = (cudaStream_t)stream;
  BatchPtrs bp = make_ptrs(h, &io);
  bp.K = nullptr; bp.k = nullptr; bp.kkt = nullptr; bp.first = nullptr; bp.status = io.status;
  bp.gX = v->gX; bp.gU = v->gU; bp.wX = v->wX; bp.wU = v->wU; bp.wL = v->wL; bp.gx0 = v->gx0; bp.gref = v->gref;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cap) != cudaSuccess) {
    cudaGetLastError();
    return fail(h, MPXG_ERR_CUDA, "mpxg_solve_vjp: cudaStreamIsCapturing failed");
  }
  int r;
  if (cap == cudaStreamCaptureStatusNone) {
    r = h->ring_next;
    h->ring_next = (r + 1) % mpxg_handle::kRing;
    if (h->ring_used[r]) {
      cudaError_t e = cudaStreamWaitEvent(st, h->ring_ev[r], 0);
      if (e != cudaSuccess) return cuda_fail(h, e, "cudaStreamWaitEvent");
    }
  } else {
    r = mpxg_handle::kRing + h->capture_next;
    h->capture_next = (h->capture_next + 1) % mpxg_handle::kRing;
  }
  bp.counter = h->counters + (size_t)r * mpxg_handle::kCounterStride;
  cudaError_t e = cudaMemsetAsync(bp.counter, 0, sizeof(int), st);
  if (e != cudaSuccess) return cuda_fail(h, e, "cudaMemsetAsync");
  const int wpb = h->warps_per_block;
  int blocks = h->num_sms * h->blocks_per_sm_lat;
  const int need = (io.batch + wpb - 1) / wpb;
  if (need < blocks) blocks = need;
  const SqpOps* ops = sqp_ops(h->desc.model);
  if (!ops) return fail(h, MPXG_ERR_UNSUPPORTED, "mpxg_solve_vjp: model");
  e = ops->launch_vjp(h->mc, h->sp, bp, blocks, wpb, st);
  s = e == cudaSuccess ? MPXG_OK : cuda_fail(h, e, "sqp_vjp_kernel launch");
  if (s != MPXG_OK || cap != cudaStreamCaptureStatusNone) return s;
  e = cudaEventRecord(h->ring_ev[r], st);
  if (e != cudaSuccess) return cuda_fail(h, e, "cudaEventRecord");
  h->ring_used[r] = true;
  return MPXG_OK;
}

mpxg_status mpxg_evaluate(mpxg_handle* h, void* stream, int batch, const int* horizon, const float* x0,
                          const float* X, const float* U, const float* reference, const float* parameter,
                          const float* w, float* g, float* c) {
  if (!h) return fail(nullptr, MPXG_ERR_INVALID_ARG, "null handle");
  if (batch < 0 || batch > h->desc.batch_max || !x0 || !X || !U || !reference || !parameter || !w || !g || !c)
    return fail(h, MPXG_ERR_INVALID_ARG, "mpxg_evaluate: bad arguments");
  if (batch == 0) return MPXG_OK;
  const SqpOps* ops = sqp_ops(h->desc.model);
  if (!ops) return fail(h, MPXG_ERR_UNSUPPORTED, "mpxg_evaluate: model");
  const cudaError_t e = ops->launch_evaluate(h->mc, batch, h->desc.n_max, horizon, x0, X, U, reference, parameter,
                                             w, g, c, (cudaStream_t)stream);
  return e == cudaSuccess ? MPXG_OK : cuda_fail(h, e, "evaluate_kernel launch");
}

mpxg_status mpxg_timer_run(void* stream, int batch, int n_legs, float duty_factor, float step_freq, float dt,
                           float* leg_time, int* contact) {
  if (batch < 0 || n_legs < 1 || !leg_time || !contact) return fail(nullptr, MPXG_ERR_INVALID_ARG, "mpxg_timer_run");
  const int n = batch * n_legs;
  if (n == 0) return MPXG_OK;
  timer_kernel<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(n, n_legs, duty_factor, step_freq, dt, leg_time, contact);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MPXG_OK : cuda_fail(nullptr, e, "timer_kernel launch");
}

mpxg_status mpxg_gait_tables(void* stream, const mpxg_gait_args* a) {
  if (!a) return fail(nullptr, MPXG_ERR_INVALID_ARG, "mpxg_gait_tables: null args");
  int nx, nu, legs, rc, pc, cc;
  if (a->model == MPXG_MODEL_SRBD_QUAT13) { nx = 13; nu = 12; legs = 4; rc = 17; pc = 16; cc = 13; }
  else if (a->model == MPXG_MODEL_SRBD_RPY12) { nx = 12; nu = 12; legs = 4; rc = 16; pc = 16; cc = 12; }
  else if (a->model == MPXG_MODEL_BIPED_WRENCH12) { nx = 12; nu = 12; legs = 2; rc = 14; pc = 8; cc = 12; }
  else return fail(nullptr, MPXG_ERR_UNSUPPORTED, "mpxg_gait_tables: model");
  if (a->batch < 0 || a->n_max < 1 || a->mode < 0 || a->mode > 2 || !a->x0 || !a->X || !a->v_ref ||
      !a->leg_time || !a->reference || !a->parameter || (a->mode == 0 && (!a->U || !a->V)))
    return fail(nullptr, MPXG_ERR_INVALID_ARG, "mpxg_gait_tables: bad arguments");
  if (a->batch == 0) return MPXG_OK;
  gait_tables_kernel<<<(a->batch + 3) / 4, 128, 0, (cudaStream_t)stream>>>(*a, nx, nu, legs, rc, pc, cc);  // warp per entry
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MPXG_OK : cuda_fail(nullptr, e, "gait_tables_kernel launch");
}

mpxg_status mpxg_refgen_srbd(void* stream, int batch, int N, int n_max, float dt, const float* foot0,
                             float duty_factor, float step_freq, float step_height, float clearence_speed,
                             const float* t_timer, const float* x, const float* foot, const float* input,
                             const float* contact, float* liftoff, float* reference, float* parameter,
                             float* foot_ref_dot) {
  if (batch < 0 || N < 1 || n_max < N || !foot0 || !t_timer || !x || !foot || !input || !contact || !liftoff ||
      !reference || !parameter || !foot_ref_dot)
    return fail(nullptr, MPXG_ERR_INVALID_ARG, "mpxg_refgen_srbd: bad arguments");
  if (batch == 0) return MPXG_OK;
  RefGenArgs g;
  g.batch = batch; g.N = N; g.n_max = n_max; g.dt = dt;
  for (int i = 0; i < 12; ++i) g.foot0[i] = foot0[i];  // host array
  g.duty = duty_factor; g.step_freq = step_freq; g.step_height = step_height; g.clearence = clearence_speed;
  g.t_timer = t_timer; g.x = x; g.foot = foot; g.input = input; g.contact = contact;
  g.liftoff = liftoff; g.reference = reference; g.parameter = parameter; g.foot_ref_dot = foot_ref_dot;
  refgen_srbd_kernel<<<(batch + 127) / 128, 128, 0, (cudaStream_t)stream>>>(g);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MPXG_OK : cuda_fail(nullptr, e, "refgen_srbd_kernel launch");
}

mpxg_status mpxg_refgen_wb(void* stream, int batch, int N, int n_joints, float dt, float mass, const float* foot0,
                           const float* q0, float duty_factor, float step_freq, float step_height,
                           float clearence_speed, int use_terrain_estimation, const float* t_timer, const float* x,
                           const float* foot, const float* input, const float* contact, float* liftoff,
                           float* reference, float* parameter) {
  if (batch < 0 || N < 1 || n_joints < 0 || n_joints > MPXG_WB_MAX_DOF || !foot0 || !q0 || !t_timer || !x ||
      !foot || !input || !contact || !liftoff || !reference || !parameter)
    return fail(nullptr, MPXG_ERR_INVALID_ARG, "mpxg_refgen_wb: bad arguments");
  if (batch == 0) return MPXG_OK;
  RefGenWbArgs g;
  g.batch = batch; g.N = N; g.nj = n_joints; g.nx = 13 + 2 * n_joints + 24; g.terrain = use_terrain_estimation != 0;
  g.dt = dt; g.mass = mass;
  for (int i = 0; i < 12; ++i) g.foot0[i] = foot0[i];  // host arrays
  for (int i = 0; i < MPXG_WB_MAX_DOF; ++i) g.q0[i] = i < n_joints ? q0[i] : 0.0f;
  g.duty = duty_factor; g.step_freq = step_freq; g.step_height = step_height; g.clearence = clearence_speed;
  g.t_timer = t_timer; g.x = x; g.foot = foot; g.input = input; g.contact = contact;
  g.liftoff = liftoff; g.reference = reference; g.parameter = parameter;
  refgen_wb_kernel<<<(batch + 127) / 128, 128, 0, (cudaStream_t)stream>>>(g);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MPXG_OK : cuda_fail(nullptr, e, "refgen_wb_kernel launch");
}

}  // extern "C"

// ============================================================================
// Allocation-free batched solve.
//
// Some callers cannot allocate device memory at solve time: a host process
// that must not call cudaMalloc after start-up (real-time control loops, where
// an allocation can block for milliseconds), or a plugin whose host framework
// owns every allocation and hands the plugin only the input and output buffers
// (e.g. an XLA custom call without a workspace).  mpxg_solve_noalloc serves
// them: it needs no handle and takes its per-warp scratch from the file-scope
// device array below instead of a cudaMalloc'd workspace.
//
// Limits and sharing rules:
//  - the array is kNoAllocScratchBytes (64 MiB) on every GPU that loads this
//    library, held until the process exits;
//  - one warp needs scratch_floats(n_max) floats; the array must hold at
//    least one warp per SM, otherwise the call is rejected with
//    MPXG_ERR_INVALID_ARG (on a 152-SM GB300: n_max <= 141 for the
//    roll-pitch-yaw quadruped, 135 for the biped, 116 for the quaternion
//    model); the persistent grid is shrunk to the warps that fit;
//  - all calls share the array (and the work counter, which each call clears
//    on its stream first), so two calls that overlap on the GPU race: issue
//    them on one stream or order them with events;
//  - the first call on a device resolves the array's device address with
//    cudaGetSymbolAddress (a host-side symbol is not a device address); make
//    that first call before any stream capture;
//  - the resolved address is kept for the life of the process: after a
//    cudaDeviceReset (or anything else that destroys the device's primary
//    context) this entry point must not be called again in that process.
// ============================================================================
static constexpr size_t kNoAllocScratchBytes = size_t(64) << 20;
static __device__ __align__(256) float g_noalloc_scratch[kNoAllocScratchBytes / sizeof(float)];
static __device__ __align__(256) int g_noalloc_counter[64];

namespace {
struct NoAllocDevice {
  bool ready = false;
  float* scratch = nullptr;
  int* counter = nullptr;
  int num_sms = 0;
};
constexpr int kMaxDevices = 64;
NoAllocDevice g_noalloc_dev[kMaxDevices];
std::mutex g_noalloc_mu;

mpxg_status noalloc_setup(int dev, NoAllocDevice** out) {
  if (dev < 0 || dev >= kMaxDevices) return fail(nullptr, MPXG_ERR_UNSUPPORTED, "mpxg_solve_noalloc: device index");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  NoAllocDevice& d = g_noalloc_dev[dev];
  if (!d.ready) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "mpxg_solve_noalloc: cudaGetSymbolAddress(scratch)");
    d.scratch = static_cast<float*>(p);
    e = cudaGetSymbolAddress(&p, g_noalloc_counter);
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "mpxg_solve_noalloc: cudaGetSymbolAddress(counter)");
    d.counter = static_cast<int*>(p);
    e = cudaDeviceGetAttribute(&d.num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "mpxg_solve_noalloc: cudaDeviceGetAttribute");
    d.ready = true;
  }
  *out = &d;
  return MPXG_OK;
}

}  // namespace

extern "C" mpxg_status mpxg_solve_noalloc(const mpxg_problem_desc* d, const mpxg_solver_opts* o, void* stream,
                                          const mpxg_batch_io* io) {
  if (!d || !o || !io) return fail(nullptr, MPXG_ERR_INVALID_ARG, "mpxg_solve_noalloc: null argument");
  int nx, nu;
  if (!model_dims(d->model, &nx, &nu)) return fail(nullptr, MPXG_ERR_UNSUPPORTED, "mpxg_solve_noalloc: model id");
  if (d->n != nx || d->m != nu) return fail(nullptr, MPXG_ERR_INVALID_ARG, "mpxg_solve_noalloc: n/m do not match the model");
  if (d->n_max < 1 || d->n_max > 4096) return fail(nullptr, MPXG_ERR_INVALID_ARG, "mpxg_solve_noalloc: n_max out of range");
  if (o->sqp_iters < 0 || o->ls_max_trials < 1) return fail(nullptr, MPXG_ERR_INVALID_ARG, "mpxg_solve_noalloc: bad options");
  if (o->warps_per_block < 0 || o->warps_per_block > 4 || o->blocks_per_sm < 0)
    return fail(nullptr, MPXG_ERR_INVALID_ARG, "mpxg_solve_noalloc: warps_per_block must be 0..4 (128-thread blocks)");
  if (!(d->dt > 0.0f) || !(d->mass > 0.0f)) return fail(nullptr, MPXG_ERR_INVALID_ARG, "mpxg_solve_noalloc: dt and mass must be > 0");
  if (io->batch < 0 || !io->x0 || !io->X_in || !io->U_in || !io->V_in || !io->reference || !io->parameter ||
      !io->w || !io->X || !io->U || !io->V)
    return fail(nullptr, MPXG_ERR_INVALID_ARG, "mpxg_solve_noalloc: required pointer is null");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "mpxg_solve_noalloc: cudaGetDevice");
  NoAllocDevice* nd = nullptr;
  mpxg_status s = noalloc_setup(dev, &nd);
  if (s != MPXG_OK) return s;
  const long long stride = scratch_stride_for(d->model, d->n_max);
  const long long warps_fit = (long long)(kNoAllocScratchBytes / sizeof(float)) / stride;
  if (warps_fit < nd->num_sms)
    return fail(nullptr, MPXG_ERR_INVALID_ARG,
                "mpxg_solve_noalloc: n_max too large: one warp needs " + std::to_string(stride * 4) +
                    " bytes of scratch, the 64 MiB static array must hold one warp per SM (" +
                    std::to_string(nd->num_sms) + ")");
  if (io->batch == 0) return MPXG_OK;

  const ModelConst mc = model_const(d);
  SqpParams sp{};
  sp.sqp_iters = o->sqp_iters; sp.ls_max_trials = o->ls_max_trials; sp.ls_beta = o->ls_beta; sp.ls_eta = o->ls_eta;
  sp.reg = o->reg; sp.rho0 = o->rho0; sp.ls_skip_tol = o->ls_skip_tol; sp.compute_kkt = o->compute_kkt;

  // persistent grid limited by the warps whose scratch fits in the array
  int wpb = o->warps_per_block > 0 ? o->warps_per_block : 4;
  long long max_warps = (long long)nd->num_sms * 2 * wpb;
  if (max_warps > warps_fit) max_warps = warps_fit;
  if (wpb > max_warps) wpb = (int)max_warps;
  long long blocks = max_warps / wpb;
  const long long need = (io->batch + wpb - 1) / wpb;
  if (blocks > need) blocks = need;
  if (blocks < 1) blocks = 1;

  BatchPtrs bp;
  bp.batch = io->batch; bp.n_max = d->n_max; bp.slot = io->slot; bp.horizon = io->horizon;
  bp.x0 = io->x0; bp.X_in = io->X_in; bp.U_in = io->U_in; bp.V_in = io->V_in;
  bp.ref = io->reference; bp.par = io->parameter; bp.w = io->w;
  bp.X = io->X; bp.U = io->U; bp.V = io->V; bp.K = io->K; bp.k = io->k; bp.kkt = io->kkt; bp.status = io->status;
  bp.first = io->first;
  bp.counter = nd->counter; bp.scratch = nd->scratch; bp.scratch_stride = stride;
  bp.single_instance = -1;

  cudaStream_t st = (cudaStream_t)stream;
  e = cudaMemsetAsync(nd->counter, 0, sizeof(int), st);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "mpxg_solve_noalloc: cudaMemsetAsync");
  e = sqp_ops(d->model)->launch(mc, sp, bp, (int)blocks, wpb, /*tput=*/false, st);
  return e == cudaSuccess ? MPXG_OK : cuda_fail(nullptr, e, "mpxg_solve_noalloc: launch");
}

// ============================================================================
// XLA custom-call target (status-returning custom-call signature).
//
// The reference jit-compiles the solve (jax.jit(jax.vmap(...)),
// mpx/utils/mpc_wrapper_srbd.py:68,77); registering this target with XLA keeps
// that call inside a compiled JAX program.  Operands and results arrive as
// device buffers in the order of optimizers.mpc(reference, parameter, W, x0,
// X0, U0, V0) -> (X, U, V), with W passed as its diagonal [B,24].  The opaque
// string is an mpxg_xla_opaque.  The handle of each (device, opaque) is
// created by mpxg_xla_prepare ahead of the jitted program's first run (the
// JAX binding calls it when it builds the solve), so the custom call itself
// allocates nothing: it may run under XLA's command-buffer capture, where a
// cudaMalloc would fail.  Handles are kept for the life of the process.
// ============================================================================
namespace {

std::mutex g_xla_mu;
std::map<std::string, mpxg_handle*> g_xla_handles;

typedef void (*xla_status_set_failure_fn)(void*, const char*, size_t);

void xla_fail(void* status, const std::string& msg) {
  g_lib_err = msg;
  static xla_status_set_failure_fn setter =
      (xla_status_set_failure_fn)dlsym(RTLD_DEFAULT, "XlaCustomCallStatusSetFailure");
  if (status && setter) setter(status, msg.c_str(), msg.size());
}

}  // namespace

// Checked opaque of an XLA call and the handle key of (current device, opaque).
static bool xla_key(const char* opaque, size_t opaque_len, mpxg_xla_opaque* op, std::string* key, std::string* err,
                    const char* who) {
  if (!opaque || opaque_len != sizeof(mpxg_xla_opaque)) {
    *err = std::string(who) + ": opaque must be an mpxg_xla_opaque (" + std::to_string(sizeof(mpxg_xla_opaque)) +
           " bytes), got " + std::to_string(opaque_len);
    return false;
  }
  std::memcpy(op, opaque, sizeof(*op));
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    *err = std::string(who) + ": cudaGetDevice failed";
    return false;
  }
  if (op->batch < 0 || op->batch > op->desc.batch_max) {
    *err = std::string(who) + ": batch exceeds desc.batch_max";
    return false;
  }
  key->assign(reinterpret_cast<const char*>(&dev), sizeof(dev));
  key->append(reinterpret_cast<const char*>(&op->desc), sizeof(op->desc));
  key->append(reinterpret_cast<const char*>(&op->opts), sizeof(op->opts));
  return true;
}

// Handle of (device, opaque) prepared by mpxg_xla_prepare; null (and the
// failure reported to XLA) when there is none.
static mpxg_handle* xla_handle(const char* opaque, size_t opaque_len, void* status, mpxg_xla_opaque* op,
                               const char* who) {
  std::string key, err;
  if (!xla_key(opaque, opaque_len, op, &key, &err, who)) {
    xla_fail(status, err);
    return nullptr;
  }
  std::lock_guard<std::mutex> lock(g_xla_mu);
  auto it = g_xla_handles.find(key);
  if (it != g_xla_handles.end()) return it->second;
  xla_fail(status, std::string(who) + ": no handle for this opaque on this device: call mpxg_xla_prepare with it "
                                      "(and this device current) before the program runs");
  return nullptr;
}

extern "C" mpxg_status mpxg_xla_prepare(const char* opaque, size_t opaque_len) {
  mpxg_xla_opaque op;
  std::string key, err;
  if (!xla_key(opaque, opaque_len, &op, &key, &err, "mpxg_xla_prepare"))
    return fail(nullptr, MPXG_ERR_INVALID_ARG, err);
  std::lock_guard<std::mutex> lock(g_xla_mu);
  if (g_xla_handles.count(key)) return MPXG_OK;
  mpxg_handle* h = nullptr;
  const mpxg_status s = mpxg_create(&op.desc, &op.opts, &h);
  if (s != MPXG_OK) return s;
  g_xla_handles[key] = h;
  return MPXG_OK;
}

extern "C" void mpxg_xla_solve(void* stream, void** buffers, const char* opaque, size_t opaque_len, void* status) {
  mpxg_xla_opaque op;
  if (!buffers) { xla_fail(status, "mpxg_xla_solve: null buffers"); return; }
  mpxg_handle* h = xla_handle(opaque, opaque_len, status, &op, "mpxg_xla_solve");
  if (!h) return;
  mpxg_batch_io io;
  std::memset(&io, 0, sizeof(io));
  io.batch = op.batch;
  io.reference = (const float*)buffers[0];
  io.parameter = (const float*)buffers[1];
  io.w = (const float*)buffers[2];
  io.x0 = (const float*)buffers[3];
  io.X_in = (const float*)buffers[4];
  io.U_in = (const float*)buffers[5];
  io.V_in = (const float*)buffers[6];
  io.X = (float*)buffers[7];
  io.U = (float*)buffers[8];
  io.V = (float*)buffers[9];
  std::lock_guard<std::mutex> lock(g_xla_mu);  // a handle is used by one host thread at a time
  if (mpxg_solve(h, stream, &io) != MPXG_OK) xla_fail(status, std::string("mpxg_xla_solve: ") + h->err);
}

extern "C" void mpxg_xla_solve_vjp(void* stream, void** buffers, const char* opaque, size_t opaque_len,
                                   void* status) {
  mpxg_xla_opaque op;
  if (!buffers) { xla_fail(status, "mpxg_xla_solve_vjp: null buffers"); return; }
  mpxg_handle* h = xla_handle(opaque, opaque_len, status, &op, "mpxg_xla_solve_vjp");
  if (!h) return;
  mpxg_vjp_io v;
  std::memset(&v, 0, sizeof(v));
  v.io.batch = op.batch;
  v.io.reference = (const float*)buffers[0];
  v.io.parameter = (const float*)buffers[1];
  v.io.w = (const float*)buffers[2];
  v.io.x0 = (const float*)buffers[3];
  v.io.X_in = (const float*)buffers[4];
  v.io.U_in = (const float*)buffers[5];
  v.io.V_in = (const float*)buffers[6];
  v.gX = (const float*)buffers[7];
  v.gU = (const float*)buffers[8];
  v.gx0 = (float*)buffers[9];
  v.gref = (float*)buffers[10];
  std::lock_guard<std::mutex> lock(g_xla_mu);
  if (mpxg_solve_vjp(h, stream, &v) != MPXG_OK) xla_fail(status, std::string("mpxg_xla_solve_vjp: ") + h->err);
}

// ============================================================================
// Served MPC stream (mpxg_server_*): host runtime over the entry points above.
// ============================================================================
#include "server.cuh"
