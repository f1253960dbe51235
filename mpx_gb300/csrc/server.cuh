// Host runtime of the served MPC stream (mpxg_server_* in include/mpxg.h):
// per-model slot pools resident on the device, continuous batching over CUDA
// streams, admission by a device-memory budget.  Included at the end of
// mpxg_abi.cu; uses only the library's own C entry points for device work.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <deque>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/mpxg.h"

namespace mpxg_srv {

struct Staging {
  int* slot_h = nullptr;   // pinned: [batch slots | warm slots | cold slots]
  int* slot_d = nullptr;
  float* res_h = nullptr;  // mapped pinned result rows [cap, m+4], written by the solve kernels
  float* res_d = nullptr;  // the device address of res_h
  cudaEvent_t ev = nullptr;
};

struct Pool {
  mpxg_served_model m;
  int cap = 0, n = 0, mu = 0, legs = 0, rc = 0, pc = 0;
  float *x0 = nullptr, *X = nullptr, *U = nullptr, *V = nullptr, *ref = nullptr, *par = nullptr, *w = nullptr;
  float *kkt = nullptr, *vref = nullptr, *lt = nullptr;
  int *horizon = nullptr, *status = nullptr;
  mpxg_handle* h = nullptr;
  int total_warps = 0;
  std::vector<int> free_slots;
  std::vector<Staging*> idle;
  std::vector<long long> pending;
};

struct Episode {
  int model = 0, slot = 0, horizon = 0;
  bool cold = true, running = false, retiring = false;
  int busy = 0;  // ticks queued or running
};

struct Ticket {
  int episode = 0;
  bool done = false;
  mpxg_result res;
};

// A launched batch: one model's tickets, or (mixed launch) two models' parts.
struct Part {
  int model = 0;
  Staging* st = nullptr;
  std::vector<long long> tickets;
  std::vector<char> got;     // ticket i's result row already delivered
  std::vector<int> episode;  // ticket i's episode, and its result status once delivered (a
  std::vector<int> status;   // delivered ticket may be consumed by the client before the reap)
  size_t next = 0;           // rows before this one are all delivered
};
struct Batch {
  int stream = 0;
  std::vector<Part> parts;
  cudaEvent_t ev() const { return parts.front().st->ev; }
};

inline bool model_layout(int model, int* n, int* m, int* legs, int* rc, int* pc) {
  switch (model) {
    case MPXG_MODEL_SRBD_QUAT13: *n = 13; *m = 12; *legs = 4; *rc = 17; *pc = 16; return true;
    case MPXG_MODEL_SRBD_RPY12: *n = 12; *m = 12; *legs = 4; *rc = 16; *pc = 16; return true;
    case MPXG_MODEL_BIPED_WRENCH12: *n = 12; *m = 12; *legs = 2; *rc = 14; *pc = 8; return true;
    default: return false;
  }
}

// Device bytes of one episode slot (pool arrays) plus its share of the
// solver's per-solve order arrays.
inline size_t slot_bytes(int n, int m, int legs, int rc, int pc, int n_max) {
  size_t f = (size_t)(n_max + 1) * n * 2 + (size_t)n_max * m + (size_t)(n_max + 1) * (rc + pc);
  f += n + 24 + 3 + legs + 1;
  return 4 * f + 4 * 2 + 2 * 64 * sizeof(int);
}

}  // namespace mpxg_srv

struct mpxg_server {
  mpxg_server_desc d;
  std::vector<mpxg_srv::Pool> pools;
  std::vector<cudaStream_t> streams;
  std::vector<char> stream_busy;   // a batch is running on the stream
  std::unordered_map<int, mpxg_srv::Episode> eps;
  int next_episode = 1;
  std::unordered_map<long long, mpxg_srv::Ticket> tickets;
  long long next_ticket = 1;
  std::vector<mpxg_srv::Batch> inflight;
  mpxg_mixed* mixed = nullptr;  // mixed-model launches (mixed_launch): pools mix[0], mix[1]
  int mix[2] = {0, 1};
  std::deque<long long> done;
  unsigned int seed = 0;
  long long launches = 0;
  int queued = 0;
  std::string err;
};

namespace mpxg_srv {

// Library-level error (no server yet): reported through mpxg_last_error(NULL).
inline mpxg_status fail_lib(mpxg_status st, const std::string& msg) {
  g_lib_err = msg;
  return st;
}

inline mpxg_status fail(mpxg_server* s, mpxg_status st, const std::string& msg) {
  s->err = msg;
  return st;
}
inline mpxg_status cuda_err(mpxg_server* s, cudaError_t e, const char* where) {
  return fail(s, MPXG_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

inline void free_pool(Pool& p) {
  for (void* q : {(void*)p.x0, (void*)p.X, (void*)p.U, (void*)p.V, (void*)p.ref, (void*)p.par, (void*)p.w,
                  (void*)p.kkt, (void*)p.vref, (void*)p.lt, (void*)p.horizon, (void*)p.status})
    if (q) cudaFree(q);
  for (Staging* st : p.idle) {
    cudaFreeHost(st->slot_h);
    cudaFree(st->slot_d);
    cudaFreeHost(st->res_h);
    cudaEventDestroy(st->ev);
    delete st;
  }
  p.idle.clear();
  if (p.h) mpxg_destroy(p.h);
  p.h = nullptr;
}

inline Staging* get_staging(mpxg_server* s, Pool& p) {
  if (!p.idle.empty()) {
    Staging* st = p.idle.back();
    p.idle.pop_back();
    return st;
  }
  Staging* st = new Staging();
  const size_t rows = (size_t)p.cap * (p.mu + 4) * sizeof(float);
  if (cudaMallocHost(&st->slot_h, 3 * (size_t)p.cap * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&st->slot_d, 3 * (size_t)p.cap * sizeof(int)) != cudaSuccess ||
      cudaHostAlloc((void**)&st->res_h, rows, cudaHostAllocMapped) != cudaSuccess ||
      cudaHostGetDevicePointer((void**)&st->res_d, st->res_h, 0) != cudaSuccess ||
      cudaEventCreateWithFlags(&st->ev, cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();
    s->err = "server: staging allocation failed";
    if (st->slot_h) cudaFreeHost(st->slot_h);
    if (st->slot_d) cudaFree(st->slot_d);
    if (st->res_h) cudaFreeHost(st->res_h);
    delete st;
    return nullptr;
  }
  return st;
}

inline void fill_gait(const Pool& p, int n_max, mpxg_gait_args* a) {
  std::memset(a, 0, sizeof(*a));
  a->model = p.m.desc.model;
  a->n_max = n_max;
  a->horizon = p.horizon;
  a->dt = p.m.desc.dt;
  a->duty_factor = p.m.duty_factor;
  a->step_freq = p.m.step_freq;
  a->height = p.m.height;
  a->weight = p.m.desc.mass * p.m.desc.gravity;
  for (int i = 0; i < 12; ++i) a->offsets[i] = p.m.offsets[i];
  a->x0 = p.x0; a->X = p.X; a->U = p.U; a->V = p.V;
  a->v_ref = p.vref; a->leg_time = p.lt; a->reference = p.ref; a->parameter = p.par;
}

// Stage one model's part of a batch on `stream`: order the tickets longest
// horizon first, upload their slots, shift the warm starts and rebuild the
// gait tables.  Fills the solve io of the part.
inline mpxg_status prepare_part(mpxg_server* s, Part& part, cudaStream_t stream, mpxg_batch_io* io) {
  Pool& p = s->pools[part.model];
  std::vector<long long>& ticks = part.tickets;
  std::sort(ticks.begin(), ticks.end(), [&](long long a, long long b) {
    return s->eps[s->tickets[a].episode].horizon > s->eps[s->tickets[b].episode].horizon;
  });
  const int nb = (int)ticks.size();
  Staging* st = get_staging(s, p);
  if (!st) return MPXG_ERR_OUT_OF_MEMORY;
  part.st = st;
  int nw = 0, nc = 0;
  for (int i = 0; i < nb; ++i) {
    const Episode& e = s->eps[s->tickets[ticks[i]].episode];
    st->slot_h[i] = e.slot;
    if (!e.cold) ++nw;
  }
  int iw = nb, ic = nb + nw;
  for (int i = 0; i < nb; ++i) {
    Episode& e = s->eps[s->tickets[ticks[i]].episode];
    if (e.cold) st->slot_h[ic++] = e.slot; else st->slot_h[iw++] = e.slot;
    nc += e.cold ? 1 : 0;
    e.cold = false;
    e.running = true;
  }
  cudaError_t ce = cudaMemcpyAsync(st->slot_d, st->slot_h, (size_t)(nb + nw + nc) * sizeof(int),
                                   cudaMemcpyHostToDevice, stream);
  if (ce != cudaSuccess) return cuda_err(s, ce, "server: slot copy");
  const int n_max = s->d.n_max;
  mpxg_status r;
  if (nw) {
    r = mpxg_shift_warm_start(p.h, stream, nw, st->slot_d + nb, p.horizon, 1, p.X, p.U, p.V, p.X, p.U, p.V);
    if (r != MPXG_OK) return fail(s, r, std::string("server: shift: ") + mpxg_last_error(p.h));
    mpxg_gait_args a;
    fill_gait(p, n_max, &a);
    a.batch = nw; a.mode = 1; a.slot = st->slot_d + nb; a.drift_std = s->d.drift_std; a.seed = ++s->seed;
    r = mpxg_gait_tables(stream, &a);
    if (r != MPXG_OK) return fail(s, r, std::string("server: gait tables: ") + mpxg_last_error(nullptr));
  }
  if (nc) {
    mpxg_gait_args a;
    fill_gait(p, n_max, &a);
    a.batch = nc; a.mode = 0; a.slot = st->slot_d + nb + nw;
    r = mpxg_gait_tables(stream, &a);
    if (r != MPXG_OK) return fail(s, r, std::string("server: gait tables: ") + mpxg_last_error(nullptr));
  }
  // the rows' status entries read "not yet written" until the kernel writes them
  for (int i = 0; i < nb; ++i) st->res_h[(size_t)i * (p.mu + 4) + p.mu + 3] = std::nanf("");
  __atomic_thread_fence(__ATOMIC_SEQ_CST);  // visible before the launch that overwrites them
  std::memset(io, 0, sizeof(*io));
  io->batch = nb; io->slot = st->slot_d; io->horizon = p.horizon;
  io->x0 = p.x0; io->X_in = p.X; io->U_in = p.U; io->V_in = p.V;
  io->reference = p.ref; io->parameter = p.par; io->w = p.w;
  io->X = p.X; io->U = p.U; io->V = p.V; io->kkt = p.kkt; io->status = p.status; io->first = st->res_d;
  s->launches += (nw ? 2 : 0) + (nc ? 1 : 0);
  return MPXG_OK;
}

// Launch one batch: the parts' tickets (per part one model, episodes
// distinct and idle); one part goes through mpxg_solve of its pool's handle,
// two parts through one mixed-model solve.
inline mpxg_status launch(mpxg_server* s, std::vector<Part> parts) {
  int si = 0;  // an idle stream (the caller checked that one exists)
  while (si < (int)s->streams.size() && s->stream_busy[si]) ++si;
  if (si == (int)s->streams.size()) return fail(s, MPXG_ERR_INVALID_ARG, "server: no idle stream");
  cudaStream_t stream = s->streams[si];
  mpxg_batch_io io[2];
  int nt = 0;
  for (size_t k = 0; k < parts.size(); ++k) {
    mpxg_status r = prepare_part(s, parts[k], stream, &io[k]);
    if (r != MPXG_OK) return r;
    nt += io[k].batch;
  }
  mpxg_status r;
  if (parts.size() == 2) {
    r = mpxg_solve_mixed(s->mixed, stream, &io[0], &io[1]);
    if (r != MPXG_OK) return fail(s, r, std::string("server: mixed solve: ") + mpxg_last_error(nullptr));
    s->launches += 2;  // order + solve
  } else {
    Pool& p = s->pools[parts[0].model];
    r = mpxg_solve(p.h, stream, &io[0]);
    if (r != MPXG_OK) return fail(s, r, std::string("server: solve: ") + mpxg_last_error(p.h));
    s->launches += io[0].batch > p.total_warps ? 2 : 1;
  }
  // the result rows arrive in mapped host memory as each instance finishes;
  // the event marks the batch's end (its warm starts written, its streams free)
  cudaError_t ce = cudaEventRecord(parts[0].st->ev, stream);
  if (ce != cudaSuccess) return cuda_err(s, ce, "server: event");
  for (Part& part : parts) {
    part.got.assign(part.tickets.size(), 0);
    part.status.assign(part.tickets.size(), 0);
    part.episode.resize(part.tickets.size());
    for (size_t i = 0; i < part.tickets.size(); ++i) part.episode[i] = s->tickets[part.tickets[i]].episode;
    part.next = 0;
  }
  Batch b;
  b.stream = si;
  s->stream_busy[si] = 1;
  b.parts = std::move(parts);
  s->inflight.push_back(std::move(b));
  s->queued -= nt;
  return MPXG_OK;
}

inline void retire(mpxg_server* s, int episode) {
  auto it = s->eps.find(episode);
  if (it == s->eps.end()) return;
  s->pools[it->second.model].free_slots.push_back(it->second.slot);
  s->eps.erase(it);
}

// Deliver ticket i of a part from its result row (in mapped host memory).
inline void deliver(mpxg_server* s, Part& part, size_t i) {
  const Pool& p = s->pools[part.model];
  Ticket& t = s->tickets[part.tickets[i]];
  const float* row = part.st->res_h + i * (p.mu + 4);
  t.res.ticket = part.tickets[i];
  t.res.episode = t.episode;
  for (int a = 0; a < 12; ++a) t.res.u0[a] = a < p.mu ? row[a] : 0.0f;
  for (int k = 0; k < 3; ++k) t.res.kkt[k] = row[p.mu + k];
  const float sv = row[p.mu + 3];
  t.res.status = sv == sv ? (int)sv : MPXG_INST_NAN;  // a row the solve never wrote reads as failed
  t.done = true;
  s->done.push_back(part.tickets[i]);
  part.got[i] = 1;
  part.status[i] = t.res.status;
}

// Deliver the rows of running batches that have arrived: a row whose status
// entry is no longer the NaN written before the launch (the kernel writes it
// last, after a system-scope fence; the acquire load orders the reads of the
// row's other entries after it).  The episodes stay claimed until the batch
// is reaped, when its warm starts are complete on the device.
inline int deliver_arrived(mpxg_server* s) {
  int n = 0;
  for (Batch& b : s->inflight)
    for (Part& part : b.parts) {
      const Pool& p = s->pools[part.model];
      for (size_t i = part.next; i < part.tickets.size(); ++i) {
        if (part.got[i]) continue;
        const unsigned* w = reinterpret_cast<const unsigned*>(part.st->res_h + i * (p.mu + 4) + p.mu + 3);
        const unsigned bits = __atomic_load_n(w, __ATOMIC_ACQUIRE);
        float v;
        std::memcpy(&v, &bits, sizeof(v));
        if (v != v) continue;  // not written yet
        deliver(s, part, i);
        ++n;
      }
      while (part.next < part.tickets.size() && part.got[part.next]) ++part.next;
    }
  return n;
}

// Reap running batch i (its event has completed): deliver the rows not yet
// delivered, release the episodes and the staging.
inline void reap(mpxg_server* s, size_t i) {
  Batch b = std::move(s->inflight[i]);
  s->inflight.erase(s->inflight.begin() + i);
  s->stream_busy[b.stream] = 0;
  for (Part& part : b.parts) {
    Pool& p = s->pools[part.model];
    for (size_t k = 0; k < part.tickets.size(); ++k) {
      if (!part.got[k]) deliver(s, part, k);  // the event has completed: every row is written
      auto it = s->eps.find(part.episode[k]);
      if (it != s->eps.end()) {
        Episode& e = it->second;
        if (part.status[k] & MPXG_INST_NAN) e.cold = true;  // NaN fallback: cold start next tick
        e.running = false;
        if (--e.busy == 0 && e.retiring) retire(s, part.episode[k]);
      }
    }
    p.idle.push_back(part.st);
  }
}

}  // namespace mpxg_srv

extern "C" {

mpxg_status mpxg_server_create(const mpxg_server_desc* d, mpxg_server** out) {
  using namespace mpxg_srv;
  if (!d || !out || d->n_models < 1 || !d->models || d->n_max < 1 || d->streams < 1 || d->streams > 64)
    return fail_lib(MPXG_ERR_INVALID_ARG, "mpxg_server_create: bad arguments");
  *out = nullptr;
  mpxg_server* s = new mpxg_server();
  s->d = *d;
  s->seed = d->seed;
  size_t budget = d->budget_bytes;
  const MixedOps* mops = nullptr;
  if (d->mixed_launch) {  // one mixed-model solve per step: a built pair of two models, its scratch off the budget
    if (d->n_models == 2) {
      const int m0 = d->models[0].desc.model, m1 = d->models[1].desc.model;
      if ((mops = mixed_ops(m0, m1))) { s->mix[0] = 0; s->mix[1] = 1; }
      else if ((mops = mixed_ops(m1, m0))) { s->mix[0] = 1; s->mix[1] = 0; }
    }
    if (!mops) {
      mpxg_server_destroy(s);
      return fail_lib(MPXG_ERR_UNSUPPORTED, "mpxg_server_create: mixed_launch needs two models of a built pair");
    }
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const size_t mixed = (size_t)mops->scratch_floats(d->n_max) * sizeof(float) *
                         ((size_t)sms * mops->resident_blocks(4) * 4);
    if (mixed >= budget) {
      mpxg_server_destroy(s);
      return fail_lib(MPXG_ERR_BUDGET, "mpxg_server_create: the budget does not hold the mixed-model scratch");
    }
    budget -= mixed;
  }
  const size_t share = budget / (size_t)d->n_models;
  s->pools.resize(d->n_models);
  for (int i = 0; i < d->n_models; ++i) {
    Pool& p = s->pools[i];
    p.m = d->models[i];
    if (!model_layout(p.m.desc.model, &p.n, &p.mu, &p.legs, &p.rc, &p.pc) || p.m.desc.n != p.n ||
        p.m.desc.m != p.mu) {
      mpxg_server_destroy(s);
      return fail_lib(MPXG_ERR_UNSUPPORTED, "mpxg_server_create: unsupported model");
    }
    mpxg_problem_desc pd = p.m.desc;
    pd.n_max = d->n_max;
    pd.batch_max = 1;
    const size_t scratch = mpxg_workspace_bytes(&pd, &d->opts);
    const size_t per = slot_bytes(p.n, p.mu, p.legs, p.rc, p.pc, d->n_max);
    long long cap = share > scratch ? (long long)((share - scratch) / per) : 0;
    if (d->max_slots > 0) cap = std::min<long long>(cap, d->max_slots);
    if (cap < 1) {
      mpxg_server_destroy(s);
      return fail_lib(MPXG_ERR_BUDGET, "mpxg_server_create: the budget leaves no slot for a model");
    }
    p.cap = (int)cap;
    pd.batch_max = p.cap;
    if (mpxg_create(&pd, &d->opts, &p.h) != MPXG_OK) {
      std::string m = mpxg_last_error(nullptr);
      mpxg_server_destroy(s);
      return fail_lib(MPXG_ERR_OUT_OF_MEMORY, "mpxg_server_create: " + m);
    }
    int wpb, bps, sms;
    mpxg_query_geometry(p.h, &wpb, &bps, &sms);
    p.total_warps = wpb * bps * sms;
    const size_t C = (size_t)p.cap, NM = (size_t)d->n_max;
    bool ok = cudaMalloc(&p.x0, C * p.n * 4) == cudaSuccess && cudaMalloc(&p.X, C * (NM + 1) * p.n * 4) == cudaSuccess &&
              cudaMalloc(&p.U, C * NM * p.mu * 4) == cudaSuccess && cudaMalloc(&p.V, C * (NM + 1) * p.n * 4) == cudaSuccess &&
              cudaMalloc(&p.ref, C * (NM + 1) * p.rc * 4) == cudaSuccess &&
              cudaMalloc(&p.par, C * (NM + 1) * p.pc * 4) == cudaSuccess && cudaMalloc(&p.w, C * 24 * 4) == cudaSuccess &&
              cudaMalloc(&p.kkt, C * 3 * 4) == cudaSuccess && cudaMalloc(&p.vref, C * 4) == cudaSuccess &&
              cudaMalloc(&p.lt, C * p.legs * 4) == cudaSuccess && cudaMalloc(&p.horizon, C * 4) == cudaSuccess &&
              cudaMalloc(&p.status, C * 4) == cudaSuccess;
    if (ok) ok = cudaMemset(p.horizon, 0, C * 4) == cudaSuccess && cudaMemset(p.X, 0, C * (NM + 1) * p.n * 4) == cudaSuccess &&
                 cudaMemset(p.U, 0, C * NM * p.mu * 4) == cudaSuccess && cudaMemset(p.V, 0, C * (NM + 1) * p.n * 4) == cudaSuccess;
    if (!ok) {
      cudaGetLastError();
      mpxg_server_destroy(s);
      return fail_lib(MPXG_ERR_OUT_OF_MEMORY, "mpxg_server_create: pool allocation failed");
    }
    p.free_slots.reserve(p.cap);
    for (int k = p.cap - 1; k >= 0; --k) p.free_slots.push_back(k);
  }
  if (mops && mpxg_mixed_create(s->pools[s->mix[0]].h, s->pools[s->mix[1]].h, &s->mixed) != MPXG_OK) {
    std::string m = mpxg_last_error(nullptr);
    mpxg_server_destroy(s);
    return fail_lib(MPXG_ERR_OUT_OF_MEMORY, "mpxg_server_create: " + m);
  }
  for (int k = 0; k < d->streams; ++k) {
    cudaStream_t st;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
      cudaGetLastError();
      mpxg_server_destroy(s);
      return fail_lib(MPXG_ERR_CUDA, "mpxg_server_create: stream creation failed");
    }
    s->streams.push_back(st);
    s->stream_busy.push_back(0);
  }
  // A batch's staging (pinned slot ids and mapped result rows) is taken per
  // launch; allocate as many per pool as batches can run at once now, so
  // that no pinned allocation (milliseconds, and synchronising) lands in the
  // served stream
  for (Pool& p : s->pools) {
    std::vector<Staging*> made;
    for (int k = 0; k < d->streams; ++k) {
      Staging* st = get_staging(s, p);
      if (!st) {
        for (Staging* m : made) p.idle.push_back(m);
        mpxg_server_destroy(s);
        return fail_lib(MPXG_ERR_OUT_OF_MEMORY, "mpxg_server_create: staging allocation failed");
      }
      made.push_back(st);
    }
    for (Staging* m : made) p.idle.push_back(m);
  }
  *out = s;
  return MPXG_OK;
}

void mpxg_server_destroy(mpxg_server* s) {
  if (!s) return;
  for (cudaStream_t st : s->streams) cudaStreamSynchronize(st);
  for (auto& b : s->inflight)
    for (auto& part : b.parts) s->pools[part.model].idle.push_back(part.st);
  s->inflight.clear();
  if (s->mixed) mpxg_mixed_destroy(s->mixed);
  for (auto& p : s->pools) mpxg_srv::free_pool(p);
  for (cudaStream_t st : s->streams) cudaStreamDestroy(st);
  delete s;
}

int mpxg_server_capacity(const mpxg_server* s, int model) {
  if (!s || model < 0 || model >= (int)s->pools.size()) return 0;
  return s->pools[model].cap;
}

mpxg_status mpxg_server_admit(mpxg_server* s, int model, const float* x0, int horizon, float v_ref, float phase,
                              int* episode) {
  using namespace mpxg_srv;
  if (!s || !x0 || !episode || model < 0 || model >= (int)s->pools.size())
    return s ? fail(s, MPXG_ERR_INVALID_ARG, "mpxg_server_admit: bad arguments") : MPXG_ERR_INVALID_ARG;
  if (horizon < 1 || horizon > s->d.n_max) return fail(s, MPXG_ERR_INVALID_ARG, "mpxg_server_admit: horizon");
  Pool& p = s->pools[model];
  if (p.free_slots.empty())
    return fail(s, MPXG_ERR_BUDGET, "mpxg_server_admit: device-memory budget exhausted for this model");
  const int slot = p.free_slots.back();
  float lt[4];
  for (int i = 0; i < p.legs; ++i) {
    float v = p.m.phase0[i] + phase;
    lt[i] = v - std::floor(v);
  }
  // synchronous copies into the free slot (no batch can be using it)
  cudaError_t e = cudaMemcpy(p.x0 + (size_t)slot * p.n, x0, p.n * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(p.horizon + slot, &horizon, 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(p.vref + slot, &v_ref, 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(p.lt + (size_t)slot * p.legs, lt, p.legs * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(p.w + (size_t)slot * 24, p.m.w, 24 * 4, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_err(s, e, "mpxg_server_admit");
  p.free_slots.pop_back();
  Episode ep;
  ep.model = model;
  ep.slot = slot;
  ep.horizon = horizon;
  const int id = s->next_episode++;
  s->eps[id] = ep;
  *episode = id;
  return MPXG_OK;
}

mpxg_status mpxg_server_reset(mpxg_server* s, int episode, const float* x0) {
  using namespace mpxg_srv;
  if (!s) return MPXG_ERR_INVALID_ARG;
  auto it = s->eps.find(episode);
  if (it == s->eps.end()) return fail(s, MPXG_ERR_INVALID_ARG, "mpxg_server_reset: unknown episode");
  if (x0) {
    if (it->second.busy > 0) return fail(s, MPXG_ERR_NOT_READY, "mpxg_server_reset: episode has ticks in flight");
    Pool& p = s->pools[it->second.model];
    cudaError_t e = cudaMemcpy(p.x0 + (size_t)it->second.slot * p.n, x0, p.n * 4, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_err(s, e, "mpxg_server_reset");
  }
  it->second.cold = true;
  return MPXG_OK;
}

mpxg_status mpxg_server_release(mpxg_server* s, int episode) {
  using namespace mpxg_srv;
  if (!s) return MPXG_ERR_INVALID_ARG;
  auto it = s->eps.find(episode);
  if (it == s->eps.end()) return fail(s, MPXG_ERR_INVALID_ARG, "mpxg_server_release: unknown episode");
  if (it->second.busy > 0) it->second.retiring = true;
  else retire(s, episode);
  return MPXG_OK;
}

mpxg_status mpxg_submit(mpxg_server* s, int episode, long long* ticket) {
  using namespace mpxg_srv;
  if (!s || !ticket) return MPXG_ERR_INVALID_ARG;
  auto it = s->eps.find(episode);
  if (it == s->eps.end() || it->second.retiring)
    return fail(s, MPXG_ERR_INVALID_ARG, "mpxg_submit: unknown or released episode");
  const long long id = s->next_ticket++;
  Ticket t;
  t.episode = episode;
  std::memset(&t.res, 0, sizeof(t.res));
  s->tickets[id] = t;
  it->second.busy += 1;
  s->pools[it->second.model].pending.push_back(id);
  s->queued += 1;
  *ticket = id;
  return MPXG_OK;
}

mpxg_status mpxg_submit_many(mpxg_server* s, const int* episodes, int n, long long* tickets) {
  if (!s || n < 0 || (n > 0 && (!episodes || !tickets))) return MPXG_ERR_INVALID_ARG;
  for (int i = 0; i < n; ++i) {
    mpxg_status r = mpxg_submit(s, episodes[i], tickets + i);
    if (r != MPXG_OK) return r;
  }
  return MPXG_OK;
}

mpxg_status mpxg_server_step(mpxg_server* s, int block, int* launched, int* finished) {
  using namespace mpxg_srv;
  if (!s) return MPXG_ERR_INVALID_ARG;
  int nfin = 0, nlaunch = 0;
  if (block && !s->inflight.empty()) {  // wait for the oldest running batch
    cudaError_t e = cudaEventSynchronize(s->inflight.front().ev());
    if (e != cudaSuccess) return cuda_err(s, e, "mpxg_server_step");
  }
  nfin += deliver_arrived(s);  // results of instances that finished, before their batch ends
  for (size_t i = 0; i < s->inflight.size();) {  // collect every finished batch, in any order
    cudaError_t e = cudaEventQuery(s->inflight[i].ev());
    if (e == cudaErrorNotReady) { ++i; continue; }
    if (e != cudaSuccess) return cuda_err(s, e, "mpxg_server_step");
    for (const auto& part : s->inflight[i].parts)
      for (char g : part.got) nfin += g ? 0 : 1;
    reap(s, i);
  }
  // the idle episodes' pending tickets of pool mi (claimed for a batch)
  auto take = [&](int mi) {
    Pool& p = s->pools[mi];
    std::vector<long long> batch, later;
    batch.reserve(p.pending.size());
    for (long long tk : p.pending) {
      Episode& e = s->eps[s->tickets[tk].episode];
      if (e.running) { later.push_back(tk); continue; }
      e.running = true;  // claims the episode for this batch
      batch.push_back(tk);
    }
    p.pending.swap(later);
    for (long long tk : batch) s->eps[s->tickets[tk].episode].running = false;
    return batch;
  };
  if (s->mixed) {  // both models' ticks in one mixed-model solve
    if ((int)s->inflight.size() < (int)s->streams.size()) {
      std::vector<Part> parts(2);
      for (int k = 0; k < 2; ++k) {
        parts[k].model = s->mix[k];
        parts[k].tickets = take(s->mix[k]);
      }
      const int n = (int)(parts[0].tickets.size() + parts[1].tickets.size());
      if (n > 0) {
        mpxg_status r = launch(s, std::move(parts));
        if (r != MPXG_OK) return r;
        nlaunch += n;
      }
    }
  } else {
    for (size_t mi = 0; mi < s->pools.size() && (int)s->inflight.size() < (int)s->streams.size(); ++mi) {
      std::vector<Part> parts(1);
      parts[0].model = (int)mi;
      parts[0].tickets = take((int)mi);
      const int n = (int)parts[0].tickets.size();
      if (n == 0) continue;
      mpxg_status r = launch(s, std::move(parts));
      if (r != MPXG_OK) return r;
      nlaunch += n;
    }
  }
  if (launched) *launched = nlaunch;
  if (finished) *finished = nfin;
  return MPXG_OK;
}

mpxg_status mpxg_poll(mpxg_server* s, long long ticket, mpxg_result* result) {
  if (!s || !result) return MPXG_ERR_INVALID_ARG;
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end()) return mpxg_srv::fail(s, MPXG_ERR_INVALID_ARG, "mpxg_poll: unknown ticket");
  if (!it->second.done) return MPXG_ERR_NOT_READY;
  *result = it->second.res;
  s->tickets.erase(it);
  return MPXG_OK;
}

mpxg_status mpxg_server_completed(mpxg_server* s, mpxg_result* results, int max, int* count) {
  if (!s || !count || (max > 0 && !results)) return MPXG_ERR_INVALID_ARG;
  int n = 0;
  while (n < max && !s->done.empty()) {
    const long long tk = s->done.front();
    s->done.pop_front();
    auto it = s->tickets.find(tk);
    if (it == s->tickets.end()) continue;  // already taken by mpxg_poll
    results[n++] = it->second.res;
    s->tickets.erase(it);
  }
  *count = n;
  return MPXG_OK;
}

mpxg_status mpxg_server_stats(const mpxg_server* s, int* queued, int* running, long long* launches) {
  if (!s) return MPXG_ERR_INVALID_ARG;
  int run = 0;
  for (const auto& b : s->inflight)
    for (const auto& part : b.parts) run += (int)part.tickets.size();
  if (queued) *queued = s->queued;
  if (running) *running = run;
  if (launches) *launches = s->launches;
  return MPXG_OK;
}

const char* mpxg_server_last_error(const mpxg_server* s) { return s ? s->err.c_str() : ""; }

}  // extern "C"
