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
  float* res_h = nullptr;  // pinned result rows [cap, m+4]
  float* res_d = nullptr;
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

struct Batch {
  int model = 0, stream = 0;
  Staging* st = nullptr;
  std::vector<long long> tickets;
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
    cudaFree(st->res_d);
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
      cudaMallocHost(&st->res_h, rows) != cudaSuccess || cudaMalloc(&st->res_d, rows) != cudaSuccess ||
      cudaEventCreateWithFlags(&st->ev, cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();
    s->err = "server: staging allocation failed";
    if (st->slot_h) cudaFreeHost(st->slot_h);
    if (st->slot_d) cudaFree(st->slot_d);
    if (st->res_h) cudaFreeHost(st->res_h);
    if (st->res_d) cudaFree(st->res_d);
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

// Launch one batch of `ticks` (all of model `mi`, episodes distinct and idle).
inline mpxg_status launch(mpxg_server* s, int mi, std::vector<long long>& ticks) {
  Pool& p = s->pools[mi];
  std::sort(ticks.begin(), ticks.end(), [&](long long a, long long b) {
    return s->eps[s->tickets[a].episode].horizon > s->eps[s->tickets[b].episode].horizon;
  });
  const int nb = (int)ticks.size();
  Staging* st = get_staging(s, p);
  if (!st) return MPXG_ERR_OUT_OF_MEMORY;
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
  int si = 0;  // an idle stream (the caller checked that one exists)
  while (si < (int)s->streams.size() && s->stream_busy[si]) ++si;
  if (si == (int)s->streams.size()) return fail(s, MPXG_ERR_INVALID_ARG, "server: no idle stream");
  cudaStream_t stream = s->streams[si];
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
  mpxg_batch_io io;
  std::memset(&io, 0, sizeof(io));
  io.batch = nb; io.slot = st->slot_d; io.horizon = p.horizon;
  io.x0 = p.x0; io.X_in = p.X; io.U_in = p.U; io.V_in = p.V;
  io.reference = p.ref; io.parameter = p.par; io.w = p.w;
  io.X = p.X; io.U = p.U; io.V = p.V; io.kkt = p.kkt; io.status = p.status; io.first = st->res_d;
  r = mpxg_solve(p.h, stream, &io);
  if (r != MPXG_OK) return fail(s, r, std::string("server: solve: ") + mpxg_last_error(p.h));
  ce = cudaMemcpyAsync(st->res_h, st->res_d, (size_t)nb * (p.mu + 4) * sizeof(float), cudaMemcpyDeviceToHost,
                       stream);
  if (ce == cudaSuccess) ce = cudaEventRecord(st->ev, stream);
  if (ce != cudaSuccess) return cuda_err(s, ce, "server: result copy");
  s->launches += (nw ? 2 : 0) + (nc ? 1 : 0) + (nb > p.total_warps ? 2 : 1);
  Batch b;
  b.model = mi;
  b.stream = si;
  s->stream_busy[si] = 1;
  b.st = st;
  b.tickets = ticks;
  s->inflight.push_back(std::move(b));
  s->queued -= nb;
  return MPXG_OK;
}

inline void retire(mpxg_server* s, int episode) {
  auto it = s->eps.find(episode);
  if (it == s->eps.end()) return;
  s->pools[it->second.model].free_slots.push_back(it->second.slot);
  s->eps.erase(it);
}

// Reap running batch i (its event has completed).
inline void reap(mpxg_server* s, size_t i) {
  Batch b = std::move(s->inflight[i]);
  s->inflight.erase(s->inflight.begin() + i);
  s->stream_busy[b.stream] = 0;
  Pool& p = s->pools[b.model];
  for (size_t i = 0; i < b.tickets.size(); ++i) {
    Ticket& t = s->tickets[b.tickets[i]];
    const float* row = b.st->res_h + i * (p.mu + 4);
    t.res.ticket = b.tickets[i];
    t.res.episode = t.episode;
    for (int a = 0; a < 12; ++a) t.res.u0[a] = a < p.mu ? row[a] : 0.0f;
    for (int k = 0; k < 3; ++k) t.res.kkt[k] = row[p.mu + k];
    t.res.status = (int)row[p.mu + 3];
    t.done = true;
    s->done.push_back(b.tickets[i]);
    auto it = s->eps.find(t.episode);
    if (it != s->eps.end()) {
      Episode& e = it->second;
      if (t.res.status & MPXG_INST_NAN) e.cold = true;  // NaN fallback: cold start next tick
      e.running = false;
      if (--e.busy == 0 && e.retiring) retire(s, t.episode);
    }
  }
  p.idle.push_back(b.st);
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
  const size_t share = d->budget_bytes / (size_t)d->n_models;
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
  *out = s;
  return MPXG_OK;
}

void mpxg_server_destroy(mpxg_server* s) {
  if (!s) return;
  for (cudaStream_t st : s->streams) cudaStreamSynchronize(st);
  for (auto& b : s->inflight) s->pools[b.model].idle.push_back(b.st);
  s->inflight.clear();
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
    cudaError_t e = cudaEventSynchronize(s->inflight.front().st->ev);
    if (e != cudaSuccess) return cuda_err(s, e, "mpxg_server_step");
  }
  for (size_t i = 0; i < s->inflight.size();) {  // collect every finished batch, in any order
    cudaError_t e = cudaEventQuery(s->inflight[i].st->ev);
    if (e == cudaErrorNotReady) { ++i; continue; }
    if (e != cudaSuccess) return cuda_err(s, e, "mpxg_server_step");
    nfin += (int)s->inflight[i].tickets.size();
    reap(s, i);
  }
  for (size_t mi = 0; mi < s->pools.size() && (int)s->inflight.size() < (int)s->streams.size(); ++mi) {
    Pool& p = s->pools[mi];
    if (p.pending.empty()) continue;
    std::vector<long long> batch, later;
    batch.reserve(p.pending.size());
    for (long long tk : p.pending) {
      Episode& e = s->eps[s->tickets[tk].episode];
      if (e.running) { later.push_back(tk); continue; }
      e.running = true;  // claims the episode for this batch
      batch.push_back(tk);
    }
    p.pending.swap(later);
    if (batch.empty()) continue;
    for (long long tk : batch) s->eps[s->tickets[tk].episode].running = false;
    const int n = (int)batch.size();
    mpxg_status r = launch(s, (int)mi, batch);
    if (r != MPXG_OK) return r;
    nlaunch += n;
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
  for (const auto& b : s->inflight) run += (int)b.tickets.size();
  if (queued) *queued = s->queued;
  if (running) *running = run;
  if (launches) *launches = s->launches;
  return MPXG_OK;
}

const char* mpxg_server_last_error(const mpxg_server* s) { return s ? s->err.c_str() : ""; }

}  // extern "C"
