"""Serving: continuous batching of MPC control ticks on one GPU.

Python face of the native serving runtime (`mpxg_server_*` in
include/mpxg.h, implemented in mpx_gb300/csrc/server.cuh).  Each request is
one control tick of a persistent episode (a robot).  The runtime keeps every
admitted episode's warm start -- X, U, V, gait timers, horizon, weights --
resident on the device in per-model slot pools, so a tick moves only slot
ids in and one result row (first control, KKT residual, status) out.
Requests submitted while earlier batches run form the next batch, launched
on the next free CUDA stream so that batches overlap on the device
(continuous batching); a batch is the warm-start shift and gait tables of its
episodes followed by one persistent solve over their scattered slots.

Admission is by a device-memory budget: an episode that does not fit is
refused with BudgetError (MPXG_ERR_BUDGET).  A slot whose solve returns
non-finite values is cold-started at its next tick (the NaN fallback of
mpx/utils/mpc_wrapper.py:79-98,261-282).
"""
import collections
import ctypes
import gc
import time

import numpy as np
import torch

from . import _lib
from . import problem as P
from .solver import problem_desc, solver_opts

MPXG_ERR_INVALID_ARG = 1
MPXG_ERR_BUDGET = 3


class BudgetError(RuntimeError):
    """No slot left inside the device-memory budget (MPXG_ERR_BUDGET)."""


class _PoolInfo:
    def __init__(self, index, desc, gait, cap):
        self.index, self.desc, self.gait, self.cap = index, desc, gait, cap


class MPCServer:
    """Continuous-batching server for several compiled models.

    models: {name: (ModelDesc, gait)} with gait = dict(duty, step_freq, height,
    offsets (legs x 3), W (24 x 24 diagonal), phase0 (legs,)).  The budget is
    split evenly between the models; each model's pool holds as many slots as
    fit after its solver scratch.  `completed` keeps the last `keep_completed`
    results that poll() returned, oldest first.  mixed_launch=True (two
    models of a built pair, e.g. the rpy12 quadruped and the biped): every
    step solves both models' ticks in one mixed-model launch
    (mpxg_solve_mixed), whose scratch is taken off the budget first."""

    def __init__(self, models, n_max=200, budget_bytes=8 << 30, opts=None, streams=32, device=None, drift_std=0.01,
                 seed=0, max_slots=None, keep_completed=1 << 16, mixed_launch=False):
        self.dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.opts = opts or P.SolverOptions()
        self.n_max = int(n_max)
        self.L = _lib.load()
        names = list(models)
        arr = (_lib.ServedModel * len(names))()
        for i, name in enumerate(names):
            desc, g = models[name]
            sm = arr[i]
            sm.desc = problem_desc(desc, self.n_max, 1)
            sm.duty_factor, sm.step_freq, sm.height = float(g["duty"]), float(g["step_freq"]), float(g["height"])
            off = np.zeros(12, dtype=np.float32)
            o = np.asarray(g["offsets"], dtype=np.float32).reshape(-1)
            off[:o.size] = o
            ph = np.zeros(4, dtype=np.float32)
            p0 = np.asarray(g["phase0"], dtype=np.float32).reshape(-1)
            ph[:p0.size] = p0
            w = np.diag(np.asarray(g["W"], dtype=np.float64)).astype(np.float32)
            for k in range(12):
                sm.offsets[k] = float(off[k])
            for k in range(4):
                sm.phase0[k] = float(ph[k])
            for k in range(24):
                sm.w[k] = float(w[k])
        d = _lib.ServerDesc()
        d.n_models, d.models, d.n_max = len(names), arr, self.n_max
        d.budget_bytes, d.max_slots, d.streams = int(budget_bytes), int(max_slots or 0), int(streams)
        d.drift_std, d.seed, d.opts = float(drift_std), int(seed) & 0xFFFFFFFF, solver_opts(self.opts)
        d.mixed_launch = int(bool(mixed_launch))
        self._models = arr
        h = ctypes.c_void_p()
        with torch.cuda.device(self.dev):
            st = self.L.mpxg_server_create(ctypes.byref(d), ctypes.byref(h))
        if st == MPXG_ERR_BUDGET:
            raise BudgetError(self.L.mpxg_last_error(None).decode())
        _lib.check(st, None, "mpxg_server_create")
        self.handle = h
        self.pools = {name: _PoolInfo(i, models[name][0], models[name][1],
                                      int(self.L.mpxg_server_capacity(h, i))) for i, name in enumerate(names)}
        self.streams = int(streams)
        self.episodes = {}     # key -> episode id
        self._m = {}           # key -> controls per result row
        self._mi = {}          # key -> model index (order of `models`)
        self.model_names = list(names)
        self._arrival = {}     # ticket -> (key, m, arrival time)
        # arrival time and model index of tickets _t_base, _t_base + 1, ...
        # (the vectorised poll_fast path)
        self._t_arr = np.zeros(1 << 16)
        self._t_mod = np.zeros(1 << 16, dtype=np.int8)
        self._t_base = 0
        self.completed = collections.deque(maxlen=int(keep_completed))
        self._res = (_lib.Result * 4096)()
        self._res_np = np.frombuffer(self._res, dtype=np.dtype(
            {"names": ["ticket", "episode", "status", "u0", "kkt"],
             "formats": ["<i8", "<i4", "<i4", ("<f4", 12), ("<f4", 3)],
             "offsets": [_lib.Result.ticket.offset, _lib.Result.episode.offset, _lib.Result.status.offset,
                         _lib.Result.u0.offset, _lib.Result.kkt.offset],
             "itemsize": ctypes.sizeof(_lib.Result)}))

    def close(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            self.L.mpxg_server_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st, what):
        if st != 0:
            raise _lib.MpxgError("%s: %s" % (what, self.L.mpxg_server_last_error(self.handle).decode()))

    # ------------------------------------------------------------ admission
    def capacity(self, name):
        return self.pools[name].cap

    def admit(self, episode, name, x0, horizon, v_ref=0.0, phase=0.0):
        """Give `episode` (any hashable key) a resident slot or raise
        BudgetError.  Its first tick cold-starts the warm start from x0."""
        pool = self.pools[name]
        x = np.ascontiguousarray(np.asarray(x0, dtype=np.float32).reshape(-1))
        eid = ctypes.c_int()
        st = self.L.mpxg_server_admit(self.handle, pool.index, x.ctypes.data, int(horizon), float(v_ref),
                                      float(phase), ctypes.byref(eid))
        if st == MPXG_ERR_BUDGET:
            raise BudgetError("device-memory budget exhausted for model %s (%d slots)" % (name, pool.cap))
        if st == MPXG_ERR_INVALID_ARG:
            raise ValueError(self.L.mpxg_server_last_error(self.handle).decode())
        self._check(st, "admit")
        self.episodes[episode] = eid.value
        self._m[episode] = pool.desc.m
        self._mi[episode] = pool.index
        return eid.value

    def reset_slot(self, episode, x0=None):
        """Cold-start the episode's next tick (optionally from a new x0)."""
        ptr = None
        if x0 is not None:
            x = np.ascontiguousarray(np.asarray(x0, dtype=np.float32).reshape(-1))
            ptr = x.ctypes.data
        self._check(self.L.mpxg_server_reset(self.handle, self.episodes[episode], ptr), "reset")

    def release(self, episode):
        """Free the episode's slot once its queued and running ticks are done."""
        self._check(self.L.mpxg_server_release(self.handle, self.episodes.pop(episode)), "release")

    # ------------------------------------------------------------ requests
    def submit(self, episode, arrival=None):
        """Queue the next control tick of an admitted episode; returns its ticket."""
        t = ctypes.c_longlong()
        self._check(self.L.mpxg_submit(self.handle, self.episodes[episode], ctypes.byref(t)), "submit")
        a = time.perf_counter() if arrival is None else arrival
        self._arrival[t.value] = (episode, self._m[episode], a)
        self._note_arrival(np.array([t.value]), np.array([a]), np.array([self._mi[episode]], dtype=np.int8))
        return t.value

    def _note_arrival(self, tickets, times, models):
        """Record the arrival time and model of new tickets.  The arrays cover
        the tickets from the oldest one still outstanding upwards: when a
        ticket runs past their end they are shifted down to that ticket (and
        doubled only if the tickets in flight need it), so their size follows
        the tickets in flight, not the tickets ever issued."""
        top = int(tickets.max())
        size = self._t_arr.shape[0]
        if top - self._t_base >= size:
            low = min(self._arrival) if self._arrival else int(tickets.min())
            new = size
            while top - low >= new:
                new *= 2
            live = self._t_base + size - low  # entries [low, old end) stay
            arr = np.zeros(new)
            mod = np.zeros(new, dtype=np.int8)
            if live > 0:
                arr[:live] = self._t_arr[low - self._t_base:]
                mod[:live] = self._t_mod[low - self._t_base:]
            self._t_arr, self._t_mod, self._t_base = arr, mod, low
        idx = tickets - self._t_base
        self._t_arr[idx] = times
        self._t_mod[idx] = models

    def _arrivals(self, tickets):
        """(arrival times, model indices) of outstanding tickets."""
        idx = tickets - self._t_base
        return self._t_arr[idx], self._t_mod[idx]

    def submit_many(self, episodes, arrival=None):
        """Queue the next tick of several episodes in one call; returns their tickets."""
        n = len(episodes)
        if n == 0:
            return []
        ids = np.fromiter((self.episodes[e] for e in episodes), dtype=np.int32, count=n)
        t = np.empty(n, dtype=np.int64)
        self._check(self.L.mpxg_submit_many(self.handle, ids.ctypes.data, n, t.ctypes.data), "submit_many")
        times = np.full(n, time.perf_counter()) if arrival is None else np.asarray(arrival, dtype=np.float64)
        for k, e in enumerate(episodes):
            self._arrival[int(t[k])] = (e, self._m[e], times[k])
        self._note_arrival(t, times, np.fromiter((self._mi[e] for e in episodes), dtype=np.int8, count=n))
        return t.tolist()

    def launch_pending(self):
        """Launch queued ticks on free streams (and collect finished batches)."""
        n = ctypes.c_int()
        self._check(self.L.mpxg_server_step(self.handle, 0, ctypes.byref(n), None), "step")
        return n.value

    def stats(self):
        """(ticks queued, ticks running, kernel launches so far)."""
        q, r, launches = ctypes.c_int(), ctypes.c_int(), ctypes.c_longlong()
        self._check(self.L.mpxg_server_stats(self.handle, ctypes.byref(q), ctypes.byref(r), ctypes.byref(launches)),
                    "stats")
        return q.value, r.value, launches.value

    @property
    def launches(self):
        return self.stats()[2]

    def poll(self, block=False):
        """Make progress (collect finished batches, launch queued ticks) and
        return the finished ticks as
        [(ticket, episode, latency_s, first control, kkt, status)]."""
        self._check(self.L.mpxg_server_step(self.handle, 1 if block else 0, None, None), "step")
        now = time.perf_counter()
        done = []
        while True:
            cnt = ctypes.c_int()
            self._check(self.L.mpxg_server_completed(self.handle, self._res, len(self._res), ctypes.byref(cnt)),
                        "completed")
            for i in range(cnt.value):
                r = self._res[i]
                key, m, arrival = self._arrival.pop(r.ticket)
                done.append((r.ticket, key, now - arrival, np.array(r.u0[:m], dtype=np.float32),
                             np.array(r.kkt[:], dtype=np.float32), int(r.status)))
            if cnt.value < len(self._res):
                break
        self.completed.extend(done)
        return done

    def poll_fast(self, block=False, with_model=False):
        """poll() without per-result Python objects: returns (latency_s,
        status, kkt) arrays of the ticks finished now, and with_model their
        model indices (order of `model_names`) as a fourth array (for high
        request rates; the tickets' episodes are not reported)."""
        self._check(self.L.mpxg_server_step(self.handle, 1 if block else 0, None, None), "step")
        now = time.perf_counter()
        lat, st, kk, md = [], [], [], []
        while True:
            cnt = ctypes.c_int()
            self._check(self.L.mpxg_server_completed(self.handle, self._res, len(self._res), ctypes.byref(cnt)),
                        "completed")
            r = self._res_np[:cnt.value]
            tk = r["ticket"]
            t_arr, t_mod = self._arrivals(tk)
            lat.append(now - t_arr)
            st.append(r["status"].copy())
            kk.append(r["kkt"][:, 2].copy())
            md.append(t_mod)
            for t in tk.tolist():
                self._arrival.pop(t, None)
            if cnt.value < len(self._res):
                break
        out = (np.concatenate(lat), np.concatenate(st), np.concatenate(kk))
        return out + (np.concatenate(md),) if with_model else out

    def drain(self):
        """Wait for every queued and running tick."""
        while True:
            q, r, _ = self.stats()
            if q == 0 and r == 0:
                self.poll()
                return
            self.poll(block=True)


class EpisodeStream:
    """Concurrent episodes of a served stream, carried from one call of
    served_workload to the next (so that a measured window can start with
    episodes already warm).  close() releases the episodes still open."""

    def __init__(self, server, seed=0):
        self.server = server
        self.rng = np.random.default_rng(seed)
        self.eps = collections.deque()
        self.counter = 0
        self.seed = seed

    def close(self):
        for ep, _ in self.eps:
            self.server.release(ep)
        self.eps.clear()


def served_workload(server, n_episodes, rate_hz, duration_s, seed=0, horizon_range=(20, 200), episode_ticks=200,
                    models=("quadruped", "biped"), v_range=(-0.5, 0.5), stream=None, stagger=False):
    """Poisson request stream (rate_hz) over `n_episodes` concurrent episodes
    of `episode_ticks` ticks; finished episodes are replaced by new ones.
    Runs in real time; returns (latencies in s, wall time in s); the statuses,
    KKT residuals and model indices of the completed ticks are left in
    server.last_status, server.last_kkt and server.last_model.

    stream: an EpisodeStream to continue (its episodes stay open at return,
    and new ones are admitted only up to n_episodes); None: fresh episodes,
    all released at return.  stagger: the episodes admitted to fill the
    stream start at uniformly drawn ages, so that their ends (and their
    successors' cold starts) spread over time as in a steady stream.

    The loop runs with Python's cyclic garbage collector paused (collected
    once before): a full collection over the process's objects can stall the
    host loop for ~0.1 s, which every request in flight would wait out."""
    own = stream is None
    st = EpisodeStream(server, seed) if own else stream
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate_hz, size=int(rate_hz * duration_s * 1.2) + 16)
    arrivals = np.cumsum(gaps)
    arrivals = arrivals[arrivals < duration_s]
    eps = st.eps

    def new_episode(age=0):
        st.counter += 1
        name = models[st.counter % len(models)]
        pool = server.pools[name]
        x0 = np.zeros(pool.desc.n, dtype=np.float32)
        x0[2] = pool.gait["height"]
        x0 += st.rng.normal(0, 0.02, pool.desc.n).astype(np.float32)
        hz = int(st.rng.integers(horizon_range[0], horizon_range[1] + 1))
        ep = ("ep", st.seed, st.counter)
        server.admit(ep, name, x0, hz, v_ref=float(st.rng.uniform(*v_range)), phase=float(st.rng.uniform()))
        eps.append([ep, age])

    while len(eps) < n_episodes:
        new_episode(int(st.rng.integers(0, episode_ticks)) if stagger else 0)
    gc.collect()
    gc_was_enabled = gc.isenabled()
    gc.disable()
    try:
        return _run_stream(server, st, eps, arrivals, episode_ticks, new_episode, own)
    finally:
        if gc_was_enabled:
            gc.enable()


def _run_stream(server, st, eps, arrivals, episode_ticks, new_episode, own):
    t0 = time.perf_counter()
    i = 0
    lat, stats, kkts, mods = [], [], [], []
    while True:
        now = time.perf_counter() - t0
        keys, arr = [], []
        while i < len(arrivals) and arrivals[i] <= now:
            ep = eps[0]
            eps.rotate(-1)
            keys.append(ep[0])
            arr.append(t0 + arrivals[i])
            ep[1] += 1
            if ep[1] >= episode_ticks:
                eps.remove(ep)
                server.submit_many(keys, arr)
                keys, arr = [], []
                server.release(ep[0])  # deferred until its last tick completes
                new_episode()
            i += 1
        if keys:
            server.submit_many(keys, arr)
        la, stt, kk, md = server.poll_fast(with_model=True)
        lat.append(la); stats.append(stt); kkts.append(kk); mods.append(md)
        if i >= len(arrivals):
            q, r, _ = server.stats()
            if q == 0 and r == 0:
                la, stt, kk, md = server.poll_fast(with_model=True)
                lat.append(la); stats.append(stt); kkts.append(kk); mods.append(md)
                break
    wall = time.perf_counter() - t0
    server.last_status = np.concatenate(stats) if stats else np.zeros(0, np.int32)
    server.last_kkt = np.concatenate(kkts) if kkts else np.zeros(0, np.float32)
    server.last_model = np.concatenate(mods) if mods else np.zeros(0, np.int8)
    if own:
        st.close()
    return np.concatenate(lat) if lat else np.zeros(0), wall


def default_models():
    """The served mix: SRBD trot quadruped and SRBD walking biped."""
    q = P.quadruped_rpy12()
    b = P.biped_wrench12()
    quad = dict(duty=0.6, step_freq=2.0, height=0.30, offsets=P.HIP_OFFSETS, W=P.quadruped_weights(),
                phase0=P.TROT_PHASE)
    bip = dict(duty=0.6, step_freq=1.25, height=0.90, offsets=P.BIPED_HIP_OFFSETS, W=P.biped_weights(),
               phase0=P.WALK_PHASE)
    return {"quadruped": (q, quad), "biped": (b, bip)}
