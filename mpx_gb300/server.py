"""Serving: continuous batching of MPC control ticks on one GPU.

Each request is one control tick of a persistent episode (a robot).  The
server keeps every admitted episode's warm start -- X, U, V, gait timers,
horizon, weights -- resident on the device in a fixed pool of slots, so a tick
moves only slot indices in and one result row (first control, KKT residual,
status) out.  Requests that arrive while earlier batches are still running go
into the next batch, launched on another CUDA stream so that it overlaps the
running ones on the device (continuous batching); a batch is one persistent
solve launch over the scattered pool rows of its requests
(mpxg_batch_io.slot), preceded by the warm-start shift and the gait tables of
those rows.  Cold starts and the per-tick state drift are made on the device
by the gait-table kernel, so the host issues four launches and two copies per
batch and nothing per request.

Admission is by a device-memory budget: pool slots plus the solver scratch
must fit; an episode that does not fit is refused with BudgetError (the C ABI
status MPXG_ERR_BUDGET).  A slot whose solve returns non-finite values is
cold-started at its next tick (the NaN fallback of
mpx/utils/mpc_wrapper.py:79-98,261-282).
"""
import collections
import ctypes
import time

import numpy as np
import torch

from . import _lib
from . import problem as P
from .solver import Solver, _ptr, _stream_handle, gait_tables, problem_desc, solver_opts


class BudgetError(RuntimeError):
    """No slot left inside the device-memory budget (MPXG_ERR_BUDGET)."""


Request = collections.namedtuple("Request", "rid episode arrival")


def slot_bytes(desc, n_max):
    """Device bytes of one episode slot."""
    n, m = desc.n, desc.m
    f = (n_max + 1) * n * 2 + n_max * m + (n_max + 1) * (desc.ref_cols + desc.par_cols)
    f += n + 24 + 3 + desc.n_contact + 1     # x0, w, kkt, leg timers, v_ref
    return 4 * f + 4 * 2                    # + horizon and status


class _Pool:
    """Slots of one model: device arrays with a leading slot dimension."""

    def __init__(self, name, desc, gait, capacity, n_max, opts, dev):
        self.name, self.desc, self.gait, self.cap, self.n_max, self.dev = name, desc, gait, capacity, n_max, dev
        n, m, rc, pc = desc.n, desc.m, desc.ref_cols, desc.par_cols
        z = lambda *s, dt=torch.float32: torch.zeros(*s, device=dev, dtype=dt)
        self.x0 = z(capacity, n)
        self.X, self.U, self.V = z(capacity, n_max + 1, n), z(capacity, n_max, m), z(capacity, n_max + 1, n)
        self.ref, self.par = z(capacity, n_max + 1, rc), z(capacity, n_max + 1, pc)
        self.w, self.kkt = z(capacity, 24), z(capacity, 3)
        self.status = z(capacity, dt=torch.int32)
        self.horizon = torch.ones(capacity, device=dev, dtype=torch.int32)
        self.v_ref = z(capacity)
        self.leg_time = z(capacity, desc.n_contact)
        # one handle serves the batches of every stream: its warps claim
        # scratch slots per launch and each solve takes its own work counter
        self.solver = Solver(desc, opts, n_max=n_max, batch_max=capacity, device=dev)
        self.out = dict(X=self.X, U=self.U, V=self.V, kkt=self.kkt, status=self.status)
        self.free = list(range(capacity))[::-1]
        # reusable (pinned slot ids, device slot ids, pinned results, device results, event)
        self.staging = []
        self.W = np.diag(gait["W"]).astype(np.float32)


class MPCServer:
    """Continuous-batching server for several compiled models.

    models: {name: (ModelDesc, gait)} with gait = dict(duty, step_freq, height,
    offsets (legs x 3), W (24 x 24 diagonal), phase0 (legs,)).  The budget is
    split evenly between the models; each model's pool holds as many slots as
    fit after its solver scratch."""

    def __init__(self, models, n_max=200, budget_bytes=8 << 30, opts=None, streams=4, device=None, drift_std=0.01,
                 seed=0, max_slots=None):
        self.dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.opts = opts or P.SolverOptions()
        self.n_max = int(n_max)
        self.L = _lib.load()
        self.drift_std = float(drift_std)
        self.seed = int(seed)
        self.pools = {}
        share = budget_bytes // max(len(models), 1)
        for name, (desc, gait) in models.items():
            scratch = int(self.L.mpxg_workspace_bytes(ctypes.byref(problem_desc(desc, self.n_max, 1)),
                                                      ctypes.byref(solver_opts(self.opts))))
            cap = (share - scratch) // slot_bytes(desc, self.n_max)
            if max_slots is not None:
                cap = min(cap, int(max_slots))
            if cap < 1:
                raise BudgetError("budget %d B leaves no slot for model %s" % (budget_bytes, name))
            self.pools[name] = _Pool(name, desc, gait, int(cap), self.n_max, self.opts, self.dev)
        self.episodes = {}          # episode -> [pool name, slot, ticks done, cold start pending, horizon]
        self.pending = collections.defaultdict(list)
        self.streams = [torch.cuda.Stream(device=self.dev) for _ in range(streams)]
        self.next_stream = 0
        self.inflight = collections.deque()
        self.completed = []
        self._rid = 0
        self.launches = 0
        self.busy = collections.Counter()   # episode -> ticks queued or in flight
        self.running = set()                # episodes with a tick in flight
        self.retiring = set()

    # ------------------------------------------------------------ admission
    def capacity(self, name):
        return self.pools[name].cap

    def admit(self, episode, name, x0, horizon, v_ref=0.0, phase=0.0):
        """Give `episode` a resident slot or raise BudgetError.  Its first tick
        cold-starts the warm start from x0 on the device."""
        pool = self.pools[name]
        if not pool.free:
            raise BudgetError("device-memory budget exhausted for model %s (%d slots)" % (name, pool.cap))
        if not (1 <= int(horizon) <= self.n_max):
            raise ValueError("horizon must be in 1..%d" % self.n_max)
        s = pool.free.pop()
        self.episodes[episode] = [name, s, 0, True, int(horizon)]
        n, nc = pool.desc.n, pool.desc.n_contact
        row = np.zeros(n + 2 + nc + 24, dtype=np.float32)
        row[:n] = np.asarray(x0, dtype=np.float32)
        row[n] = float(v_ref)
        row[n + 1] = float(int(horizon))
        row[n + 2:n + 2 + nc] = np.mod(np.asarray(pool.gait["phase0"]) + phase, 1.0)
        row[n + 2 + nc:] = pool.W
        r = torch.from_numpy(row).to(self.dev)
        with torch.no_grad():
            pool.x0[s] = r[:n]
            pool.v_ref[s] = r[n]
            pool.horizon[s] = r[n + 1].to(torch.int32)
            pool.leg_time[s] = r[n + 2:n + 2 + nc]
            pool.w[s] = r[n + 2 + nc:]
        return s

    def reset_slot(self, episode, x0=None):
        """Cold-start the episode's next tick (optionally from a new x0)."""
        name, s = self.episodes[episode][:2]
        if x0 is not None:
            with torch.no_grad():
                self.pools[name].x0[s] = torch.as_tensor(np.asarray(x0, dtype=np.float32), device=self.dev)
        self.episodes[episode][3] = True

    def release(self, episode):
        """Free the episode's slot (deferred until its queued and in-flight ticks complete)."""
        if self.busy.get(episode, 0) > 0:
            self.retiring.add(episode)
            return
        name, s = self.episodes.pop(episode)[:2]
        self.pools[name].free.append(s)

    # ------------------------------------------------------------ requests
    def submit(self, episode, arrival=None):
        """Queue the next control tick of an admitted episode."""
        self._rid += 1
        r = Request(self._rid, episode, time.perf_counter() if arrival is None else arrival)
        self.pending[self.episodes[episode][0]].append(r)
        self.busy[episode] += 1
        return r.rid

    def launch_pending(self):
        """Launch one batch per model with every launchable pending request
        (continuous batching: call whenever requests have arrived)."""
        n = 0
        for name, reqs in list(self.pending.items()):
            if not reqs:
                continue
            self.pending[name] = []
            n += self._launch(self.pools[name], reqs)
        return n

    def _staging(self, pool):
        if pool.staging:
            return pool.staging.pop()
        cap = pool.cap
        return (torch.empty(3 * cap, dtype=torch.int32, pin_memory=True),
                torch.empty(3 * cap, dtype=torch.int32, device=self.dev),
                torch.empty(cap, pool.desc.m + 4, pin_memory=True),
                torch.empty(cap, pool.desc.m + 4, device=self.dev),
                torch.cuda.Event())

    def _launch(self, pool, reqs):
        # one tick per episode at a time: a tick whose episode is still in
        # flight (or repeated in this batch) waits for a later batch
        seen, batch, later = set(), [], []
        for r in reqs:
            (later if (r.episode in seen or r.episode in self.running) else batch).append(r)
            seen.add(r.episode)
        if later:
            self.pending[pool.name].extend(later)
        if not batch:
            return 0
        # longest horizons first: the persistent grid hands out instances in
        # batch order, so this shortens the batch's tail
        batch.sort(key=lambda r: -self.episodes[r.episode][4])
        self.running.update(r.episode for r in batch)
        k = self.next_stream
        st, solver = self.streams[k], pool.solver
        self.next_stream = (k + 1) % len(self.streams)
        st.wait_stream(torch.cuda.current_stream(self.dev))  # admissions are issued on the current stream
        nb = len(batch)
        slots = np.array([self.episodes[r.episode][1] for r in batch], dtype=np.int32)
        first = np.array([self.episodes[r.episode][3] for r in batch], dtype=bool)
        for r in batch:
            self.episodes[r.episode][3] = False
            self.episodes[r.episode][2] += 1
        warm_s, cold_s = slots[~first], slots[first]
        nw, nc = len(warm_s), len(cold_s)
        stg = self._staging(pool)
        slot_h, slot_all, res_h, res_d, ev = stg
        packed = slot_h.numpy()
        packed[:nb] = slots
        packed[nb:nb + nw] = warm_s
        packed[nb + nw:nb + nw + nc] = cold_s
        self.seed += 1
        with torch.cuda.stream(st):
            slot_all[:nb + nw + nc].copy_(slot_h[:nb + nw + nc], non_blocking=True)
            slot_d = slot_all[:nb]
            warm = slot_all[nb:nb + nw]
            cold = slot_all[nb + nw:nb + nw + nc]
            hs = _stream_handle(st)
            if nw:
                _lib.check(self.L.mpxg_shift_warm_start(solver.handle, hs, nw, _ptr(warm), _ptr(pool.horizon), 1,
                                                        _ptr(pool.X), _ptr(pool.U), _ptr(pool.V), _ptr(pool.X),
                                                        _ptr(pool.U), _ptr(pool.V)), solver.handle, "shift")
                gait_tables(st, pool.desc, nw, self.n_max, pool.x0, pool.X, pool.U, pool.V, pool.v_ref,
                            pool.leg_time, pool.ref, pool.par, pool.gait, 1, slot=warm, horizon=pool.horizon,
                            drift_std=self.drift_std, seed=self.seed)
            if nc:
                gait_tables(st, pool.desc, nc, self.n_max, pool.x0, pool.X, pool.U, pool.V, pool.v_ref,
                            pool.leg_time, pool.ref, pool.par, pool.gait, 0, slot=cold, horizon=pool.horizon)
            out = dict(pool.out, first=res_d)
            io = solver.io(pool.x0, pool.X, pool.U, pool.V, pool.ref, pool.par, pool.w, pool.horizon, out, slot=slot_d)
            _lib.check(self.L.mpxg_solve(solver.handle, hs, ctypes.byref(io)), solver.handle, "mpxg_solve")
            res_h[:nb].copy_(res_d[:nb], non_blocking=True)
            ev.record(st)
        self.launches += (2 if nw else 0) + (1 if nc else 0) + solver.launches_per_solve(nb)
        self.inflight.append((ev, pool, batch, stg))
        return nb

    def poll(self, block=False):
        """Collect finished batches; returns [(rid, episode, latency_s, first control, kkt, status)]."""
        done = []
        while self.inflight:
            ev, pool, batch, stg = self.inflight[0]
            if not block and not ev.query():
                break
            ev.synchronize()
            now = time.perf_counter()
            self.inflight.popleft()
            res = stg[2][:len(batch)].numpy().copy()
            pool.staging.append(stg)
            m = pool.desc.m
            for i, r in enumerate(batch):
                status = int(res[i, m + 3])
                if status & _lib.INST_NAN and r.episode in self.episodes:
                    self.episodes[r.episode][3] = True  # cold start next tick (NaN fallback)
                done.append((r.rid, r.episode, now - r.arrival, res[i, :m].copy(), res[i, m:m + 3].copy(), status))
                self.busy[r.episode] -= 1
                self.running.discard(r.episode)
                if r.episode in self.retiring and self.busy[r.episode] == 0:
                    self.retiring.discard(r.episode)
                    self.release(r.episode)
        self.completed.extend(done)
        return done

    def drain(self):
        while self.inflight:
            self.poll(block=True)


def served_workload(server, n_episodes, rate_hz, duration_s, seed=0, horizon_range=(20, 200), episode_ticks=200,
                    models=("quadruped", "biped"), v_range=(-0.5, 0.5)):
    """Poisson request stream (rate_hz) over `n_episodes` concurrent episodes
    of `episode_ticks` ticks; finished episodes are replaced by new ones.
    Runs in real time; returns (latencies in s, wall time in s)."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate_hz, size=int(rate_hz * duration_s * 1.2) + 16)
    arrivals = np.cumsum(gaps)
    arrivals = arrivals[arrivals < duration_s]
    eps = collections.deque()
    counter = [0]

    def new_episode():
        counter[0] += 1
        name = models[counter[0] % len(models)]
        pool = server.pools[name]
        x0 = np.zeros(pool.desc.n, dtype=np.float32)
        x0[2] = pool.gait["height"]
        x0 += rng.normal(0, 0.02, pool.desc.n).astype(np.float32)
        hz = int(rng.integers(horizon_range[0], horizon_range[1] + 1))
        ep = ("ep", seed, counter[0])
        server.admit(ep, name, x0, hz, v_ref=float(rng.uniform(*v_range)), phase=float(rng.uniform()))
        eps.append([ep, 0])

    for _ in range(n_episodes):
        new_episode()
    t0 = time.perf_counter()
    i = 0
    lat = []
    while True:
        now = time.perf_counter() - t0
        while i < len(arrivals) and arrivals[i] <= now:
            ep = eps[0]
            eps.rotate(-1)
            server.submit(ep[0], arrival=t0 + arrivals[i])
            ep[1] += 1
            if ep[1] >= episode_ticks:
                eps.remove(ep)
                server.release(ep[0])  # deferred until its last tick completes
                new_episode()
            i += 1
        if any(server.pending.values()) and len(server.inflight) < len(server.streams):
            server.launch_pending()
        lat.extend(d[2] for d in server.poll())
        if i >= len(arrivals) and not any(server.pending.values()) and not server.inflight:
            break
    wall = time.perf_counter() - t0
    for ep, _ in eps:
        server.release(ep)
    return np.asarray(lat), wall


def default_models():
    """The served mix: SRBD trot quadruped and SRBD walking biped."""
    q = P.quadruped_rpy12()
    b = P.biped_wrench12()
    quad = dict(duty=0.6, step_freq=2.0, height=0.30, offsets=P.HIP_OFFSETS, W=P.quadruped_weights(),
                phase0=P.TROT_PHASE)
    bip = dict(duty=0.6, step_freq=1.25, height=0.90, offsets=P.BIPED_HIP_OFFSETS, W=P.biped_weights(),
               phase0=P.WALK_PHASE)
    return {"quadruped": (q, quad), "biped": (b, bip)}
