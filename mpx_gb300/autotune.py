"""Launch-geometry autotuner for the batched solve.

The persistent solve kernel runs one instance per warp; its grid is
(SMs x blocks per SM) blocks of `warps_per_block` warps.  Long horizons can
instead go to the time-parallel team kernel, 8 warps per instance, from a
horizon threshold on (`team_warps`, `team_min_horizon`).  The best choice
depends on the model (registers, shared memory per warp), the horizon mix and
the batch size, so it is measured: each candidate (warps per block, blocks
per SM, warps per instance, team threshold) solves the caller's own batch a
few times (CUDA events, after a warm-up solve) and the fastest is kept.  A
batched solve ends when its last instance does, so the time measured is both
the batch's latency and its throughput.  Results are cached per (GPU,
model, n_max, batch, SQP iterations) in a JSON file (MPXG_TUNE_CACHE,
default ~/.cache/mpxg/tune.json).
"""
import dataclasses
import json
import os

import torch

from .solver import Solver

# (warps per block, blocks per SM, warps per instance, team threshold); 0 = default
DEFAULT_CANDIDATES = ([(wpb, bps, 0, 0) for wpb in (1, 2, 4) for bps in (0, 2, 3, 4)] +
                      [(4, 0, tw, tmin) for tw in (4, 8) for tmin in (32, 64, 128)])


def _full(c):
    """A candidate as (wpb, bps, team_warps, team_min_horizon)."""
    c = tuple(c)
    return c + (0, 0) if len(c) == 2 else c


def _cache_path():
    return os.environ.get("MPXG_TUNE_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "mpxg", "tune.json"))


def _key(desc, opts, n_max, batch, tag=""):
    name = torch.cuda.get_device_name() if torch.cuda.is_available() else "cpu"
    key = "%s|model%d|n_max%d|batch%d|iters%d" % (name, desc.model, n_max, batch, opts.sqp_iters)
    return key + ("|" + tag if tag else "")


def _load():
    try:
        with open(_cache_path()) as f:
            return json.load(f)
    except Exception:
        return {}


def _store(cache):
    p = _cache_path()
    try:
        os.makedirs(os.path.dirname(p), exist_ok=True)
        with open(p, "w") as f:
            json.dump(cache, f, indent=1)
    except OSError:
        pass


def warm_workload(wl, opts, ticks=3, device=None, drift_std=0.0):
    """The inputs of a steady-state control tick of `wl`: `ticks` warm ticks
    (shift, tables, solve) with the default geometry, then the next tick's
    shift and tables, copied back as a host Workload."""
    from . import problem as P
    from .tick import TickRunner
    tr = TickRunner(wl, opts, device=device, drift_std=drift_std)
    try:
        tr.first_tick()
        for _ in range(ticks):
            tr.tick()
        tr.shift()
        tr.tables()
        torch.cuda.synchronize()
        h = lambda t: t.cpu().numpy()
        return P.Workload(wl.desc, h(tr.x0), h(tr.X), h(tr.U), h(tr.V), h(tr.ref), h(tr.par), wl.W, h(tr.horizon))
    finally:
        tr.solver.close()


def time_geometry(wl, opts, warps_per_block, blocks_per_sm, reps=5, device=None, team_warps=0, team_min_horizon=0):
    """Mean ms of one batched solve of workload `wl` with this geometry."""
    if team_warps:
        opts = dataclasses.replace(opts, team_warps=team_warps, team_min_horizon=team_min_horizon)
    s = Solver(wl.desc, opts, n_max=wl.n_max, batch_max=wl.batch, device=device,
               warps_per_block=warps_per_block, blocks_per_sm=blocks_per_sm)
    try:
        args = s.prepare(wl.x0, wl.X0, wl.U0, wl.V0, wl.reference, wl.parameter, wl.W, wl.horizon)
        out = s.empty_outputs(wl.batch)
        s.solve(*args, out=out)  # warm-up (args: prepared device tensors, w as [B, 24])
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):
            s.solve(*args, out=out)
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps, s.geometry()
    finally:
        s.close()


def tune(wl, opts, candidates=None, reps=5, use_cache=True, device=None, tag=""):
    """Measure every candidate (warps_per_block, blocks_per_sm[, team_warps,
    team_min_horizon]) on `wl` (0 = the occupancy-derived default, no team
    path) and return dict(best=(wpb, bps, team_warps, team_min_horizon),
    ms=..., table=[{wpb, bps, team_warps, team_min_horizon, ms, geometry},
    ...], cached=bool).  `tag` names the kind of state `wl` holds (e.g.
    "warm" for a steady-state tick, whose line searches and convergence
    differ from a cold start's) in the cache key."""
    key = _key(wl.desc, opts, wl.n_max, wl.batch, tag)
    cache = _load() if use_cache else {}
    if use_cache and key in cache:
        r = dict(cache[key])
        r["best"] = tuple(r["best"])
        r["cached"] = True
        return r
    table = []
    for wpb, bps, tw, tm in map(_full, candidates or DEFAULT_CANDIDATES):
        row = dict(wpb=wpb, bps=bps, team_warps=tw, team_min_horizon=tm)
        try:
            if tw:
                ms, geo = time_geometry(wl, opts, wpb, bps, reps=reps, device=device, team_warps=tw,
                                        team_min_horizon=tm)
            else:
                ms, geo = time_geometry(wl, opts, wpb, bps, reps=reps, device=device)
        except Exception as e:  # e.g. a geometry the device cannot hold
            table.append(dict(row, ms=None, error=str(e)[:120]))
            continue
        table.append(dict(row, ms=ms, geometry=geo))
    ok = [r for r in table if r.get("ms") is not None]
    if not ok:
        raise RuntimeError("autotune: no candidate geometry ran: %s" % table)
    best = min(ok, key=lambda r: r["ms"])
    res = dict(best=(best["wpb"], best["bps"], best["team_warps"], best["team_min_horizon"]), ms=best["ms"],
               table=table, cached=False)
    if use_cache:
        cache[key] = dict(best=list(res["best"]), ms=res["ms"], table=table)
        _store(cache)
    return res
