"""Launch-geometry autotuner for the batched solve.

The persistent solve kernel runs one instance per warp; its grid is
(SMs x blocks per SM) blocks of `warps_per_block` warps.  The best pair
depends on the model (registers, shared memory per warp), the horizon mix and
the batch size, so it is measured: each candidate solves the caller's own
batch a few times (CUDA events, after a warm-up solve) and the fastest is
kept.  Results are cached per (GPU, model, n_max, batch, SQP iterations) in a
JSON file (MPXG_TUNE_CACHE, default ~/.cache/mpxg/tune.json).
"""
import json
import os

import torch

from .solver import Solver

DEFAULT_CANDIDATES = [(wpb, bps) for wpb in (1, 2, 4) for bps in (0, 2, 3, 4)]


def _cache_path():
    return os.environ.get("MPXG_TUNE_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "mpxg", "tune.json"))


def _key(desc, opts, n_max, batch):
    name = torch.cuda.get_device_name() if torch.cuda.is_available() else "cpu"
    return "%s|model%d|n_max%d|batch%d|iters%d" % (name, desc.model, n_max, batch, opts.sqp_iters)


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


def time_geometry(wl, opts, warps_per_block, blocks_per_sm, reps=5, device=None):
    """Mean ms of one batched solve of workload `wl` with this geometry."""
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


def tune(wl, opts, candidates=None, reps=5, use_cache=True, device=None):
    """Measure every (warps_per_block, blocks_per_sm) candidate on `wl` (0 =
    the occupancy-derived default) and return dict(best=(wpb, bps),
    ms=..., table=[{wpb, bps, ms, geometry}, ...], cached=bool)."""
    key = _key(wl.desc, opts, wl.n_max, wl.batch)
    cache = _load() if use_cache else {}
    if use_cache and key in cache:
        r = dict(cache[key])
        r["best"] = tuple(r["best"])
        r["cached"] = True
        return r
    table = []
    for wpb, bps in (candidates or DEFAULT_CANDIDATES):
        try:
            ms, geo = time_geometry(wl, opts, wpb, bps, reps=reps, device=device)
        except Exception as e:  # e.g. a geometry the device cannot hold
            table.append(dict(wpb=wpb, bps=bps, ms=None, error=str(e)[:120]))
            continue
        table.append(dict(wpb=wpb, bps=bps, ms=ms, geometry=geo))
    ok = [r for r in table if r.get("ms") is not None]
    if not ok:
        raise RuntimeError("autotune: no candidate geometry ran: %s" % table)
    best = min(ok, key=lambda r: r["ms"])
    res = dict(best=(best["wpb"], best["bps"]), ms=best["ms"], table=table, cached=False)
    if use_cache:
        cache[key] = dict(best=list(res["best"]), ms=res["ms"], table=table)
        _store(cache)
    return res
