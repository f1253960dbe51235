"""The autotuner's host logic on the CPU, with the timing call replaced by a
fake: it keeps the fastest candidate that ran, records the ones that failed,
caches by (GPU, model, n_max, batch, SQP iterations), and says so when no
candidate runs."""
import json
import types

import pytest

from mpx_gb300 import autotune


def _workload(batch=64, n_max=50, model=1):
    return types.SimpleNamespace(desc=types.SimpleNamespace(model=model), n_max=n_max, batch=batch)


def _fake_timer(times, calls):
    def time_geometry(wl, opts, wpb, bps, reps=5, device=None, team_warps=0, team_min_horizon=0):
        key = (wpb, bps) if not team_warps else (wpb, bps, team_warps, team_min_horizon)
        calls.append(key)
        t = times[key]
        if t is None:
            raise RuntimeError("too many resources requested for launch")
        return t, (wpb, bps or 3, 152)
    return time_geometry


def test_keeps_the_fastest_and_records_failures(tmp_path, monkeypatch):
    monkeypatch.setenv("MPXG_TUNE_CACHE", str(tmp_path / "tune.json"))
    times = {(1, 0): 3.0, (2, 0): 1.5, (4, 0): None, (4, 2): 2.0}
    calls = []
    monkeypatch.setattr(autotune, "time_geometry", _fake_timer(times, calls))
    opts = types.SimpleNamespace(sqp_iters=5)
    r = autotune.tune(_workload(), opts, candidates=list(times), reps=1)
    assert r["best"] == (2, 0, 0, 0) and r["ms"] == 1.5 and not r["cached"]
    assert calls == list(times)
    failed = [t for t in r["table"] if t["ms"] is None]
    assert [(t["wpb"], t["bps"]) for t in failed] == [(4, 0)] and "resources" in failed[0]["error"]
    # the second call is answered from the cache, without timing anything
    calls.clear()
    r2 = autotune.tune(_workload(), opts, candidates=list(times), reps=1)
    assert r2["cached"] and r2["best"] == (2, 0, 0, 0) and calls == []
    stored = json.load(open(tmp_path / "tune.json"))
    assert len(stored) == 1 and list(stored.values())[0]["best"] == [2, 0, 0, 0]


def test_cache_key_separates_workloads(tmp_path, monkeypatch):
    monkeypatch.setenv("MPXG_TUNE_CACHE", str(tmp_path / "tune.json"))
    calls = []
    monkeypatch.setattr(autotune, "time_geometry", _fake_timer({(1, 0): 1.0, (2, 0): 2.0}, calls))
    opts = types.SimpleNamespace(sqp_iters=5)
    for wl in (_workload(batch=64), _workload(batch=128), _workload(n_max=100), _workload(model=2)):
        assert not autotune.tune(wl, opts, candidates=[(1, 0), (2, 0)], reps=1)["cached"]
    assert not autotune.tune(_workload(), types.SimpleNamespace(sqp_iters=3), candidates=[(1, 0)], reps=1)["cached"]
    # a warm-tick state is tuned and cached apart from the cold start of the same shape
    assert not autotune.tune(_workload(), opts, candidates=[(1, 0)], reps=1, tag="warm")["cached"]
    assert autotune.tune(_workload(), opts, candidates=[(1, 0)], reps=1, tag="warm")["cached"]
    assert len(json.load(open(tmp_path / "tune.json"))) == 6


def test_no_candidate_runs(tmp_path, monkeypatch):
    monkeypatch.setenv("MPXG_TUNE_CACHE", str(tmp_path / "tune.json"))
    monkeypatch.setattr(autotune, "time_geometry", _fake_timer({(8, 0): None}, []))
    with pytest.raises(RuntimeError, match="no candidate"):
        autotune.tune(_workload(), types.SimpleNamespace(sqp_iters=5), candidates=[(8, 0)], reps=1)
    assert not (tmp_path / "tune.json").exists()


def test_unreadable_cache_is_ignored(tmp_path, monkeypatch):
    p = tmp_path / "tune.json"
    p.write_text("{not json")
    monkeypatch.setenv("MPXG_TUNE_CACHE", str(p))
    monkeypatch.setattr(autotune, "time_geometry", _fake_timer({(1, 0): 1.0}, []))
    r = autotune.tune(_workload(), types.SimpleNamespace(sqp_iters=5), candidates=[(1, 0)], reps=1)
    assert r["best"] == (1, 0, 0, 0) and not r["cached"]
    assert json.load(open(p))  # rewritten


def test_warps_per_instance_is_a_candidate(tmp_path, monkeypatch):
    """The time-parallel team path (8 warps per instance from a horizon
    threshold on) is searched beside the one-warp geometries, timed with its
    own options, and kept when it is fastest."""
    monkeypatch.setenv("MPXG_TUNE_CACHE", str(tmp_path / "tune.json"))
    times = {(4, 0): 2.0, (4, 0, 8, 64): 1.2, (4, 0, 8, 128): 1.5}
    calls = []
    monkeypatch.setattr(autotune, "time_geometry", _fake_timer(times, calls))
    r = autotune.tune(_workload(), types.SimpleNamespace(sqp_iters=5), candidates=list(times), reps=1)
    assert r["best"] == (4, 0, 8, 64) and calls == list(times)
    assert {(row["team_warps"], row["team_min_horizon"]) for row in r["table"]} == {(0, 0), (8, 64), (8, 128)}
    assert all(len(c) == 4 for c in autotune.DEFAULT_CANDIDATES)
    assert any(c[2] == 8 for c in autotune.DEFAULT_CANDIDATES)
    assert any(c[2] == 4 for c in autotune.DEFAULT_CANDIDATES)
