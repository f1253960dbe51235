"""Benchmark: batched SRBD-quadruped MPC control ticks on GB300.

Workload (the batched configuration the headline metric is quoted on):
4096 roll-pitch-yaw SRBD quadruped MPC instances (n = 12, m = 12), horizons
drawn uniformly from {25, 50, 100}, gait phase offsets uniform on [0, 1),
forward reference speeds uniform on [-1, 1] m/s, trot gait (period 0.5 s,
duty 0.6), 5 SQP iterations per solve, warm start from the shifted previous
solution.  One bench "step" = one control tick of the whole batch (gait
tables + batched solve + warm-start shift), all resident in HBM.

Prints one JSON line (see the keys below).  `--impl reference` times the CPU
restatement of the reference's solver path (the oracle, C++ with OpenMP) on
the host cores instead.
"""
import argparse
import ctypes
import dataclasses
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

BATCH = 4096
HORIZONS = (25, 50, 100)
SQP_ITERS = 5
SEED = 7
DRIFT = 0.0


def f_lqr(n, m):
    """Work-efficient Riccati FLOPs per stage per SQP iteration (backward, forward, costates)."""
    return 4 * n ** 3 + 8 * n * n * m + 4 * n * m * m + m ** 3 / 3 + 4 * n * n + 2 * n * m


# Model FLOPs of one stage and SQP iteration of the roll-pitch-yaw quadruped:
# the linearisation (dynamics with [A B], residual and cone Jacobians, cost,
# Gauss-Newton blocks, gradient, barrier curvature) plus one line-search
# trial, counted by the oracle's counting scalar (oracle/flops.hpp) and
# averaged over the stage rows of the benchmark batch (1181 + 268).
MODEL_FLOPS_RPY12 = 1449


def status_bits(status):
    """Instances with each per-instance status bit set (1 non-finite, 2
    non-positive pivot, 4 line search at its smallest step, 8 bad horizon)."""
    st = np.asarray(status).astype(np.int64)
    return {name: int(((st & bit) != 0).sum())
            for name, bit in (("nonfinite", 1), ("pivot", 2), ("line_search", 4), ("bad_horizon", 8))}


def algorithmic_bytes(n, m, horizon, ref_cols, par_cols):
    """Compulsory HBM bytes of one batched solve: inputs x0, X0, U0, V0,
    reference, parameter, w; outputs X, U, V, kkt, status (float32/int32)."""
    N = np.asarray(horizon, dtype=np.int64)
    per = (n + (N + 1) * n * 2 + N * m + (N + 1) * (ref_cols + par_cols) + 24) + ((N + 1) * n * 2 + N * m + 3 + 1)
    return int(per.sum() * 4)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--batch", type=int, default=BATCH)
    ap.add_argument("--plain-sample", type=int, default=256)
    ap.add_argument("--cpu-sample", type=int, default=1024, help="instances per step of --impl reference")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="CPU baseline sample length")
    ap.add_argument("--no-served", action="store_true", help="skip the served-stream section")
    ap.add_argument("--no-n50", action="store_true", help="skip the fixed-horizon N=50 section")
    ap.add_argument("--no-dropin", action="store_true", help="skip the drop-in wrapper end-to-end section")
    ap.add_argument("--no-autotune", action="store_true", help="use the default launch geometry")
    ap.add_argument("--workload", default="mpc", choices=["mpc", "lqr", "lqr_eq", "wb", "wb_sqp"],
                    help="mpc: the batched SRBD MPC tick (default); lqr: the isolated LQR solve; lqr_eq: the "
                         "equality-constrained n=72 LQ solve")
    ap.add_argument("--lqr-method", type=int, default=0, choices=[0, 1],
                    help="lqr: 0 sequential Riccati, 1 associative scan; lqr_eq: 0 tensor cores, 1 CUDA cores")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-other", action="store_true", help="skip the short LQ runs attached to the MPC line")
    ap.add_argument("--no-graph", action="store_true")
    ap.add_argument("--profile", action="store_true", help="small run for ncu (no clocks, no CPU, no plain)")
    return ap.parse_args()


# ------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons while running."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------ CPU (oracle) timing
class CpuTicks:
    """The oracle port ticking a sample of the batch the way the GPU arm ticks
    the whole batch: warm-start shift, x0 <- the shifted X[0] (no drift), gait
    timers advanced one tick, tables rebuilt, FP32 SQP solve (5 iterations)
    with OpenMP over instances.  Tick 0 is the cold start."""

    def __init__(self, wl, idx, threads):
        from mpx_gb300 import problem as P
        self.P = P
        self.wl = _subset(wl, idx)
        self.threads = threads
        w = self.wl
        self.x0, self.X, self.U, self.V = w.x0.copy(), w.X0.copy(), w.U0.copy(), w.V0.copy()
        self.ref, self.par, self.lt = w.reference, w.parameter, w.leg_time.copy()
        self.ticks = 0

    def tick(self):
        """One control tick of the sample; returns its wall time in s."""
        from oracle import oracle as O
        P, w = self.P, self.wl
        t0 = time.perf_counter()
        if self.ticks > 0:
            self.X, self.U, self.V = P.shift_warm_start(self.X, self.U, self.V, w.horizon)
            _, self.lt = P.timer_run_np(w.duty, w.step_freq, self.lt, w.desc.dt)
            self.x0 = self.X[:, 0].astype(np.float32)
            self.ref, self.par = P.quadruped_tables(w.desc, self.x0, self.lt, w.v_ref, w.horizon, w.n_max,
                                                    duty=w.duty, step_freq=w.step_freq, height=w.height)
        out = O.sqp_solve(w.desc, P.SolverOptions(sqp_iters=SQP_ITERS), self.x0, self.X, self.U, self.V, self.ref,
                          self.par, w.W, w.horizon, precision=32, n_threads=self.threads, want_kkt=False)
        self.X, self.U, self.V = (out[k].astype(np.float32) for k in ("X", "U", "V"))
        self.ticks += 1
        return time.perf_counter() - t0


def _subset(wl, idx):
    from mpx_gb300 import problem as P
    return P.Workload(wl.desc, wl.x0[idx], wl.X0[idx], wl.U0[idx], wl.V0[idx], wl.reference[idx], wl.parameter[idx],
                      wl.W[idx], wl.horizon[idx], leg_time=wl.leg_time[idx], v_ref=wl.v_ref[idx], duty=wl.duty,
                      step_freq=wl.step_freq, height=wl.height)


def cpu_warm_ticks(wl, threads, seconds, sample=512, warm=3):
    """Oracle solves/s of warm-started steady-state ticks: `sample` instances
    of the batch are ticked `warm` times untimed (cold start first), then
    timed tick after tick until `seconds` have elapsed."""
    ct = CpuTicks(wl, np.arange(min(sample, wl.batch)), threads)
    for _ in range(warm):
        ct.tick()
    tot, done = 0.0, 0
    while tot < seconds:
        tot += ct.tick()
        done += ct.wl.batch
    return done / tot, tot, done


def host_info():
    info = {"cpu_count": os.cpu_count()}
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            k, _, v = ln.partition(":")
            if k.strip() in ("Architecture", "Model name", "CPU(s)", "Thread(s) per core", "CPU max MHz"):
                info[k.strip()] = v.strip()
    except Exception:
        pass
    return info


def run_reference(args, rank, world):
    """--impl reference: the oracle (CPU restatement of the path) on host
    cores, ticking a sample of the same workload warm as the GPU arm does."""
    from mpx_gb300 import problem as P
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    wl = P.quadruped_workload(args.batch, horizons=HORIZONS, seed=SEED, model=P.MODEL_SRBD_RPY12, v_range=(-1, 1),
                              random_phase=True)
    sample = min(args.cpu_sample, args.batch)
    ct = CpuTicks(wl, np.arange(sample), threads)
    for _ in range(max(args.warmup, 3)):  # cold start, then warm ticks
        ct.tick()
    times = [ct.tick() for _ in range(args.steps)]
    tot = sum(times)
    value = sample * args.steps / tot
    line = {
        "metric": "MPC solves/s @4096 envs (batched SRBD quadruped, 5 SQP iterations)",
        "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * tot / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32", "data": "synthetic (seeded)", "impl": "reference",
        "config": config_dict(args.batch),
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": threads, "kind": "port",
                         "sample": "the first %d instances of the batch ticked warm (shift, timers, tables, FP32 "
                                   "SQP of 5 iterations; %d untimed ticks from the cold start first), one tick per "
                                   "step; FP32 oracle (C++), OpenMP over instances" % (sample, max(args.warmup, 3)),
                         "host": host_info()},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def _rel_errors(a, o, horizon):
    """Max |a - o| over each instance's valid rows of X, U, V, K, k, relative to
    max |o| (k relative to max |U|: the feedforward tends to 0 at convergence)."""
    out = {}
    for key in ("X", "U", "V", "K", "k"):
        rows = (lambda N: N + 1) if key in ("X", "V") else (lambda N: N)
        err = max(float(np.abs(a[key][i, :rows(N)] - o[key][i, :rows(N)]).max()) for i, N in enumerate(horizon))
        ref = "U" if key == "k" else key
        scale = max(float(np.abs(o[ref][i, :rows(N)]).max()) for i, N in enumerate(horizon))
        out[key] = err / max(scale, 1e-30)
    return out


def fp64_error(tr, opts, stream, sample=64):
    """Error of one steady-state tick of the benchmarked batch against the FP64
    oracle on the same inputs, for `sample` instances drawn from the batch; the
    oracle's own FP32 run on those inputs gives float32's floor.  The tick's
    solution is kept as the batch's state."""
    import torch
    from oracle import oracle as O
    with torch.cuda.stream(stream):
        tr.shift(stream)
        tr.tables(stream)
    torch.cuda.synchronize()
    idx = np.sort(np.random.default_rng(11).choice(tr.wl.batch, size=min(sample, tr.wl.batch), replace=False))
    ins = {k: getattr(tr, k)[idx].cpu().numpy() for k in ("x0", "X", "U", "V", "ref", "par", "w", "horizon")}
    with torch.cuda.stream(stream):
        out = tr.solver.solve(tr.x0, tr.X, tr.U, tr.V, tr.ref, tr.par, tr.w, tr.horizon, stream=stream,
                              want_gains=True)
        for k in ("X", "U", "V"):
            tr.out[k].copy_(out[k])
    torch.cuda.synchronize()
    g = {k: out[k][idx].cpu().numpy() for k in ("X", "U", "V", "K", "k")}
    W = np.stack([np.diag(w) for w in ins["w"]])
    a = (tr.desc, opts, ins["x0"], ins["X"], ins["U"], ins["V"], ins["ref"], ins["par"], W, ins["horizon"])
    o = O.sqp_solve(*a)
    o32 = O.sqp_solve(*a, precision=32)
    kg = O.kkt_residual(tr.desc, ins["x0"], g["X"], g["U"], g["V"], ins["ref"], ins["par"], W, ins["horizon"])
    return {"sample": int(len(idx)), "gpu_vs_fp64": _rel_errors(g, o, ins["horizon"]),
            "oracle_fp32_vs_fp64": _rel_errors(o32, o, ins["horizon"]),
            "kkt_fp64_eval": {"gpu_max": float(kg[:, 2].max()), "oracle_fp64_max": float(o["kkt"][:, 2].max())},
            "what": "one warm tick of the benchmarked batch re-solved with gains; max |gpu - fp64| over each "
                    "instance's valid rows, relative to max |fp64| (k relative to max |U|), over %d sampled "
                    "instances" % len(idx)}


def dropin_wrapper(dev, steps, warmup, n_env=BATCH, smooth=False):
    """End to end through the drop-in API: BatchedMPCControllerWrapper.run (the
    interface of mpx/utils/mpc_wrapper_srbd.py:91-141) on the reference's SRBD
    model and config (quaternion state, N = 25, the reference's barrier) for
    n_env environments.  Every tick passes host numpy arrays in (x0, input,
    foot_op, contact) and reads the first controls back, plus the plan's next
    state, foot references and contact flags, which stand in for the
    simulator's measurements at the next tick."""
    import torch
    from mpx_gb300 import configs
    from mpx_gb300.wrappers import BatchedMPCControllerWrapper
    from mpx_gb300 import problem as P
    cfg = configs.srbd_quadruped()
    desc = None
    if smooth:
        desc = dataclasses.replace(P.quadruped_quat13(cfg), barrier_kind=1, barrier_masked=1, cone_eps2=1.0)
    w = BatchedMPCControllerWrapper(cfg, n_env, device=dev, desc=desc)
    rng = np.random.default_rng(5)
    x0 = np.tile(w.initial_state, (n_env, 1)).astype(np.float32)
    x0[:, :3] += rng.normal(0.0, 0.01, (n_env, 3)).astype(np.float32)
    inp = np.zeros((n_env, 7), dtype=np.float32)
    inp[:, 0] = rng.uniform(-0.5, 0.5, n_env)
    inp[:, 6] = cfg.robot_height
    foot = (np.tile(cfg.p_legs0, (n_env, 1)) + np.tile(x0[:, :3], (1, 4)) * np.array([1, 1, 0] * 4)).astype(np.float32)
    contact = np.ones((n_env, 4), dtype=np.float32)
    state = {"x0": x0, "foot": foot, "contact": contact}

    def tick():
        w.run(state["x0"], inp, state["foot"], state["contact"])
        grf = w.grf.cpu().numpy()
        state["x0"] = w.X[:, 1].cpu().numpy()
        state["foot"] = w.foot_ref.cpu().numpy()
        state["contact"] = w.contact.cpu().numpy().astype(np.float32)
        return grf

    for _ in range(max(warmup, 3)):
        tick()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        tick()
    wall = time.perf_counter() - t0
    kkt = w.kkt[:, 2].cpu().numpy()
    res = {"value": n_env * steps / wall, "unit": "solves/s", "ms_per_tick": 1e3 * wall / steps,
           "h2d_bytes_per_step": n_env * (13 + 7 + 12 + 4) * 4, "d2h_bytes_per_step": n_env * (12 + 13 + 12 + 4) * 4,
           "kkt_frac_le_1e-5": float((kkt <= 1e-5).mean()), "kkt_median": float(np.median(kkt)),
           "what": "%d environments through BatchedMPCControllerWrapper.run with host numpy arrays every tick "
                   "(timer, reference generator, solve, shift: 4 launches), host wall clock; model SRBD_QUAT13 "
                   "with %s, config mpx/config/config_srbd.py (N = 25)" %
                   (n_env, "the smooth stance-masked barrier (cone smoothing 1 N)" if smooth else
                    "the reference's penalty barrier")}
    w.solver.close()
    return res


def _served_entry(srv, lat, wall, offered):
    sk = srv.last_kkt
    return {"offered_req_per_s": offered, "completed_req_per_s": len(lat) / wall, "requests": int(len(lat)),
            "latency_ms": {"p50": 1e3 * float(np.percentile(lat, 50)), "p99": 1e3 * float(np.percentile(lat, 99)),
                           "p999": 1e3 * float(np.percentile(lat, 99.9)), "max": 1e3 * float(np.max(lat))},
            "frac_over_2ms": float((lat > 2e-3).mean()),
            "kkt_frac_le_1e-5": float((sk <= 1e-5).mean()),
            "nan_status": int(((srv.last_status & 1) != 0).sum())}


def queue_latency(dev, opts, N=50, pool=64, reps=200):
    """Round trip of one request through the device work queue (a persistent
    kernel already running; push -> result row on the host, no launch per
    request), and the time to drain `pool` requests pushed at once."""
    import time
    from mpx_gb300 import problem as P
    from mpx_gb300.solver import SolveQueue, Solver
    wl = P.quadruped_workload(pool, horizons=(N,), seed=3, model=P.MODEL_SRBD_RPY12, v_range=(-1, 1),
                              random_phase=True)
    s = Solver(wl.desc, opts, n_max=N, batch_max=pool, device=dev)
    q = SolveQueue(s, (wl.x0, wl.X0, wl.U0, wl.V0, wl.reference, wl.parameter, wl.W, wl.horizon), capacity=4096,
                   idle_timeout_s=10.0)

    def wait(t):
        while True:
            r = q.result(t)
            if r is not None:
                return r

    lat = []
    for k in range(reps + 10):
        t0 = time.perf_counter()
        wait(q.push(k % pool))
        if k >= 10:
            lat.append(time.perf_counter() - t0)
    t0 = time.perf_counter()
    ts = [q.push(r) for r in range(pool)]
    for t in ts:
        wait(t)
    burst = time.perf_counter() - t0
    q.finish()
    s.close()
    lat = np.asarray(lat)
    return {"round_trip_ms": {"p50": 1e3 * float(np.percentile(lat, 50)), "p99": 1e3 * float(np.percentile(lat, 99))},
            "burst_%d_ms" % pool: 1e3 * burst,
            "what": "quadruped SRBD N = %d, 5 SQP iterations: one request pushed into the running queue kernel's "
                    "ring and its result row read back on the host, %d times; then %d requests at once" %
                    (N, reps, pool)}


def lone_latency(dev, opts, horizons=(50, 100, 200), reps=10):
    """Latency of one lone solve (batch 1, CUDA events around the launch) of
    the roll-pitch-yaw quadruped and the biped: one warp per instance (the
    plain path's kernel) and the time-parallel team kernel (8 warps)."""
    import torch
    from mpx_gb300 import problem as P
    from mpx_gb300.solver import Solver
    out = {}
    for name, make in (("quadruped", lambda N: P.quadruped_workload(1, horizons=(N,), seed=3, model=P.MODEL_SRBD_RPY12,
                                                                   v_range=(-1, 1), random_phase=True)),
                       ("biped", lambda N: P.biped_workload(1, horizons=(N,), seed=3))):
        for N in horizons:
            wl = make(N)
            row = {}
            for mode, kw in (("one_warp", {}), ("team8", dict(team_warps=8, team_min_horizon=8))):
                s = Solver(wl.desc, dataclasses.replace(opts, **kw), n_max=N, batch_max=1, device=dev)
                ins = s.prepare(wl.x0, wl.X0, wl.U0, wl.V0, wl.reference, wl.parameter, wl.W, wl.horizon)
                io = s.io(*ins, s.empty_outputs(1))
                st = torch.cuda.current_stream(dev)
                ts = []
                for rep in range(reps + 2):
                    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    a.record(st)
                    assert s.L.mpxg_solve(s.handle, ctypes.c_void_p(st.cuda_stream), ctypes.byref(io)) == 0
                    b.record(st)
                    torch.cuda.synchronize()
                    if rep >= 2:
                        ts.append(a.elapsed_time(b))
                row[mode] = float(np.median(ts))
                s.close()
            row["speedup"] = row["one_warp"] / row["team8"]
            out["%s_N%d_ms" % (name, N)] = row
    return out


def run_served(dev, opts):
    """Served request streams (continuous batching).  Latency is submit to
    result row on the host, with real-time Poisson arrivals; every measured
    window continues episodes that were already running, so it sees the
    stream's steady state rather than a cold start of every episode."""
    from mpx_gb300.server import EpisodeStream, MPCServer, default_models, served_workload
    out = {}
    # config 3: the mixed stream, 200-tick episodes with state drift, one warp per instance; then the same
    # stream with horizons of 64 and more on the time-parallel team kernel (8 warps per instance), and with
    # both models' ticks of a step in one mixed-model launch
    for key, o3, mixed in (("mixed", opts, False),
                           ("mixed_team8", dataclasses.replace(opts, team_warps=8, team_min_horizon=64,
                                                               team_exact_last=True), False),
                           ("mixed_one_launch", opts, True)):
        srv = MPCServer(default_models(), n_max=200, budget_bytes=8 << 30, opts=o3, drift_std=0.01, streams=32,
                        device=dev, mixed_launch=mixed)
        es = EpisodeStream(srv, seed=1)
        served_workload(srv, 400, 20000.0, 0.5, seed=1, stream=es, stagger=True)
        launches0 = srv.launches
        lat, wall = served_workload(srv, 400, 20000.0, 2.0, seed=2, stream=es, stagger=True)
        e = _served_entry(srv, lat, wall, 20000.0)
        e["kkt_frac_le_1e-5_by_model"] = {name: float((srv.last_kkt[srv.last_model == i] <= 1e-5).mean())
                                          for i, name in enumerate(srv.model_names) if (srv.last_model == i).any()}
        e["gpu_launches"] = srv.launches - launches0
        e["workload"] = ("Poisson 20k req/s over 400 concurrent episodes (quadruped SRBD and biped SRBD, "
                         "alternating), N uniform in [20, 200], 200-tick episodes at staggered ages (ended episodes "
                         "are replaced by cold ones), state drift N(0, 0.01^2) per tick, 8 GB admission budget, "
                         "32 streams; 0.5 s warm-up of the same episodes, then 2 s measured; " +
                         {"mixed": "one warp per instance",
                          "mixed_team8": "horizons >= 64 on the time-parallel team kernel (8 warps per instance, "
                                         "the last SQP iteration's KKT step as one sequential sweep: "
                                         "team_exact_last)",
                          "mixed_one_launch": "one warp per instance, both models' ticks of a step in one "
                                              "mixed-model launch (mpxg_solve_mixed)"}[key])
        if key == "mixed":
            out.update(e)
        else:
            out[key] = e
        es.close()
        srv.close()
    # the latency target's case: 4096 robots (N = 50 quadruped episodes that keep running) at rising rates
    for drift, key in ((0.0, "envs4096_n50"), (0.01, "envs4096_n50_drift")):
        srv = MPCServer(default_models(), n_max=50, budget_bytes=8 << 30, opts=opts, drift_std=drift, streams=32,
                        device=dev)
        es = EpisodeStream(srv, seed=3)
        kw = dict(horizon_range=(50, 50), models=("quadruped",), episode_ticks=1 << 30, stream=es)
        served_workload(srv, 4096, 300000.0, 4096 * 10 / 300000.0, seed=3, **kw)  # ~10 ticks per robot first
        sweep = []
        for rate in ((50000.0, 150000.0, 300000.0) if drift == 0.0 else (150000.0,)):
            served_workload(srv, 4096, rate, 0.5, seed=4, **kw)
            l4, w4 = served_workload(srv, 4096, rate, 1.0, seed=5, **kw)
            sweep.append(_served_entry(srv, l4, w4, rate))
        out[key] = {"sweep": sweep,
                    "workload": "4096 concurrent quadruped SRBD episodes, N = 50, 5 SQP iterations, %s; each tick "
                                "x0 <- X[1] of the shifted warm start%s; 32 streams; ~10 ticks per robot before the "
                                "first window, 0.5 s warm-up per rate, 1 s measured" %
                                ("no drift" if drift == 0.0 else "drift N(0, 0.01^2)",
                                 "" if drift == 0.0 else " + drift")}
        es.close()
        srv.close()
    return out


def config_dict(batch):
    return {"workload": "batched SRBD quadruped trot MPC: %d instances, horizons uniform in {25,50,100}, random gait "
                        "phase, v_ref uniform in [-1,1] m/s, 5 SQP iterations, warm-started control ticks" % batch,
            "model": "SRBD_RPY12 (n=12, m=12)", "batch": batch, "horizons": list(HORIZONS), "sqp_iters": SQP_ITERS,
            "l2": "working set larger than L2 (inputs + per-warp scratch)", "parallelism": "replicas"}


# ------------------------------------------------------------ GPU arm
def run_ours(args, rank, world, local_rank):
    import torch
    from mpx_gb300 import problem as P
    from mpx_gb300.replicas import max_over_ranks
    from mpx_gb300.tick import TickRunner

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    B = args.batch
    wl = P.quadruped_workload(B, horizons=HORIZONS, seed=SEED + rank, model=P.MODEL_SRBD_RPY12, v_range=(-1, 1),
                              random_phase=True)
    opts = P.SolverOptions(sqp_iters=SQP_ITERS)
    tuned = None
    wpb, bps, tw, tm = 0, 0, 0, 0
    if not args.no_autotune and not args.profile:
        # geometry measured on the steady-state tick this bench times (a cold
        # first tick runs more line-search trials and favours other shapes)
        from mpx_gb300.autotune import tune, warm_workload
        tuned = tune(warm_workload(wl, opts, device=dev, drift_std=DRIFT), opts, device=dev, tag="warm")
        wpb, bps, tw, tm = tuned["best"]
    tick_opts = dataclasses.replace(opts, team_warps=tw, team_min_horizon=tm) if tw else opts
    tr = TickRunner(wl, tick_opts, device=dev, drift_std=DRIFT, warps_per_block=wpb, blocks_per_sm=bps)
    stream = torch.cuda.Stream(device=dev)
    n, m = wl.desc.n, wl.desc.m
    with torch.cuda.stream(stream):
        tr.first_tick(stream)
        for _ in range(max(args.warmup, 3)):
            tr.tick(stream)
    torch.cuda.synchronize()
    use_graph = not args.no_graph
    if use_graph:
        with torch.cuda.stream(stream):
            tr.capture(stream)
            tr.replay()
        torch.cuda.synchronize()

    # ---------------- device-timed steady-state ticks
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    sev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    clocks = ClockSampler(local_rank) if not args.profile else None
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    if clocks:
        clocks.start()
    with torch.cuda.stream(stream):
        ev[0].record(stream)
        for k in range(args.steps):
            if use_graph:
                tr.replay()
            else:
                tr.shift(stream)
                tr.tables(stream)
                sev[k][0].record(stream)
                tr.solve(stream)
                sev[k][1].record(stream)
            ev[k + 1].record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop() if clocks else None
    tick_ms = [ev[k].elapsed_time(ev[k + 1]) for k in range(args.steps)]
    total_ms = ev[0].elapsed_time(ev[-1])
    total_ms = max_over_ranks(total_ms, device=dev)  # the job ends with its slowest replica
    value = world * B * args.steps / (total_ms / 1000.0)

    # ---------------- solve kernel alone (roofline): ungraphed ticks with events around the solve
    solve_ms = []
    with torch.cuda.stream(stream):
        for k in range(min(args.steps, 10)):
            tr.shift(stream)
            tr.tables(stream)
            sev[k][0].record(stream)
            tr.solve(stream)
            sev[k][1].record(stream)
    torch.cuda.synchronize()
    solve_ms = [sev[k][0].elapsed_time(sev[k][1]) for k in range(min(args.steps, 10))]
    solve_avg = sum(solve_ms) / len(solve_ms)
    kkt = tr.out["kkt"][:, 2].float().cpu().numpy()
    status = tr.out["status"].cpu().numpy()
    # the reference's own stopping test (mpx/utils/mpc_wrapper.py:452-465): the squared defects of each
    # instance's solution summed, sum(c * c) < 1e-5, by the library's residual evaluator
    _, c_ev = tr.solver.evaluate(tr.x0, tr.X, tr.U, tr.ref, tr.par, tr.w, tr.horizon, stream=stream)
    torch.cuda.synchronize()
    sum_c2 = (c_ev.double() ** 2).sum(dim=(1, 2)).cpu().numpy()

    # ---------------- the batch's error against the FP64 oracle (64 sampled instances)
    fp64 = fp64_error(tr, opts, stream) if (not args.profile and rank == 0) else None

    # ---------------- end to end through the public API with host buffers
    x0_host = torch.empty(B, n, pin_memory=True)
    x0_host.copy_(tr.x0.cpu())
    res_host = torch.empty(B, m + 4, pin_memory=True)
    res_dev = torch.empty(B, m + 4, device=dev)
    tr.set_result_rows(res_dev)  # the solve writes [first control | kkt | status] per instance
    e2e_ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    e2e_steps = args.steps
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    t_host0 = time.perf_counter()
    with torch.cuda.stream(stream):
        e2e_ev[0].record(stream)
        for k in range(e2e_steps):
            tr.x0.copy_(x0_host, non_blocking=True)             # measured states in
            tr.shift(stream)
            tr.tables(stream, measured=True)
            tr.solve(stream)
            res_host.copy_(res_dev, non_blocking=True)             # result rows out
        e2e_ev[1].record(stream)
    torch.cuda.synchronize()
    e2e_ms = max_over_ranks(e2e_ev[0].elapsed_time(e2e_ev[1]), device=dev)
    e2e_value = world * B * e2e_steps / (e2e_ms / 1000.0)
    h2d = B * n * 4
    d2h = B * (m + 4) * 4

    # ---------------- plain path comparator (one launch per instance)
    plain = None
    if args.plain_sample > 0 and not args.profile:
        ps = min(args.plain_sample, B)
        sub = P.Workload(wl.desc, wl.x0[:ps], wl.X0[:ps], wl.U0[:ps], wl.V0[:ps], wl.reference[:ps],
                         wl.parameter[:ps], wl.W[:ps], wl.horizon[:ps], leg_time=wl.leg_time[:ps],
                         v_ref=wl.v_ref[:ps])
        tp = TickRunner(sub, opts, device=dev, drift_std=DRIFT)
        with torch.cuda.stream(stream):
            tp.first_tick(stream)
            for _ in range(max(args.warmup, 3)):
                tp.tick(stream)
            tp.shift(stream)
            tp.tables(stream)
        torch.cuda.synchronize()
        from mpx_gb300 import _lib
        from mpx_gb300.solver import _stream_handle
        L = _lib.load()
        # the whole plain sweep: one launch per instance, back to back
        pa, pb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            pa.record(stream)
            st = L.mpxg_solve_plain(tp.solver.handle, _stream_handle(stream), ctypes.byref(tp.io))
            pb.record(stream)
        torch.cuda.synchronize()
        assert st == 0
        plain_ms = pa.elapsed_time(pb)
        # per-launch latency of single-instance plain solves
        lat = []
        nl = min(ps, 64)
        pev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(nl)]
        with torch.cuda.stream(stream):
            for i in range(nl):
                sl = slice(i, i + 1)
                o1 = {k: v[sl] for k, v in tp.out.items()}
                io1 = tp.solver.io(tp.x0[sl], tp.X[sl], tp.U[sl], tp.V[sl], tp.ref[sl], tp.par[sl], tp.w[sl],
                                   tp.horizon[sl], o1)
                pev[i][0].record(stream)
                st = L.mpxg_solve_plain(tp.solver.handle, _stream_handle(stream), ctypes.byref(io1))
                pev[i][1].record(stream)
                assert st == 0
        torch.cuda.synchronize()
        lat = [a.elapsed_time(b) for a, b in pev]
        plain = {"solves_per_s": ps / (plain_ms / 1000.0), "sample": ps, "launches": ps,
                 "ms_per_solve": plain_ms / ps,
                 "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                                "what": "one launch of one instance (%d launches timed)" % nl}}
        tp.solver.close()

    # ---------------- vector-Jacobian product of the converged 4096-instance solve
    vjp = None
    if not args.profile:
        sx, sX, sU, sV = tr.x0.clone(), tr.X.clone(), tr.U.clone(), tr.V.clone()
        gen = torch.Generator(device=dev).manual_seed(5)
        gX = torch.randn(sX.shape, generator=gen, device=dev)
        gU = torch.randn(sU.shape, generator=gen, device=dev)
        vst = torch.cuda.current_stream()
        tr.solver.vjp(sx, sX, sU, sV, tr.ref, tr.par, tr.w, gX, gU, tr.horizon, stream=vst)  # warm-up
        torch.cuda.synchronize()
        va, vb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        va.record(vst)
        for _ in range(10):
            vout = tr.solver.vjp(sx, sX, sU, sV, tr.ref, tr.par, tr.w, gX, gU, tr.horizon, stream=vst)
        vb.record(vst)
        torch.cuda.synchronize()
        vms = va.elapsed_time(vb) / 10
        vjp = {"ms_per_batch": vms, "instances_per_s": B / (vms / 1000.0),
               "what": "mpxg_solve_vjp on the converged %d-instance tick: gradients w.r.t. x0 and the reference "
                       "for random cotangents of X, U (one adjoint LQR per instance)" % B,
               "finite": bool(torch.isfinite(vout["gx0"]).all().item())}

    # ---------------- the same batch with every horizon N = 50
    n50 = None
    if not args.no_n50 and not args.profile:
        wl50 = P.quadruped_workload(B, horizons=(50,), seed=SEED + rank, model=P.MODEL_SRBD_RPY12, v_range=(-1, 1),
                                    random_phase=True)
        t50 = TickRunner(wl50, opts, device=dev, drift_std=DRIFT)
        with torch.cuda.stream(stream):
            t50.first_tick(stream)
            for _ in range(max(args.warmup, 3)):
                t50.tick(stream)
        torch.cuda.synchronize()
        a50, b50 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            a50.record(stream)
            for _ in range(args.steps):
                t50.tick(stream)
            b50.record(stream)
        torch.cuda.synchronize()
        ms50 = a50.elapsed_time(b50) / args.steps
        k50 = t50.out["kkt"][:, 2].float().cpu().numpy()
        n50 = {"solves_per_s_per_gpu": B / (ms50 / 1000.0), "ms_per_tick": ms50, "horizon": 50,
               "kkt_frac_le_1e-5": float((k50 <= 1e-5).mean())}
        t50.solver.close()
        del t50

    # ---------------- served request stream (continuous batching), rank 0
    served = None
    if not args.no_served and not args.profile and rank == 0:
        served = run_served(dev, opts)

    # ---------------- one lone solve: one warp vs the time-parallel team kernel
    lone = lone_latency(dev, opts) if (not args.profile and rank == 0) else None
    queue = queue_latency(dev, opts) if (not args.profile and rank == 0) else None

    # ---------------- end to end through the drop-in wrapper API (reference model and config)
    dropin = None
    if not args.profile and rank == 0 and not args.no_dropin:
        dropin = dropin_wrapper(dev, min(args.steps, 20), args.warmup)
        dropin["smooth_barrier"] = dropin_wrapper(dev, min(args.steps, 20), args.warmup, smooth=True)

    # ---------------- CPU baseline (oracle, rank 0)
    cpu = None
    if rank == 0 and not args.no_cpu and not args.profile:
        threads = os.cpu_count() or 1
        v, dt, done = cpu_warm_ticks(wl, threads, args.cpu_seconds, sample=min(1024, B))
        cpu = {"value": v, "unit": "solves/s", "cores": threads, "kind": "port",
               "sample": "%d solves in %.1f s: the first %d instances of the batch ticked warm (shift, timers, "
                         "tables, 5 SQP iterations) after 3 untimed ticks from the cold start; FP32 oracle (C++, "
                         "-O3), OpenMP over instances" % (done, dt, min(1024, B)),
               "host": host_info()}
        # secondary figure: the same port on one thread
        v1, dt1, done1 = cpu_warm_ticks(wl, 1, 3.0, sample=64)
        cpu["single_thread"] = {"value": v1, "unit": "solves/s", "cores": 1,
                                "sample": "%d solves in %.1f s (64 instances ticked warm), one thread" % (done1, dt1)}

    # ---------------- roofline of the solve kernel
    import json as _json
    peaks = {}
    try:
        peaks = _json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    alg_bytes = algorithmic_bytes(n, m, wl.horizon, wl.desc.ref_cols, wl.desc.par_cols)
    achieved = alg_bytes / (solve_avg / 1000.0) / 1e9
    traffic = None
    try:
        tj = _json.load(open(os.path.join(ROOT, "profiles", "sqp_rpy12_traffic.json")))
        # bytes per (instance x stage) from a small capture, scaled to this launch
        traffic = float(tj["dram_bytes_per_instance_stage"]) * float(np.sum(wl.horizon))
    except Exception:
        traffic = None
    flops = float(np.sum(wl.horizon)) * SQP_ITERS * f_lqr(n, m)
    model_flops = float(np.sum(wl.horizon)) * SQP_ITERS * MODEL_FLOPS_RPY12
    fp32_nominal = 152 * 128 * 2 * 2.07e9 / 1e12

    line = {
        "metric": "MPC solves/s @4096 envs (batched SRBD quadruped, 5 SQP iterations)",
        "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32", "data": "synthetic (seeded)", "config": config_dict(B),
        "latency_ms": {"p50": float(np.percentile(tick_ms, 50)), "p99": float(np.percentile(tick_ms, 99)),
                       "what": "per-solve latency = one batched control tick (all instances complete together)"},
        "plain": plain,
        "batched_vs_plain": (value / world) / plain["solves_per_s"] if plain else None,
        "kkt": {"median": float(np.median(kkt)), "p99": float(np.percentile(kkt, 99)),
                "frac_le_1e-5": float((kkt <= 1e-5).mean()), "status_nonzero": int((status != 0).sum()),
                "status_bits": status_bits(status),
                "sum_c2": {"median": float(np.median(sum_c2)), "max": float(sum_c2.max()),
                           "frac_lt_1e-5": float((sum_c2 < 1e-5).mean()),
                           "what": "the reference's stopping test, sum of squared dynamics and initial-state "
                                   "defects per instance (mpc_wrapper.py:465)"}},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "traffic": traffic, "kernel": "sqp_kernel<ModelRpy12>",
                     "solve_ms": solve_avg, "algorithmic_bytes": alg_bytes, "peak_source": "MEASURED_PEAKS.json hbm_gbs"},
        "fp32": {"achieved_tflops": flops / (solve_avg / 1000.0) / 1e12, "nominal_peak_tflops": fp32_nominal,
                 "frac": flops / (solve_avg / 1000.0) / 1e12 / fp32_nominal,
                 "flops": "work-efficient Riccati count per stage per iteration",
                 "model_flops_per_stage_iter": MODEL_FLOPS_RPY12,
                 "achieved_tflops_with_model": (flops + model_flops) / (solve_avg / 1000.0) / 1e12,
                 "frac_with_model": (flops + model_flops) / (solve_avg / 1000.0) / 1e12 / fp32_nominal},
        "n50": n50,
        "fp64_error": fp64,
        "lone_solve_latency_ms": lone,
        "device_queue": queue,
        "e2e_dropin": dropin,
        "vjp": vjp,
        "served": served,
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": tr.launches_per_tick * args.steps,
        "graph": use_graph,
        "clocks": clk,
        "geometry": tr.solver.geometry(),
        "autotune": None if tuned is None else {
            "best": {"warps_per_block": tuned["best"][0], "blocks_per_sm": tuned["best"][1] or "auto",
                     "warps_per_instance": tuned["best"][2] or 1, "team_min_horizon": tuned["best"][3]},
            "cached": tuned["cached"],
            "ms_per_solve": {("%dx%s" % (r["wpb"], r["bps"] or "auto")) +
                             (" team%d>=%d" % (r["team_warps"], r["team_min_horizon"]) if r.get("team_warps") else ""): r.get("ms")
                             for r in tuned["table"]}},
    }
    if not args.no_other and not args.profile:
        line["other_configs"] = other_configs(args, rank, world, local_rank)
    if rank == 0:
        print(json.dumps(line), flush=True)


def other_configs(args, rank, world, local_rank):
    """Short runs of the other workloads (their full lines: --workload lqr /
    lqr_eq / wb): the isolated LQR of 1024 x (n=24, m=12, N=128), sequential
    Riccati; the constrained LQ of 512 x (n=72, m=30, 12 rows, N=100) on the
    tensor cores and on the CUDA cores; the whole-body interface for 4096
    aliengo environments."""
    import copy
    a = copy.copy(args)
    a.steps, a.warmup, a.no_cpu, a.batch = 5, 3, True, BATCH
    out = {}
    a.lqr_method = 0
    l1 = run_lqr(a, rank, world, local_rank, emit=False)
    out["lqr_1024_n24_m12_N128"] = {"metric": "LQR solves/s", "value": l1["value"], "ms_per_step": l1["ms_per_step"],
                                    "method": "sequential Riccati", "fp32_tflops": l1["fp32"]["achieved_tflops"]}
    for method, label in ((0, "tensor_cores"), (1, "cuda_cores")):
        a.lqr_method = method
        l4 = run_lqr_eq(a, rank, world, local_rank, emit=False)
        entry = {"metric": "constrained LQR solves/s", "value": l4["value"], "ms_per_step": l4["ms_per_step"],
                 "kernel": l4["roofline"]["kernel"], "fp32_tflops": l4["fp32"]["achieved_tflops"]}
        if "tensor" in l4:
            entry["tf32_mma_tflops"] = l4["tensor"]["achieved_tflops"]
            entry["tensor_frac"] = l4["tensor"]["frac"]
        entry["sqp"] = {k: l4["sqp"][k] for k in ("value", "ms_per_step", "iters", "kkt_max", "kkt_median")}
        out["lqr_eq_512_n72_m30_p12_N100_" + label] = entry
    w = run_wb(a, rank, world, local_rank, emit=False)
    out["wb_interface_4096_aliengo"] = {"metric": "whole-body interface evaluations/s", "value": w["value"],
                                        "us_per_call": w["us_per_call"], "e2e": w["e2e"]["value"]}
    a.steps = 10
    ws = run_wb_sqp(a, rank, world, local_rank, emit=False)
    out["wb_sqp_aliengo_N25"] = {"metric": ws["metric"], "value": ws["value"], "ms_per_step": ws["ms_per_step"],
                                 "lone": ws["lone"], "batch": ws["batch"], "wrapper": ws["wrapper"]}
    return out


# ------------------------------------------------------------ isolated LQR (KKT) workload
LQR_B, LQR_N, LQR_NX, LQR_NU = 1024, 128, 24, 12


def lqr_data(B, N, n, m, seed, chunk=64):
    """Seeded random time-varying LQR problems (float32), generated in chunks."""
    from mpx_gb300 import problem as P
    parts = [P.random_lq(min(chunk, B - i), n, m, N, seed=seed + i) for i in range(0, B, chunk)]
    return {k: np.concatenate([p[k] for p in parts], 0).astype(np.float32) for k in parts[0]}


def run_lqr(args, rank, world, local_rank, emit=True):
    """--workload lqr: the isolated KKT/LQR solve, B=1024 problems with n=24,
    m=12, N=128 (mpxg_lqr_solve; --lqr-method 0 sequential Riccati, 1 scan)."""
    import torch
    from mpx_gb300 import _lib
    from mpx_gb300.replicas import max_over_ranks
    from mpx_gb300.solver import _ptr, _stream_handle
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    B, N, n, m = LQR_B, LQR_N, LQR_NX, LQR_NU
    d = lqr_data(B, N, n, m, seed=11 + 1000 * rank)
    names = ("A", "B", "c", "Q", "R", "M", "q", "r", "x0")
    host = {k: torch.from_numpy(d[k]).pin_memory() for k in names}
    dv = {k: host[k].to(dev) for k in names}
    outs = dict(K=torch.empty(B, N, m, n, device=dev), k=torch.empty(B, N, m, device=dev),
                X=torch.empty(B, N + 1, n, device=dev), U=torch.empty(B, N, m, device=dev),
                lam=torch.empty(B, N + 1, n, device=dev))
    L = _lib.load()
    method = int(args.lqr_method)
    ws = torch.empty(max(int(L.mpxg_lqr_workspace_bytes(B, N, n, m, method)) // 4, 1), device=dev)
    io = _lib.LqIO()
    io.batch, io.N, io.n, io.m = B, N, n, m
    for name, key in zip(("A", "Bm", "c", "Q", "R", "M", "q", "r", "x0"), names):
        setattr(io, name, _ptr(dv[key]))
    for key in ("K", "k", "X", "U", "lam"):
        setattr(io, key, _ptr(outs[key]))
    io.workspace = _ptr(ws)
    stream = torch.cuda.Stream(device=dev)
    hs = _stream_handle(stream)

    def solve():
        _lib.check(L.mpxg_lqr_solve(hs, ctypes.byref(io), method), None, "mpxg_lqr_solve")

    with torch.cuda.stream(stream):
        for _ in range(max(args.warmup, 3)):
            solve()
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    clocks = ClockSampler(local_rank)
    clocks.start()
    with torch.cuda.stream(stream):
        ev[0].record(stream)
        for k in range(args.steps):
            solve()
            ev[k + 1].record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    per = [ev[k].elapsed_time(ev[k + 1]) for k in range(args.steps)]
    total_ms = max_over_ranks(ev[0].elapsed_time(ev[-1]), device=dev)
    value = world * B * args.steps / (total_ms / 1000.0)
    # end to end: inputs from pinned host memory in, all outputs back
    out_h = {k: torch.empty(v.shape, pin_memory=True) for k, v in outs.items()}
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    esteps = max(2, min(args.steps, 5))
    with torch.cuda.stream(stream):
        e0.record(stream)
        for _ in range(esteps):
            for k in names:
                dv[k].copy_(host[k], non_blocking=True)
            solve()
            for k in outs:
                out_h[k].copy_(outs[k], non_blocking=True)
        e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = max_over_ranks(e0.elapsed_time(e1), device=dev)
    h2d = sum(host[k].numel() * 4 for k in names)
    d2h = sum(v.numel() * 4 for v in outs.values())
    # roofline: compulsory bytes and work-efficient Riccati FLOPs per launch
    avg_s = (sum(per) / len(per)) / 1000.0
    flops = B * N * f_lqr(n, m)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    fp32_nominal = 152 * 128 * 2 * 2.07e9 / 1e12
    gbs = (h2d + d2h) / avg_s / 1e9
    tfs = flops / avg_s / 1e12
    cpu = None
    if rank == 0 and not args.no_cpu:
        from oracle import oracle as O
        threads = os.cpu_count() or 1
        done, tot, i = 0, 0.0, 0
        while tot < args.cpu_seconds:
            sl = slice(i, i + 64)
            t0 = time.perf_counter()
            O.lqr_solve(*[d[k][sl] for k in names], precision=32, n_threads=threads)
            tot += time.perf_counter() - t0
            done += 64
            i = (i + 64) % B
        cpu = {"value": done / tot, "unit": "solves/s", "cores": threads, "kind": "port",
               "sample": "%d LQR solves (64-problem chunks of the batch) in %.1f s: sequential Riccati, FP32 oracle "
                         "(C++, -O3), OpenMP over problems" % (done, tot), "host": host_info()}
    line = {
        "metric": "LQR solves/s (isolated KKT solve, n=24, m=12, N=128, batch 1024)",
        "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32", "data": "synthetic (seeded)",
        "config": {"workload": "1024 random time-varying LQR problems, n=24, m=12, N=128 (A = I + 0.05 G rescaled "
                               "to spectral radius 0.98, B ~ N(0,1/m), Q = M M^T/n + 0.1 I, R = 0.1 I, S = 0)",
                   "method": ["sequential Riccati", "associative scan"][method],
                   "l2": "inputs (1.2 GB) larger than L2", "parallelism": "replicas"},
        "roofline": {"bound": "hbm" if gbs / hbm_peak >= tfs / fp32_nominal else "fp32", "achieved": gbs,
                     "peak": hbm_peak, "unit": "GB/s", "frac": gbs / hbm_peak, "traffic": None,
                     "algorithmic_bytes": h2d + d2h, "kernel": "mpxg_lqr_solve method %d" % method},
        "fp32": {"achieved_tflops": tfs, "nominal_peak_tflops": fp32_nominal, "frac": tfs / fp32_nominal,
                 "flops": "work-efficient Riccati count F_LQR(24,12) = 127,872 per stage"},
        "cpu_baseline": cpu,
        "e2e": {"value": world * B * esteps / (e2e_ms / 1000.0), "unit": "solves/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": args.steps * (1 if method == 0 else 1),
        "clocks": clk,
    }
    if rank == 0 and emit:
        print(json.dumps(line), flush=True)
    return line


def run_lqr_eq(args, rank, world, local_rank, emit=True):
    """--workload lqr_eq: 512 equality-constrained LQ problems, n=72, m=30,
    12 equality rows per stage, N=100 (mpxg_lqr_eq_solve_method; --lqr-method
    0: stage products on the tensor cores, 1: on the CUDA cores)."""
    import torch
    from mpx_gb300 import _lib
    from mpx_gb300 import problem as P
    from mpx_gb300.replicas import max_over_ranks
    from mpx_gb300.solver import _ptr, _stream_handle
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    B = 512 if args.batch == BATCH else int(args.batch)  # --batch: a smaller case for profiling
    N, n, m, ne = 100, 72, 30, 12
    parts = [P.random_lq_eq(min(32, B - i), n, m, ne, N, seed=31 + i + 1000 * rank) for i in range(0, B, 32)]
    d = {k: np.concatenate([p[k] for p in parts], 0).astype(np.float32) for k in parts[0]}
    names = ("A", "B", "c", "Q", "R", "M", "q", "r", "C", "D", "e", "x0")
    dv = {k: torch.from_numpy(d[k]).to(dev) for k in names}
    outs = dict(K=torch.empty(B, N, m, n, device=dev), k=torch.empty(B, N, m, device=dev),
                Knu=torch.empty(B, N, ne, n, device=dev), knu=torch.empty(B, N, ne, device=dev),
                X=torch.empty(B, N + 1, n, device=dev), U=torch.empty(B, N, m, device=dev),
                lam=torch.empty(B, N + 1, n, device=dev), nu=torch.empty(B, N, ne, device=dev))
    L = _lib.load()
    ws = torch.empty(int(L.mpxg_lqr_eq_workspace_bytes(B, N, n)) // 4, device=dev)
    io = _lib.LqEqIO()
    io.batch, io.N, io.n, io.m, io.n_eq = B, N, n, m, ne
    for name, key in zip(("A", "Bm", "c", "Q", "R", "M", "q", "r", "C", "D", "e", "x0"), names):
        setattr(io, name, _ptr(dv[key]))
    for key in outs:
        setattr(io, key, _ptr(outs[key]))
    io.workspace = _ptr(ws)
    stream = torch.cuda.Stream(device=dev)
    hs = _stream_handle(stream)

    method = int(args.lqr_method)

    def solve():
        _lib.check(L.mpxg_lqr_eq_solve_method(hs, ctypes.byref(io), method), None, "mpxg_lqr_eq_solve")

    with torch.cuda.stream(stream):
        for _ in range(max(args.warmup, 3)):
            solve()
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    clocks = ClockSampler(local_rank)
    clocks.start()
    with torch.cuda.stream(stream):
        ev[0].record(stream)
        for _ in range(args.steps):
            solve()
        ev[1].record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    total_ms = max_over_ranks(ev[0].elapsed_time(ev[1]), device=dev)
    avg_s = total_ms / args.steps / 1000.0
    # work: Riccati count + the constraint elimination (Schur complement) per stage
    f_eq = f_lqr(n, m) + 2 * (m * m * ne + m * ne * n + ne * ne * n + ne * n * n)
    flops = B * N * f_eq
    in_bytes = sum(dv[k].numel() * 4 for k in names)
    out_bytes = sum(v.numel() * 4 for v in outs.values())
    fp32_nominal = 152 * 128 * 2 * 2.07e9 / 1e12
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    gbs = (in_bytes + out_bytes) / avg_s / 1e9
    line = {
        "metric": "constrained LQR solves/s (n=72, m=30, 12 equality rows, N=100, batch %d)" % B,
        "value": world * B / avg_s, "unit": "solves/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32", "data": "synthetic (seeded)",
        "config": {"workload": "512 equality-constrained LQ problems: A = I + 0.1 J (J ~ N(0,1/n), spectral radius "
                               "<= 1.01), B ~ N(0,0.1/m), Q diagonal log-uniform [1e-2,1e2], R = 1e-3 I, 12 rows "
                               "[C D] ~ N(0,1) per stage", "parallelism": "replicas"},
        "roofline": {"bound": "hbm", "achieved": gbs, "peak": hbm_peak, "unit": "GB/s", "frac": gbs / hbm_peak,
                     "traffic": None, "algorithmic_bytes": in_bytes + out_bytes,
                     "kernel": ["lqr_eq_tc_kernel<72,30,12>", "lqr_eq_kernel<72,30,12>"][method]},
        "fp32": {"achieved_tflops": flops / avg_s / 1e12, "nominal_peak_tflops": fp32_nominal,
                 "frac": flops / avg_s / 1e12 / fp32_nominal,
                 "flops": "F_LQR(72,30) + Schur-complement elimination per stage = %d" % f_eq},
        "method": ["tensor cores (tcgen05 split-TF32 stage products)", "CUDA cores (float32)"][method],
        "gpu_launches": args.steps,
        "clocks": clk,
    }
    if method == 0:
        # MMA work issued per stage: alpha and beta 128 x 112 x 72, gamma
        # 128 x 80 x 48 (tiles padded to M = 128), three TF32 MMAs per product
        mma = 3 * 2 * (2 * 128 * 112 * 72 + 128 * 80 * 48)
        tf32_peak = float(peaks.get("bf16_tflops", 1900.0)) / 2.0
        ach = B * N * mma / avg_s / 1e12
        line["tensor"] = {"achieved_tflops": ach, "peak_tflops": tf32_peak, "frac": ach / tf32_peak,
                          "peak_source": "TF32 = half the measured bf16 dense rate (MEASURED_PEAKS.json bf16_tflops)",
                          "flops": "TF32 MMA work issued per stage (padded tiles, 3 MMAs per split product) = %d"
                                   % mma}
    line["sqp"] = lqr_eq_sqp_leg(L, io, dv, outs, ws, stream, method, args.steps, dev)
    if rank == 0 and emit:
        print(json.dumps(line), flush=True)
    return line


def lqr_eq_sqp_leg(L, io, dv, outs, ws, stream, method, steps, dev, iters=2):
    """The same problems through SQP iterations (mpxg_lqr_eq_sqp): every step
    restarts from the zero iterate, forms the step problem at the iterate,
    solves it with the constrained Riccati and takes the full step, `iters`
    times, then evaluates the KKT residual.  Reports solves/s and the KKT
    residuals reached."""
    import torch
    from mpx_gb300 import _lib
    from mpx_gb300.solver import _ptr, _stream_handle
    B, N, n, m, ne = io.batch, io.N, io.n, io.m, io.n_eq
    sio = _lib.LqEqSqpIO()
    sio.lq = io
    step = torch.empty(int(L.mpxg_lqr_eq_sqp_workspace_bytes(B, N, n, m, ne)) // 4, device=dev)
    kkt = torch.empty(B, 3, device=dev)
    sio.iters, sio.method, sio.kkt, sio.step = iters, method, _ptr(kkt), _ptr(step)
    hs = _stream_handle(stream)

    def solve():
        outs["X"].zero_()
        outs["U"].zero_()
        _lib.check(L.mpxg_lqr_eq_sqp(hs, ctypes.byref(sio)), None, "mpxg_lqr_eq_sqp")

    with torch.cuda.stream(stream):
        for _ in range(3):
            solve()
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    with torch.cuda.stream(stream):
        ev[0].record(stream)
        for _ in range(steps):
            solve()
        ev[1].record(stream)
    torch.cuda.synchronize()
    ms = ev[0].elapsed_time(ev[1]) / steps
    k = kkt.cpu().numpy()
    return {"metric": "constrained LQ SQP solves/s (%d iterations from the zero iterate + KKT)" % iters,
            "value": B / (ms / 1000.0), "ms_per_step": ms, "iters": iters,
            "kkt_max": float(np.nanmax(k[:, 2])), "kkt_median": float(np.median(k[:, 2])),
            "primal_max": float(np.nanmax(k[:, 0])), "dual_rel_max": float(np.nanmax(k[:, 1])),
            "launches_per_step": 3 * iters + 2,
            "note": "launches: per iteration step data, constrained Riccati, step; then KKT and its finish "
                    "(plus two memsets of the iterate)"}


# ------------------------------------------------------------ whole-body interface workload
WB_B = 4096


def run_wb(args, rank, world, local_rank, emit=True):
    """--workload wb: the SRBD controller's whole-body torque interface
    (mpc_utils.py:276-313, mpxg_wb_interface) for 4096 aliengo environments
    at seeded random states; outputs tau and the contact Jacobians."""
    import torch
    from mpx_gb300 import configs, mjcf
    from mpx_gb300.replicas import max_over_ranks
    from mpx_gb300.wholebody import WholeBodyModel
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    B = WB_B if args.batch == BATCH else int(args.batch)
    model = mjcf.load_npz(os.path.join(ROOT, "tests", "golden", "aliengo_wb.npz"))
    wb = WholeBodyModel(model, device=dev)
    cfg = configs.srbd_quadruped()
    rng = np.random.default_rng(41 + 1000 * rank)
    q0 = np.load(os.path.join(ROOT, "tests", "golden", "aliengo_wb.npz"))["q0"]
    quat = rng.normal(size=(B, 4))
    quat /= np.linalg.norm(quat, axis=1, keepdims=True)
    host = dict(qpos=np.concatenate([rng.normal(size=(B, 3)) * 0.3 + [0, 0, 0.3], quat,
                                     q0 + rng.normal(size=(B, 12)) * 0.2], axis=1),
                qvel=rng.normal(size=(B, 18)), grf=rng.normal(size=(B, 12)) * 30,
                foot_ref=rng.normal(size=(B, 12)) * 0.05, foot_ref_dot=rng.normal(size=(B, 12)) * 0.2)
    host = {k: torch.from_numpy(v.astype(np.float32)).pin_memory() for k, v in host.items()}
    host["contact"] = torch.from_numpy(rng.integers(0, 2, size=(B, 4)).astype(np.int32)).pin_memory()
    dv = {k: v.to(dev) for k, v in host.items()}
    Kp = torch.as_tensor(cfg.Kp, dtype=torch.float32, device=dev)
    Kd = torch.as_tensor(cfg.Kd, dtype=torch.float32, device=dev)
    stream = torch.cuda.Stream(device=dev)

    def step(d):
        return wb.interface(d["qpos"], d["qvel"], d["grf"], d["foot_ref"], d["foot_ref_dot"], d["contact"], Kp, Kd,
                            stream=stream)

    tau_host = torch.empty(B, 12).pin_memory()
    with torch.cuda.stream(stream):
        for _ in range(max(args.warmup, 3)):
            step(dv)
    torch.cuda.synchronize()
    # the per-tick call replayed as CUDA graphs: the kernel alone, and end to
    # end (host inputs copied in and tau read back inside the graph)
    g_kernel, g_e2e = torch.cuda.CUDAGraph(), torch.cuda.CUDAGraph()
    with torch.cuda.graph(g_kernel, stream=stream):
        step(dv)
    with torch.cuda.graph(g_e2e, stream=stream):
        for k in host:
            dv[k].copy_(host[k], non_blocking=True)
        tau_e2e, _ = step(dv)
        tau_host.copy_(tau_e2e, non_blocking=True)
    with torch.cuda.stream(stream):
        for _ in range(max(args.warmup, 3)):
            g_kernel.replay()
            g_e2e.replay()
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(6)]
    clocks = ClockSampler(local_rank)
    clocks.start()
    with torch.cuda.stream(stream):
        ev[0].record(stream)
        for _ in range(args.steps):
            g_kernel.replay()
        ev[1].record(stream)
        ev[2].record(stream)
        for _ in range(args.steps):
            g_e2e.replay()
        ev[3].record(stream)
        ev[4].record(stream)
        for _ in range(args.steps):
            step(dv)
        ev[5].record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    eager_ms = max_over_ranks(ev[4].elapsed_time(ev[5]), device=dev)
    total_ms = max_over_ranks(ev[0].elapsed_time(ev[1]), device=dev)
    e2e_ms = max_over_ranks(ev[2].elapsed_time(ev[3]), device=dev)
    avg_s = total_ms / args.steps / 1000.0
    h2d = sum(v.numel() * v.element_size() for v in host.values())
    out_bytes = B * (12 + 18 * 12) * 4
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    gbs = (h2d + out_bytes) / avg_s / 1e9
    line = {
        "metric": "whole-body interface evaluations/s (aliengo, nv = 18, 4 contacts)",
        "value": world * B / avg_s, "unit": "evaluations/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "us_per_call": total_ms / args.steps * 1e3,
        "eager_us_per_call": eager_ms / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32",
        "data": "synthetic (seeded states around the reference's q0)",
        "config": {"workload": "%d environments: whole_body_interface (mpc_utils.py:276-313) with config_srbd Kp, Kd"
                               % B, "parallelism": "replicas", "l2": "inputs (%.1f MB) stay in L2: the call is "
                               "latency-bound" % ((h2d + out_bytes) / 1e6),
                   "timing": "CUDA graph replays of the call (eager_us_per_call: the Python call per step)"},
        "roofline": {"bound": "hbm", "achieved": gbs, "peak": hbm_peak, "unit": "GB/s", "frac": gbs / hbm_peak,
                     "traffic": None, "algorithmic_bytes": h2d + out_bytes, "kernel": "wb_kernel<true>"},
        "e2e": {"value": world * B / (e2e_ms / args.steps / 1000.0), "unit": "evaluations/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": B * 12 * 4},
        "gpu_launches": 3 * args.steps,  # wb_kernel: graph, end-to-end graph, eager
        "clocks": clk,
    }
    if not args.no_cpu and rank == 0:
        sys.path.insert(0, ROOT)
        from oracle import wholebody as W
        n, t0 = 0, time.perf_counter()
        hq = {k: v.numpy() for k, v in host.items()}
        while time.perf_counter() - t0 < min(args.cpu_seconds, 5.0) and n < B:
            W.interface(model, cfg.Kp, cfg.Kd, hq["qpos"][n], hq["qvel"][n], hq["grf"][n], hq["foot_ref"][n],
                        hq["foot_ref_dot"][n], hq["contact"][n])
            n += 1
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": n / dt, "unit": "evaluations/s", "cores": 1, "kind": "port",
                                "sample": "%d environments through the float64 numpy oracle (one thread)" % n}
    if rank == 0 and emit:
        print(json.dumps(line), flush=True)
    return line


# ------------------------------------------------------------ whole-body SQP workload
WBS_N, WBS_ITERS, WBS_BATCH = 25, 5, 64


def run_wb_sqp(args, rank, world, local_rank, emit=True):
    """--workload wb_sqp: the whole-body MPC solve of mpc_wrapper.py's
    wrappers (mpxg_wb_sqp; aliengo, config_aliengo.py: N = 25, dt = 0.02,
    its W), 5 SQP iterations per control tick, warm-started from the shifted
    previous solution with x0 = X[1] of it, on seeded synthetic instances
    (problem.wb_workload).  Two figures: one instance per solve (the
    single-environment MPCControllerWrapper; p50/p99 over the timed ticks),
    and a batch of 64 (the batched wrapper) in solves/s."""
    import torch
    from mpx_gb300 import configs, mjcf, problem
    from mpx_gb300.replicas import max_over_ranks
    from mpx_gb300.wholebody import WholeBodyModel, WholeBodySQP
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    fix = os.path.join(ROOT, "tests", "golden", "aliengo_wb.npz")
    model = mjcf.load_npz(fix)
    d = np.load(fix)
    cfg = configs.aliengo_wb()
    wb = WholeBodyModel(model, device=dev)
    N = WBS_N
    Bb = WBS_BATCH if args.batch == BATCH else int(args.batch)
    steps = max(3, min(args.steps, 30))
    res = {}
    clocks = ClockSampler(local_rank)
    clocks.start()
    for label, B in (("lone", 1), ("batch", Bb)):
        wl = problem.wb_workload(B, N, d["q0"], d["p_legs0"], float(np.sum(model.mass)), seed=21 + 1000 * rank)
        sqp = WholeBodySQP(wb, N=N, batch_max=B, iters=WBS_ITERS)
        ref = torch.as_tensor(wl["reference"], device=dev)
        cont = torch.as_tensor(wl["contact"], device=dev)
        Wd = torch.as_tensor(cfg.W_diag, device=dev)
        out = sqp.solve(wl["x0"], wl["X0"], wl["U0"], wl["V0"], ref, cont, Wd, iters=12)
        sh = lambda a: torch.cat([a[:, 1:], a[:, -1:]], 1)
        times, kkts = [], []
        for tick in range(max(args.warmup, 3) + steps):
            X, U, V = out["X"], out["U"], out["V"]
            ref, cont = sh(ref), sh(cont)
            x0, Xs, Us, Vs = X[:, 1].contiguous(), sh(X), sh(U), sh(V)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            out = sqp.solve(x0, Xs, Us, Vs, ref, cont, Wd, inplace=True)
            e1.record()
            torch.cuda.synchronize()
            if tick >= max(args.warmup, 3):
                times.append(e0.elapsed_time(e1))
                kkts.append(out["kkt"][:, 2].cpu().numpy())
        t = np.array(times)
        kk = np.concatenate(kkts)
        res[label] = {"batch": B, "ms_p50": float(np.percentile(t, 50)), "ms_p99": float(np.percentile(t, 99)),
                      "solves_per_s": B / (float(np.mean(t)) / 1000.0),
                      "kkt_frac_le_1e-5": float(np.mean(kk <= 1e-5)), "kkt_median": float(np.median(kk)),
                      "ticks": len(times)}
    # the drop-in controller end to end: MPCControllerWrapper(config_aliengo).run(qpos, qvel, input,
    # contact) from host arrays to (tau, q, dq) on the host -- feet by forward kinematics, timer,
    # reference generator, solve, shift (mpc_wrapper.py:297-365)
    from mpx_gb300.mpc_wrapper import MPCControllerWrapper
    ctrl = MPCControllerWrapper(cfg, model=model, device=dev)
    rng = np.random.default_rng(5 + rank)
    qpos = np.concatenate([cfg.p0 + rng.normal(0, 0.01, 3), [1.0, 0.0, 0.0, 0.0], cfg.q0]).astype(np.float32)
    qvel = rng.normal(0, 0.05, 18).astype(np.float32)
    inp = np.array([0.3, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0], dtype=np.float32)
    cont = np.ones(4, dtype=np.float32)
    import contextlib
    with contextlib.redirect_stdout(sys.stderr):  # reset() prints as the reference's does
        ctrl.reset(qpos, qvel)
    wt = []
    for tick in range(max(args.warmup, 3) + steps):
        t0 = time.perf_counter()
        tau, q, dq = ctrl.run(qpos, qvel, inp, cont)
        t1 = time.perf_counter()
        if tick >= max(args.warmup, 3):
            wt.append((t1 - t0) * 1e3)
    wt = np.array(wt)
    res["wrapper"] = {"what": "MPCControllerWrapper(config_aliengo).run(qpos, qvel, input, contact) -> (tau, q, dq), "
                              "host numpy in and out, wall clock per call",
                      "ms_p50": float(np.percentile(wt, 50)), "ms_p99": float(np.percentile(wt, 99)),
                      "h2d_bytes_per_step": int(qpos.nbytes + qvel.nbytes + inp.nbytes + cont.nbytes),
                      "d2h_bytes_per_step": int(3 * 12 * 4), "finite": bool(np.all(np.isfinite(tau)))}
    clk = clocks.stop()
    ms = max_over_ranks(res["batch"]["ms_p50"], device=dev)
    line = {
        "metric": "whole-body MPC solves/s (aliengo, 61 states, N = 25, 5 SQP iterations)",
        "value": world * Bb / (ms / 1000.0), "unit": "solves/s", "n_gpus": world, "steps": steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32 (derivatives, Riccati) / fp64 (model step, merit)",
        "data": "synthetic (seeded trotting references and perturbed standing states)",
        "config": {"workload": "%d aliengo whole-body MPCs, N = %d, %d SQP iterations per warm tick" % (Bb, N, WBS_ITERS),
                   "parallelism": "replicas"},
        "lone": res["lone"], "batch": res["batch"], "wrapper": res["wrapper"],
        "gpu_launches": (8 * WBS_ITERS + 4) * steps,
        "clocks": clk,
    }
    if rank == 0 and emit:
        print(json.dumps(line), flush=True)
    return line


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    if args.workload == "lqr":
        run_lqr(args, rank, world, local_rank)
    elif args.workload == "lqr_eq":
        run_lqr_eq(args, rank, world, local_rank)
    elif args.workload == "wb":
        run_wb(args, rank, world, local_rank)
    elif args.workload == "wb_sqp":
        run_wb_sqp(args, rank, world, local_rank)
    else:
        run_ours(args, rank, world, local_rank)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
