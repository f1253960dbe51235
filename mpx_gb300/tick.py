"""Device-resident control-tick loop of a batch of SRBD MPC instances.

One tick does what mpx/utils/mpc_wrapper_srbd.py:91-141 does per call of
`run()`: advance the gait timers, build the reference / parameter tables,
solve from the warm start, and shift the warm start for the next tick -- but
for the whole batch, with every array resident in HBM and three of our
kernels per tick (gait tables, SQP solve, shift).  Optionally the ticks are
captured into one CUDA graph and replayed.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from . import problem as P
from .solver import Solver, _ptr, _stream_handle, gait_tables


class TickRunner:
    def __init__(self, wl: P.Workload, opts: P.SolverOptions, device=None, drift_std=0.0, seed=0,
                 warps_per_block=0, blocks_per_sm=0, offsets=None):
        self.wl = wl
        self.desc = wl.desc
        self.dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.solver = Solver(wl.desc, opts, n_max=wl.n_max, batch_max=wl.batch, device=self.dev,
                             warps_per_block=warps_per_block, blocks_per_sm=blocks_per_sm)
        self.L = _lib.load()
        d = lambda a, dt=torch.float32: torch.as_tensor(np.ascontiguousarray(a)).to(self.dev, dt)
        self.x0 = d(wl.x0)
        self.X = d(wl.X0)
        self.U = d(wl.U0)
        self.V = d(wl.V0)
        self.ref = d(wl.reference)
        self.par = d(wl.parameter)
        self.w = self.solver.prepare(wl.x0, wl.X0, wl.U0, wl.V0, wl.reference, wl.parameter, wl.W)[6]
        self.horizon = d(wl.horizon, torch.int32)
        self.v_ref = d(wl.v_ref)
        self.leg_time = d(wl.leg_time)
        self.drift_std = float(drift_std)
        if offsets is None:
            offsets = P.BIPED_HIP_OFFSETS if wl.desc.model == P.MODEL_BIPED_WRENCH12 else P.HIP_OFFSETS
        self.gait = dict(duty=wl.duty, step_freq=wl.step_freq, height=wl.height, offsets=offsets)
        self.seed = int(seed)
        self.out = dict(X=self.X, U=self.U, V=self.V, kkt=torch.zeros(wl.batch, 3, device=self.dev),
                        status=torch.zeros(wl.batch, dtype=torch.int32, device=self.dev))
        self.io = self.solver.io(self.x0, self.X, self.U, self.V, self.ref, self.par, self.w, self.horizon, self.out)
        self.launches_per_tick = 2 + self.solver.launches_per_solve(wl.batch)  # tables, shift, (order,) solve
        self.graph = None

    def set_result_rows(self, first):
        """Have each solve also write one row per instance into `first`
        ([batch, m+4] float32 device tensor: first control, KKT residuals,
        status) -- the rows a caller copies back to the host each tick."""
        self.out["first"] = first
        self.io = self.solver.io(self.x0, self.X, self.U, self.V, self.ref, self.par, self.w, self.horizon, self.out)

    # ------------------------------------------------------------ pieces
    def tables(self, stream=None, first=False, measured=False):
        """Gait tables for all instances.  first=True also cold-starts X, U, V;
        measured=True keeps the x0 already in place (copied from the host)."""
        self.seed += 1
        mode = 0 if first else (2 if measured else 1)
        gait_tables(stream, self.desc, self.wl.batch, self.wl.n_max, self.x0, self.X, self.U, self.V, self.v_ref,
                    self.leg_time, self.ref, self.par, self.gait, mode, horizon=self.horizon,
                    drift_std=self.drift_std, seed=self.seed)

    def solve(self, stream=None, plain=False):
        fn = self.L.mpxg_solve_plain if plain else self.L.mpxg_solve
        st = fn(self.solver.handle, _stream_handle(stream), ctypes.byref(self.io))
        _lib.check(st, self.solver.handle, "mpxg_solve")

    def shift(self, stream=None):
        st = self.L.mpxg_shift_warm_start(self.solver.handle, _stream_handle(stream), int(self.wl.batch), None,
                                          _ptr(self.horizon), 1, _ptr(self.X), _ptr(self.U), _ptr(self.V),
                                          _ptr(self.X), _ptr(self.U), _ptr(self.V))
        _lib.check(st, self.solver.handle, "mpxg_shift_warm_start")

    # ------------------------------------------------------------ one tick
    def first_tick(self, stream=None):
        """Tick 0: cold start from the given x0 and timers, then solve."""
        self.tables(stream, first=True)
        self.solve(stream)

    def tick(self, stream=None):
        """Shift the previous solution, x0 <- its second state (+ drift), advance
        the gait one tick, rebuild the tables, solve."""
        self.shift(stream)
        self.tables(stream, first=False)
        self.solve(stream)

    def capture(self, stream):
        """Capture one tick into a CUDA graph (replayed by replay()).  The
        drift seed is frozen into the graph, so replays repeat one drift draw."""
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=stream):
            self.tick(torch.cuda.current_stream())
        self.graph = g
        return g

    def replay(self):
        self.graph.replay()
