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
from .solver import Solver, _ptr, _stream_handle


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
        self.gen = torch.Generator(device=self.dev)
        self.gen.manual_seed(seed)
        self.drift = torch.zeros_like(self.x0)
        if offsets is None:
            offsets = P.BIPED_HIP_OFFSETS if wl.desc.model == P.MODEL_BIPED_WRENCH12 else P.HIP_OFFSETS
        self.offsets = (ctypes.c_float * 12)(*np.asarray(offsets, dtype=np.float32).reshape(-1).tolist(),
                                             *([0.0] * (12 - np.asarray(offsets).size)))
        self.out = dict(X=self.X, U=self.U, V=self.V, kkt=torch.zeros(wl.batch, 3, device=self.dev),
                        status=torch.zeros(wl.batch, dtype=torch.int32, device=self.dev))
        self.io = self.solver.io(self.x0, self.X, self.U, self.V, self.ref, self.par, self.w, self.horizon, self.out)
        self.launches_per_tick = 3
        self.graph = None

    # ------------------------------------------------------------ pieces
    def tables(self, stream=None, from_warm_start=True, advance=True):
        L = self.L
        st = L.mpxg_gait_tables(_stream_handle(stream), int(self.desc.model), int(self.wl.batch), int(self.wl.n_max),
                                _ptr(self.horizon), float(self.desc.dt), float(self.wl.duty),
                                float(self.wl.step_freq), float(self.wl.height), self.offsets,
                                _ptr(self.X) if from_warm_start else None,
                                _ptr(self.drift) if (from_warm_start and self.drift_std > 0) else None,
                                _ptr(self.x0), _ptr(self.v_ref), _ptr(self.leg_time), int(advance),
                                _ptr(self.ref), _ptr(self.par))
        _lib.check(st, None, "mpxg_gait_tables")

    def solve(self, stream=None, plain=False):
        fn = self.L.mpxg_solve_plain if plain else self.L.mpxg_solve
        st = fn(self.solver.handle, _stream_handle(stream), ctypes.byref(self.io))
        _lib.check(st, self.solver.handle, "mpxg_solve")

    def shift(self, stream=None):
        st = self.L.mpxg_shift_warm_start(self.solver.handle, _stream_handle(stream), int(self.wl.batch),
                                          _ptr(self.horizon), 1, _ptr(self.X), _ptr(self.U), _ptr(self.V),
                                          _ptr(self.X), _ptr(self.U), _ptr(self.V))
        _lib.check(st, self.solver.handle, "mpxg_shift_warm_start")

    def new_drift(self):
        if self.drift_std > 0:
            self.drift.normal_(0.0, self.drift_std, generator=self.gen)

    # ------------------------------------------------------------ one tick
    def first_tick(self, stream=None):
        """Tick 0: tables from the given x0 and timers, then solve."""
        self.tables(stream, from_warm_start=False, advance=False)
        self.solve(stream)

    def tick(self, stream=None):
        """Shift the previous solution, x0 <- its second state (+ drift), advance
        the gait one tick, rebuild the tables, solve."""
        self.shift(stream)
        self.tables(stream, from_warm_start=True, advance=True)
        self.solve(stream)

    def capture(self, stream):
        """Capture one tick into a CUDA graph (replayed by replay())."""
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=stream):
            self.tick(torch.cuda.current_stream())
        self.graph = g
        return g

    def replay(self):
        self.graph.replay()
