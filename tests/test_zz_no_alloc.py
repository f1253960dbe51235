"""The allocation-free entry point mpxg_solve_noalloc.

It exists for callers that cannot allocate device memory when they solve --
a real-time control loop that forbids cudaMalloc after start-up, or a plugin
whose host framework hands over only the input and output buffers.  This test
calls it through the C ABI (ctypes) twice in a row on the same inputs and
checks each result against the handle-based mpxg_solve.  Both run the same
kernel on the same inputs, so the results must be equal bit for bit.  The
test allocates its own input/output tensors before the calls; free device
memory is the same before and after the second call (the first may still
let the driver size its per-launch local memory).
"""
import ctypes

import numpy as np
import pytest
import torch

from mpx_gb300 import _lib
from mpx_gb300 import problem as P
from mpx_gb300.solver import Solver, _stream_handle, problem_desc, solver_opts

pytestmark = pytest.mark.gpu


def test_noalloc_matches_handle_solve_twice():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    wl = P.quadruped_workload(96, horizons=(25, 50, 100), seed=21, model=P.MODEL_SRBD_RPY12, v_range=(-1, 1),
                              random_phase=True)
    opts = P.SolverOptions(sqp_iters=5)
    s = Solver(wl.desc, opts, n_max=wl.n_max, batch_max=wl.batch)
    ref = s.solve(wl.x0, wl.X0, wl.U0, wl.V0, wl.reference, wl.parameter, wl.W, wl.horizon)
    torch.cuda.synchronize()
    x0, X0, U0, V0, reference, parameter, w, horizon = ref["_keep"]
    L = _lib.load()
    pd = problem_desc(wl.desc, wl.n_max, wl.batch)
    po = solver_opts(opts)
    outs = [s.empty_outputs(wl.batch) for _ in range(2)]
    for call in range(2):
        out = outs[call]
        io = s.io(x0, X0, U0, V0, reference, parameter, w, horizon, out)
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        st = L.mpxg_solve_noalloc(ctypes.byref(pd), ctypes.byref(po), _stream_handle(None), ctypes.byref(io))
        assert st == 0, L.mpxg_last_error(None)
        torch.cuda.synchronize()
        if call == 1:
            assert torch.cuda.mem_get_info()[0] == free0
        for key in ("X", "U", "V", "kkt", "status"):
            a, b = out[key].cpu().numpy(), ref[key].cpu().numpy()
            for i, N in enumerate(wl.horizon):
                if key in ("kkt", "status"):
                    assert np.array_equal(a[i], b[i]), (call, key, i)
                else:
                    rows = (N + 1) if key in ("X", "V") else N
                    assert np.array_equal(a[i, :rows], b[i, :rows]), (call, key, i)
    s.close()


def _empty_io():
    io = _lib.BatchIO()
    io.batch = 0  # no kernel can launch even if a check below regressed
    dummy = torch.zeros(16, device="cuda")
    for name in ("x0", "X_in", "U_in", "V_in", "reference", "parameter", "w", "X", "U", "V"):
        setattr(io, name, ctypes.c_void_p(dummy.data_ptr()))
    return io, dummy


def test_noalloc_rejects_oversized_problem():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    L = _lib.load()
    desc = P.quadruped_rpy12()
    pd = problem_desc(desc, 1000, 1)  # one warp of scratch per SM no longer fits in 64 MiB
    po = solver_opts(P.SolverOptions())
    io, _keep = _empty_io()
    st = L.mpxg_solve_noalloc(ctypes.byref(pd), ctypes.byref(po), _stream_handle(None), ctypes.byref(io))
    assert st == 1
    assert b"n_max too large" in L.mpxg_last_error(None)


def test_noalloc_rejects_launch_geometry_beyond_its_blocks():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    L = _lib.load()
    pd = problem_desc(P.quadruped_rpy12(), 50, 1)
    io, _keep = _empty_io()
    for wpb, bps in ((5, 0), (-1, 0), (2, -1)):
        po = solver_opts(P.SolverOptions(), warps_per_block=wpb, blocks_per_sm=bps)
        st = L.mpxg_solve_noalloc(ctypes.byref(pd), ctypes.byref(po), _stream_handle(None), ctypes.byref(io))
        assert st == 1, (wpb, bps)
        assert b"warps_per_block" in L.mpxg_last_error(None)
