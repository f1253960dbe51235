"""The model-FLOP figure of the roofline and the bench line's status counts (CPU).

The bench's FP32 work per stage and SQP iteration is the work-efficient
Riccati count plus the model work of the stage, counted by running the
oracle's model functions on the counting scalar of oracle/flops.hpp.  These
tests pin the bench's constant to that count over the benchmark batch and
check the properties the count must have.
"""
import numpy as np

import bench
from mpx_gb300 import problem as P
from oracle import oracle as O


def _bench_batch():
    return P.quadruped_workload(bench.BATCH, horizons=bench.HORIZONS, seed=bench.SEED, model=P.MODEL_SRBD_RPY12,
                                v_range=(-1, 1), random_phase=True)


def test_bench_constant_is_the_counted_mean_over_the_benchmark_batch():
    wl = _bench_batch()
    W = P.quadruped_weights().astype(np.float64)
    per = []
    for b in range(0, wl.batch, 32):
        for t in range(int(wl.horizon[b])):
            f = O.stage_flops(wl.desc, wl.X0[b, t], wl.U0[b, t], wl.reference[b, t], wl.parameter[b, t], W)
            per.append(f["linearisation"] + f["trial"])
    assert abs(np.mean(per) - bench.MODEL_FLOPS_RPY12) <= 0.02 * bench.MODEL_FLOPS_RPY12
    # the model work is a small share of the stage's algorithmic FLOPs
    assert bench.MODEL_FLOPS_RPY12 < 0.1 * bench.f_lqr(12, 12)


def test_count_properties():
    wl = P.quadruped_workload(16, horizons=(50,), seed=3, model=P.MODEL_SRBD_RPY12, random_phase=True)
    W = P.quadruped_weights().astype(np.float64)
    by_contact = {}
    for b in range(wl.batch):
        for t in range(0, 50, 5):
            x, u, ref, par = wl.X0[b, t], wl.U0[b, t].astype(np.float64), wl.reference[b, t], wl.parameter[b, t]
            f = O.stage_flops(wl.desc, x, u, ref, par, W)
            # a Jacobian costs more than a value; a linearisation more than a trial
            assert f["dyn_jacobian"] > f["dyn_value"] > 0
            assert f["linearisation"] > f["trial"] > f["dyn_value"]
            # values that happen to be zero still cost: moving the tangential
            # forces off zero changes no count
            u2 = u.copy()
            u2[0::3] += 0.3
            u2[1::3] -= 0.2
            assert O.stage_flops(wl.desc, x, u2, ref, par, W) == f
            by_contact.setdefault(tuple(par[:4].astype(int)), set()).add(tuple(f.values()))
    # the count depends on the contact pattern only; more legs in stance, more work
    assert all(len(v) == 1 for v in by_contact.values())
    legs = {sum(k): next(iter(v))[3] for k, v in by_contact.items()}
    assert len(legs) >= 2 and all(legs[a] < legs[b] for a in legs for b in legs if a < b)


def test_status_bits_counts_each_flag_of_the_header():
    """The bench line's status_bits counts instances per MPXG_INST_* bit
    (include/mpxg.h: 1 non-finite, 2 non-positive pivot, 4 line search at
    its smallest step, 8 bad horizon)."""
    st = np.array([0, 1, 2, 3, 4, 12, 0, 8], dtype=np.int32)
    assert bench.status_bits(st) == {"nonfinite": 2, "pivot": 2, "line_search": 2, "bad_horizon": 2}
    assert bench.status_bits(np.zeros(5, dtype=np.int32)) == {"nonfinite": 0, "pivot": 0, "line_search": 0,
                                                               "bad_horizon": 0}
