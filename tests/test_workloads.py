"""The seeded synthetic workloads follow the recipes they are quoted on (CPU).

Each workload stands in for a benchmark configuration, so its shapes, sizes
and value distributions are part of what a measurement means:
  - the plain quadruped: mass 15 kg, inertia diag(0.10, 0.25, 0.30), feet at
    the hip offsets (+-0.20, +-0.12, -0.30) m, trot of period 0.5 s and duty
    0.6, N = 50, dt = 0.02, Q = diag(50, 20, 5, 1 per 3-block), R = 1e-4 I,
    v_ref = 0.5 m/s, mu = 0.6, x0 perturbed by N(0, 0.05^2);
  - the isolated LQR: 1024 x (n 24, m 12, N 128), A = I + 0.05 G rescaled to
    spectral radius 0.98, B ~ N(0, 1/m), Q = M M'/n + 0.1 I, R = 0.1 I, S = 0;
  - the batched quadruped: horizons uniform on {25, 50, 100}, gait phase
    uniform on [0, 1), v_ref uniform on [-1, 1];
  - the served biped: mass 60 kg, inertia diag(6, 5, 1.5), 0.2 x 0.1 m feet;
  - the large LQ: n 72, m 30, 12 equality rows, spectral radius <= 1.01,
    Q diagonal log-uniform in [1e-2, 1e2], R = 1e-3 I.
"""
import numpy as np

from mpx_gb300 import problem as P


def test_plain_quadruped():
    wl = P.quadruped_workload(400, horizons=(50,), seed=0, model=P.MODEL_SRBD_RPY12, v_range=(0.5, 0.5))
    d = wl.desc
    assert (d.n, d.m, d.mass, d.mu) == (12, 12, 15.0, 0.6)
    assert abs(d.dt - 0.02) < 1e-9
    assert np.allclose(np.asarray(d.inertia), np.diag([0.10, 0.25, 0.30]))
    assert np.all(wl.horizon == 50) and wl.n_max == 50
    assert np.all(wl.v_ref == np.float32(0.5))
    w = np.diag(wl.W[0])
    assert np.allclose(w, [50] * 3 + [20] * 3 + [5] * 3 + [1] * 3 + [1e-4] * 12)
    assert np.count_nonzero(wl.W[0] - np.diag(w)) == 0
    # x0 = nominal standing state + N(0, 0.05^2)
    nominal = np.zeros(12)
    nominal[2] = 0.30
    pert = wl.x0 - nominal
    assert abs(pert.std() - 0.05) < 0.003 and abs(pert.mean()) < 0.003
    # feet at the hip offsets below the CoM reference, contacts from the trot timer
    par, ref = wl.parameter, wl.reference
    for i, off in enumerate(P.HIP_OFFSETS):
        for k in range(3):
            com = ref[:, :, k] if k < 2 else np.float32(0.30)
            assert np.allclose(par[:, :, 4 + 3 * i + k], com + np.float32(off[k]), atol=1e-6)
    assert np.array_equal(par[:, :, :4], ref[:, :, 12:16])
    # trot: diagonal pairs share a phase, the two pairs are half a period apart,
    # and each leg is in stance for 60 % of the 25-stage (0.5 s) period
    c = par[:, :, :4]
    assert np.array_equal(c[:, :, 0], c[:, :, 3]) and np.array_equal(c[:, :, 1], c[:, :, 2])
    duty = c[:, :50, 0].mean()
    assert abs(duty - 0.6) < 0.03
    # nominal forces carry the weight over the legs in stance
    fz = wl.U0[:, :, 2::3].sum(-1)
    stance = c[:, :-1].sum(-1) > 0
    assert np.allclose(fz[stance], 15.0 * d.gravity, rtol=1e-5)


def test_isolated_lqr():
    d = P.random_lq(4, 24, 12, 16, seed=0)
    assert d["A"].shape == (4, 16, 24, 24) and d["B"].shape == (4, 16, 24, 12)
    assert d["Q"].shape == (4, 17, 24, 24) and d["R"].shape == (4, 16, 12, 12)
    assert np.allclose(np.abs(np.linalg.eigvals(d["A"])).max(-1), 0.98)
    assert np.all(d["M"] == 0) and np.all(d["R"] == 0.1 * np.eye(12))
    assert np.linalg.eigvalsh(d["Q"]).min() >= 0.1 - 1e-9
    assert abs(d["B"].std() - np.sqrt(1.0 / 12)) < 0.01
    for k in ("q", "r", "c", "x0"):
        assert abs(d[k].std() - 1.0) < 0.15, k


def test_batched_quadruped():
    wl = P.quadruped_workload(4096, horizons=(25, 50, 100), seed=7, model=P.MODEL_SRBD_RPY12, v_range=(-1, 1),
                              random_phase=True)
    assert wl.batch == 4096 and wl.n_max == 100
    counts = np.array([(wl.horizon == h).sum() for h in (25, 50, 100)])
    assert counts.sum() == 4096 and counts.min() > 4096 / 3 - 150
    assert wl.v_ref.min() >= -1 and wl.v_ref.max() <= 1 and wl.v_ref.std() > 0.5
    phase = np.mod(wl.leg_time[:, 0] - P.TROT_PHASE[0], 1.0)
    assert phase.min() >= 0 and phase.max() < 1 and abs(phase.mean() - 0.5) < 0.03
    assert np.allclose(np.mod(wl.leg_time[:, 1] - wl.leg_time[:, 0], 1.0), 0.5, atol=1e-6)


def test_served_biped():
    d = P.biped_wrench12()
    assert (d.n, d.m, d.mass, d.n_contact) == (12, 12, 60.0, 2)
    assert np.allclose(np.asarray(d.inertia), np.diag([6.0, 5.0, 1.5]))
    assert abs(d.foot_length - 0.2) < 1e-7 and abs(d.foot_width - 0.1) < 1e-7
    wl = P.biped_workload(64, horizons=(20, 200), seed=1)
    assert wl.n_max == 200 and set(np.unique(wl.horizon)) <= {20, 200}


def test_large_lq():
    d = P.random_lq_eq(3, n=72, m=30, n_eq=12, N=4, seed=2)
    diag = np.diagonal(d["Q"], axis1=-2, axis2=-1)
    assert diag.min() >= 1e-2 and diag.max() <= 1e2
    assert np.count_nonzero(d["Q"] - np.einsum("...i,ij->...ij", diag, np.eye(72))) == 0
    assert np.all(d["R"] == 1e-3 * np.eye(30))
    assert np.abs(np.linalg.eigvals(d["A"])).max() <= 1.01 + 1e-9
    assert abs(d["B"].std() - np.sqrt(0.1 / 30)) < 0.003


def test_solver_shape_check_accepts_the_workloads_and_names_a_short_buffer():
    """Solver.prepare's check (raised, not asserted) passes every workload
    as built and rejects a buffer shorter than the kernels index."""
    import pytest
    import torch
    from mpx_gb300.solver import check_shapes, weights_diagonal
    for wl in (P.quadruped_workload(6, horizons=(10, 20), seed=1, model=P.MODEL_SRBD_RPY12),
               P.quadruped_workload(3, horizons=(15,), seed=2, model=P.MODEL_SRBD_QUAT13),
               P.biped_workload(4, horizons=(12, 30), seed=3)):
        B = wl.batch
        arrays = dict(x0=wl.x0, X0=wl.X0, U0=wl.U0, V0=wl.V0, reference=wl.reference, parameter=wl.parameter,
                      w=weights_diagonal(torch.as_tensor(wl.W), B), horizon=wl.horizon)
        check_shapes(wl.desc, wl.n_max, B, **arrays)
        for name in arrays:
            short = dict(arrays)
            short[name] = np.asarray(arrays[name])[:B - 1]
            with pytest.raises(ValueError, match=name):
                check_shapes(wl.desc, wl.n_max, B, **short)
        with pytest.raises(ValueError, match="X0"):
            check_shapes(wl.desc, wl.n_max + 1, B, X0=wl.X0)
