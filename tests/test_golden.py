"""The oracle against golden vectors produced by executing the reference's own
Python source (tests/golden/make_golden.py): gait timer (bit-exact), SRBD
reference generator, dynamics, stage cost and Gauss-Newton Hessian."""
import os

import numpy as np
import pytest

from mpx_gb300 import problem as P

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "srbd_golden.npz"))


def ref_model():
    """config_srbd's body (mpx/config/config_srbd.py:20-90) as the quat13 model."""
    mass, dt = G["dyn_const"]
    return P.ModelDesc(P.MODEL_SRBD_QUAT13, 13, 12, dt=float(dt), mass=float(mass), inertia=G["dyn_inertia"],
                       n_contact=4, mu=0.7)


@pytest.mark.parametrize("tag", ["srbd", "trot"])
def test_timer_bit_exact(oracle, tag):
    duty, freq, dt = G["timer_%s_params" % tag]
    lt = G["timer_%s_init" % tag].copy()
    for k in range(G["timer_%s_contact" % tag].shape[0]):
        for b in range(lt.shape[0]):
            c, lt[b] = oracle.timer_run(duty, freq, dt, lt[b])
            assert np.array_equal(c, G["timer_%s_contact" % tag][k, b])
        assert np.array_equal(lt.view(np.uint32), G["timer_%s_time" % tag][k].view(np.uint32))


def test_host_timer_bit_exact():
    """The product's host-side timer (used to build workload tables) too."""
    duty, freq, dt = G["timer_trot_params"]
    lt = G["timer_trot_init"].copy()
    for k in range(G["timer_trot_contact"].shape[0]):
        c, lt = P.timer_run_np(duty, freq, lt, dt)
        assert np.array_equal(c, G["timer_trot_contact"][k])
        assert np.array_equal(lt.view(np.uint32), G["timer_trot_time"][k].view(np.uint32))


def test_reference_generator(oracle):
    N, dt, mass, duty, freq, sh, cl = G["refgen_cfg"]
    N = int(N)
    for r in range(G["refgen_in_x"].shape[0]):
        ref, par, lo, frd = oracle.refgen_srbd(N, dt, mass, G["refgen_foot0"], duty, freq, sh, cl,
                                               G["refgen_in_t_timer"][r], G["refgen_in_x"][r],
                                               G["refgen_in_foot"][r], G["refgen_in_input"][r],
                                               G["refgen_in_contact"][r], G["refgen_in_liftoff"][r])
        gref, gpar = G["refgen_out_reference"][r], G["refgen_out_parameter"][r]
        assert np.array_equal(ref[:, 13:17], gref[:, 13:17])  # contact schedule
        assert np.array_equal(par[:, 0:4], gpar[:, 0:4])
        np.testing.assert_allclose(ref, gref, rtol=2e-6, atol=2e-6)
        np.testing.assert_allclose(par, gpar, rtol=2e-6, atol=2e-6)
        np.testing.assert_allclose(lo, G["refgen_out_liftoff"][r], rtol=2e-6, atol=2e-6)
        np.testing.assert_allclose(frd, G["refgen_out_foot_ref_dot"][r], rtol=1e-5, atol=1e-5)


@pytest.mark.parametrize("precision", [32, 64])
def test_dynamics(oracle, precision):
    d = ref_model()
    for i in range(G["dyn_x"].shape[0]):
        xn = oracle.dynamics(d, G["dyn_x"][i], G["dyn_u"][i], G["dyn_par"][i], precision=precision)
        np.testing.assert_allclose(xn, G["dyn_xnext"][i], rtol=2e-5, atol=2e-6)


@pytest.mark.parametrize("precision", [32, 64])
def test_stage_cost(oracle, precision):
    d = ref_model()
    for i in range(G["cost_x"].shape[0]):
        v = oracle.cost(d, G["cost_x"][i], G["cost_u"][i], G["cost_ref"][i], G["cost_W"],
                        terminal=bool(G["cost_terminal"][i]), precision=precision)
        assert abs(v - G["cost_val"][i]) <= 2e-5 * max(1.0, abs(G["cost_val"][i])), (i, v, G["cost_val"][i])


def test_gauss_newton_hessian(oracle):
    d = ref_model()
    for i in range(G["hess_x"].shape[0]):
        ref = G["hess_ref"][i]
        par = np.concatenate([ref[13:17], np.zeros(12)])
        A, B, fx, g, H, l = oracle.linearize(d, G["hess_x"][i], G["hess_u"][i], ref, par, G["cost_W"])
        n = 13
        for blk, gold in ((H[:n, :n], G["hess_Q"][i]), (H[n:, n:], G["hess_R"][i]), (H[:n, n:], G["hess_M"][i])):
            scale = max(1.0, np.abs(gold).max())
            assert np.abs(blk - gold).max() <= 1e-5 * scale, (i, np.abs(blk - gold).max(), scale)


def test_oracle_wb_refgen_matches_golden():
    """oracle.refgen_wb (the whole-body generator, mpc_utils.py:15-145) against
    the reference's own reference_generator run under the numpy stand-in
    (tests/golden/wb_refgen.npz), both terrain settings: the contact schedule
    and liftoff bookkeeping exactly, the float rows to 1e-6 relative (the
    yaw's float32 sin/cos differ by an ulp between numpy and glibc)."""
    from oracle import oracle as O
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "wb_refgen.npz"))
    cfg = g["wbref_cfg"]
    N = int(cfg[0])
    for tag, terrain in (("flat", 0), ("terrain", 1)):
        for r in range(g["wbref_in_x"].shape[0]):
            ref, par, lo = O.refgen_wb(N, 12, cfg[1], cfg[2], g["wbref_foot0"], g["wbref_q0"], cfg[3], cfg[4],
                                       cfg[5], cfg[6], terrain, *(g["wbref_in_" + k][r] for k in
                                                                 ("t_timer", "x", "foot", "input", "contact",
                                                                  "liftoff")))
            want = g["wbref_%s_reference" % tag][r]
            assert np.array_equal(par, g["wbref_%s_parameter" % tag][r]), (tag, r)
            assert np.array_equal(ref[:, 37:41], want[:, 37:41]), (tag, r)
            assert (np.abs(ref - want) / (1.0 + np.abs(want))).max() < 1e-6, (tag, r)
            assert np.abs(lo - g["wbref_%s_liftoff" % tag][r]).max() < 1e-6, (tag, r)
