"""CPU checks of the oracle itself: adjoint vs frozen-step central finite
differences, a closed-form discrete adjoint, controller invariants, and the
multi-cost (Nout > 1) write-back semantics of the reference's adjointSolve
(detail/backpropagation.hpp:280-348)."""
import numpy as np
import pytest

from vectorizedadjoint_gb300 import workloads as W


def _fd(oracle, pb, y0, p, times, cost, eps=1e-6):
    def G(y, q):
        yT = oracle.forward_frozen(pb, y, q, times)
        return np.sum(yT ** 2) if cost == "sumsq" else np.sum(yT)
    gy = np.array([(G(y0 + eps * e, p) - G(y0 - eps * e, p)) / (2 * eps) for e in np.eye(len(y0))])
    gp = np.array([(G(y0, p + eps * e) - G(y0, p - eps * e)) / (2 * eps) for e in np.eye(len(p))])
    return gy, gp


@pytest.mark.parametrize("name", ["vdp1", "dho", "vdpb", "glv10"])
def test_adjoint_matches_frozen_step_fd(oracle, name):
    w = W.make(name, batch=3)
    c = w["cfg"]
    pb = oracle.problem(c["model"], c["tableau"], c["n"], c["npar"], c["tol"], c["tol"])
    for b in range(3):
        g = oracle.gradient(pb, c["cost"], w["y0"][b], w["params"][b], 0.0, w["t1"][b])
        assert g["status"] == 0
        fw = oracle.forward(pb, w["y0"][b], w["params"][b], 0.0, w["t1"][b])
        assert fw["n_acc"] == g["n_acc"]
        gy, gp = _fd(oracle, pb, w["y0"][b], w["params"][b], fw["times"], c["cost"])
        scale = max(np.abs(gy).max(), np.abs(gp).max(), 1e-3)
        assert np.abs(g["dy0"] - gy).max() / scale < 2e-6
        assert np.abs(g["dp"] - gp).max() / scale < 2e-6


def test_decay_closed_form(oracle):
    """y' = -k y with a frozen step sequence: every DOPRI5 step multiplies y by
    R(-k h) = sum_{j<=5} (-k h)^j / j! + (-k h)^6/600 (the pair's stability
    polynomial), so dy(T)/dy0 = prod R and the discrete adjoint must equal it."""
    pb = oracle.problem("decay", "dopri5", 1, 1, 1e-9, 1e-9)
    k, y0 = 0.7, 1.3
    fw = oracle.forward(pb, [y0], [k], 0.0, 3.0)
    h = np.diff(fw["times"])
    z = -k * h
    R = 1 + z + z ** 2 / 2 + z ** 3 / 6 + z ** 4 / 24 + z ** 5 / 120 + z ** 6 / 600
    lam, mu, st = oracle.adjoint(pb, [k], fw["times"], fw["states"], [[1.0]], [[0.0]])
    assert st == 0
    np.testing.assert_allclose(lam[0, 0], np.prod(R), rtol=1e-13)
    np.testing.assert_allclose(fw["yT"][0], y0 * np.prod(R), rtol=1e-13)


def test_controller_invariants(oracle):
    w = W.make("vdp1")
    c = w["cfg"]
    pb = oracle.problem(c["model"], c["tableau"], 2, 1, c["tol"], c["tol"])
    fw = oracle.forward(pb, w["y0"][0], w["params"][0], 0.0, 10.0)
    t = fw["times"]
    assert fw["status"] == 0 and t[0] == 0.0
    assert np.all(np.diff(t) > 0)
    assert abs(t[-1] - 10.0) <= 1e-12
    # the trial step grows by at most 0.9 * 5 per accepted step (odeint's limiter)
    dt = fw["dt_trial"]
    assert np.all(dt[1:] / dt[:-1] <= 4.5 * (1 + 1e-12))


def test_failed_step_checker(oracle):
    """odeint's failed_step_checker: more than max_fail attempts on one step
    is an error (a first step of 1.0 at tol 1e-12 needs several rejections)."""
    pb = oracle.problem("vdp", "dopri5", 2, 1, 1e-12, 1e-12, dt0=1.0, max_fail=2)
    fw = oracle.forward(pb, [2.0, 0.0], [5.0], 0.0, 1.0)
    assert oracle.STATUS[fw["status"]] == "MAX_REJECTS"
    pb = oracle.problem("vdp", "dopri5", 2, 1, 1e-12, 1e-12, dt0=1.0, max_fail=500)
    fw = oracle.forward(pb, [2.0, 0.0], [5.0], 0.0, 1.0)
    assert fw["status"] == 0 and fw["n_rej"] > 2


def test_multi_cost_seeds_match_single_runs(oracle):
    """nout cost rows (the reference's SIMD lanes) equal nout separate sweeps,
    with mu accumulated onto the direct partials (:317-321)."""
    w = W.make("glv10", batch=1)
    c = w["cfg"]
    pb = oracle.problem("glv", "dopri5", 10, 110, 1e-7, 1e-7)
    fw = oracle.forward(pb, w["y0"][0], w["params"][0], 0.0, 20.0)
    rng = np.random.default_rng(0)
    lam = rng.normal(size=(5, 10))
    mu = rng.normal(size=(5, 110))
    L, M, st = oracle.adjoint(pb, w["params"][0], fw["times"], fw["states"], lam, mu)
    assert st == 0
    for q in range(5):
        l1, m1, _ = oracle.adjoint(pb, w["params"][0], fw["times"], fw["states"], lam[q:q + 1], mu[q:q + 1])
        np.testing.assert_array_equal(L[q], l1[0])
        np.testing.assert_array_equal(M[q], m1[0])


def test_batch_threads_equal_serial(oracle):
    w = W.make("dho", batch=16)
    c = w["cfg"]
    pb = oracle.problem("dho", "ck54", 2, 2, 1e-8, 1e-8)
    a = oracle.gradient_batch(pb, "sumsq", w["y0"], w["params"], w["t0"], w["t1"], nthreads=4)
    b = oracle.gradient_batch(pb, "sumsq", w["y0"], w["params"], w["t0"], w["t1"], nthreads=1)
    np.testing.assert_array_equal(a["dp"], b["dp"])
    np.testing.assert_array_equal(a["n_acc"], b["n_acc"])


@pytest.mark.parametrize("name", ["vdp1", "dho", "vdpb", "glv10"])
def test_checkpoint_traffic_counts(oracle, name):
    """The instrumented oracle's checkpoint bytes: the forward stores one time
    and one state per accepted point (StateStorage.hpp:22-43, T + 1 points);
    the adjoint reads t_n, t_{n+1} and y_n once per step
    (detail/backpropagation.hpp:256-278) -- (1 + N) 8 and (2 + N) 8 bytes per
    accepted step, VdP 24 and 32."""
    w = W.make(name, batch=2)
    c = w["cfg"]
    n = c["n"]
    pb = oracle.problem(c["model"], c["tableau"], n, c["npar"], c["tol"], c["tol"])
    for b in range(2):
        tr = oracle.gradient_traffic(pb, c["cost"], w["y0"][b], w["params"][b], 0.0, w["t1"][b])
        g = oracle.gradient(pb, c["cost"], w["y0"][b], w["params"][b], 0.0, w["t1"][b])
        T = g["n_acc"]
        assert tr["status"] == 0 and tr["n_acc"] == T > 0
        assert tr["store_bytes"] == (T + 1) * (1 + n) * 8
        assert tr["load_bytes"] == T * (2 + n) * 8
