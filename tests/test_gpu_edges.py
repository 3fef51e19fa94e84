"""Edge cases of the time interval, as the reference's loop treats them
(lib/include/detail/runge_kutta.hpp:37-72, :137-180): empty and reversed
intervals take no step (the adjoint then returns its seed and mu_direct),
an interval shorter than DBL_EPSILON takes none either, and start times
other than zero -- negative, or with a negative end time, where the
double-word sweeps' integer time tests fall back to FP64 -- give the
oracle's step sequence."""
import numpy as np
import pytest
import torch

from vectorizedadjoint_gb300 import Solver

pytestmark = pytest.mark.gpu


def dev(a):
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def vdp_batch(B, t0, t1, seed=21):
    rng = np.random.Generator(np.random.PCG64(seed))
    mu = 10.0 ** rng.uniform(-1, 0.5, B)
    y0 = rng.uniform(-2, 2, (B, 2))
    return y0, mu[:, None], np.asarray(t0, dtype=np.float64), np.asarray(t1, dtype=np.float64)


def solve(precision, y0, p, t0, t1, tableau="dopri5", dt0=1e-3, tol=1e-8):
    B = y0.shape[0]
    s = Solver("vdp", 2, 1, B, tableau=tableau, precision=precision, atol=tol, rtol=tol, dt0=dt0)
    out = s.gradient("sumsq", dev(y0), dev(p), dev(t0), dev(t1))
    torch.cuda.synchronize()
    res = {k: v.cpu().numpy() for k, v in out.items()}
    s.close()
    return res


def spans(B, seed=5):
    """Start times in [-3, 3]; spans: empty, reversed, below eps, regular."""
    rng = np.random.Generator(np.random.PCG64(seed))
    t0 = rng.uniform(-3, 3, B)
    kind = np.arange(B) % 4
    span = np.where(kind == 0, 0.0, np.where(kind == 1, -1.0, np.where(kind == 2, 1e-17, rng.uniform(0.5, 8, B))))
    return t0, t0 + span, kind


@pytest.mark.parametrize("precision", ["fp64", "mixed_dw", "mixed"])
def test_empty_reversed_and_tiny_intervals(oracle, cuda, precision):
    B = 64
    t0, t1, kind = spans(B)
    y0, p, t0, t1 = vdp_batch(B, t0, t1)
    r = solve(precision, y0, p, t0, t1)
    assert (r["status"] == 0).all()
    still = kind <= 2
    assert (r["n_acc"][still] == 0).all()
    # no step: y(T) = y0, dG/dy0 = the seed 2 y0, dG/dp = 0 (exactly; a
    # double-word state holds y0 to 48 bits)
    rt = 4e-15 if precision == "mixed_dw" else 0.0
    np.testing.assert_allclose(r["yT"][still], y0[still], rtol=rt, atol=0)
    np.testing.assert_allclose(r["dy0"][still], 2.0 * y0[still], rtol=rt, atol=0)
    assert (r["dp"][still] == 0.0).all()
    pb = oracle.problem("vdp", "dopri5", 2, 1, 1e-8, 1e-8)
    for b in range(B):
        g = oracle.gradient(pb, "sumsq", y0[b], p[b], t0[b], t1[b])
        assert g["status"] == 0
        if precision == "fp64":
            assert int(r["n_acc"][b]) == g["n_acc"]
            np.testing.assert_array_equal(r["yT"][b], g["yT"])
            np.testing.assert_array_equal(r["dy0"][b], g["dy0"])
            np.testing.assert_array_equal(r["dp"][b], g["dp"])
        elif precision == "mixed_dw":
            ref = np.concatenate([g["dy0"], g["dp"]])
            got = np.concatenate([r["dy0"][b], r["dp"][b]])
            assert np.abs(got - ref).max() <= 1e-7 * max(np.abs(ref).max(), 1e-8)


@pytest.mark.parametrize("t0,t1", [(-20.0, -12.0), (-6.0, 2.0), (1e3, 1e3 + 6.0)])
def test_shifted_intervals(oracle, cuda, t0, t1):
    """Autonomous models: only the time bookkeeping sees t0.  FP64 equals the
    oracle bit for bit; double-word takes the same accepted steps with
    gradients within 1e-7 (negative end times use the FP64 time tests)."""
    B = 32
    y0, p, tt0, tt1 = vdp_batch(B, np.full(B, t0), np.full(B, t1))
    r64 = solve("fp64", y0, p, tt0, tt1)
    rdw = solve("mixed_dw", y0, p, tt0, tt1)
    assert (r64["status"] == 0).all() and (rdw["status"] == 0).all()
    pb = oracle.problem("vdp", "dopri5", 2, 1, 1e-8, 1e-8)
    for b in range(0, B, 4):
        g = oracle.gradient(pb, "sumsq", y0[b], p[b], t0, t1)
        assert int(r64["n_acc"][b]) == g["n_acc"]
        np.testing.assert_array_equal(r64["dy0"][b], g["dy0"])
        np.testing.assert_array_equal(r64["dp"][b], g["dp"])
    assert (rdw["n_acc"] == r64["n_acc"]).mean() >= 0.9
    g64 = np.concatenate([r64["dy0"], r64["dp"]], 1)
    gdw = np.concatenate([rdw["dy0"], rdw["dp"]], 1)
    err = np.abs(gdw - g64).max(1) / np.abs(g64).max(1)
    assert np.median(err) < 1e-9 and err.max() < 1e-5


@pytest.mark.parametrize("tableau,dt0", [("rk4", 0.01), ("euler", 1e-3)])
def test_fixed_step_shifted_start(oracle, cuda, tableau, dt0):
    """Fixed steps from t0 != 0: t_n = t0 + n dt, as the reference forms it."""
    B = 16
    t0 = np.linspace(-5.0, 5.0, B)
    y0, p, tt0, tt1 = vdp_batch(B, t0, t0 + 3.0)
    r = solve("fp64", y0, p, tt0, tt1, tableau=tableau, dt0=dt0)
    pb = oracle.problem("vdp", tableau, 2, 1, 1e-8, 1e-8, dt0=dt0)
    for b in range(B):
        g = oracle.gradient(pb, "sumsq", y0[b], p[b], t0[b], t0[b] + 3.0)
        assert int(r["n_acc"][b]) == g["n_acc"]
        np.testing.assert_array_equal(r["dy0"][b], g["dy0"])
        np.testing.assert_array_equal(r["dp"][b], g["dp"])
