"""Fixed-step runge_kutta4 and euler (the reference's non-controlled loop,
lib/include/detail/runge_kutta.hpp:37-72: t_n = t0 + n dt while
t_n + dt <= t1 to within DBL_EPSILON, every step recorded): the FP64 sweeps
reproduce the oracle bit for bit, the double-word sweeps take the same steps
and stay within 1e-9 of them, and two-level checkpointing gives the same
bits as every-step checkpointing.  The reference itself is pinned in
tests/test_golden.py (rk4 and euler cases)."""
import numpy as np
import pytest
import torch

from vectorizedadjoint_gb300 import Solver
from vectorizedadjoint_gb300 import workloads as W

pytestmark = pytest.mark.gpu

DT = {"rk4": 1e-2, "euler": 1e-3}


def dev(a):
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def run(name, B, tableau, **kw):
    w = W.make(name, batch=B)
    c = w["cfg"]
    s = Solver(c["model"], c["n"], c["npar"], B, tableau=tableau, atol=c["tol"], rtol=c["tol"], dt0=DT[tableau],
               **kw)
    out = s.gradient(c["cost"], dev(w["y0"]), dev(w["params"]), dev(w["t0"]), dev(w["t1"]))
    torch.cuda.synchronize()
    res = {k: v.cpu().numpy() for k, v in out.items()}
    s.close()
    return w, res


def rel_rows(g, g64, y0):
    """Per-instance error relative to the instance's largest FP64 entry, with
    a floor of 1e-8 |y0|: strongly damped oscillators decay to ~1e-55 by
    t1 = 50, below the float exponent range that double-word and float
    stages share, where only an absolute bound means anything."""
    scale = np.maximum(np.abs(g64).max(1), 1e-8 * np.abs(y0).max(1))
    return (np.abs(g - g64).max(1) / scale)


@pytest.mark.parametrize("tableau", ["rk4", "euler"])
@pytest.mark.parametrize("name,B", [("vdpb", 128), ("dho", 64), ("vdp1", 1), ("glv10", 16)])
def test_fixed_fp64_bit_exact(oracle, cuda, name, B, tableau):
    w, r = run(name, B, tableau, precision="fp64")
    assert (r["status"] == 0).all()
    c = w["cfg"]
    pb = oracle.problem(c["model"], tableau, c["n"], c["npar"], c["tol"], c["tol"], dt0=DT[tableau])
    for b in range(0, B, max(1, B // 12)):
        g = oracle.gradient(pb, c["cost"], w["y0"][b], w["params"][b], 0.0, w["t1"][b])
        assert g["status"] == 0
        assert int(r["n_acc"][b]) == g["n_acc"]
        np.testing.assert_array_equal(r["yT"][b], g["yT"])
        np.testing.assert_array_equal(r["dy0"][b], g["dy0"])
        np.testing.assert_array_equal(r["dp"][b], g["dp"])


@pytest.mark.parametrize("tableau", ["rk4", "euler"])
@pytest.mark.parametrize("name,B", [("vdpb", 256), ("dho", 128), ("glv10", 32)])
def test_fixed_reduced_precision(cuda, name, B, tableau):
    """Without a controller the step sequence cannot drift: double-word and
    float sweeps take exactly the FP64 steps.  Double-word gradients within
    1e-9 of FP64, float-stage sweeps within 1e-3 (rel_rows)."""
    w, r64 = run(name, B, tableau, precision="fp64")
    g64 = np.concatenate([r64["dy0"], r64["dp"]], 1)
    for precision, tol in (("mixed_dw", 1e-9), ("mixed", 1e-3)):
        _, r = run(name, B, tableau, precision=precision)
        assert (r["status"] == 0).all()
        np.testing.assert_array_equal(r["n_acc"], r64["n_acc"])
        g = np.concatenate([r["dy0"], r["dp"]], 1)
        err = rel_rows(g, g64, w["y0"])
        assert err.max() < tol, (precision, err.max())


@pytest.mark.parametrize("tableau", ["rk4", "euler"])
@pytest.mark.parametrize("precision", ["fp64", "mixed_dw"])
def test_fixed_two_level_same_bits(cuda, tableau, precision):
    """Segments re-run from their checkpoints with t = t0 + n dt land on the
    next checkpoint exactly; the adjoint equals the every-step one bit for
    bit (double-word: the stage-record layout in both)."""
    _, ref = run("vdpb", 128, tableau, precision=precision)
    _, r = run("vdpb", 128, tableau, precision=precision, ckpt_stride=7)
    assert (r["status"] == 0).all()
    for k in ("n_acc", "yT", "dy0", "dp"):
        np.testing.assert_array_equal(r[k], ref[k])


def test_fixed_trajectory_times(oracle, cuda):
    """The recorded times are t0 + n dt, rounded as the reference computes
    them, and the last one falls short of t1 when dt does not divide it."""
    w = W.make("vdpb", batch=4)
    c = w["cfg"]
    s = Solver(c["model"], c["n"], c["npar"], 4, tableau="rk4", atol=c["tol"], rtol=c["tol"], dt0=0.03)
    P = dev(w["params"])
    f = s.forward(dev(w["y0"]), P, dev(w["t0"]), dev(w["t1"]))
    torch.cuda.synchronize()
    pb = oracle.problem(c["model"], "rk4", c["n"], c["npar"], c["tol"], c["tol"], dt0=0.03)
    for b in range(4):
        times, _, states = s.trajectory(b)
        fw = oracle.forward(pb, w["y0"][b], w["params"][b], 0.0, w["t1"][b])
        assert int(f["n_acc"][b]) == fw["n_acc"]
        np.testing.assert_array_equal(times, fw["times"])
        np.testing.assert_array_equal(states, fw["states"])
        assert times[-1] <= w["t1"][b]
    s.close()


@pytest.mark.parametrize("tableau", ["rk4", "euler"])
def test_fixed_shared_matrix(oracle, cuda, tableau):
    """GLV with one shared A (bundle sweeps), fixed steps: FP64 per instance
    equals the oracle bit for bit (steps, y(T), dy0, dr), dA equals the sum
    of the oracle's per-instance dA to rounding; double-word within 1e-9."""
    N, B, T = 64, 6, 3.0
    rng = np.random.Generator(np.random.PCG64(17))
    A = rng.normal(0.0, 0.5 / np.sqrt(N), (N, N))
    A[np.arange(N), np.arange(N)] = -1.0
    r = rng.uniform(0.5, 1.5, (B, N))
    x0 = rng.uniform(0.1, 1.0, (B, N))
    res = {}
    for precision in ("fp64", "mixed_dw"):
        s = Solver("glv_shared", N, N, B, tableau=tableau, precision=precision, dt0=DT[tableau])
        dA = torch.empty(N, N, dtype=torch.float64, device="cuda")
        s.set_shared(dev(A), dA)
        out = s.gradient("sum", dev(x0), dev(r), dev(np.zeros(B)), dev(np.full(B, T)))
        torch.cuda.synchronize()
        res[precision] = {k: v.cpu().numpy() for k, v in out.items()}
        res[precision]["dA"] = dA.cpu().numpy()
        s.close()
    r64 = res["fp64"]
    pb = oracle.problem("glv", tableau, N, N + N * N, 1e-6, 1e-6, dt0=DT[tableau])
    dA = np.zeros((N, N))
    for b in range(B):
        g = oracle.gradient(pb, "sum", x0[b], np.concatenate([r[b], A.ravel()]), 0.0, T)
        assert int(r64["n_acc"][b]) == g["n_acc"]
        np.testing.assert_array_equal(r64["yT"][b], g["yT"])
        np.testing.assert_array_equal(r64["dy0"][b], g["dy0"])
        np.testing.assert_array_equal(r64["dp"][b], g["dp"][:N])
        dA += g["dp"][N:].reshape(N, N)
    assert np.abs(r64["dA"] - dA).max() <= 1e-12 * np.abs(dA).max()
    rdw = res["mixed_dw"]
    np.testing.assert_array_equal(rdw["n_acc"], r64["n_acc"])
    for k in ("dy0", "dp", "dA"):
        assert np.abs(rdw[k] - r64[k]).max() <= 1e-9 * np.abs(r64[k]).max()


def test_rkf78_rejected_for_shared_matrix(cuda):
    with pytest.raises(Exception):
        Solver("glv_shared", 64, 64, 4, tableau="rkf78")
