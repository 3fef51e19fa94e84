"""Gradients against central finite differences of the GPU forward sweep.

The backward sweep is the exact derivative of the forward map with the
accepted step sizes frozen (h_n = t_{n+1} - t_n; the reference's
back_prop_step, lib/include/detail/backpropagation.hpp:83-158).  For every
model and tableau: run the FP64 forward + backward on a small batch, read
each instance's accepted-step record back, and differentiate the GPU's
frozen-step replay of that record (va_forward_frozen) by central
differences in every initial-state component and every parameter (for the
shared matrix of the shared-matrix model, a sample of its entries: the
derivative of the batch's summed cost).  Fourth-order central stencil
(f(-2e), f(-e), f(e), f(2e)) at a relative step of 1e-4 (floor 0.1): the
truncation error is O(e^4) and the rounding error of the replayed cost is
divided by a step large enough that neither reaches 1e-8 (measured with
the oracle's replay: at most 6e-9 over these cases).  Bound: 1e-7
relative to the instance's largest gradient entry.

The adaptive map (step sizes chosen by the controller, so they move with
the parameters) is differentiated separately: it differs from the
frozen-step gradient by terms of the order of the tolerance, which the
last test measures and bounds loosely.
"""
import numpy as np
import pytest
import torch

from vectorizedadjoint_gb300 import Solver
from vectorizedadjoint_gb300 import workloads as W

pytestmark = pytest.mark.gpu

EPS, FLOOR = 1e-4, 1e-1
TOL_FD = 1e-7
STENCIL = (-2.0, -1.0, 1.0, 2.0)


def stencil_derivative(f):
    """f[s] for s in STENCIL, in units of the step -> fourth-order derivative times the step"""
    return (8.0 * (f[2] - f[1]) - (f[3] - f[0])) / 12.0


def dev(a, dtype=torch.float64):
    return torch.tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda")


def cost(yT, kind):
    return (yT ** 2).sum(-1) if kind == "sumsq" else yT.sum(-1)


def fd_lanes(y0, p, k_list):
    """Perturbed copies of one instance's (y0, p): lanes 4j .. 4j+3 move input
    k = k_list[j] (k < n: y0[k], else p[k - n]) by STENCIL x its step.
    Returns (Y0, P, steps)."""
    n = y0.size
    S = len(STENCIL)
    L = S * len(k_list)
    Y0 = np.repeat(y0[None, :], L, 0)
    P = np.repeat(p[None, :], L, 0)
    steps = []
    for j, k in enumerate(k_list):
        v = y0[k] if k < n else p[k - n]
        e = EPS * max(abs(v), FLOOR)
        steps.append(e)
        for q, sgn in enumerate(STENCIL):
            if k < n:
                Y0[S * j + q, k] = v + sgn * e
            else:
                P[S * j + q, k - n] = v + sgn * e
    return Y0, P, np.array(steps)


def check_instance(s, b, t, y0, p, grad, kind, k_list=None):
    n = y0.size
    k_list = list(range(n + p.size)) if k_list is None else k_list
    Y0, P, e = fd_lanes(y0, p, k_list)
    yT = s.forward_frozen([t] * len(Y0), dev(Y0), dev(P)).cpu().numpy()
    g = cost(yT, kind).reshape(len(k_list), len(STENCIL))
    fd = stencil_derivative(g.T) / e
    want = grad[k_list]
    scale = max(np.abs(grad).max(), 1e-300)
    err = np.abs(fd - want).max() / scale
    assert err < TOL_FD, (b, err, fd, want)
    return err


ONE_THREAD = [("vdpb", "dopri5"), ("vdpb", "ck54"), ("vdpb", "rkf78"), ("vdpb", "rk4"), ("vdpb", "euler"),
              ("dho", "ck54"), ("dho", "dopri5"), ("dho", "rkf78"), ("dho", "rk4"), ("vdp1", "dopri5"),
              ("glv10", "dopri5"), ("glv10", "ck54"), ("glv10", "rkf78"), ("glv10", "rk4"), ("glv10", "euler")]


@pytest.mark.parametrize("name,tableau", ONE_THREAD)
def test_gradient_vs_fd_of_gpu_forward(cuda, name, tableau):
    B = 3
    w = W.make(name, batch=B)
    c = w["cfg"]
    dt0 = 1e-2 if tableau == "rk4" else (2e-3 if tableau == "euler" else 1e-3)
    t1 = np.minimum(w["t1"], 5.0) if tableau in ("rk4", "euler") else w["t1"]
    s = Solver(c["model"], c["n"], c["npar"], B, tableau=tableau, precision="fp64", atol=c["tol"], rtol=c["tol"],
               dt0=dt0)
    out = s.gradient(c["cost"], dev(w["y0"]), dev(w["params"]), dev(w["t0"]), dev(t1))
    torch.cuda.synchronize()
    assert (out["status"].cpu().numpy() == 0).all()
    dy0, dp = out["dy0"].cpu().numpy(), out["dp"].cpu().numpy()
    for b in range(B):
        t, _, _ = s.trajectory(b)
        check_instance(s, b, t, w["y0"][b], w["params"][b], np.concatenate([dy0[b], dp[b]]), c["cost"])
    s.close()


def test_replay_reproduces_forward(cuda):
    """Unperturbed, the replay lands on the forward sweep's y(T) (to the
    rounding of h_n = t_{n+1} - t_n against the step the forward took)."""
    B = 8
    w = W.make("vdpb", batch=B)
    c = w["cfg"]
    s = Solver(c["model"], c["n"], c["npar"], B, tableau=c["tableau"], atol=c["tol"], rtol=c["tol"])
    f = s.forward(dev(w["y0"]), dev(w["params"]), dev(w["t0"]), dev(w["t1"]))
    torch.cuda.synchronize()
    times = [s.trajectory(b)[0] for b in range(B)]
    yT = s.forward_frozen(times, dev(w["y0"]), dev(w["params"])).cpu().numpy()
    np.testing.assert_allclose(yT, f["yT"].cpu().numpy(), rtol=1e-10, atol=1e-12)
    s.close()


@pytest.mark.parametrize("N,tableau", [(64, "dopri5"), (64, "ck54"), (64, "rk4")])
def test_shared_glv_gradient_vs_fd(cuda, N, tableau):
    """Shared-matrix GLV: per-instance dr and dx0 in full, and sampled
    entries of the shared dA as the derivative of the batch's summed cost."""
    B, T, tol = 4, 5.0, 1e-7
    rng = np.random.Generator(np.random.PCG64(3))
    A = rng.normal(0.0, 0.5 / np.sqrt(N), (N, N))
    A[np.arange(N), np.arange(N)] = -1.0
    r = rng.uniform(0.5, 1.5, (B, N))
    x0 = rng.uniform(0.1, 1.0, (B, N))
    dt0 = 1e-2 if tableau == "rk4" else 1e-3
    s = Solver("glv_shared", N, N, B, tableau=tableau, precision="fp64", atol=tol, rtol=tol, dt0=dt0)
    dA = torch.empty(N, N, dtype=torch.float64, device="cuda")
    Ad = dev(A)
    s.set_shared(Ad, dA)
    out = s.gradient("sum", dev(x0), dev(r), dev(np.zeros(B)), dev(np.full(B, T)))
    torch.cuda.synchronize()
    assert (out["status"].cpu().numpy() == 0).all()
    dy0, dr, dAh = out["dy0"].cpu().numpy(), out["dp"].cpu().numpy(), dA.cpu().numpy()
    times = [s.trajectory(b)[0] for b in range(B)]
    for b in range(B):
        check_instance(s, b, times[b], x0[b], r[b], np.concatenate([dy0[b], dr[b]]), "sum")
    rng = np.random.default_rng(0)
    entries = [(0, 0), (N - 1, N - 1), (3, 7)] + [tuple(rng.integers(0, N, 2)) for _ in range(5)]
    scale = np.abs(dAh).max()
    for i, j in entries:
        e = EPS * max(abs(A[i, j]), FLOOR)
        g = []
        for sgn in STENCIL:
            Ap = A.copy()
            Ap[i, j] += sgn * e
            yT = s.forward_frozen(times, dev(x0), dev(r), shared=dev(Ap)).cpu().numpy()
            g.append(yT.sum())
        fd = stencil_derivative(g) / e
        assert abs(fd - dAh[i, j]) / scale < TOL_FD, (i, j, fd, dAh[i, j])
    s.close()


@pytest.mark.parametrize("name", ["dho", "vdpb"])
def test_adaptive_map_fd_differs_by_tolerance_terms(cuda, name):
    """Central differences of the ADAPTIVE forward (controller active, step
    sizes move with the inputs) against the frozen-step gradient: the two
    differ by the neglected dh/dp terms, of the order of the tolerance, and
    the adaptive map itself jitters at that order, so the step is 1e-3
    relative (floor 0.1) and the error is taken relative to the instance's
    gradient scale with the floor 1e-8 max|y0|.  Instances whose step count
    changes under a perturbation are skipped.  Measured with the oracle's
    identical forward: median 7e-7 (DHO) / 1.3e-5 (VdP), max 2.3e-4 / 5.3e-4."""
    B = 8
    w = W.make(name, batch=B)
    c = w["cfg"]
    s = Solver(c["model"], c["n"], c["npar"], B, tableau=c["tableau"], atol=c["tol"], rtol=c["tol"])
    out = s.gradient(c["cost"], dev(w["y0"]), dev(w["params"]), dev(w["t0"]), dev(w["t1"]))
    torch.cuda.synchronize()
    g = np.concatenate([out["dy0"].cpu().numpy(), out["dp"].cpu().numpy()], 1)
    nacc = out["n_acc"].cpu().numpy()
    scale = np.maximum(np.abs(g).max(1), 1e-8 * np.abs(w["y0"]).max(1))
    n = c["n"]
    errs = []
    for k in range(n + c["npar"]):
        vals, same = [], np.ones(B, dtype=bool)
        src0 = w["y0"] if k < n else w["params"]
        kk = k if k < n else k - n
        e = 1e-3 * np.maximum(np.abs(src0[:, kk]), 0.1)
        for sgn in STENCIL:
            y0, p = w["y0"].copy(), w["params"].copy()
            (y0 if k < n else p)[:, kk] += sgn * e
            f = s.forward(dev(y0), dev(p), dev(w["t0"]), dev(w["t1"]))
            torch.cuda.synchronize()
            vals.append(cost(f["yT"].cpu().numpy(), c["cost"]))
            same &= f["n_acc"].cpu().numpy() == nacc
        fd = stencil_derivative(vals) / e
        errs += list((np.abs(fd - g[:, k]) / scale)[same])
    errs = np.array(errs)
    assert errs.size >= 8
    assert np.median(errs) < 1e-4 and errs.max() < 1e-2, (np.median(errs), errs.max())
    s.close()
