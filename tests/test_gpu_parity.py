"""GPU parity through the C ABI against the CPU oracle.

FP64 path (the drop-in): per instance the same accepted-step count, the
accepted (t_n, y_n) within 1e-12 relative, y(T) within 1e-12 and gradients
within 1e-9 relative (tolerances of the drop-in contract; the GPU contracts
products into FMAs, the oracle does not, so results agree to rounding, not
bit for bit).  Mixed path: gradient error against the FP64 oracle stated per
config.
"""
import numpy as np
import pytest
import torch

from vectorizedadjoint_gb300 import Solver
from vectorizedadjoint_gb300 import workloads as W

pytestmark = pytest.mark.gpu

REL_Y = 1e-12
REL_G = 1e-9


def dev(a, dtype=torch.float64):
    return torch.tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda")


def rel_err(a, b, floor=1e-12):
    a, b = np.asarray(a), np.asarray(b)
    scale = np.maximum(np.abs(b), floor)
    return float(np.max(np.abs(a - b) / scale)) if a.size else 0.0


def grad_rel(a, b):
    """max |a-b| / max|b| per instance (gradient components share a scale)."""
    a, b = np.atleast_2d(a), np.atleast_2d(b)
    s = np.maximum(np.abs(b).max(axis=1, keepdims=True), 1e-300)
    return float(np.max(np.abs(a - b) / s))


def run_gpu(name, B, precision="fp64", **kw):
    w = W.make(name, batch=B)
    c = w["cfg"]
    s = Solver(c["model"], c["n"], c["npar"], B, tableau=c["tableau"], precision=precision,
               atol=c["tol"], rtol=c["tol"], **kw)
    out = s.gradient(c["cost"], dev(w["y0"]), dev(w["params"]), dev(w["t0"]), dev(w["t1"]))
    torch.cuda.synchronize()
    res = {k: v.cpu().numpy() for k, v in out.items()}
    return s, w, res


def oracle_batch(oracle, w, idx):
    c = w["cfg"]
    pb = oracle.problem(c["model"], c["tableau"], c["n"], c["npar"], c["tol"], c["tol"])
    return pb, [oracle.gradient(pb, c["cost"], w["y0"][b], w["params"][b], 0.0, w["t1"][b]) for b in idx]


@pytest.mark.parametrize("name,B", [("vdp1", 1), ("dho", 256), ("vdpb", 512)])
def test_fp64_gradients_match_oracle(oracle, cuda, name, B):
    s, w, r = run_gpu(name, B)
    assert (r["status"] == 0).all()
    idx = list(range(0, B, max(1, B // 64)))
    pb, ref = oracle_batch(oracle, w, idx)
    for b, g in zip(idx, ref):
        assert g["status"] == 0
        assert int(r["n_acc"][b]) == g["n_acc"], (b, int(r["n_acc"][b]), g["n_acc"])
        # relative to the trajectory's scale: a decayed oscillator ends near 0
        yscale = max(np.abs(w["y0"][b]).max(), np.abs(g["yT"]).max())
        assert np.abs(r["yT"][b] - g["yT"]).max() / yscale < REL_Y * 100, b
        assert grad_rel(r["dy0"][b], g["dy0"]) < REL_G, b
        assert grad_rel(r["dp"][b], g["dp"]) < REL_G, b
    s.close()


@pytest.mark.parametrize("name,B", [("vdp1", 1), ("dho", 64), ("vdpb", 64)])
def test_fp64_accepted_step_sequence(oracle, cuda, name, B):
    """Same accepted steps: count, t_n (hence h_n) and y_n within 1e-12 relative."""
    w = W.make(name, batch=B)
    c = w["cfg"]
    s = Solver(c["model"], c["n"], c["npar"], B, tableau=c["tableau"], precision="fp64",
               atol=c["tol"], rtol=c["tol"])
    f = s.forward(dev(w["y0"]), dev(w["params"]), dev(w["t0"]), dev(w["t1"]))
    torch.cuda.synchronize()
    pb = oracle.problem(c["model"], c["tableau"], c["n"], c["npar"], c["tol"], c["tol"])
    worst_t = worst_y = 0.0
    for b in range(0, B, max(1, B // 16)):
        fw = oracle.forward(pb, w["y0"][b], w["params"][b], 0.0, w["t1"][b])
        t, dt, y = s.trajectory(b)
        assert len(t) == fw["n_acc"] + 1
        h_gpu, h_ref = np.diff(t), np.diff(fw["times"])
        worst_t = max(worst_t, rel_err(h_gpu, h_ref))
        scale = np.maximum(np.abs(fw["states"]), 1e-3)
        worst_y = max(worst_y, float(np.max(np.abs(y - fw["states"]) / scale)))
        assert int(f["n_rej"][b]) == fw["n_rej"]
    # h_n = t_{n+1} - t_n inherits the absolute error of t, so compare on t's scale
    assert worst_t < 1e-9, worst_t
    assert worst_y < 1e-11, worst_y
    s.close()


def test_forward_backward_pair_equals_gradient(oracle, cuda):
    """va_forward + va_backward with explicit seeds == va_gradient (cost sumsq)."""
    B = 128
    w = W.make("dho", batch=B)
    c = w["cfg"]
    s = Solver("dho", 2, 2, B, tableau="ck54", atol=1e-8, rtol=1e-8)
    P = dev(w["params"])
    f = s.forward(dev(w["y0"]), P, dev(w["t0"]), dev(w["t1"]))
    lam = (2.0 * f["yT"]).reshape(B, 1, 2).contiguous()
    mu = torch.zeros(B, 1, 2, dtype=torch.float64, device="cuda")
    bw = s.backward(P, lam, mu)
    torch.cuda.synchronize()
    s2, _, r = run_gpu("dho", B)
    np.testing.assert_array_equal(bw["dy0"].cpu().numpy()[:, 0], r["dy0"])
    np.testing.assert_array_equal(bw["dp"].cpu().numpy()[:, 0], r["dp"])
    s.close()
    s2.close()


def test_multi_cost_seeds(oracle, cuda):
    """nout > 1 (the reference's seed lanes): each row equals the oracle's."""
    B, Q = 32, 3
    w = W.make("vdpb", batch=B)
    s = Solver("vdp", 2, 1, B, nout=Q, tableau="dopri5", atol=1e-6, rtol=1e-6)
    P = dev(w["params"])
    s.forward(dev(w["y0"]), P, dev(w["t0"]), dev(w["t1"]))
    rng = np.random.default_rng(3)
    lam = rng.normal(size=(B, Q, 2))
    mu = rng.normal(size=(B, Q, 1))
    bw = s.backward(P, dev(lam), dev(mu))
    torch.cuda.synchronize()
    dy0, dp = bw["dy0"].cpu().numpy(), bw["dp"].cpu().numpy()
    pb = oracle.problem("vdp", "dopri5", 2, 1, 1e-6, 1e-6)
    for b in range(0, B, 5):
        fw = oracle.forward(pb, w["y0"][b], w["params"][b], 0.0, w["t1"][b])
        L, M, st = oracle.adjoint(pb, w["params"][b], fw["times"], fw["states"], lam[b], mu[b])
        assert grad_rel(dy0[b], L) < REL_G
        assert grad_rel(dp[b], M) < REL_G
    s.close()


def test_deterministic_repeat(cuda):
    """No atomics on the result path: two runs are bitwise equal."""
    s, w, r1 = run_gpu("vdpb", 4096)
    c = w["cfg"]
    out = s.gradient(c["cost"], dev(w["y0"]), dev(w["params"]), dev(w["t0"]), dev(w["t1"]))
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out["dp"].cpu().numpy(), r1["dp"])
    np.testing.assert_array_equal(out["dy0"].cpu().numpy(), r1["dy0"])
    s.close()


def test_host_entry_point_matches_device(cuda):
    B = 256
    w = W.make("vdpb", batch=B)
    s, _, r = run_gpu("vdpb", B)
    h = s.gradient_host("sumsq", w["y0"], w["params"], w["t0"], w["t1"])
    np.testing.assert_array_equal(h["dp"], r["dp"])
    np.testing.assert_array_equal(h["n_acc"], r["n_acc"])
    s.close()


@pytest.mark.parametrize("name,B,bound", [("vdp1", 1, 1e-5), ("dho", 256, 1e-5), ("vdpb", 512, 1e-4)])
def test_mixed_precision_error_vs_fp64(oracle, cuda, name, B, bound):
    """Plain FP32 stages/VJPs (FP64 controller and accumulators): median
    gradient error against the FP64 oracle, bounded per config."""
    s, w, r = run_gpu(name, B, precision="mixed")
    assert (r["status"] == 0).all()
    idx = list(range(0, B, max(1, B // 32)))
    pb, ref = oracle_batch(oracle, w, idx)
    errs = [max(grad_rel(r["dy0"][b], g["dy0"]), grad_rel(r["dp"][b], g["dp"])) for b, g in zip(idx, ref)]
    assert np.median(errs) < bound, (np.median(errs), max(errs))
    s.close()


@pytest.mark.parametrize("name,B", [("vdp1", 1), ("dho", 256), ("vdpb", 512)])
def test_mixed_dw_error_vs_fp64(oracle, cuda, name, B):
    """Double-word stages/VJPs on the FP32 pipe: gradient error against the FP64
    oracle at most 1e-6 for every instance (the mixed-path target), median
    below 1e-9, and the same accepted-step counts."""
    s, w, r = run_gpu(name, B, precision="mixed_dw")
    assert (r["status"] == 0).all()
    idx = list(range(0, B, max(1, B // 32)))
    pb, ref = oracle_batch(oracle, w, idx)
    errs = [max(grad_rel(r["dy0"][b], g["dy0"]), grad_rel(r["dp"][b], g["dp"])) for b, g in zip(idx, ref)]
    assert max(errs) <= 1e-6, (np.median(errs), max(errs))
    assert np.median(errs) < 1e-9, np.median(errs)
    same = [int(r["n_acc"][b]) == g["n_acc"] for b, g in zip(idx, ref)]
    assert np.mean(same) >= 0.95
    s.close()
