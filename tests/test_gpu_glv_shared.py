"""Generalized Lotka-Volterra with one interaction matrix A shared by the
batch (bundle kernels).  Per instance the FP64 sweep reproduces the oracle's
GLV model (parameters r and the common A) bit for bit: step counts, y(T),
dy0 and dr.  The shared gradient dA is the sum over instances of the
oracle's per-instance dA, equal to rounding (the GPU sums in another order)."""
import numpy as np
import pytest
import torch

from vectorizedadjoint_gb300 import Solver
from vectorizedadjoint_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def dev(a):
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def make_small(N, B, seed=11):
    """The GLV-256 recipe at size N (diag -1, off-diagonal N(0, (0.5/sqrt N)^2))."""
    rng = np.random.Generator(np.random.PCG64(seed))
    A = rng.normal(0.0, 0.5 / np.sqrt(N), (N, N))
    A[np.arange(N), np.arange(N)] = -1.0
    r = rng.uniform(0.5, 1.5, (B, N))
    x0 = rng.uniform(0.1, 1.0, (B, N))
    return A, r, x0


def run(N, B, A, r, x0, T, precision, tol=1e-7, traj=None, **kw):
    s = Solver("glv_shared", N, N, B, tableau="dopri5", precision=precision, atol=tol, rtol=tol, **kw)
    dA = torch.empty(N, N, dtype=torch.float64, device="cuda")
    Ad = dev(A)
    s.set_shared(Ad, dA)
    out = s.gradient("sum", dev(x0), dev(r), dev(np.zeros(B)), dev(np.full(B, T)))
    torch.cuda.synchronize()
    res = {k: v.cpu().numpy() for k, v in out.items()}
    res["dA"] = dA.cpu().numpy()
    if traj is not None:
        res["traj"] = [s.trajectory(b) for b in traj]
    s.close()
    return res


def oracle_ref(oracle, N, A, r, x0, T, idx, tol=1e-7):
    pb = oracle.problem("glv", "dopri5", N, N + N * N, tol, tol)
    out = []
    for b in idx:
        p = np.concatenate([r[b], A.ravel()])
        out.append(oracle.gradient(pb, "sum", x0[b], p, 0.0, T))
    return out


@pytest.mark.parametrize("N,B,T", [(64, 10, 10.0), (256, 6, 10.0)])
def test_shared_glv_fp64_bit_exact(oracle, cuda, N, B, T):
    A, r, x0 = make_small(N, B)
    res = run(N, B, A, r, x0, T, "fp64")
    assert (res["status"] == 0).all()
    ref = oracle_ref(oracle, N, A, r, x0, T, range(B))
    dA = np.zeros((N, N))
    for b, g in enumerate(ref):
        assert g["status"] == 0
        assert int(res["n_acc"][b]) == g["n_acc"]
        np.testing.assert_array_equal(res["yT"][b], g["yT"])
        np.testing.assert_array_equal(res["dy0"][b], g["dy0"])
        np.testing.assert_array_equal(res["dp"][b], g["dp"][:N])
        dA += g["dp"][N:].reshape(N, N)
    scale = np.abs(dA).max()
    assert np.abs(res["dA"] - dA).max() <= 1e-12 * scale


@pytest.mark.parametrize("stage_records", [1, 0])
@pytest.mark.parametrize("N,B,T", [(64, 10, 10.0), (256, 6, 10.0)])
def test_shared_glv_mixed_dw(oracle, cuda, N, B, T, stage_records):
    """Double-word bundles against FP64, with stage records (the backward
    reads the forward's stage points and A X products) and without (the
    reference's recompute); the record read-back decodes either layout."""
    A, r, x0 = make_small(N, B)
    r64 = run(N, B, A, r, x0, T, "fp64", traj=[0, B - 1])
    rdw = run(N, B, A, r, x0, T, "mixed_dw", traj=[0, B - 1], stage_records=stage_records)
    for (t64, dt64, y64), (tdw, dtdw, ydw) in zip(r64["traj"], rdw["traj"]):
        # the double-word step sizes follow FP64 to ~1e-9 (the records decode
        # to the states, not to packed bits)
        assert len(t64) == len(tdw)
        np.testing.assert_allclose(tdw, t64, rtol=1e-7, atol=0)
        np.testing.assert_allclose(ydw, y64, rtol=1e-7, atol=1e-10)
    assert (rdw["status"] == 0).all()
    for b in range(B):
        g = np.concatenate([r64["dy0"][b], r64["dp"][b]])
        gd = np.concatenate([rdw["dy0"][b], rdw["dp"][b]])
        assert np.abs(gd - g).max() <= 1e-6 * np.abs(g).max()
    assert np.abs(rdw["dA"] - r64["dA"]).max() <= 1e-6 * np.abs(r64["dA"]).max()


def test_shared_glv_workload_smoke(cuda):
    """The benchmark configuration's inputs (N = 256) run to completion."""
    w = W.make("glv256", batch=8)
    res = run(256, 8, w["shared"], w["params"], w["y0"], 10.0, "mixed_dw")
    assert (res["status"] == 0).all()
    assert np.isfinite(res["dA"]).all()


def test_shared_glv256_tensor_core_dA_vs_fp64(cuda):
    """N = 256, double-word sweeps with stage records: the backward writes
    factor rows and dA comes from the tcgen05 contraction
    (csrc/va_contract.cu); against the FP64 path's dA (FP64 CTA partials)
    within 1e-8 of its largest entry, and against the double-word sweeps
    without stage records (which keep the fused double-word partials) to the
    same bound."""
    N, B, T = 256, 12, 10.0
    A, r, x0 = make_small(N, B, seed=21)
    r64 = run(N, B, A, r, x0, T, "fp64")
    rtc = run(N, B, A, r, x0, T, "mixed_dw", stage_records=1)
    rfu = run(N, B, A, r, x0, T, "mixed_dw", stage_records=0)
    scale = np.abs(r64["dA"]).max()
    assert np.isfinite(rtc["dA"]).all()
    assert np.abs(rtc["dA"] - r64["dA"]).max() <= 1e-8 * scale, np.abs(rtc["dA"] - r64["dA"]).max() / scale
    assert np.abs(rtc["dA"] - rfu["dA"]).max() <= 1e-8 * scale
