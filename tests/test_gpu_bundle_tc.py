"""The shared-matrix GLV sweeps with tensor-core stage products
(csrc/va_bundle_tc.cuh): clusters of 8 CTAs carry 64 instances in lockstep and
form each stage's A X (forward, DOPRI5) and A^T v (backward, the 5(4) pairs)
for the whole tile on tcgen05 with an error-free digit split.  Against the
double-word bundle sweeps (FP32-pipe dot products) and against the FP64
path: the same accepted steps, y(T) and per-instance gradients at the
double-word level, dA (the tensor-core contraction over nearly identical
factor rows) to 1e-8 of its largest entry."""
import numpy as np
import pytest
import torch

from vectorizedadjoint_gb300 import Solver
from vectorizedadjoint_gb300 import workloads as W

pytestmark = pytest.mark.gpu

N = 256


def dev(a):
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def make(B, seed):
    """The GLV-256 recipe (diag -1, off-diagonal N(0, (0.5/sqrt N)^2))."""
    rng = np.random.Generator(np.random.PCG64(seed))
    A = rng.normal(0.0, 0.5 / np.sqrt(N), (N, N))
    A[np.arange(N), np.arange(N)] = -1.0
    r = rng.uniform(0.5, 1.5, (B, N))
    x0 = rng.uniform(0.1, 1.0, (B, N))
    return A, r, x0


def run(A, r, x0, t1, precision, tensor_products=0, tol=1e-7, cost="sum", **kw):
    B = r.shape[0]
    s = Solver("glv_shared", N, N, B, tableau=kw.pop("tableau", "dopri5"), precision=precision, atol=tol,
               rtol=tol, tensor_products=tensor_products, **kw)
    dA = torch.empty(N, N, dtype=torch.float64, device="cuda")
    s.set_shared(dev(A), dA)
    out = s.gradient(cost, dev(x0), dev(r), dev(np.zeros(B)), dev(t1))
    torch.cuda.synchronize()
    res = {k: v.cpu().numpy() for k, v in out.items()}
    res["dA"] = dA.cpu().numpy()
    res["launch"] = s.launch()
    s.close()
    return res


def rel_inst(a, b):
    """per-instance max |a - b| / max |b| over [dy0, dr]"""
    ga = np.concatenate([a["dy0"], a["dp"]], axis=1)
    gb = np.concatenate([b["dy0"], b["dp"]], axis=1)
    return np.abs(ga - gb).max(axis=1) / np.abs(gb).max(axis=1)


def rel_y(a, b):
    """per-instance max |a - b| / max |b| of y(T)"""
    return np.abs(a["yT"] - b["yT"]).max(axis=1) / np.abs(b["yT"]).max(axis=1)


@pytest.mark.parametrize("tableau", ["dopri5", "ck54"])
@pytest.mark.parametrize("B", [1, 100])
def test_tc_sweeps_vs_fp32_pipe_and_fp64(cuda, B, tableau):
    """Ragged tiles (1 and 100 instances: one partly filled cluster, then
    one full and one partly filled), both 5(4) pairs (CK54, not FSAL, keeps
    the bundle forward)."""
    A, r, x0 = make(B, seed=31 + B)
    t1 = np.full(B, 10.0)
    tc = run(A, r, x0, t1, "mixed_dw", 0, tableau=tableau)
    pipe = run(A, r, x0, t1, "mixed_dw", -1, tableau=tableau)
    f64 = run(A, r, x0, t1, "fp64", tableau=tableau)
    assert tc["launch"]["bwd_block"] == 512, tc["launch"]  # the cluster kernels ran
    assert tc["launch"]["fwd_block"] == (512 if tableau == "dopri5" else N), tc["launch"]
    assert pipe["launch"]["bwd_block"] == N and pipe["launch"]["fwd_block"] == N
    assert (tc["status"] == 0).all() and (pipe["status"] == 0).all()
    # the accepted steps of the FP64 sweep, y(T) to the double-word level
    np.testing.assert_array_equal(tc["n_acc"], f64["n_acc"])
    np.testing.assert_array_equal(pipe["n_acc"], f64["n_acc"])
    assert rel_y(tc, f64).max() <= 1e-12, rel_y(tc, f64).max()
    assert rel_inst(tc, pipe).max() <= 1e-11, rel_inst(tc, pipe).max()
    assert rel_inst(tc, f64).max() <= 1e-11, rel_inst(tc, f64).max()
    scale = np.abs(f64["dA"]).max()
    assert np.isfinite(tc["dA"]).all()
    assert np.abs(tc["dA"] - pipe["dA"]).max() <= 1e-8 * scale
    assert np.abs(tc["dA"] - f64["dA"]).max() <= 1e-8 * scale


def test_tc_forward_trajectory(cuda):
    """The cluster forward's checkpoint records decode to the FP64 sweep's
    steps: the same step count, t_n and y_n as close to FP64 as the
    FP32-pipe double-word forward's (the double-word controller's dt
    differs from FP64's at ~1e-9, so mid-trajectory states do too)."""
    B = 70
    A, r, x0 = make(B, seed=5)
    t1 = np.full(B, 10.0)
    out = {}
    for prec, tp in (("fp64", 0), ("mixed_dw", 0), ("mixed_dw", -1)):
        s = Solver("glv_shared", N, N, B, precision=prec, atol=1e-7, rtol=1e-7, tensor_products=tp)
        dA = torch.empty(N, N, dtype=torch.float64, device="cuda")
        s.set_shared(dev(A), dA)
        s.gradient("sum", dev(x0), dev(r), dev(np.zeros(B)), dev(t1))
        torch.cuda.synchronize()
        out[(prec, tp)] = [s.trajectory(b) for b in (0, 33, 69)]
        if prec == "mixed_dw":
            assert s.launch()["fwd_block"] == (512 if tp == 0 else N)
        s.close()
    dev_t = {"tc": 0.0, "pipe": 0.0}
    dev_y = {"tc": 0.0, "pipe": 0.0}
    for k, key in (("tc", ("mixed_dw", 0)), ("pipe", ("mixed_dw", -1))):
        for (t64, _, y64), (tdw, _, ydw) in zip(out[("fp64", 0)], out[key]):
            assert len(t64) == len(tdw)
            np.testing.assert_allclose(tdw, t64, rtol=1e-7, atol=0)
            np.testing.assert_allclose(ydw, y64, rtol=1e-7, atol=1e-10)
            dev_t[k] = max(dev_t[k], float(np.abs(tdw - t64).max()))
            dev_y[k] = max(dev_y[k], float(np.abs(ydw - y64).max()))
    assert dev_t["tc"] <= 10 * dev_t["pipe"] + 1e-13, dev_t
    assert dev_y["tc"] <= 10 * dev_y["pipe"] + 1e-13, dev_y


def test_tc_backward_uneven_lengths_and_failed_instance(cuda):
    """Instances of very different lengths share a tile (the lockstep runs
    the longest; finished instances contribute zero columns), and one
    instance whose forward fails (a NaN initial state) reports the forward's
    status with NaN gradients while the others match the FP32-pipe backward."""
    B = 70
    A, r, x0 = make(B, seed=7)
    x0[5] = np.nan
    t1 = np.linspace(0.2, 12.0, B)
    tc = run(A, r, x0, t1, "mixed_dw", 0)
    pipe = run(A, r, x0, t1, "mixed_dw", -1)
    assert tc["launch"]["bwd_block"] == 512
    np.testing.assert_array_equal(tc["status"], pipe["status"])
    assert tc["status"][5] != 0 and (np.delete(tc["status"], 5) == 0).all(), tc["status"]
    assert np.isnan(tc["dy0"][5]).all() and np.isnan(tc["dp"][5]).all()
    ok = np.arange(B) != 5
    assert rel_inst({k: tc[k][ok] for k in ("dy0", "dp")}, {k: pipe[k][ok] for k in ("dy0", "dp")}).max() <= 1e-11
    n = tc["n_acc"][ok]
    assert n.max() >= 3 * n.min(), (n.min(), n.max())  # the tile really is uneven


def test_tc_backward_sumsq_cost_and_workload(cuda):
    """The benchmark recipe (glv256) with the sum-of-squares cost, 130
    instances (three clusters), against FP64."""
    B = 130
    w = W.make("glv256", batch=B)
    t1 = np.full(B, 10.0)
    tc = run(w["shared"], w["params"], w["y0"], t1, "mixed_dw", 0, cost="sumsq")
    f64 = run(w["shared"], w["params"], w["y0"], t1, "fp64", cost="sumsq")
    assert tc["launch"]["bwd_block"] == 512
    assert (tc["status"] == 0).all()
    assert rel_inst(tc, f64).max() <= 1e-11, rel_inst(tc, f64).max()
    scale = np.abs(f64["dA"]).max()
    assert np.abs(tc["dA"] - f64["dA"]).max() <= 1e-8 * scale


def test_tc_backward_repeatable(cuda):
    """Two gradients of one handle (the second replays the captured graph)
    give the same bits."""
    B = 64
    A, r, x0 = make(B, seed=3)
    s = Solver("glv_shared", N, N, B, precision="mixed_dw", atol=1e-7, rtol=1e-7)
    dA = torch.empty(N, N, dtype=torch.float64, device="cuda")
    s.set_shared(dev(A), dA)
    outs = []
    for _ in range(2):
        o = s.gradient("sum", dev(x0), dev(r), dev(np.zeros(B)), dev(np.full(B, 10.0)))
        torch.cuda.synchronize()
        outs.append({k: v.cpu().numpy().copy() for k, v in o.items()} | {"dA": dA.cpu().numpy().copy()})
    assert s.launch()["bwd_block"] == 512
    s.close()
    for k in ("dy0", "dp", "dA"):
        np.testing.assert_array_equal(outs[0][k], outs[1][k])


def test_tc_forward_limits(cuda):
    """A zero-length instance (y(T) = y_0, no step), an instance that reaches
    max_steps, and ordinary ones share the tiles; counters, statuses and y(T)
    match the FP32-pipe sweeps, the failed instance's gradients are NaN."""
    B = 66
    A, r, x0 = make(B, seed=9)
    t1 = np.full(B, 10.0)
    t1[0] = 0.0   # t0 = t1
    t1[65] = 400.0
    kw = dict(max_steps=80)
    tc = run(A, r, x0, t1, "mixed_dw", 0, **kw)
    pipe = run(A, r, x0, t1, "mixed_dw", -1, **kw)
    assert tc["launch"]["fwd_block"] == 512 and tc["launch"]["bwd_block"] == 512
    np.testing.assert_array_equal(tc["status"], pipe["status"])
    np.testing.assert_array_equal(tc["n_acc"], pipe["n_acc"])
    assert tc["status"][65] != 0 and tc["n_acc"][65] == 80, (tc["status"][65], tc["n_acc"][65])
    assert tc["n_acc"][0] == 0 and tc["status"][0] == 0
    np.testing.assert_array_equal(tc["yT"][0], x0[0])
    ok = tc["status"] == 0
    assert rel_y({"yT": tc["yT"][ok]}, {"yT": pipe["yT"][ok]}).max() <= 1e-12
    assert rel_inst({k: tc[k][ok] for k in ("dy0", "dp")}, {k: pipe[k][ok] for k in ("dy0", "dp")}).max() <= 1e-11
    assert np.isnan(tc["dy0"][65]).all()


@pytest.mark.parametrize("tableau", ["dopri5", "ck54"])
def test_tc_sweeps_with_tail(cuda, tableau):
    """1,000 instances: 16 tiles, one more than the 15 clusters a GB300 holds
    at once, so the last tile's 40 instances run in the double-word bundle
    sweeps beside the clusters (a programmatic dependent launch; CK54: the
    backward only).  Every instance, tail included, against FP64; dA against
    FP64 and the FP32-pipe sweeps; two gradients give the same bits."""
    B = 1000
    w = W.make("glv256", batch=B)
    t1 = np.full(B, 10.0)
    f64 = run(w["shared"], w["params"], w["y0"], t1, "fp64", tableau=tableau)
    pipe = run(w["shared"], w["params"], w["y0"], t1, "mixed_dw", -1, tableau=tableau)
    s = Solver("glv_shared", N, N, B, tableau=tableau, precision="mixed_dw", atol=1e-7, rtol=1e-7)
    dA = torch.empty(N, N, dtype=torch.float64, device="cuda")
    s.set_shared(dev(w["shared"]), dA)
    outs = []
    for _ in range(2):
        o = s.gradient("sum", dev(w["y0"]), dev(w["params"]), dev(np.zeros(B)), dev(t1))
        torch.cuda.synchronize()
        outs.append({k: v.cpu().numpy().copy() for k, v in o.items()} | {"dA": dA.cpu().numpy().copy()})
    assert s.launch()["fwd_block"] == (512 if tableau == "dopri5" else N) and s.launch()["bwd_block"] == 512
    s.close()
    tc = outs[0]
    assert (tc["status"] == 0).all()
    np.testing.assert_array_equal(tc["n_acc"], f64["n_acc"])
    assert rel_y(tc, f64).max() <= 1e-12, rel_y(tc, f64).max()
    assert rel_inst(tc, f64).max() <= 1e-11, rel_inst(tc, f64).max()
    scale = np.abs(f64["dA"]).max()
    assert np.abs(tc["dA"] - f64["dA"]).max() <= 1e-8 * scale
    assert np.abs(tc["dA"] - pipe["dA"]).max() <= 1e-8 * scale
    for k in ("yT", "dy0", "dp", "dA"):
        np.testing.assert_array_equal(outs[0][k], outs[1][k])
