"""Two-level checkpointing: storing every k-th accepted step and
re-integrating segments in the backward sweep reproduces the every-step
gradients bit for bit (the re-integration runs the same device code from
the same bits, and each segment is checked to land on the next checkpoint).
The automatic mode picks a stride that fits an undersized budget."""
import numpy as np
import pytest
import torch

from vectorizedadjoint_gb300 import Solver
from vectorizedadjoint_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def dev(a):
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def grads(name, B, **kw):
    return grads_kw(name, B, **kw)


def grads_kw(name, B, tableau=None, **kw):
    w = W.make(name, batch=B)
    c = w["cfg"]
    s = Solver(c["model"], c["n"], c["npar"], B, tableau=tableau or c["tableau"], atol=c["tol"], rtol=c["tol"],
               **kw)
    out = s.gradient(c["cost"], dev(w["y0"]), dev(w["params"]), dev(w["t0"]), dev(w["t1"]))
    torch.cuda.synchronize()
    res = {k: v.cpu().numpy() for k, v in out.items()}
    info = s.checkpoint_info()
    s.close()
    return res, info


@pytest.mark.parametrize("name,B,precision,stride", [("vdpb", 512, "fp64", 8), ("dho", 256, "fp64", 5),
                                                     ("vdpb", 512, "mixed_dw", 16), ("dho", 128, "mixed", 3)])
def test_stride_matches_every_step(cuda, name, B, precision, stride):
    ref, _ = grads(name, B, precision=precision)
    r, info = grads(name, B, precision=precision, ckpt_stride=stride)
    assert info["stride"] == stride
    assert (r["status"] == 0).all(), np.unique(r["status"])
    np.testing.assert_array_equal(r["n_acc"], ref["n_acc"])
    np.testing.assert_array_equal(r["dy0"], ref["dy0"])
    np.testing.assert_array_equal(r["dp"], ref["dp"])


def test_automatic_stride_under_budget(cuda):
    """A pool ~1/10 of what every-step storage needs: the forward reruns with
    4x strides until the checkpoints fit, and the gradients are unchanged."""
    B = 1024
    ref, _ = grads("vdpb", B)
    need = int((ref["n_acc"].sum() + B) * 32)
    w = W.make("vdpb", batch=B)
    s = Solver("vdp", 2, 1, B, atol=1e-6, rtol=1e-6, ckpt_stride=-1, ckpt_budget_bytes=need // 10, chunk_len=8)
    P = dev(w["params"])
    f = s.forward(dev(w["y0"]), P, dev(w["t0"]), dev(w["t1"]))
    lam = (2.0 * f["yT"]).reshape(B, 1, 2).contiguous()
    bw = s.backward(P, lam)
    torch.cuda.synchronize()
    info = s.checkpoint_info()
    assert info["stride"] > 1 and info["capacity_bytes"] < need
    assert (bw["status"].cpu().numpy() == 0).all()
    np.testing.assert_array_equal(bw["dy0"].cpu().numpy()[:, 0], ref["dy0"])
    np.testing.assert_array_equal(bw["dp"].cpu().numpy()[:, 0], ref["dp"])
    s.close()


def test_stride_multi_seed(cuda):
    B, Q = 64, 3
    w = W.make("vdpb", batch=B)
    rng = np.random.default_rng(5)
    lam = dev(rng.normal(size=(B, Q, 2)))
    mu = dev(rng.normal(size=(B, Q, 1)))
    out = []
    for stride in (1, 7):
        s = Solver("vdp", 2, 1, B, nout=Q, atol=1e-6, rtol=1e-6, ckpt_stride=stride)
        P = dev(w["params"])
        s.forward(dev(w["y0"]), P, dev(w["t0"]), dev(w["t1"]))
        bw = s.backward(P, lam, mu)
        torch.cuda.synchronize()
        out.append((bw["dy0"].cpu().numpy(), bw["dp"].cpu().numpy()))
        s.close()
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])


@pytest.mark.parametrize("name,B", [("vdpb", 512), ("dho", 256)])
def test_stage_records_vs_recompute(cuda, name, B):
    """mixed_dw with every step checkpointed: stage records (the backward
    reads the forward's stage values) and the reference's stage recompute
    run the same forward bit for bit and agree on the gradients to 1e-8 of
    their scale.  (The recompute forms the stages with h = t_{n+1} - t_n,
    the forward with its double-word dt: step sizes one FP64 rounding apart,
    which stiff Van der Pol instances amplify to ~1e-9.)"""
    st, _ = grads(name, B, precision="mixed_dw", stage_records=1)
    rc, info = grads(name, B, precision="mixed_dw", stage_records=0)
    assert info["stride"] == 1
    assert (st["status"] == 0).all() and (rc["status"] == 0).all()
    np.testing.assert_array_equal(st["n_acc"], rc["n_acc"])
    np.testing.assert_array_equal(st["yT"], rc["yT"])
    for k in ("dy0", "dp"):
        scale = np.maximum(np.abs(st[k]).max(1, keepdims=True), 1e-8)
        assert (np.abs(st[k] - rc[k]) / scale).max() < 1e-8


@pytest.mark.parametrize("stage_records", [1, 0])
def test_glv_lane_group_modes(cuda, stage_records):
    """GLV N=10 lane groups, mixed_dw: the double-word stage-record sweeps
    (stage_records = 1) and the double-word-stage sweeps over FP64 records
    (0) both stay within 1e-6 of the FP64 path on every instance."""
    B = 256
    ref, _ = grads("glv10", B, precision="fp64")
    r, info = grads("glv10", B, precision="mixed_dw", stage_records=stage_records)
    assert info["stride"] == 1
    assert (r["status"] == 0).all()
    g = np.concatenate([r["dy0"], r["dp"]], 1)
    g64 = np.concatenate([ref["dy0"], ref["dp"]], 1)
    scale = np.maximum(np.abs(g64).max(1, keepdims=True), 1e-8)
    assert (np.abs(g - g64) / scale).max() < 1e-6


def test_ladder_drops_stage_values_first(cuda):
    """Automatic checkpointing with a pool that holds [t, dt, y] records of
    every step but not stage records: the stride stays 1, the stage values
    go, and the gradients are the recompute path's, bit for bit."""
    B = 1024
    ref, _ = grads("vdpb", B, precision="mixed_dw", stage_records=0)
    plain = int((ref["n_acc"].sum() + 3 * B) * 32)
    w = W.make("vdpb", batch=B)
    s = Solver("vdp", 2, 1, B, precision="mixed_dw", atol=1e-6, rtol=1e-6, ckpt_stride=-1,
               ckpt_budget_bytes=2 * plain, chunk_len=8)
    P = dev(w["params"])
    f = s.forward(dev(w["y0"]), P, dev(w["t0"]), dev(w["t1"]))
    lam = (2.0 * f["yT"]).reshape(B, 1, 2).contiguous()
    bw = s.backward(P, lam)
    torch.cuda.synchronize()
    info = s.checkpoint_info()
    assert info["stride"] == 1 and info["capacity_bytes"] < 112 * int(ref["n_acc"].sum() + B)
    assert (bw["status"].cpu().numpy() == 0).all()
    np.testing.assert_array_equal(bw["dy0"].cpu().numpy()[:, 0], ref["dy0"])
    np.testing.assert_array_equal(bw["dp"].cpu().numpy()[:, 0], ref["dp"])
    s.close()


def test_ladder_first_rung_lane_groups(cuda):
    """GLV-10 lane groups (no two-level backward): with ckpt_stride = -1 and a
    pool too small for stage records (2 + 12N doubles a step) but large
    enough for [t, dt, y] records, the forward reruns without stage records;
    the gradients are the recompute path's, bit for bit."""
    B = 96
    ref, _ = grads("glv10", B, precision="mixed_dw", stage_records=0)
    w = W.make("glv10", batch=B)
    c = w["cfg"]
    plain = int((ref["n_acc"].sum() + 3 * B) * 12 * 8)
    s = Solver(c["model"], c["n"], c["npar"], B, tableau=c["tableau"], precision="mixed_dw", atol=c["tol"],
               rtol=c["tol"], ckpt_stride=-1, ckpt_budget_bytes=3 * plain, chunk_len=8)
    P = dev(w["params"])
    s.forward(dev(w["y0"]), P, dev(w["t0"]), dev(w["t1"]))
    bw = s.backward(P, torch.ones(B, 1, c["n"], dtype=torch.float64, device="cuda"))
    torch.cuda.synchronize()
    info = s.checkpoint_info()
    assert info["stride"] == 1 and info["capacity_bytes"] <= 3 * plain
    assert (bw["status"].cpu().numpy() == 0).all()
    np.testing.assert_array_equal(bw["dy0"].cpu().numpy()[:, 0], ref["dy0"])
    np.testing.assert_array_equal(bw["dp"].cpu().numpy()[:, 0], ref["dp"])
    s.close()


@pytest.mark.parametrize("precision,stride,tableau", [("fp64", 4, None), ("mixed", 5, None), ("mixed_dw", 8, None),
                                                       ("fp64", 3, "rkf78"), ("fp64", 6, "rk4"),
                                                       ("mixed_dw", 4, "euler"), ("fp64", 64, None)])
def test_lane_group_stride_matches_every_step(cuda, precision, stride, tableau):
    """GLV N=10 lane groups: every stride-th step stored, segments re-run by
    the group (backward_group_kernel_2level) -- the gradients equal the
    every-step sweeps' bit for bit (mixed_dw: the sweeps over [t, dt, y]
    records, stage_records = 0, whose forward code the segments re-run).  A
    stride above every instance's step count (64) leaves one segment."""
    B = 96
    kw = {"tableau": tableau} if tableau else {}
    if tableau in ("rk4", "euler"):
        kw["dt0"] = 1e-2
    sr = {"stage_records": 0} if precision == "mixed_dw" else {}
    ref, _ = grads_kw("glv10", B, precision=precision, **sr, **kw)
    r, info = grads_kw("glv10", B, precision=precision, ckpt_stride=stride, **sr, **kw)
    assert info["stride"] == stride
    assert (ref["status"] == 0).all() and (r["status"] == 0).all(), np.unique(r["status"])
    np.testing.assert_array_equal(r["n_acc"], ref["n_acc"])
    np.testing.assert_array_equal(r["yT"], ref["yT"])
    np.testing.assert_array_equal(r["dy0"], ref["dy0"])
    np.testing.assert_array_equal(r["dp"], ref["dp"])


def test_lane_group_automatic_stride_under_budget(cuda):
    """GLV-10, mixed_dw, ckpt_stride = -1 with a pool ~1/8 of what [t, dt, y]
    records of every step need: the ladder drops the stage records, then
    thins the checkpoints until they fit; the gradients are the recompute
    path's, bit for bit."""
    B = 96
    ref, _ = grads("glv10", B, precision="mixed_dw", stage_records=0)
    w = W.make("glv10", batch=B)
    c = w["cfg"]
    plain = int((ref["n_acc"].sum() + B) * 12 * 8)
    s = Solver(c["model"], c["n"], c["npar"], B, tableau=c["tableau"], precision="mixed_dw", atol=c["tol"],
               rtol=c["tol"], ckpt_stride=-1, ckpt_budget_bytes=plain // 8, chunk_len=4)
    P = dev(w["params"])
    s.forward(dev(w["y0"]), P, dev(w["t0"]), dev(w["t1"]))
    bw = s.backward(P, torch.ones(B, 1, c["n"], dtype=torch.float64, device="cuda"))
    torch.cuda.synchronize()
    info = s.checkpoint_info()
    assert info["stride"] > 1 and info["capacity_bytes"] <= plain // 8
    assert (bw["status"].cpu().numpy() == 0).all()
    np.testing.assert_array_equal(bw["dy0"].cpu().numpy()[:, 0], ref["dy0"])
    np.testing.assert_array_equal(bw["dp"].cpu().numpy()[:, 0], ref["dp"])
    s.close()


def shared_problem(N, B, seed=11):
    """The GLV-256 recipe at size N (diag -1, off-diagonal N(0, (0.5/sqrt N)^2))."""
    rng = np.random.Generator(np.random.PCG64(seed))
    A = rng.normal(0.0, 0.5 / np.sqrt(N), (N, N))
    A[np.arange(N), np.arange(N)] = -1.0
    return A, rng.uniform(0.5, 1.5, (B, N)), rng.uniform(0.1, 1.0, (B, N))


def shared_grads(N, B, precision, tableau="dopri5", dt0=1e-3, **kw):
    A, r, x0 = shared_problem(N, B)
    s = Solver("glv_shared", N, N, B, tableau=tableau, precision=precision, atol=1e-7, rtol=1e-7, dt0=dt0, **kw)
    dA = torch.empty(N, N, dtype=torch.float64, device="cuda")
    s.set_shared(dev(A), dA)
    out = s.gradient("sum", dev(x0), dev(r), dev(np.zeros(B)), dev(np.full(B, 10.0)))
    torch.cuda.synchronize()
    res = {k: v.cpu().numpy() for k, v in out.items()}
    res["dA"] = dA.cpu().numpy()
    info = s.checkpoint_info()
    s.close()
    return res, info


@pytest.mark.parametrize("N,B,precision,stride,tableau", [(64, 10, "fp64", 4, "dopri5"), (64, 9, "mixed", 3, "ck54"),
                                                          (64, 10, "mixed_dw", 5, "dopri5"),
                                                          (256, 5, "mixed_dw", 8, "dopri5"),
                                                          (256, 4, "fp64", 16, "dopri5"),
                                                          (64, 6, "mixed_dw", 7, "rk4")])
def test_shared_matrix_stride_matches_every_step(cuda, N, B, precision, stride, tableau):
    """Shared-matrix GLV bundles (backward_bundle_kernel_2level): each
    instance's gradients equal the every-step sweeps' bit for bit (mixed_dw:
    the sweeps over [t, dt, y] records with the stage recompute, which the
    segments' back steps run); the shared dA, whose terms the two sweeps add
    in another order, agrees to 1e-12 of its largest entry (FP64), 1e-9
    (double-word) or 1e-5 (float stages: each step's terms are summed in
    float before they reach the FP64 partial, over the instances stepping
    together)."""
    dt0 = 1e-2 if tableau == "rk4" else 1e-3
    sr = {"stage_records": 0} if precision == "mixed_dw" else {}
    ref, _ = shared_grads(N, B, precision, tableau, dt0, **sr)
    r, info = shared_grads(N, B, precision, tableau, dt0, ckpt_stride=stride, **sr)
    assert info["stride"] == stride
    assert (ref["status"] == 0).all() and (r["status"] == 0).all(), np.unique(r["status"])
    np.testing.assert_array_equal(r["n_acc"], ref["n_acc"])
    np.testing.assert_array_equal(r["yT"], ref["yT"])
    np.testing.assert_array_equal(r["dy0"], ref["dy0"])
    np.testing.assert_array_equal(r["dp"], ref["dp"])
    tol = {"fp64": 1e-12, "mixed_dw": 1e-9, "mixed": 1e-5}[precision]
    assert np.abs(r["dA"] - ref["dA"]).max() <= tol * np.abs(ref["dA"]).max()


def test_shared_matrix_automatic_stride_under_budget(cuda):
    """GLV-256 bundles, mixed_dw, ckpt_stride = -1 with a budget far below
    every-step stage records: the ladder drops the stage records, then
    thins the checkpoints; per-instance gradients equal the recompute
    path's bit for bit."""
    N, B = 256, 6
    ref, _ = shared_grads(N, B, "mixed_dw", stage_records=0)
    plain = int((ref["n_acc"].sum() + B) * (N + 2) * 8)
    r, info = shared_grads(N, B, "mixed_dw", ckpt_stride=-1, ckpt_budget_bytes=plain // 6, chunk_len=4)
    assert info["stride"] > 1 and info["capacity_bytes"] <= plain // 6
    assert (r["status"] == 0).all()
    np.testing.assert_array_equal(r["dy0"], ref["dy0"])
    np.testing.assert_array_equal(r["dp"], ref["dp"])
    assert np.abs(r["dA"] - ref["dA"]).max() <= 1e-9 * np.abs(ref["dA"]).max()


def test_invalid_stride_rejected(cuda):
    with pytest.raises(Exception):
        Solver("glv_shared", 64, 64, 8, ckpt_stride=-2)
