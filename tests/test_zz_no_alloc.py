"""va_gradient_noalloc: the entry point for callers that may not allocate
device memory while they run (its scratch is a fixed array compiled into the
library).  Called through the C ABI, twice in a row (the second call reuses
the array with the first call's leftovers in it), it must give the same
gradients as va_gradient, which works in handle-owned, cudaMalloc'd memory;
a batch too large for the array is rejected before any GPU work.  This file
is collected last on purpose."""
import ctypes

import numpy as np
import pytest
import torch

from vectorizedadjoint_gb300 import Solver, _lib
from vectorizedadjoint_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def dev(a, dtype=torch.float64):
    return torch.tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda")


def p(t):
    return ctypes.c_void_p(t.data_ptr())


def call_noalloc(L, model, tableau, precision, tol, cost, B, y0, par, t0, t1, dt0=1e-3):
    out = dict(yT=torch.empty(B, y0.shape[1], dtype=torch.float64, device="cuda"),
               dy0=torch.empty(B, y0.shape[1], dtype=torch.float64, device="cuda"),
               dp=torch.empty(B, par.shape[1], dtype=torch.float64, device="cuda"),
               n_acc=torch.empty(B, dtype=torch.int32, device="cuda"),
               status=torch.empty(B, dtype=torch.int32, device="cuda"))
    st = L.va_gradient_noalloc(_lib.MODELS[model], _lib.TABLEAUX[tableau], _lib.PRECISIONS[precision],
                               tol, tol, dt0, 1000000, 500, _lib.COSTS[cost], B,
                               p(y0), p(par), p(t0), p(t1), p(out["yT"]), p(out["dy0"]), p(out["dp"]),
                               p(out["n_acc"]), p(out["status"]), None)
    torch.cuda.synchronize()
    return st, {k: v.cpu().numpy() for k, v in out.items()}


CASES = [  # workload, batch, precision, tableau (None: the workload's), dt0, stage records in the reference run
    ("vdpb", 2048, "fp64", None, 1e-3, 1),
    ("dho", 512, "mixed_dw", None, 1e-3, 1),
    ("vdpb", 1024, "mixed", None, 1e-3, 1),
    ("vdpb", 512, "fp64", "rkf78", 1e-3, 1),
    ("dho", 256, "mixed_dw", "rkf78", 1e-3, 1),
    ("dho", 256, "fp64", "rk4", 1e-2, 1),
    ("vdpb", 128, "mixed_dw", "euler", 1e-2, 1),
    # too many instances for stage records (4 chunks each): [t, dt, y] records
    ("vdpb", 8192, "mixed_dw", None, 1e-3, 0),
]


@pytest.mark.parametrize("name,B,precision,tableau,dt0,stages", CASES)
def test_noalloc_matches_va_gradient_twice(cuda, name, B, precision, tableau, dt0, stages):
    L = _lib.load()
    w = W.make(name, batch=B)
    c = w["cfg"]
    tab = tableau or c["tableau"]
    t1 = np.minimum(w["t1"], 10.0) if tab in ("rk4", "euler") else w["t1"]
    y0, par, t0, t1 = dev(w["y0"]), dev(w["params"]), dev(w["t0"]), dev(t1)
    s = Solver(c["model"], c["n"], c["npar"], B, tableau=tab, precision=precision,
               atol=c["tol"], rtol=c["tol"], dt0=dt0, stage_records=stages)
    ref = {k: v.cpu().numpy() for k, v in s.gradient(c["cost"], y0, par, t0, t1).items()}
    s.close()
    assert (ref["status"] == 0).all()
    for _ in range(2):
        st, r = call_noalloc(L, c["model"], tab, precision, c["tol"], c["cost"], B, y0, par, t0, t1, dt0=dt0)
        assert st == 0
        assert (r["status"] == 0).all()
        np.testing.assert_array_equal(r["n_acc"], ref["n_acc"])
        np.testing.assert_array_equal(r["yT"], ref["yT"])
        np.testing.assert_array_equal(r["dy0"], ref["dy0"])
        np.testing.assert_array_equal(r["dp"], ref["dp"])


@pytest.mark.parametrize("name,B,tableau,dt0", [("vdpb", 30000, None, 1e-3), ("dho", 2000, "rk4", 1e-2)])
def test_noalloc_pool_exhausted_at_run_time(cuda, name, B, tableau, dt0):
    """A batch whose first chunks fit but whose steps do not: the instances
    that run out report VA_CKPT_BUDGET (4), and every instance that finishes
    (status 0) has va_gradient's bits.  (Instances run concurrently and draw
    chunks from one pool, so the horizons vary here -- damped oscillators over
    5..50 time units -- and the short ones finish before it runs dry.)"""
    L = _lib.load()
    w = W.make(name, batch=B)
    c = w["cfg"]
    tab = tableau or c["tableau"]
    y0, par, t0, t1 = dev(w["y0"]), dev(w["params"]), dev(w["t0"]), dev(w["t1"])
    s = Solver(c["model"], c["n"], c["npar"], B, tableau=tab, precision="fp64", atol=c["tol"], rtol=c["tol"],
               dt0=dt0)
    ref = {k: v.cpu().numpy() for k, v in s.gradient(c["cost"], y0, par, t0, t1).items()}
    s.close()
    assert (ref["status"] == 0).all()
    st, r = call_noalloc(L, c["model"], tab, "fp64", c["tol"], c["cost"], B, y0, par, t0, t1, dt0=dt0)
    assert st == 0
    ok, out = r["status"] == 0, r["status"] == 4
    assert (ok | out).all() and ok.any() and out.any(), np.bincount(r["status"])
    for k in ("n_acc", "yT", "dy0", "dp"):
        np.testing.assert_array_equal(r[k][ok], ref[k][ok])


def test_noalloc_rejects_oversized_batch(cuda):
    """More instances than the array holds (metadata plus one checkpoint chunk
    each): VA_BAD_ARGS, nothing launched."""
    L = _lib.load()
    big = 1 << 20
    x = torch.zeros(4, 2, dtype=torch.float64, device="cuda")
    o = torch.zeros(4, 2, dtype=torch.float64, device="cuda")
    st = L.va_gradient_noalloc(_lib.MODELS["vdp"], 0, 0, 1e-6, 1e-6, 1e-3, 1000, 500, 0, big,
                               p(x), p(x), p(x), p(x), None, p(o), p(o), None, None, None)
    assert st == 5
    assert L.va_gradient_noalloc(_lib.MODELS["glv"], 0, 0, 1e-6, 1e-6, 1e-3, 1000, 500, 0, 4,
                                 p(x), p(x), p(x), p(x), None, p(o), p(o), None, None, None) == 5
