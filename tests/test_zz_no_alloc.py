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


def call_noalloc(L, model, tableau, precision, tol, cost, B, y0, par, t0, t1):
    out = dict(yT=torch.empty(B, y0.shape[1], dtype=torch.float64, device="cuda"),
               dy0=torch.empty(B, y0.shape[1], dtype=torch.float64, device="cuda"),
               dp=torch.empty(B, par.shape[1], dtype=torch.float64, device="cuda"),
               n_acc=torch.empty(B, dtype=torch.int32, device="cuda"),
               status=torch.empty(B, dtype=torch.int32, device="cuda"))
    st = L.va_gradient_noalloc(_lib.MODELS[model], _lib.TABLEAUX[tableau], _lib.PRECISIONS[precision],
                               tol, tol, 1e-3, 1000000, 500, _lib.COSTS[cost], B,
                               p(y0), p(par), p(t0), p(t1), p(out["yT"]), p(out["dy0"]), p(out["dp"]),
                               p(out["n_acc"]), p(out["status"]), None)
    torch.cuda.synchronize()
    return st, {k: v.cpu().numpy() for k, v in out.items()}


@pytest.mark.parametrize("name,B,precision", [("vdpb", 2048, "fp64"), ("dho", 512, "mixed_dw")])
def test_noalloc_matches_va_gradient_twice(cuda, name, B, precision):
    L = _lib.load()
    w = W.make(name, batch=B)
    c = w["cfg"]
    y0, par, t0, t1 = dev(w["y0"]), dev(w["params"]), dev(w["t0"]), dev(w["t1"])
    s = Solver(c["model"], c["n"], c["npar"], B, tableau=c["tableau"], precision=precision,
               atol=c["tol"], rtol=c["tol"])
    ref = {k: v.cpu().numpy() for k, v in s.gradient(c["cost"], y0, par, t0, t1).items()}
    s.close()
    assert (ref["status"] == 0).all()
    for _ in range(2):
        st, r = call_noalloc(L, c["model"], c["tableau"], precision, c["tol"], c["cost"], B, y0, par, t0, t1)
        assert st == 0
        assert (r["status"] == 0).all()
        np.testing.assert_array_equal(r["n_acc"], ref["n_acc"])
        np.testing.assert_array_equal(r["yT"], ref["yT"])
        np.testing.assert_array_equal(r["dy0"], ref["dy0"])
        np.testing.assert_array_equal(r["dp"], ref["dp"])


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
