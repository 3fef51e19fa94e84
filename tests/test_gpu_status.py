"""Per-instance failure reporting on the GPU.  Faults are injected from the
host through inputs and options (NaN parameters, a tiny step cap, an
undersized checkpoint budget, a reject limit); every device loop is bounded,
so nothing can hang.  The failing instances carry their status and the others
are unaffected, bit for bit."""
import numpy as np
import pytest
import torch

from vectorizedadjoint_gb300 import Solver, VaError
from vectorizedadjoint_gb300 import workloads as W

pytestmark = pytest.mark.gpu

MAX_REJECTS, MAX_STEPS, NONFINITE, CKPT_BUDGET, NOT_READY = 1, 2, 3, 4, 7


def dev(a):
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def grads(s, w, params=None):
    p = w["params"] if params is None else params
    out = s.gradient("sumsq", dev(w["y0"]), dev(p), dev(w["t0"]), dev(w["t1"]))
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in out.items()}


@pytest.mark.parametrize("precision", ["fp64", "mixed_dw"])
def test_nan_parameter_isolated(cuda, precision):
    B = 256
    w = W.make("vdpb", batch=B)
    ref = grads(Solver("vdp", 2, 1, B, precision=precision), w)
    p = w["params"].copy()
    bad = [3, 77, 200]
    p[bad, 0] = np.nan
    r = grads(Solver("vdp", 2, 1, B, precision=precision), w, p)
    assert all(r["status"][b] == NONFINITE for b in bad)
    good = np.setdiff1d(np.arange(B), bad)
    assert (r["status"][good] == 0).all()
    np.testing.assert_array_equal(r["dp"][good], ref["dp"][good])
    assert np.isnan(r["dp"][bad]).all()


def test_max_steps(cuda):
    B = 64
    w = W.make("vdpb", batch=B)
    ref = grads(Solver("vdp", 2, 1, B), w)
    cap = int(np.median(ref["n_acc"]))
    r = grads(Solver("vdp", 2, 1, B, max_steps=cap), w)
    over = ref["n_acc"] > cap
    assert (r["status"][over] == MAX_STEPS).all()
    assert (r["status"][~over] == 0).all()
    np.testing.assert_array_equal(r["dp"][~over], ref["dp"][~over])


def test_failed_step_checker(cuda):
    """dt0 = 1 at tol 1e-12 needs several rejections on the first step:
    max_rejects = 2 trips odeint's failed_step_checker, 500 does not."""
    B = 8
    w = W.make("vdpb", batch=B)
    s = Solver("vdp", 2, 1, B, atol=1e-12, rtol=1e-12, dt0=1.0, max_rejects=2)
    f = s.forward(dev(w["y0"]), dev(w["params"]), dev(w["t0"]), dev(w["t1"]))
    torch.cuda.synchronize()
    assert (f["status"].cpu().numpy() == MAX_REJECTS).all()
    s2 = Solver("vdp", 2, 1, B, atol=1e-8, rtol=1e-8, dt0=1.0, max_rejects=500)
    f2 = s2.forward(dev(w["y0"]), dev(w["params"]), dev(w["t0"]), dev(w["t1"]))
    torch.cuda.synchronize()
    assert (f2["status"].cpu().numpy() == 0).all()
    assert (f2["n_rej"].cpu().numpy() > 2).all()


def test_checkpoint_budget_exhaustion(cuda):
    """A pool too small for the batch (every-step storage, ckpt_stride=1):
    instances that cannot store their steps report VA_CKPT_BUDGET and NaN
    gradients; any that completed are exact; a large enough pool is clean."""
    B = 512
    w = W.make("vdpb", batch=B)
    ref = grads(Solver("vdp", 2, 1, B), w)
    need = int(ref["n_acc"].sum() + B) * 32
    r = grads(Solver("vdp", 2, 1, B, ckpt_budget_bytes=need // 3, chunk_len=16, ckpt_stride=1), w)
    st = r["status"]
    assert (st == CKPT_BUDGET).any()
    assert set(np.unique(st)) <= {0, CKPT_BUDGET}
    ok = st == 0
    np.testing.assert_array_equal(r["dp"][ok], ref["dp"][ok])
    assert np.isnan(r["dp"][~ok]).all()
    r2 = grads(Solver("vdp", 2, 1, B, ckpt_budget_bytes=2 * need + (64 << 10), chunk_len=16, ckpt_stride=1), w)
    assert (r2["status"] == 0).all()
    np.testing.assert_array_equal(r2["dp"], ref["dp"])


def test_backward_before_forward(cuda):
    s = Solver("vdp", 2, 1, 4)
    p = torch.zeros(4, 1, dtype=torch.float64, device="cuda")
    lam = torch.zeros(4, 1, 2, dtype=torch.float64, device="cuda")
    with pytest.raises(VaError) as e:
        s.backward(p, lam)
    assert e.value.code == NOT_READY


def test_pool_allocation_failure_is_clean(cuda):
    """A checkpoint pool larger than the device (a 1 TiB budget against a
    worst case of several TB) fails to allocate: va_gradient returns
    VA_CUDA_ERROR with the allocation's message on every call (the half-built
    handle is released, never run), and a handle of ordinary size then runs."""
    from vectorizedadjoint_gb300 import _lib

    B = 65536
    w = W.make("vdpb", batch=B)
    s = Solver("vdp", 2, 1, B, ckpt_budget_bytes=1 << 40)
    for _ in range(2):
        with pytest.raises(_lib.VaError) as e:
            grads(s, w)
        assert "cudaMalloc" in str(e.value)
    s.close()
    r = grads(Solver("vdp", 2, 1, 64), W.make("vdpb", batch=64))
    assert (r["status"] == 0).all()
