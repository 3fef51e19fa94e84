"""torch.autograd over va_forward / va_backward (vectorizedadjoint_gb300.autograd):
the gradients autograd delivers are the library's discrete adjoint, seeded
with the cotangent of y(T) exactly as setCostGradients seeds the reference."""
import numpy as np
import pytest
import torch

from vectorizedadjoint_gb300 import Solver, odeint_adjoint
from vectorizedadjoint_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def dev(a, grad=False):
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda", requires_grad=grad)


def solver_for(w, B, precision="fp64"):
    c = w["cfg"]
    return Solver(c["model"], c["n"], c["npar"], B, tableau=c["tableau"], precision=precision,
                  atol=c["tol"], rtol=c["tol"])


@pytest.mark.parametrize("name,B", [("vdpb", 256), ("dho", 128), ("glv10", 32)])
def test_autograd_equals_gradient_entry(cuda, name, B):
    """loss = sum y(T)^2 through autograd gives va_gradient's bits (FP64)."""
    w = W.make(name, batch=B)
    y0, p = dev(w["y0"], True), dev(w["params"], True)
    s = solver_for(w, B)
    yT, status = odeint_adjoint(s, y0, p, dev(w["t0"]), dev(w["t1"]))
    (yT ** 2).sum().backward()
    torch.cuda.synchronize()
    assert (status.cpu().numpy() == 0).all()
    s2 = solver_for(w, B)
    ref = s2.gradient("sumsq", dev(w["y0"]), dev(w["params"]), dev(w["t0"]), dev(w["t1"]))
    torch.cuda.synchronize()
    np.testing.assert_array_equal(yT.detach().cpu().numpy(), ref["yT"].cpu().numpy())
    np.testing.assert_array_equal(y0.grad.cpu().numpy(), ref["dy0"].cpu().numpy())
    np.testing.assert_array_equal(p.grad.cpu().numpy(), ref["dp"].cpu().numpy())
    s.close()
    s2.close()


def test_autograd_general_cotangent_vs_oracle(oracle, cuda):
    """An arbitrary downstream loss: the cotangent reaches the adjoint as its
    seed; the result equals the oracle's adjoint of the same trajectory."""
    B = 16
    w = W.make("vdpb", batch=B)
    c = w["cfg"]
    y0, p = dev(w["y0"], True), dev(w["params"], True)
    s = solver_for(w, B)
    yT, _ = odeint_adjoint(s, y0, p, dev(w["t0"]), dev(w["t1"]))
    wgt = torch.tensor(np.random.default_rng(7).normal(size=(B, 2)), device="cuda")
    (torch.sin(yT) * wgt).sum().backward()
    torch.cuda.synchronize()
    seed = (torch.cos(yT) * wgt).detach().cpu().numpy()
    pb = oracle.problem(c["model"], c["tableau"], c["n"], c["npar"], c["tol"], c["tol"])
    for b in range(B):
        fw = oracle.forward(pb, w["y0"][b], w["params"][b], 0.0, w["t1"][b])
        dy0, dp, st = oracle.adjoint(pb, w["params"][b], fw["times"], fw["states"], seed[b][None], np.zeros((1, 1)))
        assert st == 0
        np.testing.assert_allclose(y0.grad[b].cpu().numpy(), dy0[0], rtol=1e-12, atol=1e-14)
        np.testing.assert_allclose(p.grad[b].cpu().numpy(), dp[0], rtol=1e-12, atol=1e-14)
    s.close()


def test_autograd_mixed_dw_within_target(cuda):
    """The double-word path through autograd: within 1e-6 of the FP64 path."""
    B = 512
    w = W.make("vdpb", batch=B)
    grads = []
    for prec in ("fp64", "mixed_dw"):
        y0, p = dev(w["y0"], True), dev(w["params"], True)
        s = solver_for(w, B, prec)
        yT, _ = odeint_adjoint(s, y0, p, dev(w["t0"]), dev(w["t1"]))
        yT.sum().backward()
        torch.cuda.synchronize()
        grads.append(torch.cat([y0.grad, p.grad], 1).cpu().numpy())
        s.close()
    scale = np.maximum(np.abs(grads[0]).max(1, keepdims=True), 1e-8)
    assert (np.abs(grads[1] - grads[0]) / scale).max() < 1e-6


def test_one_pending_backward_per_solver(cuda):
    B = 8
    w = W.make("vdpb", batch=B)
    s = solver_for(w, B)
    args = (dev(w["y0"], True), dev(w["params"], True), dev(w["t0"]), dev(w["t1"]))
    yT, _ = odeint_adjoint(s, *args)
    with pytest.raises(RuntimeError):
        odeint_adjoint(s, *args)
    yT.sum().backward()
    yT2, _ = odeint_adjoint(s, *args)  # free again after the backward
    yT2.sum().backward()
    s.close()


def test_dropped_graph_releases_solver(cuda):
    """A forward whose graph is discarded without a backward (here: the
    outputs deleted) does not block the solver's next forward."""
    import gc
    B = 8
    w = W.make("vdpb", batch=B)
    s = solver_for(w, B)
    args = (dev(w["y0"], True), dev(w["params"], True), dev(w["t0"]), dev(w["t1"]))
    yT, st = odeint_adjoint(s, *args)
    del yT, st
    gc.collect()
    yT2, _ = odeint_adjoint(s, *args)
    yT2.sum().backward()
    with torch.no_grad():
        odeint_adjoint(s, *args)  # no graph: nothing stays pending
    odeint_adjoint(s, *args)[0].sum().backward()
    s.close()
