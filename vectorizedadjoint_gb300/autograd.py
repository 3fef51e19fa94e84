"""torch.autograd over the forward / backward pair of the C ABI.

`odeint_adjoint(solver, y0, params, t0, t1)` returns y(T) [B, n] and, when
something downstream calls backward, runs va_backward with the incoming
cotangent dL/dy(T) as the seed lambda_T: the gradients with respect to y0
and params are the discrete adjoint of the accepted step sequence, step
sizes held fixed -- the derivative the reference's adjointSolve returns
(lib/include/backpropagation.hpp:18-43, seeds as setCostGradients,
lib/include/Driver.hpp:103-114).  The step-size controller's own dependence
on the inputs is not differentiated, as in the reference.

The solver's checkpoints belong to its last forward sweep, so one solver
serves one pending backward at a time: a second forward on the same solver
while the first one's graph is alive and its backward has not run raises.
A graph that is dropped without a backward (an exception, evaluation under
grad, a discarded output) releases the solver: the pending forward is
tracked through a weak reference to its autograd node.  The library does all
arithmetic; torch only carries the device buffers and the graph bookkeeping.
"""
import weakref

import torch

from .solver import Solver


class _OdeAdjoint(torch.autograd.Function):
    @staticmethod
    def forward(ctx, solver, y0, params, t0, t1):
        pending = getattr(solver, "_pending_node", None)
        if pending is not None and pending() is not None:
            raise RuntimeError("odeint_adjoint: this solver's checkpoints still wait for a backward pass; "
                               "use one solver per pending graph")
        y0c, pc = y0.detach().contiguous(), params.detach().contiguous()
        out = solver.forward(y0c, pc, t0.detach().contiguous(), t1.detach().contiguous())
        status = out["status"]
        solver._pending_node = weakref.ref(ctx)
        ctx.solver = solver
        ctx.save_for_backward(pc)
        ctx.mark_non_differentiable(status)
        return out["yT"], status

    @staticmethod
    def backward(ctx, g_yT, _g_status):
        solver = ctx.solver
        (params,) = ctx.saved_tensors
        B, n = solver.batch, solver.n
        if g_yT is None:
            g_yT = torch.zeros(B, n, dtype=torch.float64, device=params.device)
        lam = g_yT.detach().to(torch.float64).reshape(B, 1, n).contiguous()
        try:
            bw = solver.backward(params, lam)
        finally:
            solver._pending_node = None
        return None, bw["dy0"][:, 0], bw["dp"][:, 0], None, None


def odeint_adjoint(solver: Solver, y0, params, t0, t1):
    """y(T) of every instance of the batch, differentiable in y0 and params.

    solver : a Solver with nout = 1 (one seed row; the cotangent of y(T))
    y0 [B, n], params [B, npar], t0 [B], t1 [B]: FP64 CUDA tensors.
    Returns (yT [B, n], status [B] int32); instances whose status is not 0
    have no trajectory, and their gradients come back as NaN.
    """
    if solver.nout != 1:
        raise ValueError("odeint_adjoint needs a Solver with nout = 1")
    return _OdeAdjoint.apply(solver, y0, params, t0, t1)
