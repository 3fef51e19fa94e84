"""Batched solver over the C ABI (include/va.h).

`Solver` wraps one va_handle: a batch of B instances of one built-in model.
Inputs and outputs are CUDA tensors (torch provides device memory and
streams only; all arithmetic runs in the library's CUDA kernels).  The
forward/backward pair maps one-to-one onto va_forward / va_backward, so a
torch.autograd.Function can wrap it.
"""
import ctypes

import torch

from . import _lib


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class Solver:
    """One batch of B independent instances of a built-in model.

    model     : 'vdp' | 'vdp_petsc' | 'dho' | 'glv' | 'decay' | 'glv_shared', or 'user'
                with model_kernels = the address returned by a VA_DEFINE_MODEL
                accessor (a device model compiled outside the library)
    n, npar   : state and per-instance parameter counts
    batch     : B
    nout      : cost functions (seed rows) per instance
    tableau   : 'dopri5' | 'ck54'
    precision : 'fp64' | 'mixed' (FP32 stages) | 'mixed_dw' (double-word FP32-pair stages)
    stage_records : mixed_dw, every step checkpointed: 1 stores each step's stage
                values for the backward sweep, 0 recomputes them (va_options)
    step_pow  : FP64 controller: 1 (default) the correctly rounded step factor
                (odeint's std::pow), 0 the Newton root (va_options)
    tensor_products : shared-matrix GLV N = 256, mixed_dw: 0 (default) the
                backward's stage products on the tensor cores, -1 on the FP32
                pipe (va_options)
    """

    def __init__(self, model, n, npar, batch, nout=1, tableau="dopri5", precision="fp64",
                 atol=1e-6, rtol=1e-6, dt0=1e-3, max_steps=1000000, max_rejects=500,
                 ckpt_budget_bytes=0, ckpt_stride=0, block_size=0, blocks_per_sm=0, chunk_len=0,
                 stage_records=1, step_pow=1, model_kernels=None, tensor_products=0):
        self.L = _lib.load()
        if not torch.cuda.is_available():
            raise RuntimeError("vectorizedadjoint_gb300 needs a CUDA device (no CPU fallback)")
        self.model, self.n, self.npar, self.batch, self.nout = model, n, npar, batch, nout
        self.tableau, self.precision = tableau, precision
        prob = _lib.VaProblem(_lib.MODELS[model], n, npar, batch, nout)
        opt = _lib.VaOptions()
        self.L.va_default_options(ctypes.byref(opt))
        opt.tableau = _lib.TABLEAUX[tableau]
        opt.precision = _lib.PRECISIONS[precision]
        opt.atol, opt.rtol, opt.dt0 = atol, rtol, dt0
        opt.max_steps, opt.max_rejects = max_steps, max_rejects
        opt.ckpt_budget_bytes, opt.ckpt_stride = ckpt_budget_bytes, ckpt_stride
        opt.block_size, opt.blocks_per_sm, opt.chunk_len = block_size, blocks_per_sm, chunk_len
        opt.stage_records = stage_records
        opt.step_pow = step_pow
        opt.tensor_products = tensor_products
        torch.cuda.init()
        self.h = ctypes.c_void_p()
        if model_kernels is not None:
            st = self.L.va_create_model(ctypes.byref(prob), ctypes.byref(opt), ctypes.c_void_p(model_kernels),
                                        ctypes.byref(self.h))
        else:
            st = self.L.va_create(ctypes.byref(prob), ctypes.byref(opt), ctypes.byref(self.h))
        if st != _lib.VA_OK:
            raise _lib.VaError(st, f"va_create({model}, n={n}, npar={npar}, B={batch})")

    def pow_undecided(self):
        """Step factors of the last forward sweep whose correctly rounded value
        was not decided (va_step_pow_undecided; 0 expected)."""
        c = ctypes.c_int64()
        self._check(self.L.va_step_pow_undecided(self.h, ctypes.byref(c)), "va_step_pow_undecided")
        return c.value

    def _check(self, st, what):
        if st != _lib.VA_OK:
            raise _lib.VaError(st, f"{what}: {self.L.va_last_error(self.h).decode()}")

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self.L.va_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- device-tensor entry points -------------------------------------------------
    def _alloc(self, *shape, dtype=torch.float64):
        return torch.empty(*shape, dtype=dtype, device="cuda")

    def forward(self, y0, params, t0, t1):
        """va_forward.  Returns dict(yT, n_acc, n_rej, status) of CUDA tensors."""
        B, n = self.batch, self.n
        yT = self._alloc(B, n)
        n_acc = self._alloc(B, dtype=torch.int32)
        n_rej = self._alloc(B, dtype=torch.int32)
        status = self._alloc(B, dtype=torch.int32)
        self._inputs = (y0, params, t0, t1)
        self._check(self.L.va_forward(self.h, _ptr(y0), _ptr(params), _ptr(t0), _ptr(t1), _ptr(yT),
                                      _ptr(n_acc), _ptr(n_rej), _ptr(status), _stream()), "va_forward")
        return dict(yT=yT, n_acc=n_acc, n_rej=n_rej, status=status)

    def backward(self, params, lambdaT, mu_direct=None):
        """va_backward.  lambdaT [B, nout, n], mu_direct [B, nout, npar] or None."""
        B, n, P, Q = self.batch, self.n, self.npar, self.nout
        dy0 = self._alloc(B, Q, n)
        dp = self._alloc(B, Q, P)
        status = self._alloc(B, dtype=torch.int32)
        self._check(self.L.va_backward(self.h, _ptr(params), _ptr(lambdaT), _ptr(mu_direct), _ptr(dy0),
                                       _ptr(dp), _ptr(status), _stream()), "va_backward")
        return dict(dy0=dy0, dp=dp, status=status)

    def gradient(self, cost, y0, params, t0, t1, out=None):
        """va_gradient (forward + backward, graph-captured).  cost 'sumsq' | 'sum'."""
        B, n, P = self.batch, self.n, self.npar
        if out is None:
            out = dict(yT=self._alloc(B, n), dy0=self._alloc(B, n), dp=self._alloc(B, P),
                       n_acc=self._alloc(B, dtype=torch.int32), status=self._alloc(B, dtype=torch.int32))
        self._check(self.L.va_gradient(self.h, _lib.COSTS[cost], _ptr(y0), _ptr(params), _ptr(t0), _ptr(t1),
                                       _ptr(out["yT"]), _ptr(out["dy0"]), _ptr(out["dp"]), _ptr(out["n_acc"]),
                                       _ptr(out["status"]), _stream()), "va_gradient")
        return out

    def gradient_host(self, cost, y0, params, t0, t1, out=None):
        """va_gradient_host: host (numpy / CPU tensor) buffers in and out."""
        import numpy as np
        B, n, P = self.batch, self.n, self.npar

        def hp(a):
            return ctypes.c_void_p(a.ctypes.data) if isinstance(a, np.ndarray) else ctypes.c_void_p(a.data_ptr())
        if out is None:
            out = dict(yT=np.empty((B, n)), dy0=np.empty((B, n)), dp=np.empty((B, P)),
                       n_acc=np.empty(B, np.int32), status=np.empty(B, np.int32))
        self._check(self.L.va_gradient_host(self.h, _lib.COSTS[cost], hp(y0), hp(params), hp(t0), hp(t1),
                                            hp(out["yT"]), hp(out["dy0"]), hp(out["dp"]), hp(out["n_acc"]),
                                            hp(out["status"]), _stream()), "va_gradient_host")
        return out

    def set_shared(self, A, dA=None):
        """va_set_shared (shared-matrix GLV): A [n, n] CUDA tensor read by every
        later sweep; dA [n, n] receives the gradient of the batch's summed cost."""
        self._shared = (A, dA)
        self._check(self.L.va_set_shared(self.h, _ptr(A), _ptr(dA)), "va_set_shared")

    def autotune(self, cost, y0, params, t0, t1):
        self._check(self.L.va_autotune(self.h, _lib.COSTS[cost], _ptr(y0), _ptr(params), _ptr(t0), _ptr(t1),
                                       _stream()), "va_autotune")
        return self.launch()

    def launch(self):
        v = [ctypes.c_int32() for _ in range(4)]
        self.L.va_get_launch(self.h, *[ctypes.byref(x) for x in v])
        return dict(fwd_block=v[0].value, fwd_grid=v[1].value, bwd_block=v[2].value, bwd_grid=v[3].value)

    def trajectory(self, instance, capacity=None):
        """Accepted-step record of one instance: (t[T+1], dt[T+1], y[T+1, n]) as numpy arrays."""
        import numpy as np
        nrec = ctypes.c_int32()
        self.L.va_trajectory(self.h, instance, 0, None, None, None, ctypes.byref(nrec))
        cap = nrec.value if capacity is None else capacity
        t, dt, y = np.zeros(cap), np.zeros(cap), np.zeros((cap, self.n))
        self._check(self.L.va_trajectory(self.h, instance, cap, ctypes.c_void_p(t.ctypes.data),
                                         ctypes.c_void_p(dt.ctypes.data), ctypes.c_void_p(y.ctypes.data),
                                         ctypes.byref(nrec)), "va_trajectory")
        return t[:nrec.value], dt[:nrec.value], y[:nrec.value]

    def forward_frozen(self, times, y0, params, shared=None):
        """va_forward_frozen: FP64 replay of recorded accepted-step sequences.
        times: list of 1-D arrays (t_0 .. t_T per lane); y0 [L, n], params
        [L, npar] CUDA tensors; shared: an [n, n] CUDA tensor (shared-matrix
        GLV) or None.  Returns y(T) [L, n]."""
        import numpy as np
        L = len(times)
        stride = max(len(t) for t in times)
        tt = np.zeros((L, stride))
        for k, t in enumerate(times):
            tt[k, :len(t)] = t
        dtimes = torch.tensor(tt, dtype=torch.float64, device="cuda")
        steps = torch.tensor([len(t) - 1 for t in times], dtype=torch.int32, device="cuda")
        yT = self._alloc(L, self.n)
        self._check(self.L.va_forward_frozen(self.h, L, stride, _ptr(dtimes), _ptr(steps), _ptr(y0), _ptr(params),
                                             _ptr(shared), _ptr(yT), _stream()), "va_forward_frozen")
        return yT

    def set_adjoint_history(self, capacity):
        """Keep lambda_n (every seed, record indices n < capacity) in later
        backward sweeps -- the reference's back_prop observer; 0 turns it off."""
        self._check(self.L.va_set_adjoint_history(self.h, capacity), "va_set_adjoint_history")
        self._hist_cap = capacity

    def adjoint_history(self, instance, capacity=None, times=True):
        """(t[k], lambda[nout, k, n]) for k = 0..T of one instance (t is None
        when times=False, e.g. with a checkpoint stride > 1)."""
        import numpy as np
        nrec = ctypes.c_int32()
        self._check(self.L.va_adjoint_history(self.h, instance, 0, None, None, ctypes.byref(nrec)),
                    "va_adjoint_history")
        cap = nrec.value if capacity is None else capacity
        t = np.zeros(cap) if times else None
        lam = np.zeros((self.nout, cap, self.n))
        self._check(self.L.va_adjoint_history(self.h, instance, cap,
                                              ctypes.c_void_p(t.ctypes.data) if times else None,
                                              ctypes.c_void_p(lam.ctypes.data), ctypes.byref(nrec)),
                    "va_adjoint_history")
        k = min(cap, nrec.value, getattr(self, "_hist_cap", 0))
        return (t[:k] if times else None), lam[:, :k]

    def checkpoint_info(self):
        cap, used, stride = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int32()
        self.L.va_checkpoint_info(self.h, ctypes.byref(cap), ctypes.byref(used), ctypes.byref(stride))
        return dict(capacity_bytes=cap.value, used_bytes=used.value, stride=stride.value)
