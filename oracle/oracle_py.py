"""ctypes binding of the CPU oracle (test infrastructure only).

The oracle restates the reference's forward loop
(lib/include/detail/runge_kutta.hpp:137-180), the Boost.odeint 1.74.0
controller it calls, and the discrete adjoint
(lib/include/detail/backpropagation.hpp:24-348) in plain C; see oracle.h.
Only the test-suite, the smoke check and the bench's CPU-baseline leg use it,
as the checker.  The product library never imports this module.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "_build", "liboracle.so")

MODEL = {"vdp": 0, "vdp_petsc": 1, "dho": 2, "glv": 3, "decay": 4, "user": 6}
TABLEAU = {"dopri5": 0, "ck54": 1, "rkf78": 2, "rk4": 3, "euler": 4}
COST = {"sumsq": 0, "sum": 1}
STATUS = {0: "OK", 1: "MAX_REJECTS", 2: "MAX_STEPS", 3: "NONFINITE", 5: "BAD_ARGS"}


class Problem(ctypes.Structure):
    _fields_ = [
        ("model", ctypes.c_int),
        ("tableau", ctypes.c_int),
        ("n", ctypes.c_int),
        ("npar", ctypes.c_int),
        ("atol", ctypes.c_double),
        ("rtol", ctypes.c_double),
        ("dt0", ctypes.c_double),
        ("max_steps", ctypes.c_long),
        ("max_fail", ctypes.c_int),
        ("pow_mode", ctypes.c_int),
        ("user_rhs", ctypes.c_void_p),
        ("user_vjp", ctypes.c_void_p),
    ]


def build():
    """Compile the oracle with its Makefile (portable C99)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


class PowTrace(ctypes.Structure):
    _fields_ = [("calls", ctypes.c_long), ("noncr", ctypes.c_long), ("first_noncr_step", ctypes.c_long),
                ("step", ctypes.c_long), ("first_noncr_arg", ctypes.c_double)]


class Traffic(ctypes.Structure):
    _fields_ = [("store_bytes", ctypes.c_longlong), ("load_bytes", ctypes.c_longlong)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_SO):
            build()
        L = ctypes.CDLL(_SO)
        P = ctypes.POINTER(Problem)
        dp = ctypes.POINTER(ctypes.c_double)
        lp = ctypes.POINTER(ctypes.c_long)
        ip = ctypes.POINTER(ctypes.c_int)
        L.orc_forward.argtypes = [P, dp, dp, ctypes.c_double, ctypes.c_double, ctypes.c_long,
                                  dp, dp, dp, dp, lp, lp]
        L.orc_forward.restype = ctypes.c_int
        L.orc_forward_frozen.argtypes = [P, dp, dp, ctypes.c_long, dp, dp]
        L.orc_forward_frozen.restype = None
        L.orc_adjoint.argtypes = [P, dp, ctypes.c_long, dp, dp, ctypes.c_int, dp, dp]
        L.orc_adjoint.restype = ctypes.c_int
        L.orc_adjoint_history.argtypes = [P, dp, ctypes.c_long, dp, dp, ctypes.c_int, dp, dp, dp]
        L.orc_adjoint_history.restype = ctypes.c_int
        L.orc_gradient.argtypes = [P, ctypes.c_int, dp, dp, ctypes.c_double, ctypes.c_double,
                                   dp, dp, dp, lp, lp]
        L.orc_gradient.restype = ctypes.c_int
        L.orc_gradient_batch.argtypes = [P, ctypes.c_int, ctypes.c_long, dp, dp, dp, dp,
                                         ctypes.c_int, dp, dp, dp, lp, lp, ip]
        L.orc_gradient_batch.restype = ctypes.c_int
        L.orc_gradient_traffic.argtypes = [P, ctypes.c_int, dp, dp, ctypes.c_double, ctypes.c_double, lp,
                                           ctypes.POINTER(Traffic)]
        L.orc_gradient_traffic.restype = ctypes.c_int
        L.orc_set_powtrace.argtypes = [ctypes.POINTER(PowTrace)]
        L.orc_set_powtrace.restype = None
        L.orc_step_pow.argtypes = [ctypes.c_double, ctypes.c_int, ctypes.c_int]
        L.orc_step_pow.restype = ctypes.c_double
        L.orc_rhs.argtypes = [P, dp, dp, ctypes.c_double, dp]
        L.orc_vjp.argtypes = [P, dp, dp, dp, ctypes.c_double, dp, dp]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def problem(model, tableau, n, npar, atol, rtol, dt0=1e-3, max_steps=200000, max_fail=500, pow_mode=2):
    """Step-factor power pow(err, -1.0/k): pow_mode 2 (default) the correctly
    rounded value, what the CUDA library's FP64 controller computes by
    default (step_pow = 1); 1: the C library's pow, as odeint calls it; 0: the
    Newton root of the library's fast controller (step_pow = 0)."""
    return Problem(MODEL[model], TABLEAU[tableau], n, npar, atol, rtol, dt0, max_steps, max_fail, pow_mode)


def user_problem(rhs, vjp, tableau, n, npar, atol, rtol, dt0=1e-3, max_steps=200000, max_fail=500, pow_mode=2):
    """A problem whose right-hand side and VJP are C callbacks (function
    pointers, e.g. ctypes.cast(lib.f, ctypes.c_void_p).value) with the
    signatures of orc_problem.user_rhs / user_vjp."""
    return Problem(MODEL["user"], TABLEAU[tableau], n, npar, atol, rtol, dt0, max_steps, max_fail, pow_mode,
                   rhs, vjp)


def step_pow(a, k, pow_mode):
    """The oracle's step factor pow(a, -1.0/k) in the given mode."""
    return lib().orc_step_pow(float(a), int(k), int(pow_mode))


def forward(pb, y0, p, t0, t1, cap=None, powtrace=False):
    """Returns dict(status, times[T+1], states[T+1,n], dt_trial[T], yT, n_acc, n_rej).
    powtrace (pow_mode 1): also pow_calls, pow_noncr (libm results that are not
    correctly rounded) and first_noncr_step (accepted-step index of the first
    such call, -1 if none)."""
    cap = cap or pb.max_steps
    n = pb.n
    times = np.zeros(cap + 1)
    states = np.zeros((cap + 1, n))
    dtt = np.zeros(cap + 1)
    yT = np.zeros(n)
    na, nr = ctypes.c_long(0), ctypes.c_long(0)
    y0 = np.ascontiguousarray(y0, dtype=np.float64)
    p = np.ascontiguousarray(p, dtype=np.float64)
    tr = PowTrace()
    if powtrace:
        lib().orc_set_powtrace(ctypes.byref(tr))
    try:
        st = lib().orc_forward(ctypes.byref(pb), _d(y0), _d(p), t0, t1, cap, _d(times), _d(states),
                               _d(dtt), _d(yT), ctypes.byref(na), ctypes.byref(nr))
    finally:
        if powtrace:
            lib().orc_set_powtrace(None)
    T = na.value
    out = dict(status=st, times=times[:T + 1].copy(), states=states[:T + 1].copy(),
               dt_trial=dtt[:T].copy(), yT=yT, n_acc=T, n_rej=nr.value)
    if powtrace:
        out.update(pow_calls=tr.calls, pow_noncr=tr.noncr, first_noncr_step=tr.first_noncr_step,
                   first_noncr_arg=tr.first_noncr_arg)
    return out


def forward_frozen(pb, y0, p, times):
    yT = np.zeros(pb.n)
    times = np.ascontiguousarray(times, dtype=np.float64)
    y0 = np.ascontiguousarray(y0, dtype=np.float64)
    p = np.ascontiguousarray(p, dtype=np.float64)
    lib().orc_forward_frozen(ctypes.byref(pb), _d(y0), _d(p), len(times) - 1, _d(times), _d(yT))
    return yT


def adjoint(pb, p, times, states, lam, mu):
    """lam[nout, n] seeds dG/dy(T); mu[nout, npar] direct partials.  Returns (dy0, dp, status)."""
    lam = np.array(lam, dtype=np.float64, order="C", ndmin=2).copy()
    mu = np.array(mu, dtype=np.float64, order="C", ndmin=2).copy()
    times = np.ascontiguousarray(times, dtype=np.float64)
    states = np.ascontiguousarray(states, dtype=np.float64)
    p = np.ascontiguousarray(p, dtype=np.float64)
    st = lib().orc_adjoint(ctypes.byref(pb), _d(p), len(times) - 1, _d(times), _d(states),
                           lam.shape[0], _d(lam), _d(mu))
    return lam, mu, st


def adjoint_history(pb, p, times, states, lam, mu):
    """adjoint() plus lambda_n of every seed: returns (dy0, dp, hist[nout, T+1, n], status)."""
    lam = np.array(lam, dtype=np.float64, order="C", ndmin=2).copy()
    mu = np.array(mu, dtype=np.float64, order="C", ndmin=2).copy()
    times = np.ascontiguousarray(times, dtype=np.float64)
    states = np.ascontiguousarray(states, dtype=np.float64)
    p = np.ascontiguousarray(p, dtype=np.float64)
    hist = np.zeros((lam.shape[0], len(times), pb.n))
    st = lib().orc_adjoint_history(ctypes.byref(pb), _d(p), len(times) - 1, _d(times), _d(states),
                                   lam.shape[0], _d(lam), _d(mu), _d(hist))
    return lam, mu, hist, st


def gradient(pb, cost, y0, p, t0, t1):
    n, npar = pb.n, pb.npar
    yT, dy0, dp = np.zeros(n), np.zeros(n), np.zeros(npar)
    na, nr = ctypes.c_long(0), ctypes.c_long(0)
    y0 = np.ascontiguousarray(y0, dtype=np.float64)
    p = np.ascontiguousarray(p, dtype=np.float64)
    st = lib().orc_gradient(ctypes.byref(pb), COST[cost], _d(y0), _d(p), t0, t1, _d(yT), _d(dy0),
                            _d(dp), ctypes.byref(na), ctypes.byref(nr))
    return dict(status=st, yT=yT, dy0=dy0, dp=dp, n_acc=na.value, n_rej=nr.value)


def gradient_traffic(pb, cost, y0, p, t0, t1):
    """Checkpoint bytes one gradient stores (forward) and reads back (adjoint)."""
    na, tr = ctypes.c_long(0), Traffic()
    y0 = np.ascontiguousarray(y0, dtype=np.float64)
    p = np.ascontiguousarray(p, dtype=np.float64)
    st = lib().orc_gradient_traffic(ctypes.byref(pb), COST[cost], _d(y0), _d(p), t0, t1, ctypes.byref(na),
                                    ctypes.byref(tr))
    return dict(status=st, n_acc=na.value, store_bytes=tr.store_bytes, load_bytes=tr.load_bytes)


def gradient_batch(pb, cost, y0, p, t0, t1, nthreads=1):
    B = y0.shape[0]
    n, npar = pb.n, pb.npar
    yT, dy0, dp = np.zeros((B, n)), np.zeros((B, n)), np.zeros((B, npar))
    na, nr = np.zeros(B, dtype=np.int64), np.zeros(B, dtype=np.int64)
    status = np.zeros(B, dtype=np.int32)
    y0 = np.ascontiguousarray(y0, dtype=np.float64)
    p = np.ascontiguousarray(p, dtype=np.float64)
    t0 = np.ascontiguousarray(t0, dtype=np.float64)
    t1 = np.ascontiguousarray(t1, dtype=np.float64)
    lib().orc_gradient_batch(ctypes.byref(pb), COST[cost], B, _d(y0), _d(p), _d(t0), _d(t1),
                             nthreads, _d(yT), _d(dy0), _d(dp),
                             na.ctypes.data_as(ctypes.POINTER(ctypes.c_long)),
                             nr.ctypes.data_as(ctypes.POINTER(ctypes.c_long)),
                             status.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
    return dict(status=status, yT=yT, dy0=dy0, dp=dp, n_acc=na, n_rej=nr)
