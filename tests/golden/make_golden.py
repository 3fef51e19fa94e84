"""Generates tests/golden/reference_cases.npz from the REFERENCE ITSELF:
its unchanged lib/include headers compiled against the project's Boost
stand-in and linked with the AADC runtime it ships (oracle/ref/, built into
oracle/_ref/libvaref.so by `make -C oracle/ref`).  Needs the reference
sources (directory from $VA_REFERENCE_DIR, default /root/reference) and an
x86-64 host (AADC is x86-only); the fixtures it writes are committed so the
tests run anywhere.

Every case stores the reference's accepted-step record (times, states) when
it has at most 5000 steps, and the trace of the C library's pow over the
same forward sweep, taken with the oracle in its libm mode (which lands on
the reference's steps bit for bit, so it makes the same pow calls): the
number of calls and of calls whose result was not the correctly rounded
power on the machine that generated the fixtures.

Cases: seeded instances of every benchmark configuration (same draws as
vectorizedadjoint_gb300.workloads), and the reference's own GLV example
(examples/GeneralizedLotkaVolterra/main.cpp: Cash-Karp, x0 = 0.1, t in
[0, 10], dt = 1e-3, identity seeds Nout = N) on its data files
data/N5/alphasfile_cpp.csv and data/N10/alphasfile_cpp.csv.

A second file, history_cases.npz, holds adjoint histories: the values the
reference's back_prop observer is shown (lambda_n after every back step)
for three instances.

Usage:  make -C oracle/ref && python tests/golden/make_golden.py
"""
import ctypes
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
REF = os.environ.get("VA_REFERENCE_DIR", "/root/reference")

from oracle import oracle_py as O  # noqa: E402
from vectorizedadjoint_gb300 import workloads as W  # noqa: E402

MAX_STORED_STEPS = 5000


def pow_trace(model, tableau, n, npar, tol, y0, p, t1, dt, first=False):
    """libm pow calls of the forward sweep and how many were not correctly
    rounded (with first=True also the accepted-step index of the first)."""
    pb = O.problem(model, tableau, n, npar, tol, tol, dt0=dt, pow_mode=1)
    fw = O.forward(pb, y0, p, 0.0, t1, powtrace=True)
    if first:
        return fw["pow_calls"], fw["pow_noncr"], fw["first_noncr_step"]
    return fw["pow_calls"], fw["pow_noncr"]


def differs_with_cr_pow(model, tableau, n, npar, tol, y0, p, t1, dt):
    """Whether the correctly rounded step factor changes the accepted steps."""
    f1 = O.forward(O.problem(model, tableau, n, npar, tol, tol, dt0=dt, pow_mode=1), y0, p, 0.0, t1)
    f2 = O.forward(O.problem(model, tableau, n, npar, tol, tol, dt0=dt, pow_mode=2), y0, p, 0.0, t1)
    return not (f1["n_acc"] == f2["n_acc"] and np.array_equal(f1["states"], f2["states"])
                and np.array_equal(f1["times"], f2["times"]))

MODEL_ID = {"vdp": 0, "vdp_petsc": 1, "dho": 2, "glv": 3, "duffing": 10, "brusselator": 11}
TABLEAU_ID = {"dopri5": 0, "ck54": 1, "rkf78": 2, "rk4": 3, "euler": 4}


def load():
    L = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libvaref.so"))
    L.ref_solve.restype = ctypes.c_int
    L.ref_history.restype = ctypes.c_int
    return L


def solve(L, model, tableau, n, npar, tol, y0, p, t1, lam, mu, cap=200000, dt=1e-3):
    nout = lam.shape[0]
    times = np.zeros(cap + 1)
    states = np.zeros((cap + 1, n))
    T = ctypes.c_long()
    yT = np.zeros(n)
    lo = np.zeros((nout, n))
    mo = np.zeros((nout, npar))
    ptr = lambda a: np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(ctypes.c_void_p)
    keep = [np.ascontiguousarray(a, dtype=np.float64) for a in (y0, p, lam, mu)]
    rc = L.ref_solve(MODEL_ID[model], TABLEAU_ID[tableau], n, nout, npar, ctypes.c_double(tol),
                     ctypes.c_double(tol), ctypes.c_double(dt), ptr(keep[0]), ptr(keep[1]),
                     ctypes.c_double(0.0), ctypes.c_double(t1), ptr(keep[2]), ptr(keep[3]), ctypes.c_long(cap),
                     times.ctypes.data_as(ctypes.c_void_p), states.ctypes.data_as(ctypes.c_void_p),
                     ctypes.byref(T), yT.ctypes.data_as(ctypes.c_void_p), lo.ctypes.data_as(ctypes.c_void_p),
                     mo.ctypes.data_as(ctypes.c_void_p))
    assert rc == 0, rc
    return T.value, times[:T.value + 1], states[:T.value + 1], yT, lo, mo


def history(L, model, tableau, n, npar, tol, y0, p, t1, lam, dt=1e-3, cap=200000):
    """The reference's back_prop observer record: (times[T+1], hist[nout][T+1][n])."""
    nout = lam.shape[0]
    times = np.zeros(cap)
    hist = np.zeros(nout * cap * n)
    T = ctypes.c_long()
    keep = [np.ascontiguousarray(a, dtype=np.float64) for a in (y0, p, lam)]
    ptr = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    rc = L.ref_history(MODEL_ID[model], TABLEAU_ID[tableau], n, nout, npar, ctypes.c_double(tol),
                       ctypes.c_double(tol), ctypes.c_double(dt), ptr(keep[0]), ptr(keep[1]), ctypes.c_double(0.0),
                       ctypes.c_double(t1), ptr(keep[2]), ctypes.c_long(cap), ptr(times), ptr(hist), ctypes.byref(T))
    assert rc == 0, rc
    k = T.value + 1
    return times[:k], hist[:nout * k * n].reshape(nout, k, n)


def main_history(L):
    """Adjoint histories (lambda_n after every back step, the values the
    reference's back_prop observer sees) -> tests/golden/history_cases.npz."""
    out = {}
    specs = [("vdp1", None, 1e-3, "eye"), ("vdpb", "rk4", 1e-2, "cost"), ("glv10", "ck54", 1e-3, "rand3")]
    for k, (name, tableau, dt, seeds) in enumerate(specs):
        w = W.make(name, batch=1)
        c = w["cfg"]
        tab = tableau or c["tableau"]
        y0, p, t1 = w["y0"][0], w["params"][0], float(w["t1"][0])
        n = c["n"]
        if seeds == "eye":
            lam = np.eye(n)
        elif seeds == "cost":
            _, _, _, yT, _, _ = solve(L, c["model"], tab, n, c["npar"], c["tol"], y0, p, t1, np.zeros((1, n)),
                                      np.zeros((1, c["npar"])), dt=dt)
            lam = 2.0 * yT[None, :]
        else:
            lam = np.random.Generator(np.random.PCG64(11)).standard_normal((3, n))
        times, hist = history(L, c["model"], tab, n, c["npar"], c["tol"], y0, p, t1, lam, dt=dt)
        case = dict(name=f"{name}_{tab}", model=c["model"], tableau=tab, n=n, npar=c["npar"], tol=c["tol"], dt=dt,
                    y0=y0, p=p, t1=t1, lam=lam, times=times, hist=hist)
        for key, v in case.items():
            out[f"c{k}_{key}"] = np.asarray(v)
    out["count"] = np.array(len(specs))
    path = os.path.join(ROOT, "tests", "golden", "history_cases.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {len(specs)} history cases to {path} ({os.path.getsize(path)} bytes)")


def user_model_draws(name, count, seed):
    """Seeded instances of the test suite's own device models
    (tests/cpp/user_models.cuh): (y0[count, 2], p[count, P], T)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    if name == "duffing":
        p = np.stack([rng.uniform(0.1, 0.5, count), rng.uniform(0.5, 2.0, count), rng.uniform(0.0, 1.0, count),
                      rng.uniform(0.5, 2.0, count), rng.uniform(0.5, 2.0, count)], axis=1)
        return rng.uniform(-1.0, 1.0, (count, 2)), p, 10.0
    p = np.stack([rng.uniform(0.8, 1.5, count), rng.uniform(1.5, 3.5, count)], axis=1)
    return rng.uniform(0.5, 2.0, (count, 2)), p, 20.0


def user_model_callbacks():
    """Host build of tests/cpp/user_models.cuh for the oracle (g++, no contraction)."""
    import subprocess
    import tempfile
    so = os.path.join(tempfile.mkdtemp(), "libuser_models_host.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC",
                    os.path.join(ROOT, "tests", "cpp", "user_models_host.cpp"), "-o", so], check=True)
    H = ctypes.CDLL(so)
    fp = lambda name: ctypes.cast(getattr(H, name), ctypes.c_void_p).value
    return H, {"duffing": (fp("duffing_rhs"), fp("duffing_vjp")),
               "brusselator": (fp("brusselator_rhs"), fp("brusselator_vjp"))}


def main_user_models(L):
    """The test models through the reference (its functor path, AADC tape):
    forward records, pow traces and gradients -> tests/golden/user_model_cases.npz.
    The forced Duffing model is non-autonomous: the reference's back-propagation
    evaluates every recomputed stage at t_n and reads its stage times one
    entry off (detail/backpropagation.hpp:48,197), so its gradients for that
    model are kept only to measure that difference."""
    keep_alive, cbs = user_model_callbacks()
    out = {}
    k = 0
    for name, seed, tabs in [("duffing", 21, ("dopri5", "ck54", "rkf78")),
                             ("brusselator", 22, ("dopri5", "ck54", "rkf78", "rk4"))]:
        y0s, ps, T = user_model_draws(name, 3, seed)
        npar = ps.shape[1]
        for tab in tabs:
            dt = 1e-2 if tab == "rk4" else 1e-3
            for b in range(3):
                y0, p = y0s[b], ps[b]
                mu = np.zeros((1, npar))
                _, _, _, yT, _, _ = solve(L, name, tab, 2, npar, 1e-8, y0, p, T, np.zeros((1, 2)), mu, dt=dt)
                lam = 2.0 * yT[None, :]
                Tn, times, states, yT, lo, mo = solve(L, name, tab, 2, npar, 1e-8, y0, p, T, lam, mu, dt=dt)
                pb = O.user_problem(*cbs[name], tab, 2, npar, 1e-8, 1e-8, dt0=dt, pow_mode=1)
                fw = O.forward(pb, y0, p, 0.0, T, powtrace=True)
                assert fw["n_acc"] == Tn and np.array_equal(fw["states"], states), name
                case = dict(name=f"{name}_{tab}[{b}]", model=name, tableau=tab, n=2, npar=npar, tol=1e-8, dt=dt,
                            y0=y0, p=p, t1=T, lam=lam, mu=mu, T=Tn, yT=yT, dy0=lo, dp=mo, times=times,
                            states=states, pow_calls=fw["pow_calls"], pow_noncr=fw["pow_noncr"],
                            first_noncr_step=fw["first_noncr_step"])
                for key, v in case.items():
                    out[f"c{k}_{key}"] = np.asarray(v)
                k += 1
    out["count"] = np.array(k)
    path = os.path.join(ROOT, "tests", "golden", "user_model_cases.npz")
    np.savez_compressed(path, **out)
    del keep_alive
    print(f"wrote {k} user-model cases to {path} ({os.path.getsize(path)} bytes)")


def main():
    L = load()
    cases = []
    # benchmark configurations: cost seeds from y(T) (sum of squares) or ones
    # (sum); then the same draws with the Fehlberg 7(8) pair (the reference's
    # ButcherTable branch for runge_kutta_fehlberg78) and with the fixed-step
    # loop (runge_kutta4 at dt = 0.01, euler at dt = 1e-3)
    for name, count, tableau, dt in [("vdp1", 1, None, 1e-3), ("dho", 4, None, 1e-3), ("vdpb", 4, None, 1e-3),
                                     ("glv10", 3, None, 1e-3), ("vdpb", 2, "rkf78", 1e-3), ("dho", 2, "rkf78", 1e-3),
                                     ("glv10", 1, "rkf78", 1e-3), ("vdpb", 2, "rk4", 1e-2), ("dho", 1, "rk4", 1e-2),
                                     ("glv10", 1, "rk4", 1e-2), ("vdpb", 1, "euler", 1e-3)]:
        w = W.make(name, batch=count)
        c = w["cfg"]
        if tableau:
            c["tableau"] = tableau
            name = f"{name}_{tableau}"
        for b in range(count):
            y0, p, t1 = w["y0"][b], w["params"][b], float(w["t1"][b])
            mu = np.zeros((1, c["npar"]))
            # forward first to get y(T) for the sum-of-squares seed
            T, times, states, yT, _, _ = solve(L, c["model"], c["tableau"], c["n"], c["npar"], c["tol"], y0, p, t1,
                                               np.zeros((1, c["n"])), mu, dt=dt)
            lam = (2.0 * yT if c["cost"] == "sumsq" else np.ones(c["n"]))[None, :]
            T, times, states, yT, lo, mo = solve(L, c["model"], c["tableau"], c["n"], c["npar"], c["tol"], y0, p,
                                                 t1, lam, mu, dt=dt)
            keep = T <= MAX_STORED_STEPS
            calls, noncr = pow_trace(c["model"], c["tableau"], c["n"], c["npar"], c["tol"], y0, p, t1, dt)
            cases.append(dict(name=f"{name}[{b}]", model=c["model"], tableau=c["tableau"], n=c["n"],
                              npar=c["npar"], tol=c["tol"], dt=dt, y0=y0, p=p, t1=t1, lam=lam, mu=mu, T=T, yT=yT,
                              dy0=lo, dp=mo, times=times if keep else None, states=states if keep else None,
                              pow_calls=calls, pow_noncr=noncr))
    # instances of the Van der Pol and damped-oscillator batches on which the
    # C library's pow returns a value that is not the correctly rounded power
    # and the accepted steps change because of it: the first two of each
    for name in ("vdpb", "dho"):
        w = W.make(name, batch=600)
        c = w["cfg"]
        found = 0
        for b in range(600):
            y0, p, t1 = w["y0"][b], w["params"][b], float(w["t1"][b])
            args = (c["model"], c["tableau"], c["n"], c["npar"], c["tol"], y0, p, t1, 1e-3)
            calls, noncr, first = pow_trace(*args, first=True)
            if noncr == 0 or not differs_with_cr_pow(*args):
                continue
            mu = np.zeros((1, c["npar"]))
            T, times, states, yT, _, _ = solve(L, c["model"], c["tableau"], c["n"], c["npar"], c["tol"], y0, p, t1,
                                               np.zeros((1, c["n"])), mu)
            lam = (2.0 * yT if c["cost"] == "sumsq" else np.ones(c["n"]))[None, :]
            T, times, states, yT, lo, mo = solve(L, c["model"], c["tableau"], c["n"], c["npar"], c["tol"], y0, p,
                                                 t1, lam, mu)
            cases.append(dict(name=f"{name}_libm_noncr[{b}]", model=c["model"], tableau=c["tableau"], n=c["n"],
                              npar=c["npar"], tol=c["tol"], dt=1e-3, y0=y0, p=p, t1=t1, lam=lam, mu=mu, T=T,
                              yT=yT, dy0=lo, dp=mo, times=times, states=states, pow_calls=calls, pow_noncr=noncr,
                              first_noncr_step=first))
            found += 1
            if found == 2:
                break
    # the reference's GLV example on its own data, identity seeds (Nout = N)
    for N in (5, 10):
        vals = np.array([float(v) for v in open(f"{REF}/examples/GeneralizedLotkaVolterra/data/N{N}/alphasfile_cpp.csv")
                         .read().replace("\n", ",").split(",") if v.strip()])
        assert vals.size == N + N * N
        y0 = np.full(N, 0.1)
        lam, mu = np.eye(N), np.zeros((N, N + N * N))
        for tol in (1e-6, 1e-9):
            T, times, states, yT, lo, mo = solve(L, "glv", "ck54", N, N + N * N, tol, y0, vals, 10.0, lam, mu)
            calls, noncr = pow_trace("glv", "ck54", N, N + N * N, tol, y0, vals, 10.0, 1e-3)
            cases.append(dict(name=f"glv_example_N{N}_tol{tol:g}", model="glv", tableau="ck54", n=N,
                              npar=N + N * N, tol=tol, dt=1e-3, y0=y0, p=vals, t1=10.0, lam=lam, mu=mu, T=T, yT=yT,
                              dy0=lo, dp=mo, times=times, states=states, pow_calls=calls, pow_noncr=noncr))
    out = {}
    for k, cs in enumerate(cases):
        for key, v in cs.items():
            if v is not None:
                out[f"c{k}_{key}"] = np.asarray(v)
    out["count"] = np.array(len(cases))
    path = os.path.join(ROOT, "tests", "golden", "reference_cases.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {len(cases)} cases to {path} ({os.path.getsize(path)} bytes)")
    main_history(L)
    main_user_models(L)


if __name__ == "__main__":
    main()
