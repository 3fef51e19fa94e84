"""A right-hand side the library has never seen: the bring-your-own-model
path (include/va_model.cuh, va_create_model).

Two models live only in tests/cpp/user_models.cuh: a Duffing oscillator
under a rational, time-dependent forcing (non-autonomous, so the stage times
t_n + c_m h matter) and the Brusselator (autonomous).  The tests build them
the way a user does -- nvcc on a unit of their own into their own shared
library (tests/cpp/user_model_*.cu) -- and, for the oracle, into host
callbacks (g++, tests/cpp/user_models_host.cpp).

Pinning (CPU): the reference itself, taping the same functors with AADC
(tests/golden/user_model_cases.npz, made by tests/golden/make_golden.py):
the oracle with the callbacks lands on the reference's accepted steps bit
for bit and, for the autonomous model, on its gradients within 1e-12.  For
the non-autonomous model the reference's back-propagation evaluates the
recomputed stages at t_n and its stage times one entry off
(detail/backpropagation.hpp:48,197), so its gradients differ; the oracle's
(stage times t_n + c_m h) are checked against central differences instead.

GPU: FP64 bit for bit with the oracle (correctly rounded controller) and with
the reference's forward records, the FP64 gradients against central
differences of the GPU's own frozen-step replay of the model, two-level
checkpointing bit for bit, and the reduced precisions against FP64.
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CPP = os.path.join(ROOT, "tests", "cpp")
FIX = os.path.join(ROOT, "tests", "golden", "user_model_cases.npz")
NPAR = {"duffing": 5, "brusselator": 2}


def cases():
    z = np.load(FIX)
    out = []
    for k in range(int(z["count"])):
        c = {key[len(f"c{k}_"):]: z[key] for key in z.files if key.startswith(f"c{k}_")}
        for s in ("name", "model", "tableau"):
            c[s] = str(c[s])
        for s in ("n", "npar", "T", "pow_noncr", "first_noncr_step"):
            c[s] = int(c[s])
        c["tol"], c["t1"], c["dt"] = float(c["tol"]), float(c["t1"]), float(c["dt"])
        out.append(c)
    return out


CASES = cases()
IDS = [c["name"] for c in CASES]


@pytest.fixture(scope="module")
def host_models(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("um") / "libuser_models_host.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC",
                    os.path.join(CPP, "user_models_host.cpp"), "-o", so], check=True)
    H = ctypes.CDLL(so)
    fp = lambda name: ctypes.cast(getattr(H, name), ctypes.c_void_p).value
    return H, {"duffing": (fp("duffing_rhs"), fp("duffing_vjp")),
               "brusselator": (fp("brusselator_rhs"), fp("brusselator_vjp"))}


def oracle_problem(oracle, host_models, c, pow_mode, tableau=None):
    rhs, vjp = host_models[1][c["model"]]
    return oracle.user_problem(rhs, vjp, tableau or c["tableau"], 2, c["npar"], c["tol"], c["tol"], dt0=c["dt"],
                               pow_mode=pow_mode)


def rel(a, b):
    a, b = np.asarray(a).ravel(), np.asarray(b).ravel()
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("c", CASES, ids=IDS)
def test_oracle_user_model_matches_reference(oracle, host_models, c):
    pb = oracle_problem(oracle, host_models, c, pow_mode=1)
    fw = oracle.forward(pb, c["y0"], c["p"], 0.0, c["t1"])
    assert fw["status"] == 0 and fw["n_acc"] == c["T"]
    np.testing.assert_array_equal(fw["times"], c["times"])
    np.testing.assert_array_equal(fw["states"], c["states"])
    lam, mu, st = oracle.adjoint(pb, c["p"], fw["times"], fw["states"], c["lam"], c["mu"])
    assert st == 0
    g = np.concatenate([lam.ravel(), mu.ravel()])
    gref = np.concatenate([c["dy0"].ravel(), c["dp"].ravel()])
    if c["model"] == "brusselator":
        assert rel(g, gref) < 1e-12
    else:
        # the reference's stage times are wrong for a time-dependent RHS; ours
        # are checked by central differences of the frozen-step map
        assert rel(g, gref) > 1e-9
        fd = []
        x = np.concatenate([c["y0"], c["p"]])
        for k in range(x.size):
            vals = []
            e = 1e-4 * max(abs(x[k]), 0.1)
            for sgn in (-2.0, -1.0, 1.0, 2.0):
                xx = x.copy()
                xx[k] += sgn * e
                yT = oracle.forward_frozen(pb, xx[:2], xx[2:], fw["times"])
                vals.append(float((yT ** 2).sum()))
            fd.append((8.0 * (vals[2] - vals[1]) - (vals[3] - vals[0])) / (12.0 * e))
        assert rel(g, np.array(fd)) < 1e-7


# ------------------------------------------------------------------- GPU


@pytest.fixture(scope="module")
def device_models(cuda, tmp_path_factory):
    """The two models built into their own shared libraries, as a user would."""
    from vectorizedadjoint_gb300 import build as vbuild
    out = tmp_path_factory.mktemp("umd")
    procs = {}
    for name, src in (("duffing", "user_model_duffing.cu"), ("brusselator", "user_model_brusselator.cu")):
        so = str(out / f"lib{name}.so")
        cmd = [vbuild.NVCC, "-gencode=arch=compute_103a,code=sm_103a", "-std=c++17", "-O3",
               "--expt-relaxed-constexpr", "-fmad=false", "-Xcompiler", "-fPIC", "-shared",
               "-I", os.path.join(ROOT, "include"), os.path.join(CPP, src), "-o", so]
        procs[name] = (so, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT))
    libs, tables = {}, {}
    for name, (so, p) in procs.items():
        log = p.communicate()[0].decode()
        assert p.returncode == 0, log
        libs[name] = ctypes.CDLL(so)
        fn = getattr(libs[name], "forced_duffing_kernels" if name == "duffing" else "brusselator_kernels")
        fn.restype = ctypes.c_void_p
        tables[name] = fn()
    return libs, tables


def solver(device_models, model, B, tableau, precision="fp64", tol=1e-8, dt0=1e-3, **kw):
    from vectorizedadjoint_gb300 import Solver
    return Solver("user", 2, NPAR[model], B, tableau=tableau, precision=precision, atol=tol, rtol=tol, dt0=dt0,
                  model_kernels=device_models[1][model], **kw)


def dev(a):
    import torch
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def draws(model, B, seed=5):
    rng = np.random.Generator(np.random.PCG64(seed))
    if model == "duffing":
        p = np.stack([rng.uniform(0.1, 0.5, B), rng.uniform(0.5, 2.0, B), rng.uniform(0.0, 1.0, B),
                      rng.uniform(0.5, 2.0, B), rng.uniform(0.5, 2.0, B)], axis=1)
        return rng.uniform(-1.0, 1.0, (B, 2)), p, np.full(B, 10.0)
    p = np.stack([rng.uniform(0.8, 1.5, B), rng.uniform(1.5, 3.5, B)], axis=1)
    return rng.uniform(0.5, 2.0, (B, 2)), p, np.full(B, 20.0)


@pytest.mark.gpu
def test_user_model_rejects_bad_tables(cuda, device_models):
    from vectorizedadjoint_gb300 import _lib
    L = _lib.load()
    o = _lib.VaOptions()
    L.va_default_options(ctypes.byref(o))
    h = ctypes.c_void_p()
    good = _lib.VaProblem(6, 2, 5, 4, 1)
    assert L.va_create_model(ctypes.byref(good), ctypes.byref(o), None, ctypes.byref(h)) == 5
    junk = (ctypes.c_uint32 * 64)()
    assert L.va_create_model(ctypes.byref(good), ctypes.byref(o), ctypes.addressof(junk), ctypes.byref(h)) == 5
    wrong_n = _lib.VaProblem(6, 3, 5, 4, 1)
    assert L.va_create_model(ctypes.byref(wrong_n), ctypes.byref(o), ctypes.c_void_p(device_models[1]["duffing"]),
                             ctypes.byref(h)) == 5
    o.precision = 2  # the Duffing table has no double-word sweeps
    assert L.va_create_model(ctypes.byref(good), ctypes.byref(o), ctypes.c_void_p(device_models[1]["duffing"]),
                             ctypes.byref(h)) == 5


@pytest.mark.gpu
@pytest.mark.parametrize("c", CASES, ids=IDS)
def test_gpu_user_model_matches_reference(oracle, host_models, device_models, c):
    """FP64: the reference's accepted steps (t_n, y_n) bit for bit where its
    libm pow rounded correctly (else up to the first step where it did not),
    and the oracle's correctly rounded run bit for bit, gradients included."""
    import torch
    s = solver(device_models, c["model"], 1, c["tableau"], dt0=c["dt"])
    P = dev(c["p"][None, :])
    f = s.forward(dev(c["y0"][None, :]), P, dev([0.0]), dev([c["t1"]]))
    bw = s.backward(P, dev(c["lam"][None]), dev(c["mu"][None]))
    torch.cuda.synchronize()
    assert int(f["status"][0]) == 0
    t, _, y = s.trajectory(0)
    k = len(c["times"]) - 1 if c["pow_noncr"] == 0 else c["first_noncr_step"]
    np.testing.assert_array_equal(t[:k + 1], c["times"][:k + 1])
    np.testing.assert_array_equal(y[:k + 1], c["states"][:k + 1])
    pb = oracle_problem(oracle, host_models, c, pow_mode=2)
    g = oracle.gradient(pb, "sumsq", c["y0"], c["p"], 0.0, c["t1"])
    fw = oracle.forward(pb, c["y0"], c["p"], 0.0, c["t1"])
    np.testing.assert_array_equal(t, fw["times"])
    np.testing.assert_array_equal(y, fw["states"])
    lam, mu, _ = oracle.adjoint(pb, c["p"], fw["times"], fw["states"], c["lam"], c["mu"])
    np.testing.assert_array_equal(bw["dy0"].cpu().numpy()[0], lam)
    np.testing.assert_array_equal(bw["dp"].cpu().numpy()[0], mu)
    if c["model"] == "brusselator" and c["pow_noncr"] == 0:
        gref = np.concatenate([c["dy0"].ravel(), c["dp"].ravel()])
        assert rel(np.concatenate([lam.ravel(), mu.ravel()]), gref) < 1e-12
    assert g["status"] == 0
    s.close()


@pytest.mark.gpu
@pytest.mark.parametrize("model,tableau", [("duffing", "dopri5"), ("duffing", "rkf78"), ("duffing", "euler"),
                                           ("brusselator", "ck54"), ("brusselator", "rk4")])
def test_gpu_user_model_batch_and_fd(oracle, host_models, device_models, model, tableau):
    """A batch through va_gradient: bit for bit with the oracle per instance,
    and the gradients against central differences of the GPU replay."""
    import torch
    B = 64
    y0, p, T = draws(model, B)
    dt0 = 1e-2 if tableau == "rk4" else (5e-3 if tableau == "euler" else 1e-3)
    s = solver(device_models, model, B, tableau, dt0=dt0)
    out = s.gradient("sumsq", dev(y0), dev(p), dev(np.zeros(B)), dev(T))
    torch.cuda.synchronize()
    r = {k: v.cpu().numpy() for k, v in out.items()}
    assert (r["status"] == 0).all()
    rhs, vjp = host_models[1][model]
    pb = oracle.user_problem(rhs, vjp, tableau, 2, NPAR[model], 1e-8, 1e-8, dt0=dt0)
    for b in range(0, B, 7):
        g = oracle.gradient(pb, "sumsq", y0[b], p[b], 0.0, T[b])
        assert int(r["n_acc"][b]) == g["n_acc"]
        np.testing.assert_array_equal(r["dy0"][b], g["dy0"])
        np.testing.assert_array_equal(r["dp"][b], g["dp"])
    # central differences of the GPU's frozen-step replay, instances 0..2
    for b in range(3):
        t, _, _ = s.trajectory(b)
        x = np.concatenate([y0[b], p[b]])
        lanes = []
        steps = []
        for k in range(x.size):
            e = 1e-4 * max(abs(x[k]), 0.1)
            steps.append(e)
            for sgn in (-2.0, -1.0, 1.0, 2.0):
                xx = x.copy()
                xx[k] += sgn * e
                lanes.append(xx)
        lanes = np.array(lanes)
        yT = s.forward_frozen([t] * len(lanes), dev(lanes[:, :2]), dev(lanes[:, 2:])).cpu().numpy()
        v = (yT ** 2).sum(1).reshape(x.size, 4)
        fd = (8.0 * (v[:, 2] - v[:, 1]) - (v[:, 3] - v[:, 0])) / (12.0 * np.array(steps))
        grad = np.concatenate([r["dy0"][b], r["dp"][b]])
        assert rel(fd, grad) < 1e-7, (b, fd, grad)
    s.close()


@pytest.mark.gpu
def test_gpu_user_model_two_level_same_bits(device_models):
    import torch
    B = 128
    y0, p, T = draws("duffing", B, seed=8)
    res = []
    for stride in (1, 5):
        s = solver(device_models, "duffing", B, "dopri5", ckpt_stride=stride)
        out = s.gradient("sumsq", dev(y0), dev(p), dev(np.zeros(B)), dev(T))
        torch.cuda.synchronize()
        res.append({k: v.cpu().numpy() for k, v in out.items()})
        s.close()
    for k in ("n_acc", "dy0", "dp", "yT"):
        np.testing.assert_array_equal(res[0][k], res[1][k])


@pytest.mark.gpu
@pytest.mark.parametrize("model,precision,bound,same_frac", [("duffing", "mixed", 1e-3, 0.5),
                                                             ("brusselator", "mixed", 1e-3, 0.5),
                                                             ("brusselator", "mixed_dw", 1e-6, 0.9)])
def test_gpu_user_model_reduced_precision(device_models, model, precision, bound, same_frac):
    """float stages and, for the Brusselator, double-word sweeps against FP64
    on the instances that take the FP64 step count (float stages flip some
    accept/reject decisions at tol 1e-7: ~23% of the Duffing instances take
    another step count; double-word stages nearly none)."""
    import torch
    B = 256
    y0, p, T = draws(model, B, seed=9)
    res = {}
    for prec in ("fp64", precision):
        s = solver(device_models, model, B, "dopri5", precision=prec, tol=1e-7)
        out = s.gradient("sumsq", dev(y0), dev(p), dev(np.zeros(B)), dev(T))
        torch.cuda.synchronize()
        res[prec] = {k: v.cpu().numpy() for k, v in out.items()}
        s.close()
    a, b = res[precision], res["fp64"]
    assert (a["status"] == 0).all()
    same = a["n_acc"] == b["n_acc"]
    assert same.mean() > same_frac, same.mean()
    g = np.concatenate([a["dy0"], a["dp"]], 1)[same]
    g64 = np.concatenate([b["dy0"], b["dp"]], 1)[same]
    err = np.abs(g - g64).max(1) / np.abs(g64).max(1)
    assert np.median(err) < bound, np.median(err)


@pytest.mark.gpu
def test_cpp_facade_with_user_model(oracle, host_models, device_models, tmp_path):
    """A reference-style C++ program names the caller's own model by a tag
    (va_driver.hpp + VA_DEFINE_MODEL table) and gets the oracle's bits."""
    lib_dir = os.path.join(ROOT, "vectorizedadjoint_gb300")
    um_so = device_models[0]["brusselator"]._name
    exe = str(tmp_path / "driver_user_model")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"),
                    os.path.join(CPP, "driver_user_model.cpp"), "-o", exe, um_so, "-L", lib_dir, "-lva_gb300",
                    f"-Wl,-rpath,{lib_dir}", f"-Wl,-rpath,{os.path.dirname(um_so)}"], check=True)
    a, b, x0, y0, t1, tol = 1.1, 2.9, 1.2, 0.7, 15.0, 1e-8
    out = subprocess.run([exe, str(a), str(b), str(x0), str(y0), str(t1), str(tol)], capture_output=True,
                         text=True, check=True).stdout.split("\n")
    vals = {}
    for line in out:
        if line.strip():
            k, *v = line.split()
            vals.setdefault(k, []).append([float(x) for x in v])
    rhs, vjp = host_models[1]["brusselator"]
    pb = oracle.user_problem(rhs, vjp, "dopri5", 2, 2, tol, tol)
    fw = oracle.forward(pb, [x0, y0], [a, b], 0.0, t1)
    assert int(vals["steps"][0][0]) == fw["n_acc"]
    np.testing.assert_array_equal(vals["x"][0], fw["yT"])
    L, M, _ = oracle.adjoint(pb, [a, b], fw["times"], fw["states"], np.eye(2), np.zeros((2, 2)))
    np.testing.assert_array_equal(np.array(vals["lambda"]), L)
    np.testing.assert_array_equal(np.array(vals["mu"]), M)
