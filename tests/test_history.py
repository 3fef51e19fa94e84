"""Adjoint history: lambda_n after every back step, the values the
reference's back_prop observer is shown (lib/include/detail/
backpropagation.hpp:256-278).  tests/golden/history_cases.npz holds what the
reference itself shows its observer (tests/golden/make_golden.py); the
oracle must reproduce it, and the CUDA library (va_set_adjoint_history /
va_adjoint_history) must reproduce the oracle: bit for bit in FP64, for every
seed, with every-step and two-level checkpoints."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = os.path.join(HERE, "golden", "history_cases.npz")


def cases():
    z = np.load(FIX)
    out = []
    for k in range(int(z["count"])):
        c = {key[len(f"c{k}_"):]: z[key] for key in z.files if key.startswith(f"c{k}_")}
        for s in ("name", "model", "tableau"):
            c[s] = str(c[s])
        for s in ("n", "npar"):
            c[s] = int(c[s])
        for s in ("tol", "dt", "t1"):
            c[s] = float(c[s])
        out.append(c)
    return out


CASES = cases()
IDS = [c["name"] for c in CASES]


def oracle_history(oracle, c):
    pb = oracle.problem(c["model"], c["tableau"], c["n"], c["npar"], c["tol"], c["tol"], dt0=c["dt"], pow_mode=1)
    fw = oracle.forward(pb, c["y0"], c["p"], 0.0, c["t1"])
    lam, mu, hist, st = oracle.adjoint_history(pb, c["p"], fw["times"], fw["states"], c["lam"],
                                               np.zeros((c["lam"].shape[0], c["npar"])))
    assert st == 0
    return fw, lam, hist


@pytest.mark.parametrize("c", CASES, ids=IDS)
def test_oracle_history_matches_reference(oracle, c):
    fw, lam, hist = oracle_history(oracle, c)
    np.testing.assert_array_equal(fw["times"], c["times"])
    assert hist.shape == c["hist"].shape
    # lambda_T is the seed itself; the rest to rounding (AADC sums in another order)
    np.testing.assert_array_equal(hist[:, -1], c["lam"])
    scale = np.abs(c["hist"]).max(axis=(1, 2), keepdims=True)
    assert (np.abs(hist - c["hist"]) / scale).max() < 1e-12
    np.testing.assert_array_equal(hist[:, 0], lam)


@pytest.mark.gpu
@pytest.mark.parametrize("c", CASES, ids=IDS)
def test_gpu_history_matches_reference(oracle, cuda, c):
    """The FP64 library's history is the oracle's (deterministic root, the
    same steps) and within 1e-9 of the reference's (odeint's pow moves some
    step factors in the last bits)."""
    import torch

    from vectorizedadjoint_gb300 import Solver
    dev = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")
    Q = c["lam"].shape[0]
    s = Solver(c["model"], c["n"], c["npar"], 1, nout=Q, tableau=c["tableau"], atol=c["tol"], rtol=c["tol"],
               dt0=c["dt"])
    s.set_adjoint_history(len(c["times"]) + 5)
    P = dev(c["p"][None, :])
    s.forward(dev(c["y0"][None, :]), P, dev([0.0]), dev([c["t1"]]))
    s.backward(P, dev(c["lam"][None]), None)
    torch.cuda.synchronize()
    t, hist = s.adjoint_history(0)
    assert hist.shape == c["hist"].shape
    scale = np.abs(c["hist"]).max(axis=(1, 2), keepdims=True)
    assert (np.abs(hist - c["hist"]) / scale).max() < 1e-9
    pb = oracle.problem(c["model"], c["tableau"], c["n"], c["npar"], c["tol"], c["tol"], dt0=c["dt"])
    fw = oracle.forward(pb, c["y0"], c["p"], 0.0, c["t1"])
    _, _, ohist, _ = oracle.adjoint_history(pb, c["p"], fw["times"], fw["states"], c["lam"],
                                            np.zeros((Q, c["npar"])))
    np.testing.assert_array_equal(t, fw["times"])
    np.testing.assert_array_equal(hist, ohist)
    s.close()


def _batch_history(name, B, precision, tableau=None, stride=0, cap=None, nout=1):
    import torch

    from vectorizedadjoint_gb300 import Solver
    from vectorizedadjoint_gb300 import workloads as W
    w = W.make(name, batch=B)
    c = w["cfg"]
    tab = tableau or c["tableau"]
    dev = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")
    s = Solver(c["model"], c["n"], c["npar"], B, nout=nout, tableau=tab, atol=c["tol"], rtol=c["tol"],
               precision=precision, ckpt_stride=stride)
    s.set_adjoint_history(cap or 4096)
    P = dev(w["params"])
    f = s.forward(dev(w["y0"]), P, dev(w["t0"]), dev(w["t1"]))
    lam = np.random.Generator(np.random.PCG64(7)).standard_normal((B, nout, c["n"]))
    bw = s.backward(P, dev(lam), None)
    torch.cuda.synchronize()
    out = [s.adjoint_history(b, times=stride <= 1) for b in range(B)]
    res = dict(n_acc=f["n_acc"].cpu().numpy(), dy0=bw["dy0"].cpu().numpy())
    s.close()
    return w, lam, out, res


@pytest.mark.gpu
@pytest.mark.parametrize("name,precision", [("vdpb", "fp64"), ("vdpb", "mixed_dw"), ("vdpb", "mixed"),
                                            ("glv10", "fp64"), ("glv10", "mixed_dw")])
def test_gpu_history_batch(oracle, cuda, name, precision):
    """Every instance of a batch, two seeds: lambda_0 of the history is dy0,
    lambda_T the seed; FP64 equals the oracle bit for bit."""
    B = 16
    w, lam, out, res = _batch_history(name, B, precision, nout=2)
    c = w["cfg"]
    pb = oracle.problem(c["model"], c["tableau"], c["n"], c["npar"], c["tol"], c["tol"])
    for b in range(B):
        t, hist = out[b]
        assert hist.shape[1] == int(res["n_acc"][b]) + 1
        if precision == "mixed_dw":  # the seed as a double-word keeps 48 bits
            np.testing.assert_allclose(hist[:, -1], lam[b], rtol=1e-14, atol=0)
        else:
            np.testing.assert_array_equal(hist[:, -1], lam[b])
        np.testing.assert_array_equal(hist[:, 0], res["dy0"][b])
        if precision == "fp64":
            fw = oracle.forward(pb, w["y0"][b], w["params"][b], 0.0, w["t1"][b])
            np.testing.assert_array_equal(t, fw["times"])
            _, _, ohist, _ = oracle.adjoint_history(pb, w["params"][b], fw["times"], fw["states"], lam[b],
                                                    np.zeros((2, c["npar"])))
            np.testing.assert_array_equal(hist, ohist)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed_dw"])
def test_gpu_history_two_level(cuda, precision):
    """Two-level checkpointing writes the same history as every-step."""
    _, _, ref, _ = _batch_history("vdpb", 8, precision)
    _, _, out, _ = _batch_history("vdpb", 8, precision, stride=5)
    for (_, h0), (_, h1) in zip(ref, out):
        np.testing.assert_array_equal(h1, h0)


@pytest.mark.gpu
def test_gpu_history_capacity(cuda):
    """A capacity below T + 1 keeps the first records; the rest is dropped."""
    _, _, full, _ = _batch_history("vdpb", 4, "fp64")
    _, _, short, _ = _batch_history("vdpb", 4, "fp64", cap=10)
    for (_, hf), (_, hs) in zip(full, short):
        assert hs.shape[1] == 10
        np.testing.assert_array_equal(hs, hf[:, :10])
