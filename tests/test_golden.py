"""Golden fixtures made by the REFERENCE ITSELF (tests/golden/make_golden.py:
the reference's lib/include headers + the AADC runtime it ships, compiled
against the project's Boost stand-in).  They pin the oracle: its adjoint must
equal the reference's to rounding (AADC's recorded reverse sweep sums in
another order) and, with the same pow as odeint (pow_mode=1), its forward
sweep must land on the same accepted steps and states bit for bit.  The GPU
check compares the CUDA library with the same fixtures."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = os.path.join(HERE, "golden", "reference_cases.npz")


def cases():
    z = np.load(FIX)
    out = []
    for k in range(int(z["count"])):
        c = {key[len(f"c{k}_"):]: z[key] for key in z.files if key.startswith(f"c{k}_")}
        for s in ("name", "model", "tableau"):
            c[s] = str(c[s])
        for s in ("n", "npar", "T"):
            c[s] = int(c[s])
        c["tol"], c["t1"], c["dt"] = float(c["tol"]), float(c["t1"]), float(c["dt"])
        out.append(c)
    return out


CASES = cases()
IDS = [c["name"] for c in CASES]


def rel(a, b):
    a, b = np.asarray(a).ravel(), np.asarray(b).ravel()
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("c", CASES, ids=IDS)
def test_oracle_matches_reference(oracle, c):
    pb = oracle.problem(c["model"], c["tableau"], c["n"], c["npar"], c["tol"], c["tol"], dt0=c["dt"], pow_mode=1)
    fw = oracle.forward(pb, c["y0"], c["p"], 0.0, c["t1"])
    assert fw["status"] == 0
    assert fw["n_acc"] == c["T"]
    np.testing.assert_array_equal(fw["yT"], c["yT"])
    if "times" in c:
        np.testing.assert_array_equal(fw["times"], c["times"])
        np.testing.assert_array_equal(fw["states"], c["states"])
    lam, mu, st = oracle.adjoint(pb, c["p"], fw["times"], fw["states"], c["lam"], c["mu"])
    assert st == 0
    g = np.concatenate([lam.ravel(), mu.ravel()])
    gref = np.concatenate([c["dy0"].ravel(), c["dp"].ravel()])
    assert rel(g, gref) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("c", CASES, ids=IDS)
def test_gpu_matches_reference(cuda, c):
    """The FP64 library (deterministic step-factor power) against the reference
    run with odeint's std::pow: same accepted-step count and gradients within
    1e-9 relative (last-bit differences of some step factors move later steps
    by ~1e-9 relative; see the oracle's pow_mode)."""
    import torch

    from vectorizedadjoint_gb300 import Solver
    dev = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")
    Q = c["lam"].shape[0]
    s = Solver(c["model"], c["n"], c["npar"], 1, nout=Q, tableau=c["tableau"], atol=c["tol"], rtol=c["tol"],
               dt0=c["dt"])
    P = dev(c["p"][None, :])
    f = s.forward(dev(c["y0"][None, :]), P, dev([0.0]), dev([c["t1"]]))
    bw = s.backward(P, dev(c["lam"][None]), dev(c["mu"][None]))
    torch.cuda.synchronize()
    assert int(f["n_acc"][0]) == c["T"]
    g = np.concatenate([bw["dy0"].cpu().numpy().ravel(), bw["dp"].cpu().numpy().ravel()])
    gref = np.concatenate([c["dy0"].ravel(), c["dp"].ravel()])
    assert rel(g, gref) < 1e-9
    s.close()
