"""Golden fixtures made by the REFERENCE ITSELF (tests/golden/make_golden.py:
the reference's lib/include headers + the AADC runtime it ships, compiled
against the project's Boost stand-in).  They pin the oracle: its adjoint must
equal the reference's to rounding (AADC's recorded reverse sweep sums in
another order) and, with the same pow as odeint (pow_mode=1), its forward
sweep must land on the same accepted steps and states bit for bit.

The CUDA library's FP64 controller computes the step factor as the correctly
rounded pow.  Each fixture records how many of the reference's pow calls
returned a value that is not the correctly rounded power (glibc's pow is
within 0.52 ulp, not correctly rounded: ~0.07% of these calls).  Where there
were none, the library must reproduce the reference's accepted-step sequence
bit for bit (t_n, y_n, hence h_n = t_{n+1} - t_n); where there were, bit for
bit up to the step of the first such call, and bit for bit with the oracle's
correctly rounded mode throughout."""
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
        for s in ("n", "npar", "T", "pow_calls", "pow_noncr"):
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


def test_fixtures_cover_libm_rounding():
    """The fixtures hold cases where glibc's pow rounded correctly at every call
    and cases where one call did not."""
    assert sum(int(c["pow_noncr"]) == 0 and "times" in c for c in CASES) >= 20
    assert sum(int(c["pow_noncr"]) > 0 for c in CASES) >= 4


@pytest.mark.parametrize("c", CASES, ids=IDS)
def test_oracle_cr_pow_reproduces_reference(oracle, c):
    """The oracle with the correctly rounded step factor (what the CUDA library
    computes) takes the reference's accepted steps bit for bit wherever the
    reference's pow rounded correctly, and up to the first step where it did
    not."""
    if "times" not in c:
        pytest.skip("trajectory not stored")
    pb = oracle.problem(c["model"], c["tableau"], c["n"], c["npar"], c["tol"], c["tol"], dt0=c["dt"], pow_mode=2)
    fw = oracle.forward(pb, c["y0"], c["p"], 0.0, c["t1"])
    assert fw["status"] == 0
    if int(c["pow_noncr"]) == 0:
        np.testing.assert_array_equal(fw["times"], c["times"])
        np.testing.assert_array_equal(fw["states"], c["states"])
        np.testing.assert_array_equal(fw["yT"], c["yT"])
    else:
        k = int(c["first_noncr_step"])
        np.testing.assert_array_equal(fw["times"][:k + 1], c["times"][:k + 1])
        np.testing.assert_array_equal(fw["states"][:k + 1], c["states"][:k + 1])
        m = min(len(fw["times"]), len(c["times"]))
        assert not (len(fw["times"]) == len(c["times"]) and np.array_equal(fw["states"][:m], c["states"][:m]))


@pytest.mark.gpu
@pytest.mark.parametrize("c", CASES, ids=IDS)
def test_gpu_matches_reference(cuda, oracle, c):
    """The FP64 library against the reference run with odeint's std::pow.
    No incorrectly rounded libm call on the case: the accepted steps (t_n,
    y_n, so h_n), the step count and y(T) are the reference's bit for bit and
    the gradients agree within 1e-12 relative (AADC's reverse sweep sums in
    another order).  Otherwise: bit for bit up to the first such step, and
    the whole sequence equals the oracle's correctly rounded run."""
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
    assert int(f["status"][0]) == 0
    assert s.pow_undecided() == 0
    t, _, y = s.trajectory(0) if "times" in c else (None, None, None)
    yT = f["yT"].cpu().numpy()[0]
    g = np.concatenate([bw["dy0"].cpu().numpy().ravel(), bw["dp"].cpu().numpy().ravel()])
    gref = np.concatenate([c["dy0"].ravel(), c["dp"].ravel()])
    if int(c["pow_noncr"]) == 0:
        assert int(f["n_acc"][0]) == c["T"]
        np.testing.assert_array_equal(yT, c["yT"])
        if t is not None:
            np.testing.assert_array_equal(t, c["times"])
            np.testing.assert_array_equal(y, c["states"])
            np.testing.assert_array_equal(np.diff(t), np.diff(c["times"]))
        assert rel(g, gref) < 1e-12
    else:
        k = int(c["first_noncr_step"])
        np.testing.assert_array_equal(t[:k + 1], c["times"][:k + 1])
        np.testing.assert_array_equal(y[:k + 1], c["states"][:k + 1])
        pb = oracle.problem(c["model"], c["tableau"], c["n"], c["npar"], c["tol"], c["tol"], dt0=c["dt"],
                            pow_mode=2)
        fw = oracle.forward(pb, c["y0"], c["p"], 0.0, c["t1"])
        np.testing.assert_array_equal(t, fw["times"])
        np.testing.assert_array_equal(y, fw["states"])
    s.close()
