"""Full-batch FP64 parity of the drop-in path (VdP batch 262,144; DHO
65,536; GLV-10 16,384), every instance checked, not a sample:

- against the oracle with the correctly rounded step factor pow(err, -1/k)
  (pow_mode 2, what the library's FP64 controller computes): every
  instance's gradient (dG/dy0, dG/dp), y(T) and accepted-step count are
  equal bit for bit;
- against the oracle with the C library's pow (pow_mode 1, odeint's
  std::pow): the instances whose results differ are exactly instances on
  which a libm pow call was not correctly rounded (the oracle's pow trace
  finds one on every such instance).  glibc's pow misrounds ~8e-4 of these
  calls, so 2-9% of the instances (one in ~1,200 calls, a few hundred
  calls per instance) take a different rounding of some step size; the
  test records the identical fraction and asserts it stays above 85%.

The oracle runs on every host thread (the C restatement, pow_mode 2 in
binary128)."""
import os

import numpy as np
import pytest
import torch

from vectorizedadjoint_gb300 import Solver
from vectorizedadjoint_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def dev(a):
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


@pytest.mark.parametrize("name", ["glv10", "dho", "vdpb"])
def test_every_instance_bit_exact(oracle, cuda, name):
    w = W.make(name)
    c = w["cfg"]
    B = len(w["y0"])
    s = Solver(c["model"], c["n"], c["npar"], B, tableau=c["tableau"], precision="fp64", atol=c["tol"],
               rtol=c["tol"])
    out = s.gradient(c["cost"], dev(w["y0"]), dev(w["params"]), dev(w["t0"]), dev(w["t1"]))
    torch.cuda.synchronize()
    g = {k: v.cpu().numpy() for k, v in out.items()}
    assert s.pow_undecided() == 0
    s.close()
    assert (g["status"] == 0).all()

    threads = os.cpu_count() or 1
    ref = {}
    for pm in (2, 1):
        pb = oracle.problem(c["model"], c["tableau"], c["n"], c["npar"], c["tol"], c["tol"], pow_mode=pm)
        ref[pm] = oracle.gradient_batch(pb, c["cost"], w["y0"], w["params"], w["t0"], w["t1"], nthreads=threads)
        assert (ref[pm]["status"] == 0).all()

    cr = ref[2]
    np.testing.assert_array_equal(g["n_acc"], cr["n_acc"])
    np.testing.assert_array_equal(g["yT"], cr["yT"])
    np.testing.assert_array_equal(g["dy0"], cr["dy0"])
    np.testing.assert_array_equal(g["dp"], cr["dp"])

    lm = ref[1]
    same = (g["dy0"] == lm["dy0"]).all(1) & (g["dp"] == lm["dp"]).all(1) & (g["yT"] == lm["yT"]).all(1)
    same &= g["n_acc"] == lm["n_acc"]
    pb = oracle.problem(c["model"], c["tableau"], c["n"], c["npar"], c["tol"], c["tol"], pow_mode=1)
    unexplained = []
    for b in np.nonzero(~same)[0]:
        fw = oracle.forward(pb, w["y0"][b], w["params"][b], w["t0"][b], w["t1"][b], cap=int(lm["n_acc"][b]) + 8,
                            powtrace=True)
        if fw["pow_noncr"] == 0:
            unexplained.append(int(b))
    assert not unexplained, unexplained[:10]
    frac = same.mean()
    print(f"{name}: {same.sum()} of {B} instances identical to the libm-pow oracle ({100 * frac:.3f}%), "
          f"{B - same.sum()} differ, each after a libm pow call that was not correctly rounded")
    assert frac > 0.85
