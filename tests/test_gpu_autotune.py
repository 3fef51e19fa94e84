"""va_autotune: the timed search, its on-disk cache and the bundle-width
axis of the shared-matrix model.

- A second handle for the same problem takes the stored launch shape from
  the cache file without timing, and gradients do not depend on the shape.
- The shared-matrix bundles have two compiled widths; a cache line that
  names the other width makes the handle run it, and the FP64 per-instance
  results are the same bits either way (an instance's arithmetic does not
  depend on its bundle mates).
"""
import os
import time

import numpy as np
import pytest
import torch

from vectorizedadjoint_gb300 import Solver
from vectorizedadjoint_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def dev(a):
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


@pytest.fixture
def cache_file(tmp_path, monkeypatch):
    path = tmp_path / "autotune.tsv"
    monkeypatch.setenv("VA_AUTOTUNE_CACHE", str(path))
    return path


def test_cache_reused_and_results_independent_of_shape(cuda, cache_file):
    B = 4096
    w = W.make("vdpb", batch=B)
    c = w["cfg"]
    args = (dev(w["y0"]), dev(w["params"]), dev(w["t0"]), dev(w["t1"]))
    s0 = Solver(c["model"], c["n"], c["npar"], B, tableau=c["tableau"], precision="mixed_dw", atol=c["tol"],
                rtol=c["tol"])
    ref = {k: v.cpu().numpy() for k, v in s0.gradient(c["cost"], *args).items()}
    s0.close()
    s1 = Solver(c["model"], c["n"], c["npar"], B, tableau=c["tableau"], precision="mixed_dw", atol=c["tol"],
                rtol=c["tol"])
    t = time.perf_counter()
    launch1 = s1.autotune(c["cost"], *args)
    t_tune = time.perf_counter() - t
    lines = cache_file.read_text().splitlines()
    assert len(lines) == 1 and "\t" in lines[0]
    out1 = {k: v.cpu().numpy() for k, v in s1.gradient(c["cost"], *args).items()}
    s1.close()
    s2 = Solver(c["model"], c["n"], c["npar"], B, tableau=c["tableau"], precision="mixed_dw", atol=c["tol"],
                rtol=c["tol"])
    t = time.perf_counter()
    launch2 = s2.autotune(c["cost"], *args)
    t_cached = time.perf_counter() - t
    assert launch2 == launch1
    assert t_cached < t_tune / 5
    assert len(cache_file.read_text().splitlines()) == 1
    out2 = {k: v.cpu().numpy() for k, v in s2.gradient(c["cost"], *args).items()}
    s2.close()
    for k in ("dy0", "dp", "n_acc", "yT"):
        np.testing.assert_array_equal(out1[k], ref[k])
        np.testing.assert_array_equal(out2[k], ref[k])


@pytest.mark.parametrize("precision", ["fp64", "mixed_dw"])
def test_bundle_width_axis(cuda, cache_file, precision):
    N, B, T = 64, 10, 5.0
    rng = np.random.Generator(np.random.PCG64(4))
    A = rng.normal(0.0, 0.5 / np.sqrt(N), (N, N))
    A[np.arange(N), np.arange(N)] = -1.0
    r = rng.uniform(0.5, 1.5, (B, N))
    x0 = rng.uniform(0.1, 1.0, (B, N))
    args = (dev(x0), dev(r), dev(np.zeros(B)), dev(np.full(B, T)))

    def run(alt):
        s = Solver("glv_shared", N, N, B, tableau="dopri5", precision=precision, atol=1e-7, rtol=1e-7)
        dA = torch.empty(N, N, dtype=torch.float64, device="cuda")
        s.set_shared(dev(A), dA)
        if alt is not None:
            # a stored shape that names the bundle width
            s.autotune("sum", *args)
            key = cache_file.read_text().splitlines()[-1].split("\t")[0]
            with open(cache_file, "a") as f:
                f.write(f"{key}\t0 0 0 0 {alt}\n")
            s.autotune("sum", *args)
        out = {k: v.cpu().numpy() for k, v in s.gradient("sum", *args).items()}
        out["dA"] = dA.cpu().numpy()
        s.close()
        return out

    base, w0, w1 = run(None), run(0), run(1)
    for o in (w0, w1):
        assert (o["status"] == 0).all()
        if precision == "fp64":
            for k in ("dy0", "dp", "n_acc", "yT"):
                np.testing.assert_array_equal(o[k], base[k])
        else:
            g, g0 = np.concatenate([o["dy0"], o["dp"]], 1), np.concatenate([base["dy0"], base["dp"]], 1)
            assert np.abs(g - g0).max() <= 1e-9 * np.abs(g0).max()
        assert np.abs(o["dA"] - base["dA"]).max() <= 1e-8 * np.abs(base["dA"]).max()
