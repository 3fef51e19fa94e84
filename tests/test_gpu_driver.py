"""The reference-style C++ facade (include/va_driver.hpp): a program with the
call sequence of the reference's VanDerPol example, compiled with g++ against
the C ABI, must print the oracle's step count, state and gradients."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("stepper,dt,observe", [("dopri5", 1e-3, False), ("rkf78", 1e-3, False), ("rk4", 0.01, False),
                                                ("euler", 1e-3, False), ("dopri5", 1e-3, True), ("rk4", 0.01, True)])
def test_cpp_driver_matches_oracle(oracle, cuda, tmp_path, stepper, dt, observe):
    exe = str(tmp_path / "driver_example")
    lib_dir = os.path.join(ROOT, "vectorizedadjoint_gb300")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "driver_example.cpp"), "-o", exe,
                    "-L", lib_dir, "-lva_gb300", f"-Wl,-rpath,{lib_dir}"], check=True)
    mu, x0, v0, t1, tol = 1.3, 1.5, -0.4, 8.0, 1e-8
    args = [exe, str(mu), str(x0), str(v0), str(t1), str(tol), stepper, str(dt)] + (["observe"] if observe else [])
    out = subprocess.run(args, capture_output=True, text=True, check=True).stdout.split("\n")
    vals = {}
    for line in out:
        if line.strip():
            k, *v = line.split()
            vals.setdefault(k, []).append([float(x) for x in v])
    pb = oracle.problem("vdp", stepper, 2, 1, tol, tol, dt0=dt)
    fw = oracle.forward(pb, [x0, v0], [mu], 0.0, t1)
    assert int(vals["steps"][0][0]) == fw["n_acc"]
    np.testing.assert_array_equal(vals["x"][0], fw["yT"])
    L, M, st = oracle.adjoint(pb, [mu], fw["times"], fw["states"], np.eye(2), np.zeros((2, 1)))
    np.testing.assert_array_equal(np.array(vals["lambda"]), L)
    np.testing.assert_array_equal(np.array(vals["mu"]), M)
    np.testing.assert_array_equal(np.array(vals["sens"]).ravel(), M.ravel())
    np.testing.assert_array_equal(np.array(vals["sens1"]).ravel(), M.ravel())
    if observe:
        # forward observer: (t_n, x_n), n = 0 .. T in order; adjoint observer:
        # (t_n, lambda_n rows), n = T .. 0 (the reference's back_prop order)
        obs = np.array(vals["obs"])
        np.testing.assert_array_equal(obs[:, 0], fw["times"])
        np.testing.assert_array_equal(obs[:, 1:], fw["states"])
        _, _, hist, _ = oracle.adjoint_history(pb, [mu], fw["times"], fw["states"], np.eye(2), np.zeros((2, 1)))
        aobs = np.array(vals["aobs"])
        np.testing.assert_array_equal(aobs[:, 0], fw["times"][::-1])
        np.testing.assert_array_equal(aobs[:, 1:].reshape(-1, 2, 2), hist.transpose(1, 0, 2)[::-1])
