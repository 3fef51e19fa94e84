"""The step-size controller's power pow(err, -1.0/k) (csrc/va_stepfactor.cuh),
built for the host with g++ (tests/cpp/stepfactor_lib.cpp, no contraction,
as the FP64 kernels are built).

- cr_step_pow is correctly rounded: equal to an arbitrary-precision power
  (mpmath, 300 bits) rounded to nearest, and to the oracle's independent
  binary128 evaluation, over the controller's whole argument range
  (increase_step: 5^-p <= err < 0.5; decrease_step: 1 < err < 1e30).
- Its double-double value before rounding is within 2^-98 of the power (the
  bound Ziv's rounding test relies on, with a window of 2^-95); the first
  pass, with ln x from the float logarithm, within 2^-71.5 (its window is
  2^-70).
- glibc's pow, which odeint calls, is not correctly rounded on a small
  fraction of these arguments: the reason the library's default controller
  is the correctly rounded one rather than a copy of one libm.
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
KS = (3, 5, 6, 8)  # -1.0/3, -1.0/5 (5(4) pairs), -1.0/6, -1.0/8 (Fehlberg 7(8))


@pytest.fixture(scope="module")
def sf(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("sf") / "libsf.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC",
                    os.path.join(ROOT, "tests", "cpp", "stepfactor_lib.cpp"), "-o", so], check=True)
    L = ctypes.CDLL(so)
    L.sf_cr_pow.restype = ctypes.c_double
    L.sf_cr_pow.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.POINTER(ctypes.c_uint)]
    L.sf_dd.restype = None
    L.sf_dd.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.POINTER(ctypes.c_double),
                        ctypes.POINTER(ctypes.c_double)]
    L.sf_dd_fastln.restype = None
    L.sf_dd_fastln.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.POINTER(ctypes.c_double),
                               ctypes.POINTER(ctypes.c_double)]
    L.sf_inv_root.restype = ctypes.c_double
    L.sf_inv_root.argtypes = [ctypes.c_int, ctypes.c_double]
    return L


def args(k, n, seed):
    """Controller arguments: 5^-p .. 0.5 (increase) and 1 .. 1e30 (decrease)."""
    rng = np.random.default_rng(seed)
    lo = np.log10(5.0 ** -8)
    return np.concatenate([10 ** rng.uniform(lo, np.log10(0.5), n), 10 ** rng.uniform(0, 30, n // 2),
                           [5.0 ** -5, 5.0 ** -8, 0.5, 1.0, 1.0 + 2 ** -52, 2.0, 1e29]])


def test_cr_pow_equals_arbitrary_precision(sf):
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.prec = 300
    und = ctypes.c_uint(0)
    for k in KS:
        y = mpmath.mpf(-1.0 / k)
        for x in args(k, 3000, k):
            x = float(x)
            want = float(mpmath.power(mpmath.mpf(x), y))  # round to nearest
            assert sf.sf_cr_pow(k, x, ctypes.byref(und)) == want, (k, x)
    assert und.value == 0


def test_dd_value_within_bound(sf):
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.prec = 300
    ph, pl = ctypes.c_double(), ctypes.c_double()
    worst = 0.0
    for k in KS:
        y = mpmath.mpf(-1.0 / k)
        for x in args(k, 1500, 10 + k):
            x = float(x)
            sf.sf_dd(k, x, ctypes.byref(ph), ctypes.byref(pl))
            ex = mpmath.power(mpmath.mpf(x), y)
            worst = max(worst, float(abs((mpmath.mpf(ph.value) + mpmath.mpf(pl.value) - ex) / ex)))
    assert worst < 2.0 ** -98, worst


def test_first_pass_within_its_window(sf):
    """cr_step_pow's first pass (ln x from logf) is within 2^-71.5 of the
    power, inside its rounding-test window of 2^-70 (the analysis bounds it
    by 2^-72.5 plus the double-double steps' 2^-98)."""
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.prec = 300
    ph, pl = ctypes.c_double(), ctypes.c_double()
    worst = 0.0
    for k in KS:
        y = mpmath.mpf(-1.0 / k)
        for x in args(k, 3000, 20 + k):
            x = float(x)
            sf.sf_dd_fastln(k, x, ctypes.byref(ph), ctypes.byref(pl))
            ex = mpmath.power(mpmath.mpf(x), y)
            worst = max(worst, float(abs((mpmath.mpf(ph.value) + mpmath.mpf(pl.value) - ex) / ex)))
    assert worst < 2.0 ** -71.5, worst


def test_cr_pow_equals_oracle_binary128(sf, oracle):
    """Two independent correctly rounded evaluations agree (50k arguments each)."""
    und = ctypes.c_uint(0)
    for k in KS:
        for x in args(k, 50000, 100 + k):
            x = float(x)
            assert sf.sf_cr_pow(k, x, ctypes.byref(und)) == oracle.step_pow(x, k, 2), (k, x)
    assert und.value == 0


def test_newton_root_matches_oracle_scheme(sf, oracle):
    for k in KS:
        for x in args(k, 5000, 200 + k):
            assert sf.sf_inv_root(k, float(x)) == oracle.step_pow(float(x), k, 0)


def test_libm_pow_is_not_always_correctly_rounded(oracle):
    """glibc's pow misses the correctly rounded value on a small fraction of
    controller arguments (0.52-ulp bound); the correctly rounded value is the
    one that does not depend on the C library."""
    noncr = total = 0
    for k in KS:
        for x in args(k, 20000, 300 + k):
            total += 1
            noncr += oracle.step_pow(float(x), k, 1) != oracle.step_pow(float(x), k, 2)
    assert noncr < 0.01 * total
