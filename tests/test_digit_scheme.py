"""The error-free digit scheme of the shared-matrix cluster sweeps
(csrc/va_bundle_tc.cuh), modelled on the CPU with the device code's float32
operations (no GPU): 6 digits of A^T and 7 of v per quarter of 64 terms,
exact integer group sums over the digit pairs s + t <= 6, and the fold that
sums the tail groups 3..6 in float32 and the head groups 0..2 with 2Sums.

- the fold adds at most 2^-46 of the scale 2^(eA + eV) to the exact value
  of the kept digit products (the float32 tail's rounding; measured 2^-47);
- the whole scheme is within 2^-44 of that scale of the exact dot product
  sum_k A_k v_k of the double-word inputs (the truncation of A after 6
  digits, 64 terms; measured 2^-47.2 over magnitudes spread up to 1e6) and,
  for inputs of similar magnitude, within 2e-15 of sum_k |A_k| |v_k|
  (measured 5.6e-16), the double-word level.
"""
from fractions import Fraction

import numpy as np

F = np.float32


def two_sum(a, b):
    s = F(a + b)
    ap = F(s - b)
    bp = F(s - ap)
    return s, F(F(a - ap) + F(b - bp))


def split_digits(hi, lo, e, q):
    """split_digits<Q> of va_contract.cuh: hi + lo = 2^e sum_s d_s 2^(-8(s+1)) + r."""
    scale = F(2.0 ** (8 - e))
    a, b = F(hi * scale), F(lo * scale)
    d = []
    for _ in range(q):
        qq = F(np.rint(a))
        d.append(int(qq))
        r = F(a - qq)
        s = F(r + b)
        bb = F(s - r)
        err = F(F(r - F(s - bb)) + F(b - bb))
        a, b = F(s * F(256.0)), F(err * F(256.0))
    return d


def bound_exponent(m):
    return int(np.floor(np.log2(m))) + 1 if m > 0 else -120


def dword(x):
    hi = F(x)
    return hi, F(x - float(hi))


def scheme(a_vals, v_vals):
    """the value the cluster sweep forms for sum_k a_k v_k over one quarter,
    with the exact value of its kept digit products"""
    A = [dword(x) for x in a_vals]
    V = [dword(x) for x in v_vals]
    eA = bound_exponent(max(abs(float(h)) for h, _ in A))
    eV = bound_exponent(max(abs(float(h)) for h, _ in V))
    dA = [split_digits(h, l, eA, 6) for h, l in A]
    dV = [split_digits(h, l, eV, 7) for h, l in V]
    R = [0] * 7
    for g in range(7):
        for s in range(max(0, g - 6), min(g, 5) + 1):
            R[g] += sum(x[s] * y[g - s] for x, y in zip(dA, dV))
    assert all(abs(x) < 2 ** 24 for x in R)  # every group sum exact in FP32
    Rf = [F(x) for x in R]
    tail = F(F(Rf[3] * F(2.0 ** -24)) + F(F(Rf[4] * F(2.0 ** -32)) + F(F(Rf[5] * F(2.0 ** -40)) + F(Rf[6] * F(2.0 ** -48)))))
    s1, e1 = two_sum(Rf[0], F(Rf[1] * F(2.0 ** -8)))
    s2, e2 = two_sum(s1, F(Rf[2] * F(2.0 ** -16)))
    hi, lo = two_sum(s2, F(F(e1 + e2) + tail))
    unit = Fraction(2) ** (eA + eV - 16)
    folded = (Fraction(float(hi)) + Fraction(float(lo))) * unit
    kept = sum(Fraction(R[g]) * Fraction(2) ** (-8 * g) for g in range(7)) * unit
    exact = sum((Fraction(float(ah)) + Fraction(float(al))) * (Fraction(float(vh)) + Fraction(float(vl)))
                for (ah, al), (vh, vl) in zip(A, V))
    return folded, kept, exact, Fraction(2) ** (eA + eV)


def test_fold_and_truncation_bounds():
    rng = np.random.Generator(np.random.PCG64(17))
    worst_fold = worst_scheme = 0.0
    for trial in range(40):
        spread = [0.0, 2.0, 6.0][trial % 3]  # magnitudes over 1, 100, 1e6
        a = rng.normal(size=64) * 10.0 ** rng.uniform(-spread, 0.0, 64)
        v = rng.normal(size=64) * 10.0 ** rng.uniform(-spread, 0.0, 64)
        folded, kept, exact, scale = scheme(a, v)
        worst_fold = max(worst_fold, float(abs(folded - kept) / scale))
        worst_scheme = max(worst_scheme, float(abs(folded - exact) / scale))
    assert worst_fold <= 2.0 ** -46, worst_fold
    assert worst_scheme <= 2.0 ** -44, worst_scheme


def test_similar_magnitudes_reach_the_double_word_level():
    rng = np.random.Generator(np.random.PCG64(5))
    for _ in range(10):
        a = rng.uniform(0.5, 1.0, 64) * rng.choice([-1.0, 1.0], 64)
        v = rng.uniform(0.5, 1.0, 64)
        folded, _, exact, _ = scheme(a, v)
        total = sum(abs(x) * abs(y) for x, y in zip(a, v))
        assert float(abs(folded - exact)) <= 2e-15 * total
