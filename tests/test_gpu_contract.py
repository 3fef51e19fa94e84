"""The tensor-core contraction dA = sum_k v_k x_k^T (csrc/va_contract.cu,
through the C ABI's va_contract_dA) that the shared-matrix GLV backward
sweep uses for its matrix gradient.

- Against an exact CPU model of the scheme (the same float32 digit split,
  integer group sums R_g over the digit pairs s + t = g < 4, power-of-two
  scaling): equal to within 2^-44 of sum_k |v_k| |x_k|^T, the double-word
  accumulation's rounding (entries that cancel are compared on that scale).
  This pins the operand layouts, the descriptors and the exactness of the
  FP32 tensor-memory accumulation of the integer digit products.
- Factors whose digit pairs all fall in the kept groups (16-bit by 16-bit
  integers, or 31-bit by 8-bit) come out exact.
- General double-word factors: within 2e-8 of FP64, measured against
  sum_k |v_k| |x_k|^T, with row magnitudes over 2 orders and column
  magnitudes over 6 (the digits are relative to each 64-row chunk's column
  maximum; the exact model of the scheme measures 7e-9 here).
- Row counts that are not a multiple of the 64-row chunk, fewer chunks than
  CTA splits (empty splits), and K = 0.
"""
import ctypes

import numpy as np
import pytest
import torch

from vectorizedadjoint_gb300 import _lib

pytestmark = pytest.mark.gpu
N, KC, Q = 256, 64, 4


def pack_dw(a):
    """double -> double-word packed in 8 bytes ({hi, lo} floats); returns the
    packed array and the value hi + lo as a double."""
    hi = a.astype(np.float32)
    lo = (a - hi.astype(np.float64)).astype(np.float32)
    packed = np.stack([hi, lo], -1).view(np.float64)[..., 0]
    return np.ascontiguousarray(packed), hi.astype(np.float64) + lo.astype(np.float64)


def contract(L, v, x, K=None):
    K = v.shape[0] if K is None else K
    dv = torch.tensor(v, dtype=torch.float64, device="cuda")
    dx = torch.tensor(x, dtype=torch.float64, device="cuda")
    dA = torch.full((N, N), np.nan, dtype=torch.float64, device="cuda")
    st = L.va_contract_dA(K, ctypes.c_void_p(dv.data_ptr()), ctypes.c_void_p(dx.data_ptr()),
                          ctypes.c_void_p(dA.data_ptr()), None)
    assert st == 0, st
    return dA.cpu().numpy()


def split(packed):
    """The kernel's digit split of one chunk [rows, cols] of packed
    double-words: digits [Q][rows][cols] (int64) and column exponents."""
    f = packed.view(np.float32).reshape(packed.shape + (2,))
    hi, lo = f[..., 0], f[..., 1]
    m = np.abs(hi).max(0)
    e = np.where(m > 0, np.floor(np.log2(np.where(m > 0, m, 1))).astype(np.int64) + 1, -120)
    a = np.ldexp(hi, 8 - e).astype(np.float32)
    b = np.ldexp(lo, 8 - e).astype(np.float32)
    ds = []
    for _ in range(Q):
        q = np.rint(a).astype(np.float32)
        ds.append(q.astype(np.int64))
        r = (a - q).astype(np.float32)
        s = (r + b).astype(np.float32)
        bb = (s - r).astype(np.float32)
        err = ((r - (s - bb)) + (b - bb)).astype(np.float32)
        a = (s * np.float32(256)).astype(np.float32)
        b = (err * np.float32(256)).astype(np.float32)
    return np.array(ds), e


def model(v, x):
    """Exact model: per chunk, integer group sums scaled by powers of two."""
    K = v.shape[0]
    out = np.zeros((N, N))
    for c0 in range(0, K, KC):
        dv, ev = split(v[c0:c0 + KC])
        dx, ex = split(x[c0:c0 + KC])
        for g in range(Q):
            R = np.zeros((N, N), dtype=np.int64)
            for s in range(g + 1):
                R += dv[s].T @ dx[g - s]
            out += R.astype(np.float64) * np.ldexp(1.0, (ev[:, None] + ex[None, :] - 16 - 8 * g))
    return out


@pytest.mark.parametrize("K", [1, 64, 65, 1000, 4097])
def test_matches_exact_model_of_the_scheme(cuda, K):
    L = _lib.load()
    rng = np.random.default_rng(K)
    v0 = rng.standard_normal((K, N)) * 10.0 ** rng.uniform(-3, 3, (K, 1))
    x0 = rng.uniform(0.01, 2.0, (K, N))
    v0[rng.random(K) < 0.1] = 0.0  # zero rows
    v, ve = pack_dw(v0)
    x, xe = pack_dw(x0)
    got = contract(L, v, x)
    want = model(v, x)
    scale = np.abs(ve).T @ np.abs(xe)
    err = np.abs(got - want) / np.maximum(scale, 1e-300)
    assert err.max() < 2.0 ** -44, err.max()


@pytest.mark.parametrize("K,bv,bx", [(64, 16, 16), (1000, 16, 16), (300, 31, 8)])
def test_integer_factors_within_kept_groups_are_exact(cuda, K, bv, bx):
    L = _lib.load()
    rng = np.random.default_rng(K + bv)
    vi = rng.integers(-(1 << (bv - 1)), 1 << (bv - 1), (K, N))
    xi = rng.integers(-(1 << (bx - 1)), 1 << (bx - 1), (K, N))
    v, _ = pack_dw(vi.astype(np.float64))
    x, _ = pack_dw(xi.astype(np.float64))
    got = contract(L, v, x)
    exact = (vi.T @ xi).astype(np.float64)  # int64: no overflow at these sizes
    np.testing.assert_array_equal(got, exact)


@pytest.mark.parametrize("K", [63, 700, 9000])
def test_general_factors_within_2e8(cuda, K):
    L = _lib.load()
    rng = np.random.default_rng(100 + K)
    v0 = rng.standard_normal((K, N)) * 10.0 ** rng.uniform(-1, 1, (K, 1)) * 10.0 ** rng.uniform(-3, 3, (1, N))
    x0 = rng.uniform(0.01, 3.0, (K, N)) * 10.0 ** rng.uniform(-1, 1, (K, 1))
    v, ve = pack_dw(v0)
    x, xe = pack_dw(x0)
    got = contract(L, v, x)
    ref = ve.T @ xe
    bound = np.abs(ve).T @ np.abs(xe)
    err = np.abs(got - ref) / np.maximum(bound, 1e-300)
    assert err.max() < 2e-8, err.max()


def test_zero_rows_and_no_rows(cuda):
    L = _lib.load()
    z = np.zeros((3, N))
    assert (contract(L, z, z) == 0).all()
    assert (contract(L, z, z, K=0) == 0).all()
