"""The batched tensor-core product G = A^T V (csrc/va_tc_matvec.cu, through
the C ABI's va_matT_tc): G[b][i] = sum_k A[k][i] V[b][k] for a batch of
double-word vectors V[b].

- Against an exact CPU model of the scheme (the same float32 digit split
  into 7 digits per factor with exponents per row / instance and K quarter
  of 64, integer group sums over the digit pairs s + t = g < 7, power-of-two
  scaling): equal within 2^-46 of sum_k |A[k][i]| |V[b][k]| (the double-word
  accumulation of the 28 group partials).  This pins the operand layouts,
  the descriptors and the exactness of the FP32 tensor-memory sums.
- Integer factors whose digits fall in the kept groups come out exact.
- General factors (the GLV matrix recipe, vectors over 6 orders of
  magnitude): within 2^-44 of FP64-exact products, relative to
  sum_k |A| |V|.
- Batches that are not a multiple of the 64-instance tile.
"""
import ctypes

import numpy as np
import pytest
import torch

from vectorizedadjoint_gb300 import _lib

pytestmark = pytest.mark.gpu
N, KQ, Q = 256, 64, 7


def pack_dw(a):
    hi = a.astype(np.float32)
    lo = (a - hi.astype(np.float64)).astype(np.float32)
    return np.ascontiguousarray(np.stack([hi, lo], -1).view(np.float64)[..., 0]), hi.astype(np.float64) + lo


def unpack_dw(p):
    f = np.ascontiguousarray(p).view(np.float32).reshape(p.shape + (2,))
    return f[..., 0].astype(np.float64) + f[..., 1].astype(np.float64)


def gpu(L, A, V):
    B = V.shape[0]
    dA, dV = (torch.tensor(x, dtype=torch.float64, device="cuda") for x in (A, V))
    dG = torch.full((B, N), np.nan, dtype=torch.float64, device="cuda")
    st = L.va_matT_tc(B, ctypes.c_void_p(dA.data_ptr()), ctypes.c_void_p(dV.data_ptr()),
                      ctypes.c_void_p(dG.data_ptr()), None)
    assert st == 0, st
    return unpack_dw(dG.cpu().numpy())


def split(hi, lo):
    """digits [Q][rows][64] (int64) and exponents [rows] of one K quarter."""
    hi = hi.astype(np.float32)
    lo = lo.astype(np.float32)
    m = np.abs(hi).max(1)
    e = np.where(m > 0, np.floor(np.log2(np.where(m > 0, m, 1))).astype(np.int64) + 1, -120)
    sc = np.ldexp(np.float32(1), (8 - e)).astype(np.float32)[:, None]
    a = (hi * sc).astype(np.float32)
    b = (lo * sc).astype(np.float32)
    ds = []
    for _ in range(Q):
        d = np.rint(a).astype(np.float32)
        ds.append(d.astype(np.int64))
        r = (a - d).astype(np.float32)
        s = (r + b).astype(np.float32)
        bb = (s - r).astype(np.float32)
        err = ((r - (s - bb)) + (b - bb)).astype(np.float32)
        a = (s * np.float32(256)).astype(np.float32)
        b = (err * np.float32(256)).astype(np.float32)
    return np.array(ds), e


def model(A, V):
    """exact scheme: per quarter, integer group sums scaled by powers of two"""
    At = A.T.copy()
    ah = At.astype(np.float32)
    al = (At - ah.astype(np.float64)).astype(np.float32)
    f = np.ascontiguousarray(V).view(np.float32).reshape(V.shape + (2,))
    vh, vl = f[..., 0], f[..., 1]
    out = np.zeros((V.shape[0], N))
    for q in range(N // KQ):
        sl = slice(q * KQ, (q + 1) * KQ)
        da, ea = split(ah[:, sl], al[:, sl])
        dv, ev = split(vh[:, sl], vl[:, sl])
        for g in range(Q):
            R = np.zeros((V.shape[0], N), dtype=np.int64)
            for s in range(g + 1):
                R += dv[g - s] @ da[s].T
            out += R.astype(np.float64) * np.ldexp(1.0, ev[:, None] + ea[None, :] - 16 - 8 * g)
    return out


def glv_matrix(rng):
    A = rng.normal(0.0, 0.5 / 16, (N, N))
    A[np.arange(N), np.arange(N)] = -1.0
    return A


@pytest.mark.parametrize("B", [1, 64, 100, 1024])
def test_matches_exact_model_of_the_scheme(cuda, B):
    L = _lib.load()
    rng = np.random.default_rng(B)
    A = glv_matrix(rng)
    v0 = rng.standard_normal((B, N)) * 10.0 ** rng.uniform(-3, 3, (B, 1))
    V, ve = pack_dw(v0)
    got = gpu(L, A, V)
    want = model(A, V)
    bound = np.abs(ve) @ np.abs(A)
    err = np.abs(got - want) / np.maximum(bound, 1e-300)
    assert err.max() < 2.0 ** -46, err.max()


def test_integer_factors_are_exact(cuda):
    L = _lib.load()
    rng = np.random.default_rng(7)
    B = 130
    Ai = rng.integers(-(1 << 15), 1 << 15, (N, N))
    Vi = rng.integers(-(1 << 15), 1 << 15, (B, N))
    V, _ = pack_dw(Vi.astype(np.float64))
    got = gpu(L, Ai.astype(np.float64), V)
    np.testing.assert_array_equal(got, (Vi @ Ai).astype(np.float64))


def test_general_factors_close_to_exact(cuda):
    L = _lib.load()
    rng = np.random.default_rng(11)
    B = 333
    A = glv_matrix(rng)
    v0 = rng.standard_normal((B, N)) * 10.0 ** rng.uniform(-3, 3, (B, 1)) * 10.0 ** rng.uniform(-1, 1, (1, N))
    V, ve = pack_dw(v0)
    got = gpu(L, A, V)
    ref = ve @ A  # FP64 products of the double-word values (each term exact to 2^-53)
    bound = np.abs(ve) @ np.abs(A)
    err = np.abs(got - ref) / np.maximum(bound, 1e-300)
    assert err.max() < 2.0 ** -44, err.max()
