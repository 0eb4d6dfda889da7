"""CPU checks of the integer arithmetic behind the FP64-accurate tensor-core
products (hcore_gb300/csrc/hc_digits.cuh), restated in numpy:

* a value x with scale 2^E becomes X = round(x 2^(55-E)), written as seven
  balanced base-256 digits in [-128, 128] that reconstruct X exactly;
* the digit products that share one FP32 accumulator stay below 2^24 for
  the chunk lengths the kernels use (128 rows with seven digit pairs, 64 rows
  in the double-buffered QR update), so the FP32 sums are exact;
* the Gram matrix of Householder vectors formed from planes 0..7 with the
  kernels' 64-bit combine (adjacent planes paired exactly, the last pair
  rounded, shift S = 48) lies within 1e-15 of an extended-precision Gram,
  closer than an FP64 BLAS Gram.
"""
from fractions import Fraction

import numpy as np
import pytest

scipy_lapack = pytest.importorskip("scipy.linalg.lapack")


def fixed55(x, E):
    """round(x 2^(55-E)), half away from zero on the magnitude."""
    v = Fraction(float(x)) * Fraction(2) ** (55 - E)
    s = -1 if v < 0 else 1
    return s * int(abs(v) + Fraction(1, 2))


def digits7(X):
    """Balanced base-256 digits a_0..a_6 of X: X = sum a_i 256^(6-i)."""
    z = X + 0x0080808080808080           # non-negative for |X| <= 2^55
    a = [((z >> (8 * (6 - i))) & 0xFF) - 128 for i in range(1, 7)]
    return [(z >> 48) - 128] + a


def test_digits_reconstruct_and_fit_bf16():
    rng = np.random.default_rng(1)
    # E = 1: every |x| < 2 (a Householder entry is at most 1)
    xs = list(rng.uniform(-1.99, 1.99, 2000)) + [1.0, -1.0, 0.0, 2.0 ** -1074, 2 - 2.0 ** -52,
                                                  -(2 - 2.0 ** -52)]
    for x in xs:
        X = fixed55(x, 1)
        assert abs(X) <= 2 ** 55
        a = digits7(X)
        assert all(-128 <= d <= 128 for d in a)
        assert sum(d * 256 ** (6 - i) for i, d in enumerate(a)) == X


@pytest.mark.parametrize("rows,pairs", [(128, 7), (64, 7), (128, 6)])
def test_plane_sums_stay_exact_in_fp32(rows, pairs):
    """Worst case: every digit product at its maximum 128 * 128."""
    assert pairs * rows * 128 * 128 < 2 ** 24


def _householder_block(rng, M, k):
    A = rng.standard_normal((M, k)) * np.logspace(0, -6, k)
    qr, tau, _, _ = scipy_lapack.dgeqrf(A)
    return np.tril(qr, -1)[:, :k] + np.eye(M, k)


def _gram_digits(Y, S=48):
    """The kernels' Gram: digits with E = 1, planes 0..7 per 128-row chunk,
    adjacent planes paired exactly and added as q 2^(88 - 16 m - S), the last
    pair rounded to nearest."""
    M, k = Y.shape
    D = np.zeros((7, M, k), dtype=np.int64)
    for j in range(k):
        for i in range(M):
            D[:, i, j] = digits7(fixed55(Y[i, j], 1))
    T = np.zeros((k, k), dtype=np.int64)
    for c0 in range(0, M, 128):
        sl = slice(c0, min(c0 + 128, M))
        acc = []
        for d in range(8):
            a = np.zeros((k, k), dtype=np.int64)
            for i in range(max(0, d - 6), min(d, 6) + 1):
                a += D[i, sl].T @ D[d - i, sl]
            assert np.abs(a).max() < 2 ** 24
            acc.append(a)
        for m in range(4):
            q = acc[2 * m] * 256 + acc[2 * m + 1]
            sh = 88 - 16 * m - S
            T += q << sh if sh >= 0 else (q + (1 << (-sh - 1))) >> (-sh)
    assert np.abs(T).max() < 2 ** 62
    return T.astype(np.float64) * 2.0 ** (S - 108)


def test_gram_of_householder_block_is_fp64_accurate():
    rng = np.random.default_rng(7)
    Y = _householder_block(rng, 300, 20)
    exact = Y.astype(np.longdouble).T @ Y.astype(np.longdouble)
    G = _gram_digits(Y)
    err = float(np.abs(G - exact).max())
    err_blas = float(np.abs(Y.T @ Y - exact).max())
    assert err < 1e-15
    assert err <= err_blas + 1e-16
    # every entry of a Householder Gram is at most 2 (||v||^2 = 2 / tau)
    assert np.abs(G).max() <= 2.0 + 1e-12
