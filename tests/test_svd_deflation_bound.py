"""CPU check of the deflation rule of the FP64 SVD kernel (gesvd_kernel in
hcore_gb300/csrc/hc_kernels.cu), restated in numpy.

The kernel factors the core T P = Q R with column pivoting and stops at the
first step j (j >= the rank rule's start) whose trailing block has
||R(j:, j:)||_F <= delta = min(1e-13 thr, 1e-16 ||T||_F); its Jacobi then
works on the first j rows of R.  Checked here on cores whose singular values
span many decades:
* every singular value of the deflated core lies within delta of the full
  one (Weyl), and within a few eps sigma_max of LAPACK's;
* the rank by the reference's absolute rule (hcore_dgemm.c:446-463: first
  i >= 1 with sigma_i < acc) is unchanged unless a singular value lies within
  1e-13 of the threshold, relative;
* the truncated product moves by at most delta.
"""
import numpy as np
import pytest

sl = pytest.importorskip("scipy.linalg")

ACC = 1e-8


def _core(rng, k, decades):
    """A graded core D1 G D2 (G Gaussian, D1 and D2 spanning `decades` each),
    as R_A R_B^T is when the stacked factors' columns are graded: its small
    singular values are carried by small entries, not by rounding noise."""
    d1 = 10.0 ** (-decades * rng.random(k))
    d2 = 10.0 ** (-decades * rng.random(k))
    return d1[:, None] * rng.standard_normal((k, k)) * d2[None, :]


def _deflate(T, acc, rank_start=1):
    k = T.shape[0]
    fro = np.linalg.norm(T)
    delta = min(1e-13 * acc, 1e-16 * fro)
    R, piv = sl.qr(T, pivoting=True, mode="r")
    tails = [np.linalg.norm(R[j:, j:]) for j in range(k + 1)]
    kk = next((j for j in range(min(rank_start, k), k + 1) if tails[j] <= delta), k)
    R1 = R.copy()
    R1[kk:, :] = 0.0
    return R, R1, piv, kk, delta


def _rank(s, acc, start=1):
    for i in range(start, len(s)):
        if s[i] < acc:
            return i
    return len(s)


@pytest.mark.parametrize("k,decades,seed", [(13, 30, 1), (42, 30, 2), (64, 40, 3), (64, 12, 4),
                                            (124, 30, 5), (35, 60, 6)])
def test_deflated_singular_values_within_bound(k, decades, seed):
    rng = np.random.default_rng(seed)
    T = _core(rng, k, decades)
    R, R1, piv, kk, delta = _deflate(T, ACC)
    s_full = np.linalg.svd(R, compute_uv=False)
    s_defl = np.linalg.svd(R1, compute_uv=False)
    s_ref = np.linalg.svd(T, compute_uv=False)
    assert kk < k                                   # part of every such core is dropped
    assert np.linalg.norm(R - R1, 2) <= delta
    assert np.abs(s_defl - s_full).max() <= delta * (1 + 1e-12)
    assert np.abs(s_defl - s_ref).max() <= 8 * np.finfo(float).eps * s_ref[0] + delta
    assert (s_defl[kk:] == 0).all()
    r_full, r_defl = _rank(s_ref, ACC), _rank(s_defl, ACC)
    near = np.any(np.abs(s_ref - ACC) <= 1e-13 * ACC)
    assert r_full == r_defl or near


def test_truncated_products_agree():
    """U_r S_r V_r^T from the deflated core against the full core's."""
    rng = np.random.default_rng(9)
    T = _core(rng, 48, 30)
    R, R1, piv, kk, delta = _deflate(T, ACC)
    P = np.eye(48)[:, piv]
    U0, s0, V0 = np.linalg.svd(R)
    U1, s1, V1 = np.linalg.svd(R1)
    r0, r1 = _rank(s0, ACC), _rank(s1, ACC)
    assert r0 == r1
    A0 = (U0[:, :r0] * s0[:r0]) @ V0[:r0] @ P.T
    A1 = (U1[:, :r1] * s1[:r1]) @ V1[:r1] @ P.T
    assert np.linalg.norm(A0 - A1, 2) <= 2 * delta + 1e-15 * s0[0]


def test_rank_start_keeps_leading_columns():
    """A core below the threshold everywhere: the QR keeps rank_start steps
    (the rule's first column is kept whatever its size), so kk >= 1."""
    rng = np.random.default_rng(11)
    T = _core(rng, 20, 20) * 1e-12
    _, R1, _, kk, _ = _deflate(T, ACC, rank_start=1)
    assert kk >= 1
    s = np.linalg.svd(R1, compute_uv=False)
    assert _rank(s, ACC) == 1
    _, _, _, kk0, _ = _deflate(T, ACC, rank_start=0)
    assert kk0 <= kk


def test_relative_threshold_lower_bound():
    """The compressor's relative rule: acc ||T||_F / sqrt(k) <= acc sigma_max,
    so the bound built from it never exceeds the one built from sigma_max."""
    rng = np.random.default_rng(13)
    for k in (8, 33, 100):
        T = _core(rng, k, 10)
        s = np.linalg.svd(T, compute_uv=False)
        assert np.linalg.norm(T) / np.sqrt(k) <= s[0] * (1 + 1e-14)
