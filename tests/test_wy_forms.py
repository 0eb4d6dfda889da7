"""CPU checks of the compact-WY recurrences the tensor-core kernels use,
against LAPACK's own reflector application (scipy's dgeqrf / dormqr):

* rebuild (hc_rebuild_tc.cu, reference hcore_dgemm.c:508-696):
  Q [X0; 0] = X - Y Z with z_j = tau_j (y_j^T X - sum_{i>j} (y_j^T y_i) z_i),
  j = k-1 .. 0 (back substitution with the Gram matrix);
* blocked QR trailing update (hc_qr_tc.cu, reference dgeqrf at
  hcore_dgemm.c:123-124): Q_p^T A_t = A_t - Y_p W' with
  w'_j = tau_j (w_j - sum_{i<j} (y_j^T y_i) w'_i), j = 0 .. 15 (forward
  substitution), and the blocked factorization's R equals dgeqrf's.
"""
import numpy as np
import pytest

la = pytest.importorskip("scipy.linalg.lapack")


def _reflectors(A):
    qr, tau, _, _ = la.dgeqrf(A.copy())
    k = A.shape[1]
    Y = np.tril(qr, -1)[:, :k] + np.eye(A.shape[0], k)
    return qr, tau, Y


def test_rebuild_back_substitution_matches_dormqr():
    rng = np.random.default_rng(3)
    M, k, r = 400, 35, 14
    A = rng.standard_normal((M, k)) * np.logspace(0, -6, k)
    qr, tau, Y = _reflectors(A)
    X0 = rng.standard_normal((k, r))
    X = np.zeros((M, r))
    X[:k] = X0
    ref, _, info = la.dormqr("L", "N", qr, tau, X, lwork=64 * r)
    assert info == 0
    G = Y.T @ Y
    Wp = Y[:k].T @ X0
    Z = np.zeros((k, r))
    for j in range(k - 1, -1, -1):
        Z[j] = tau[j] * Wp[j]
        Wp[:j] -= np.outer(G[:j, j], Z[j])
    out = X - Y @ Z
    assert np.abs(out - ref).max() <= 1e-13 * np.abs(ref).max()
    # Householder Gram entries are at most 2 (||v||^2 = 2 / tau)
    assert np.abs(G).max() <= 2.0 + 1e-12


def test_qr_trailing_update_forward_substitution():
    rng = np.random.default_rng(5)
    M, k = 300, 35
    A = rng.standard_normal((M, k)) * np.logspace(0, -5, k)
    qr, tau, Y = _reflectors(A[:, :16])
    At = A[:, 16:].copy()
    ref = At.copy()
    for j in range(16):   # H_0 first: Q^T = H_15 ... H_0
        ref -= tau[j] * np.outer(Y[:, j], Y[:, j] @ ref)
    G = Y.T @ Y
    W = Y.T @ At
    Wp = np.zeros_like(W)
    for j in range(16):
        Wp[j] = tau[j] * (W[j] - G[j, :j] @ Wp[:j])
    out = At - Y @ Wp
    assert np.abs(out - ref).max() <= 1e-13 * np.abs(ref).max()
    # the blocked factorization's R equals dgeqrf's on the whole matrix
    qr2, _, _ = _reflectors(out[16:])
    R_full = np.triu(la.dgeqrf(A.copy())[0])[:k]
    assert np.abs(np.triu(qr)[:16] - R_full[:16, :16]).max() <= 1e-13
    assert np.abs(out[:16] - R_full[:16, 16:]).max() <= 1e-13
    assert np.abs(np.triu(qr2)[:k - 16] - R_full[16:, 16:]).max() <= 1e-13
