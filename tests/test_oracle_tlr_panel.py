"""The oracle's panel-step restatement (oracle.tlr_panel_step) on the CPU: a
whole TLR Cholesky of a small covariance matrix, panel by panel, reproduces
the matrix as L L^T to the compression's accuracy.  This pins the sequence
(POTRF, TRSM of the V factors, SYRK, recompressed GEMM updates) that the GPU
panel step is compared with."""
import numpy as np

from oracle import oracle as O


def test_oracle_tlr_cholesky_reproduces_the_matrix(port):
    from hcore_gb300 import panel as pnl

    nt, nb, store, acc = 8, 128, 64, 1e-8
    P = pnl.morton_points(nt * nb, 2, 3)
    A = pnl._kernel_np(P, P, "sqexp", 0.1) + 1e-2 * np.eye(nt * nb)
    tiles = [(i, j) for j in range(nt) for i in range(j + 1, nt)]
    comp = pnl.compress_tiles(P, nb, tiles, "sqexp", 0.1, acc, store, seed=3, workers=2)
    U, V, rank = {}, {}, {}
    for t, (Ut, Vt, r) in zip(tiles, comp):
        U[t], V[t], rank[t] = np.asfortranarray(Ut.T), np.asfortranarray(Vt.T), r
    D = [np.asfortranarray(A[i * nb:(i + 1) * nb, i * nb:(i + 1) * nb]) for i in range(nt)]
    for k in range(nt):
        info, status = O.tlr_panel_step(port, D, U, V, rank, k, acc, store, store)
        assert info == 0
        assert all(s == 0 for s in status.values())
    L = np.zeros_like(A)
    for i in range(nt):
        L[i * nb:(i + 1) * nb, i * nb:(i + 1) * nb] = np.tril(D[i])
        for j in range(i):
            L[i * nb:(i + 1) * nb, j * nb:(j + 1) * nb] = U[(i, j)] @ V[(i, j)].T
    assert O.rel_fro(L @ L.T, A) < 1e-7
