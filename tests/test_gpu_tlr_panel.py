"""hcore_gpu_tlr_panel_step: a whole TLR Cholesky, one library call per panel.

The matrix: 1024 seeded points in [0,1]^2, Morton-sorted, kernel
exp(-|x-y|^2/0.1) + 1e-2 I, 8 x 8 tiles of order 128, off-diagonal tiles
compressed to 1e-8 relative (storage 64 columns; ranks 1-33, up to 40 during
the factorization).  Before every panel step
the GPU's state is copied to the host and the oracle's restatement of the
same panel (oracle.tlr_panel_step: HCORE_dpotrf, HCORE_dtrsm, HCORE_dsyrk and
the recompressed HCORE_dgemm updates in HiCMA's order) is applied to that
copy, so each step is checked on identical inputs:
* POTRF info equal, the factored diagonal tile within 1e-12 of its largest
  entry, the solved panel factors within 1e-11 relative;
* every later diagonal tile within 1e-12 of its largest entry;
* every Schur update: same status and rank, product within 1e-11 relative.
After the last panel, L L^T reproduces the matrix to the compression's
accuracy.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

NT, NB, STORE, MAXRK, ACC = 8, 128, 64, 64, 1e-8


class Tlr:
    """Device storage of the TLR matrix and its hcore_tlr_matrix view."""

    def __init__(self, hc, torch, D, U, V, rank):
        self.torch = torch
        self.D = [torch.from_numpy(np.ascontiguousarray(d.T)).cuda() for d in D]
        self.U, self.V = {}, {}
        for (i, j), r in rank.items():
            u = torch.zeros((STORE, NB), dtype=torch.float64, device="cuda")
            v = torch.zeros_like(u)
            if r:
                u[:r] = torch.from_numpy(np.ascontiguousarray(U[(i, j)].T))
                v[:r] = torch.from_numpy(np.ascontiguousarray(V[(i, j)].T))
            self.U[(i, j)], self.V[(i, j)] = u, v
        self.rank = (C.c_int * (NT * NT))()
        Dp = (C.c_void_p * NT)(*[d.data_ptr() for d in self.D])
        Up = (C.c_void_p * (NT * NT))()
        Vp = (C.c_void_p * (NT * NT))()
        for (i, j), r in rank.items():
            Up[i + j * NT] = self.U[(i, j)].data_ptr()
            Vp[i + j * NT] = self.V[(i, j)].data_ptr()
            self.rank[i + j * NT] = r
        self._keep = (Dp, Up, Vp)
        self.mat = hc.TlrMatrix(nt=NT, nb=NB, D=C.cast(Dp, C.c_void_p), ldd=NB,
                                U=C.cast(Up, C.c_void_p), V=C.cast(Vp, C.c_void_p),
                                rank=C.cast(self.rank, C.c_void_p), maxrank=STORE)

    def host(self):
        D = [np.asfortranarray(d.cpu().numpy().T) for d in self.D]
        U, V, rank = {}, {}, {}
        for (i, j) in self.U:
            r = self.rank[i + j * NT]
            rank[(i, j)] = r
            U[(i, j)] = np.asfortranarray(self.U[(i, j)][:r].cpu().numpy().T)
            V[(i, j)] = np.asfortranarray(self.V[(i, j)][:r].cpu().numpy().T)
        return D, U, V, rank


def _matrix():
    from hcore_gb300 import panel as pnl

    P = pnl.morton_points(NT * NB, 2, 3)
    A = pnl._kernel_np(P, P, "sqexp", 0.1) + 1e-2 * np.eye(NT * NB)
    tiles = [(i, j) for j in range(NT) for i in range(j + 1, NT)]
    comp = pnl.compress_tiles(P, NB, tiles, "sqexp", 0.1, ACC, STORE, seed=3, workers=4)
    U, V, rank = {}, {}, {}
    for t, (Ut, Vt, r) in zip(tiles, comp):
        U[t], V[t], rank[t] = np.asfortranarray(Ut.T), np.asfortranarray(Vt.T), r
    D = [np.asfortranarray(A[i * NB:(i + 1) * NB, i * NB:(i + 1) * NB]) for i in range(NT)]
    return A, D, U, V, rank


def test_tlr_cholesky_panel_by_panel_against_oracle(hc, port):
    import torch

    A, D, U, V, rank = _matrix()
    tlr = Tlr(hc, torch, D, U, V, rank)
    L = hc.lib()
    for k in range(NT):
        hD, hU, hV, hr = tlr.host()
        info_ref, st_ref = O.tlr_panel_step(port, hD, hU, hV, hr, k, ACC, MAXRK, STORE)
        info = C.c_int(-1)
        status = (C.c_int * (NT * NT))()
        rc = L.hcore_gpu_tlr_panel_step(C.byref(tlr.mat), k, ACC, MAXRK, C.byref(info), status,
                                        None)
        assert rc == 0, hc.last_error()
        assert info.value == info_ref == 0
        gD, gU, gV, gr = tlr.host()
        tol = lambda x: 1e-12 * max(np.abs(x).max(), 1e-300)  # noqa: E731
        assert np.abs(np.tril(gD[k]) - np.tril(hD[k])).max() <= tol(hD[k])
        for i in range(k + 1, NT):
            np.testing.assert_allclose(gD[i], hD[i], rtol=0, atol=tol(hD[i]))
            if hr[(i, k)]:
                assert O.rel_fro(gV[(i, k)], hV[(i, k)]) < 1e-11
        for (i, j), s in st_ref.items():
            assert status[i + j * NT] == s == 0
            assert gr[(i, j)] == hr[(i, j)], (k, i, j)
            P = gU[(i, j)] @ gV[(i, j)].T
            assert O.rel_fro(P, hU[(i, j)] @ hV[(i, j)].T) < 1e-11, (k, i, j)
    # L L^T = A to the compression's accuracy
    gD, gU, gV, gr = tlr.host()
    Lf = np.zeros_like(A)
    for i in range(NT):
        Lf[i * NB:(i + 1) * NB, i * NB:(i + 1) * NB] = np.tril(gD[i])
        for j in range(i):
            Lf[i * NB:(i + 1) * NB, j * NB:(j + 1) * NB] = gU[(i, j)] @ gV[(i, j)].T
    assert O.rel_fro(Lf @ Lf.T, A) < 1e-7


def test_tlr_panel_step_rejects_bad_arguments(hc):
    import torch

    A, D, U, V, rank = _matrix()
    tlr = Tlr(hc, torch, D, U, V, rank)
    L = hc.lib()
    info = C.c_int(0)
    assert L.hcore_gpu_tlr_panel_step(C.byref(tlr.mat), NT, ACC, MAXRK, C.byref(info), None,
                                      None) == -1
    tlr.rank[1] = STORE + 1                       # tile (1, 0) above its storage
    assert L.hcore_gpu_tlr_panel_step(C.byref(tlr.mat), 0, ACC, MAXRK, C.byref(info), None,
                                      None) == -1
    assert "storage" in hc.last_error()
