"""The tile steps either side of the Schur update on the GPU: HCORE_dtrsm,
HCORE_dpotrf, HCORE_duncompress and HCORE_dgemmbdcd (drop-in entry points and
batched API), against the reference's fixtures and the oracle.

Tolerances: these are FP64 solves and products whose summation order differs
from the BLAS the reference calls; every case is well conditioned
(triangles with |diagonal| in [2, 3], SPD matrices X X^T / n + I), so results
agree to 1e-12 relative to the largest entry (1e-13 for plain products).
"""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

dp = C.POINTER(C.c_double)
LEFT, RIGHT, UPPER, LOWER, NOTRANS, TRANS, NONUNIT, UNIT = 141, 142, 121, 122, 111, 112, 131, 132


def _close(x, y, tol):
    """Equal NaN pattern; finite entries within tol relative to max |y|."""
    x, y = np.asarray(x), np.asarray(y)
    assert np.array_equal(np.isnan(x), np.isnan(y))
    f = ~np.isnan(y)
    scale = max(np.abs(y[f]).max(initial=0.0), 1.0)
    err = np.abs(x[f] - y[f]).max(initial=0.0)
    assert err <= tol * scale, (err, scale)


def _p(a):
    return a.ctypes.data_as(dp)


def test_dropins_match_reference_fixtures(hc, golden_tlr):
    """Host-memory drop-in calls reproduce the reference's outputs, ranks of
    zero, both gemmbdcd row-count branches, every trsm case and potrf's info
    (including HCORE_Lower passed as uplo, which LAPACKE rejects)."""
    meta, g = golden_tlr
    L = hc.lib()
    for c in meta["uncompress"]:
        n = c["name"]
        AU, BV = g[f"{n}_AU"], g[f"{n}_BV"]
        CD = np.asfortranarray(g[f"{n}_CD"]).copy(order="F")
        ra = np.array([c["a"]], dtype=np.float64)
        L.HCORE_duncompress(NOTRANS, TRANS, c["M"], c["N"], 1.0, _p(AU), _p(ra), AU.shape[0],
                            _p(BV), _p(ra), BV.shape[0], 0.0, _p(CD), CD.shape[0])
        _close(CD, g[f"{n}_CDo"], 1e-13)
    for c in meta["gemmbdcd"]:
        n = c["name"]
        AU, AV, BD = g[f"{n}_AU"], g[f"{n}_AV"], g[f"{n}_BD"]
        CD = np.asfortranarray(g[f"{n}_CD"]).copy(order="F")
        ra = np.array([c["a"]], dtype=np.float64)
        fc = hc.FlopCounter()
        L.HCORE_dgemmbdcd(c["transA"], NOTRANS, c["M"], c["N"], c["alpha"], _p(AU), _p(AV), _p(ra),
                          AU.shape[0], _p(BD), BD.shape[0], c["beta"], _p(CD), CD.shape[0], None,
                          C.byref(fc))
        _close(CD, g[f"{n}_CDo"], 1e-13)
        assert fc.update == c["flops"]
    for c in meta["trsm"]:
        n = c["name"]
        A = g[f"{n}_A"]
        B = np.asfortranarray(g[f"{n}_B"]).copy(order="F")
        fc = hc.FlopCounter()
        L.HCORE_dtrsm(c["side"], c["uplo"], c["trans"], c["diag"], c["M"], c["N"], c["alpha"], _p(A),
                      A.shape[0], _p(B), B.shape[0], C.byref(fc))
        _close(B, g[f"{n}_Bo"], 1e-12)
        assert fc.trsm == c["flops"]
    for c in meta["potrf"]:
        n = c["name"]
        A = np.asfortranarray(g[f"{n}_A"]).copy(order="F")
        info = C.c_int(99)
        fc = hc.FlopCounter()
        L.HCORE_dpotrf(c["uplo"], c["n"], _p(A), A.shape[0], C.byref(info), C.byref(fc))
        assert info.value == c["info"] and fc.potrf == c["flops"]
        ref = g[f"{n}_Ao"]
        if c["info"] == 0:
            _close(A, ref, 1e-12)
        elif c["info"] > 0:
            # the leading factored block and the failing pivot left in place;
            # how much of the rest a blocked LAPACK has touched varies
            j = c["info"] - 1
            _close(np.tril(A[:j, :j]), np.tril(ref[:j, :j]), 1e-12)
            assert abs(A[j, j] - ref[j, j]) <= 1e-12 * abs(ref[j, j])
        else:
            assert np.array_equal(np.isnan(A), np.isnan(ref))
            assert np.array_equal(A[~np.isnan(A)], ref[~np.isnan(ref)])   # untouched


def _triangle(rng, n, uplo, unit):
    T = rng.uniform(-0.5, 0.5, (n, n)) / np.sqrt(n)
    np.fill_diagonal(T, rng.uniform(2, 3, n) * rng.choice([-1.0, 1.0], n))
    keep = np.tril(np.ones((n, n), bool)) if uplo == LOWER else np.triu(np.ones((n, n), bool))
    T = np.where(keep, T, np.nan)          # the other triangle must not be read
    if unit:
        np.fill_diagonal(T, np.nan)        # nor the diagonal of a unit triangle
    return np.asfortranarray(T)


def _spd(rng, n):
    X = rng.standard_normal((n, n))
    return np.asfortranarray(X @ X.T / n + np.eye(n))


def test_trsm_batched_every_case_multiblock(hc, port):
    """All 16 side/uplo/trans/diag cases in one batch, triangles of order 300
    (ragged last block), alpha = -0.75; an alpha = 0 task zeroes B without
    reading A; empty tasks are skipped."""
    import torch
    from hcore_gb300 import devmem

    rng = np.random.default_rng(71)
    tasks, keep, refs = [], [], []
    for side in (LEFT, RIGHT):
        for uplo in (UPPER, LOWER):
            for tr in (NOTRANS, TRANS):
                for dg in (NONUNIT, UNIT):
                    M, N = (300, 37) if side == LEFT else (45, 300)
                    na = M if side == LEFT else N
                    A = _triangle(rng, na, uplo, dg == UNIT)
                    B = np.asfortranarray(rng.standard_normal((M, N)))
                    ref, _ = port.dtrsm(side, uplo, tr, dg, M, N, -0.75, A, B)
                    dA, dB = devmem.to_device(A), devmem.to_device(B)
                    keep += [dA, dB]
                    tasks.append(hc.TrsmTask(side=side, uplo=uplo, trans=tr, diag=dg, M=M, N=N,
                                             alpha=-0.75, A=dA.data_ptr(), lda=na, B=dB.data_ptr(),
                                             ldb=M))
                    refs.append((dB, N, ref))
    Anan = np.full((64, 64), np.nan, order="F")
    dAn = devmem.to_device(Anan)
    dB0 = devmem.to_device(np.asfortranarray(rng.standard_normal((64, 5))))
    tasks.append(hc.TrsmTask(side=LEFT, uplo=LOWER, trans=NOTRANS, diag=NONUNIT, M=64, N=5,
                             alpha=0.0, A=dAn.data_ptr(), lda=64, B=dB0.data_ptr(), ldb=64))
    tasks.append(hc.TrsmTask(side=LEFT, uplo=LOWER, trans=NOTRANS, diag=NONUNIT, M=64, N=0,
                             alpha=1.0, A=dAn.data_ptr(), lda=64, B=dB0.data_ptr(), ldb=64))
    hc.trsm_batched(tasks)
    for dB, N, ref in refs:
        _close(devmem.to_host(dB, N), ref, 1e-12)
    assert float(dB0.abs().max()) == 0.0
    del keep, torch


def test_trsm_batched_tlr_panel(hc, port):
    """The TLR Cholesky use: 40 V factors (nb = 1024, ranks 1..70) solved
    against one diagonal tile's Cholesky factor in one call."""
    import torch

    rng = np.random.default_rng(72)
    nb = 1024
    Lf, info, _ = port.dpotrf(ord("L"), nb, _spd(rng, nb))
    assert info == 0
    Lf = np.asfortranarray(np.tril(Lf))
    dL = torch.from_numpy(np.ascontiguousarray(Lf.T)).cuda()        # column-major L
    ranks = rng.integers(1, 71, 40)
    Vs = [np.asfortranarray(rng.standard_normal((nb, int(r)))) for r in ranks]
    dV = [torch.from_numpy(np.ascontiguousarray(V.T)).cuda() for V in Vs]
    hc.trsm_batched([hc.TrsmTask(side=LEFT, uplo=LOWER, trans=NOTRANS, diag=NONUNIT, M=nb,
                                 N=int(r), alpha=1.0, A=dL.data_ptr(), lda=nb, B=d.data_ptr(),
                                 ldb=nb) for r, d in zip(ranks, dV)])
    for V, d in zip(Vs, dV):
        ref, _ = port.dtrsm(LEFT, LOWER, NOTRANS, NONUNIT, nb, V.shape[1], 1.0, Lf, V)
        _close(d.cpu().numpy().T, ref, 1e-12)


def test_potrf_batched_sizes_failures_and_arguments(hc, port):
    """One batch: orders 1, 63, 64, 65, 130, 1024 in both triangles (the other
    triangle NaN, untouched), a matrix whose leading minor of order 77 is not
    positive definite (info 77, as LAPACK) and an invalid uplo (info -2,
    matrix untouched)."""
    import torch

    rng = np.random.default_rng(73)
    cases = []
    for n in (1, 63, 64, 65, 130, 1024):
        for up in ("L", "U"):
            cases.append((ord(up), n, None))
    cases += [(ord("L"), 200, 77), (ord("U"), 150, 3), (LOWER, 40, None)]
    tasks, dev, refs = [], [], []
    for uplo, n, fail in cases:
        S = _spd(rng, n)
        if fail is not None:
            S[fail - 1, fail - 1] = -1.0
        other = np.tril(np.ones((n, n), bool), -1) if uplo == ord("U") else np.triu(np.ones((n, n), bool), 1)
        S = np.asfortranarray(np.where(other, np.nan, S))
        ref, info, _ = port.dpotrf(uplo, n, S)
        d = torch.from_numpy(np.ascontiguousarray(S.T)).cuda()
        dev.append(d)
        tasks.append(hc.PotrfTask(uplo=uplo, n=n, A=d.data_ptr(), lda=n))
        refs.append((S, ref, info))
    infos = hc.potrf_batched(tasks)
    for (uplo, n, fail), d, (S, ref, info), got in zip(cases, dev, refs, infos):
        out = d.cpu().numpy().T
        assert got == info, (uplo, n, fail, got, info)
        if info == 0:
            _close(out, ref, 1e-12)
        elif info > 0:  # the leading factored block and the failing pivot
            j = info - 1
            tri = np.tril if uplo == ord("L") else np.triu
            _close(tri(out[:j, :j]), tri(ref[:j, :j]), 1e-12)
            assert abs(out[j, j] - ref[j, j]) <= 1e-12 * abs(ref[j, j])
        else:
            assert np.array_equal(np.isnan(out), np.isnan(S))
            assert np.array_equal(out[~np.isnan(out)], S[~np.isnan(S)])
    assert list(infos[-3:]) == [77, 3, -2]


def test_dense_batched_uncompress_and_gemmbdcd_in_list_order(hc, port):
    """Tasks of all four kinds in one batch: two syrk/gemmcd on a square tile;
    on a 150 x 90 tile a gemmbdcd with beta = 0 over a NaN tile (not read),
    a second gemmbdcd (kdim 70 != M), an uncompress that overwrites it all and
    a last gemmbdcd; the result equals the oracle applied in list order."""
    import torch
    from hcore_gb300 import devmem

    rng = np.random.default_rng(74)
    keep = []

    def dv(x):
        d = devmem.to_device(np.asfortranarray(x))
        keep.append(d)
        return d.data_ptr()

    M, N = 150, 90
    CD = np.full((M, N), np.nan, order="F")
    dCD = devmem.to_device(CD)
    ref = CD.copy(order="F")
    tasks = []
    for i, (kind, a, kdim, alpha, beta) in enumerate([(3, 9, M, 0.5, 0.0), (3, 12, 70, -1.0, 0.75),
                                                     (2, 6, 0, 0.0, 0.0), (3, 4, M, 2.0, -1.0)]):
        if kind == 2:
            AU, BV = rng.standard_normal((M, a)), rng.standard_normal((N, a))
            ref = port.duncompress(M, N, AU, a, BV, ref)
            tasks.append(hc.DenseTask(kind=2, M=M, N=N, a=a, Au=dv(AU), lda=M, Bv=dv(BV), ldb=N,
                                      CD=dCD.data_ptr(), ldcd=M))
        else:
            lda = max(M, kdim) + 3
            AU, AV = rng.standard_normal((lda, a)), rng.standard_normal((lda, a))
            BD = rng.standard_normal((kdim, N))
            # the oracle's non-transposed branch sums over LDB = kdim rows
            ref, _ = port.dgemmbdcd(NOTRANS, M, N, alpha, AU, AV, a, BD, beta, ref)
            tasks.append(hc.DenseTask(kind=3, M=M, N=N, a=a, alpha=alpha, beta=beta, kdim=kdim,
                                      Au=dv(AU), Av=dv(AV), lda=lda, Bd=dv(BD), ldb=kdim,
                                      CD=dCD.data_ptr(), ldcd=M))
    # a square tile with a syrk and a gemmcd in the same batch
    Ms = 96
    CS = np.asfortranarray(np.tril(rng.standard_normal((Ms, Ms))))
    dCS = devmem.to_device(CS)
    AUs, AVs = rng.standard_normal((Ms, 7)), rng.standard_normal((Ms, 7))
    refS, _ = port.dsyrk(Ms, 7, -1.0, AUs, AVs, CS)
    Au, Av, Bu, Bv = (rng.standard_normal((Ms, r)) for r in (5, 5, 8, 8))
    refS = port.dgemmcd(Ms, Au, Av, 5, Bu, Bv, 8, refS)
    tasks.insert(1, hc.DenseTask(kind=0, M=Ms, a=7, alpha=-1.0, Au=dv(AUs), Av=dv(AVs), lda=Ms,
                                 CD=dCS.data_ptr(), ldcd=Ms))
    tasks.append(hc.DenseTask(kind=1, M=Ms, a=5, b=8, alpha=-1.0, Au=dv(Au), Av=dv(Av), lda=Ms,
                              Bu=dv(Bu), Bv=dv(Bv), ldb=Ms, CD=dCS.data_ptr(), ldcd=Ms))
    hc.dense_batched(tasks)
    _close(devmem.to_host(dCD, N), ref, 1e-13)
    _close(devmem.to_host(dCS, Ms), refS, 1e-13)
    del keep, torch
