"""HCORE_zgemm (complex update) on the GPU against the reference's fixtures and
the dense restatement.

The library runs the complex update as a real update of twice the order and
ranks (X -> [Re X, -Im X; Im X, Re X]) through the FP64 plan, then takes one
complex vector per pair of equal singular values.  Gates: the rank equals the
reference's, the product agrees to 1e-11 relative Frobenius, the flop count
equals the reference's; CU has orthonormal columns and CV carries the singular
values.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _clr(rng, M, k, decades):
    U, _ = np.linalg.qr(rng.standard_normal((M, k)) + 1j * rng.standard_normal((M, k)))
    V, _ = np.linalg.qr(rng.standard_normal((M, k)) + 1j * rng.standard_normal((M, k)))
    return np.asfortranarray(U * 10.0 ** (-decades * np.arange(k) / k)), np.asfortranarray(V)


def _rel(P, Q):
    return np.linalg.norm(P - Q) / np.linalg.norm(Q)


def test_zgemm_matches_reference_fixtures(hc, golden_zgemm):
    meta, g = golden_zgemm
    for c in meta:
        n = c["name"]
        r, CU, CV, fl = hc.hcore_zgemm(c["M"], complex(*c["alpha"]), g[f"{n}_AU"], g[f"{n}_AV"],
                                       c["a"], g[f"{n}_BU"], g[f"{n}_BV"], c["b"],
                                       complex(*c["beta"]), g[f"{n}_CU"], g[f"{n}_CV"], c["c"],
                                       rk=c["rk"], maxrk=c["maxrk"], acc=c["acc"])
        assert r == c["rank"], (n, r, c["rank"])
        assert _rel(CU @ CV.T, g[f"{n}_CUo"] @ g[f"{n}_CVo"].T) < 1e-11, n
        assert fl == c["flops"]
        assert np.abs(CU.conj().T @ CU - np.eye(r)).max() < 1e-12
        sv_ref = np.linalg.norm(g[f"{n}_CVo"], axis=0)
        assert np.allclose(np.linalg.norm(CV, axis=0), sv_ref, rtol=1e-10, atol=1e-15)


@pytest.mark.parametrize("M,a,c", [(512, 32, 32), (1024, 20, 24)])
def test_zgemm_large_against_dense_truncation(hc, M, a, c):
    """Orders 512 and 1024 (the largest, a real order of 2048) against the
    dense restatement; the inputs' singular values are graded, so none lies
    near the threshold (checked)."""
    rng = np.random.default_rng(M + a)
    AU, AV = _clr(rng, M, a, 10)
    BU, BV = _clr(rng, M, a, 10)
    CU, CV = _clr(rng, M, c, 10)
    rr, P, S = O.zgemm_dense_truncation(-1.0, AU, AV, BU, BV, 1.0, CU, CV, acc=1e-8)
    assert np.all(np.abs(S - 1e-8) > 1e-3 * 1e-8)
    r, CUo, CVo, _ = hc.hcore_zgemm(M, -1.0, AU, AV, a, BU, BV, a, 1.0, CU, CV, c, maxrk=2 * (a + c),
                                    acc=1e-8)
    assert r == rr
    assert _rel(CUo @ CVo.T, P) < 1e-11


def test_zgemm_repeated_singular_values(hc):
    """C = Q Q2^T with all its singular values equal (a cluster of
    multiplicity 6, split only by an A B^T of size 1e-13, below acc): in the
    real embedding the 12 equal values mix freely, and the complex factors
    still come out with the rank and the product of the dense restatement."""
    rng = np.random.default_rng(91)
    M, a, c = 128, 3, 6
    Q, _ = np.linalg.qr(rng.standard_normal((M, c)) + 1j * rng.standard_normal((M, c)))
    Q2, _ = np.linalg.qr(rng.standard_normal((M, c)) + 1j * rng.standard_normal((M, c)))
    AU, AV = _clr(rng, M, a, 4)
    BU, BV = _clr(rng, M, a, 4)
    AU *= 1e-13
    rr, P, _ = O.zgemm_dense_truncation(1.0, AU, AV, BU, BV, 1.0, Q, Q2, acc=1e-10)
    assert rr == c
    r, CUo, CVo, _ = hc.hcore_zgemm(M, 1.0, AU, AV, a, BU, BV, a, 1.0, np.asfortranarray(Q),
                                    np.asfortranarray(Q2), c, maxrk=2 * (a + c), acc=1e-10)
    assert r == rr
    assert _rel(CUo @ CVo.T, P) < 1e-11


def test_zgemm_device_memory_inputs(hc, golden_zgemm):
    """The same entry point with the factors in device memory."""
    import ctypes as C

    import torch

    meta, g = golden_zgemm
    c = meta[1]
    n = c["name"]
    M = c["M"]
    dev = {k: torch.from_numpy(np.ascontiguousarray(g[f"{n}_{k}"].T)).cuda()
           for k in ("AU", "AV", "BU", "BV")}
    k = c["a"] + c["c"]
    CU = torch.zeros((k, M), dtype=torch.complex128, device="cuda")
    CV = torch.zeros_like(CU)
    CU[:c["c"]] = torch.from_numpy(np.ascontiguousarray(g[f"{n}_CU"].T)).cuda()
    CV[:c["c"]] = torch.from_numpy(np.ascontiguousarray(g[f"{n}_CV"].T)).cuda()
    ra, rb, rc = (np.array([v], dtype=np.float64) for v in (c["a"], c["b"], c["c"]))
    dp = C.POINTER(C.c_double)
    fc = hc.FlopCounter()
    hc.lib().HCORE_zgemm(111, 112, M, M, hc.DComplex(*c["alpha"]), dev["AU"].data_ptr(),
                         dev["AV"].data_ptr(), ra.ctypes.data_as(dp), M, dev["BU"].data_ptr(),
                         dev["BV"].data_ptr(), rb.ctypes.data_as(dp), M, hc.DComplex(*c["beta"]),
                         CU.data_ptr(), CV.data_ptr(), rc.ctypes.data_as(dp), M, c["rk"],
                         c["maxrk"], c["acc"], None, C.byref(fc))
    r = int(rc[0])
    assert r == c["rank"]
    P = CU[:r].cpu().numpy().T @ CV[:r].cpu().numpy()
    assert _rel(P, g[f"{n}_CUo"] @ g[f"{n}_CVo"].T) < 1e-11


def test_zuncompress_matches_reference(hc, golden_zgemm):
    """HCORE_zuncompress (CD = AU BV^T, complex) against the reference's output."""
    import ctypes as C

    _, g = golden_zgemm
    AU, BV = g["zunc_AU"], g["zunc_BV"]
    M, r = AU.shape
    N = BV.shape[0]
    CD = np.zeros((M, N), dtype=np.complex128, order="F")
    ra = np.array([r], dtype=np.float64)
    dp = C.POINTER(C.c_double)
    hc.lib().HCORE_zuncompress(111, 112, M, N, hc.DComplex(1, 0), AU.ctypes.data,
                               ra.ctypes.data_as(dp), M, BV.ctypes.data, ra.ctypes.data_as(dp), N,
                               hc.DComplex(0, 0), CD.ctypes.data, M)
    assert np.abs(CD - g["zunc_CDo"]).max() <= 1e-13 * np.abs(g["zunc_CDo"]).max()


def test_zgemm_batched_against_port(hc, port):
    """40 complex updates of mixed ranks in one batch (one real plan), one of
    them with a degenerate singular-value cluster (extraction falls back to
    Gram-Schmidt), and one with a zero rank (status, the rest unaffected):
    every rank and product equals the restated reference's."""
    rng = np.random.default_rng(92)
    M, maxrk = 256, 64
    tasks, keep, refs = [], [], []
    for q in range(40):
        a, b, c = (int(x) for x in rng.integers(1, 16, 3))
        AU, AV = _clr(rng, M, a, 8)
        BU, BV = _clr(rng, M, b, 8)
        if q == 7:   # all of C's singular values equal, A B^T far below acc
            CU, _ = np.linalg.qr(rng.standard_normal((M, c)) + 1j * rng.standard_normal((M, c)))
            CV, _ = np.linalg.qr(rng.standard_normal((M, c)) + 1j * rng.standard_normal((M, c)))
            CU, CV = np.asfortranarray(CU), np.asfortranarray(CV)
            AU = np.asfortranarray(AU * 1e-13)
        else:
            CU, CV = _clr(rng, M, c, 8)
        alpha, beta = complex(rng.standard_normal(), rng.standard_normal()), 1.0
        ref = port.zgemm(M, alpha, AU, AV, a, BU, BV, b, beta, CU, CV, c, maxrk=maxrk, acc=1e-8)
        oU = np.zeros((M, maxrk), dtype=np.complex128, order="F")
        oV = np.zeros_like(oU)
        oU[:, :c], oV[:, :c] = CU, CV
        if q == 11:
            c = 0  # zero rank: status 1
        keep += [AU, AV, BU, BV, oU, oV]
        tasks.append(hc.ZlrTask(M=M, a=a, b=b, c=c, rk=0, maxrk=maxrk,
                                alpha=hc.DComplex(alpha.real, alpha.imag), beta=hc.DComplex(1, 0),
                                acc=1e-8, AU=AU.ctypes.data, AV=AV.ctypes.data, lda=M,
                                BU=BU.ctypes.data, BV=BV.ctypes.data, ldb=M, CU=oU.ctypes.data,
                                CV=oV.ctypes.data, ldc=M))
        refs.append((ref, oU, oV))
    ranks, status = hc.zgemm_batched(tasks)
    for q, ((ref, oU, oV), r, st) in enumerate(zip(refs, ranks, status)):
        if q == 11:
            assert st == 1
            continue
        assert st == 0 and r == ref["rank"], (q, st, r, ref["rank"])
        assert _rel(oU[:, :r] @ oV[:, :r].T, ref["CU"] @ ref["CV"].T) < 1e-11, q


def test_zgemm_batched_device_and_pinned_memory(hc):
    """The batched complex path reads its inputs where they are (device or
    pinned host memory, through the embedding kernel) and packs pageable ones;
    outputs go back to device or host memory.  The same tasks with their
    factors in pageable host, pinned host and device memory give identical
    ranks and bits."""
    import torch

    rng = np.random.default_rng(93)
    M, maxrk, n = 192, 48, 6
    cases = []
    for q in range(n):
        a, b, c = (int(x) for x in rng.integers(2, 14, 3))
        cases.append((a, b, c) + _clr(rng, M, a, 8) + _clr(rng, M, b, 8) + _clr(rng, M, c, 8))

    def run(where):
        keep, tasks = [], []
        for (a, b, c, AU, AV, BU, BV, CU, CV) in cases:
            oU = np.zeros((M, maxrk), dtype=np.complex128, order="F")
            oV = np.zeros_like(oU)
            oU[:, :c], oV[:, :c] = CU, CV
            arrs = [AU, AV, BU, BV, oU, oV]
            if where == "device":
                arrs = [torch.from_numpy(np.ascontiguousarray(x.T)).cuda() for x in arrs]
                ptr = [x.data_ptr() for x in arrs]
            elif where == "pinned":
                arrs = [torch.from_numpy(np.ascontiguousarray(x.T)).pin_memory() for x in arrs]
                ptr = [x.data_ptr() for x in arrs]
            else:
                ptr = [x.ctypes.data for x in arrs]
            keep.append(arrs)
            tasks.append(hc.ZlrTask(M=M, a=a, b=b, c=c, rk=0, maxrk=maxrk,
                                    alpha=hc.DComplex(-1, 0), beta=hc.DComplex(1, 0), acc=1e-8,
                                    AU=ptr[0], AV=ptr[1], lda=M, BU=ptr[2], BV=ptr[3], ldb=M,
                                    CU=ptr[4], CV=ptr[5], ldc=M))
        ranks, status = hc.zgemm_batched(tasks)
        outs = []
        for arrs, r in zip(keep, ranks):
            oU, oV = arrs[4], arrs[5]
            if where in ("device", "pinned"):
                oU, oV = oU.cpu().numpy().T, oV.cpu().numpy().T
            outs.append((oU[:, :r].copy(), oV[:, :r].copy()))
        return ranks.copy(), status.copy(), outs

    r0, s0, o0 = run("pageable")
    assert (s0 == 0).all()
    for where in ("pinned", "device"):
        r1, s1, o1 = run(where)
        assert np.array_equal(r0, r1) and np.array_equal(s0, s1), where
        for (u0, v0), (u1, v1) in zip(o0, o1):
            assert np.array_equal(u0, u1) and np.array_equal(v0, v1), where


def test_zgemm_native_kernels_match_the_embedding(hc, port):
    """The native complex kernels (rank sums up to the shared-memory limit)
    and the order-2M real embedding (HCORE_GPU_ZGEMM_EMBED=1 forces it) give
    the same ranks and products (1e-11), both equal to the restated
    reference's; the native factors are orthonormal in CU."""
    import os

    rng = np.random.default_rng(94)
    M, maxrk = 320, 80
    cases = []
    for q in range(12):
        a, b, c = (int(x) for x in rng.integers(1, 40, 3))
        cases.append((a, b, c, complex(rng.standard_normal(), rng.standard_normal()))
                     + _clr(rng, M, a, 8) + _clr(rng, M, b, 8) + _clr(rng, M, c, 8))

    def run():
        keep, tasks = [], []
        for (a, b, c, al, AU, AV, BU, BV, CU, CV) in cases:
            oU = np.zeros((M, maxrk), dtype=np.complex128, order="F")
            oV = np.zeros_like(oU)
            oU[:, :c], oV[:, :c] = CU, CV
            keep.append((oU, oV))
            tasks.append(hc.ZlrTask(M=M, a=a, b=b, c=c, rk=0, maxrk=maxrk,
                                    alpha=hc.DComplex(al.real, al.imag), beta=hc.DComplex(1, 0),
                                    acc=1e-8, AU=AU.ctypes.data, AV=AV.ctypes.data, lda=M,
                                    BU=BU.ctypes.data, BV=BV.ctypes.data, ldb=M, CU=oU.ctypes.data,
                                    CV=oV.ctypes.data, ldc=M))
        ranks, status = hc.zgemm_batched(tasks)
        return ranks.copy(), status.copy(), [(u[:, :r].copy(), v[:, :r].copy())
                                             for (u, v), r in zip(keep, ranks)]

    rn, sn, on = run()
    os.environ["HCORE_GPU_ZGEMM_EMBED"] = "1"
    try:
        re_, se, oe = run()
    finally:
        del os.environ["HCORE_GPU_ZGEMM_EMBED"]
    assert (sn == 0).all() and (se == 0).all()
    assert np.array_equal(rn, re_)
    for q, ((a, b, c, al, AU, AV, BU, BV, CU, CV), (un, vn), (ue, ve)) in enumerate(zip(cases, on, oe)):
        ref = port.zgemm(M, al, AU, AV, a, BU, BV, b, 1.0, CU, CV, c, maxrk=maxrk, acc=1e-8)
        assert rn[q] == ref["rank"], q
        Pr = ref["CU"] @ ref["CV"].T
        assert _rel(un @ vn.T, Pr) < 1e-11, q
        assert _rel(ue @ ve.T, Pr) < 1e-11, q
        r = int(rn[q])
        assert np.abs(un.conj().T @ un - np.eye(r)).max() < 1e-12, q
