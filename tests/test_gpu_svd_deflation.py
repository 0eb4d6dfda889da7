"""Deflation in the FP64 SVD of the core matrix (gesvd_kernel, hc_kernels.cu).

The pivoted QR of T = R_A R_B^T stops at the first step whose trailing block
has Frobenius norm at most delta = min(1e-13 acc, 1e-16 ||T||_F), and the
Jacobi sweeps rotate the leading rows of R only.  Against the oracle (the
reference's LAPACK sequence, dgesvd of the same core at hcore_dgemm.c:403-406):
* rank equal;
* product CU CV^T within 1e-11 relative;
* every singular value within 1e-13 sigma_max of LAPACK's;
* the dropped directions come out as exact zeros (the deflation ran), and
  only where LAPACK's singular values lie below delta.
The factors' spectra span 30 decades, so that part of every core lies far
below delta, as in the far-field tiles of a TLR panel.  Rank sums cover the
SVD layouts with both matrices in shared memory (k <= 119) and with V_J in
the workspace (k > 119).
"""
import numpy as np
import pytest

from oracle import oracle as O
from test_gpu_parity import FP64_TOL, _batch_case, _run_batch

pytestmark = pytest.mark.gpu

ACC = 1e-8


def _check(cases, batch, ranks, status, outs, port, expect_zeros=True):
    assert (status == 0).all()
    for i, (cs, r, (CUo, CVo)) in enumerate(zip(cases, ranks, outs)):
        AU, AV, BU, BV, CU, CV = cs["arrays"]
        M, a, b, c = cs["M"], cs["a"], cs["b"], cs["c"]
        ref = port.gemm(M, -1.0, AU, AV, a, BU, BV, b, 1.0, CU, CV, c, maxrk=cs["maxrk"],
                        acc=ACC)
        assert int(r) == ref["rank"], (a, b, c, int(r), ref["rank"])
        assert O.rel_fro(CUo @ CVo.T, ref["CU"] @ ref["CV"].T) < FP64_TOL
        sig, sref = batch.sigma(i), np.asarray(ref["sigma"])
        smax = sref[0]
        assert np.abs(sig - sref).max() <= 1e-13 * smax
        zero = sig == 0.0
        if expect_zeros:
            assert zero.any(), (a, b, c)
        assert (sref[zero] <= 1e-13 * ACC + 1e-15 * smax).all()


@pytest.mark.parametrize("M,abc", [(256, [(6, 5, 7), (20, 18, 22), (32, 30, 32)]),
                                   (512, [(28, 26, 36), (60, 40, 64)])])
def test_deflated_svd_vs_oracle(hc, port, M, abc):
    rng = np.random.default_rng(900 + M)
    cases = []
    for a, b, c in abc:
        cases.append(dict(M=M, a=a, b=b, c=c, alpha=-1.0, beta=1.0, maxrk=a + c, acc=ACC,
                          arrays=_batch_case(rng, M, a, b, c, decades=30.0)))
    _check(cases, *_run_batch(hc, cases), port)


def test_every_singular_value_below_threshold(hc, port):
    """A far-field update: every singular value below acc.  The rank rule
    keeps its first column (hcore_dgemm.c:446-463 starts the search at 1),
    so the QR keeps at least one step."""
    rng = np.random.default_rng(41)
    cases = []
    for a, b, c in [(10, 9, 12), (24, 20, 30)]:
        AU, AV, BU, BV, CU, CV = _batch_case(rng, 256, a, b, c, decades=12.0)
        cases.append(dict(M=256, a=a, b=b, c=c, alpha=-1.0, beta=1.0, maxrk=a + c, acc=ACC,
                          arrays=(AU * 1e-7, AV, BU, BV, CU * 1e-12, CV)))
    batch, ranks, status, outs = _run_batch(hc, cases)
    assert (ranks == 1).all()
    _check(cases, batch, ranks, status, outs, port)


def test_wide_spectrum_keeps_full_rank_part(hc, port):
    """Spectra of 8 decades at acc 1e-8 keep most singular values above the
    deflation bound: results as the oracle's, zeros only below the bound."""
    rng = np.random.default_rng(77)
    cases = [dict(M=256, a=a, b=b, c=c, alpha=-1.0, beta=1.0, maxrk=a + c, acc=ACC,
                  arrays=_batch_case(rng, 256, a, b, c, decades=8.0))
             for a, b, c in [(16, 16, 16), (30, 28, 34)]]
    _check(cases, *_run_batch(hc, cases), port, expect_zeros=False)


def test_deflated_complex_svd_vs_oracle(hc, port):
    """The complex kernel (zgesvd_kernel, hc_zkernels.cu) deflates the same
    way.  Complex factors with spectra of 30 decades (part of every core below
    the bound) and a far-field update with every singular value below acc,
    through hcore_gpu_zgemm_batched (native complex kernels for a + c <= 84):
    ranks equal to the restated reference's (zgesvd at hcore_zgemm.c:327),
    products within 1e-11."""
    from test_gpu_zgemm import _clr, _rel

    rng = np.random.default_rng(61)
    M, maxrk = 256, 84
    tasks, keep, refs = [], [], []
    for q, (a, b, c) in enumerate([(6, 5, 7), (20, 18, 22), (30, 28, 34), (40, 30, 40),
                                   (12, 10, 14)]):
        AU, AV = _clr(rng, M, a, 30)
        BU, BV = _clr(rng, M, b, 30)
        CU, CV = _clr(rng, M, c, 30)
        if q == 4:   # far field: every singular value below acc
            AU, CU = np.asfortranarray(AU * 1e-7), np.asfortranarray(CU * 1e-12)
        ref = port.zgemm(M, -1.0, AU, AV, a, BU, BV, b, 1.0, CU, CV, c, maxrk=maxrk, acc=ACC)
        oU = np.zeros((M, maxrk), dtype=np.complex128, order="F")
        oV = np.zeros_like(oU)
        oU[:, :c], oV[:, :c] = CU, CV
        keep += [AU, AV, BU, BV, oU, oV]
        tasks.append(hc.ZlrTask(M=M, a=a, b=b, c=c, rk=0, maxrk=maxrk,
                                alpha=hc.DComplex(-1.0, 0.0), beta=hc.DComplex(1.0, 0.0),
                                acc=ACC, AU=AU.ctypes.data, AV=AV.ctypes.data, lda=M,
                                BU=BU.ctypes.data, BV=BV.ctypes.data, ldb=M, CU=oU.ctypes.data,
                                CV=oV.ctypes.data, ldc=M))
        refs.append((ref, oU, oV))
    ranks, status = hc.zgemm_batched(tasks)
    for q, ((ref, oU, oV), r, st) in enumerate(zip(refs, ranks, status)):
        assert st == 0 and r == ref["rank"], (q, st, r, ref["rank"])
        assert _rel(oU[:, :r] @ oV[:, :r].T, ref["CU"] @ ref["CV"].T) < FP64_TOL, q
    assert ranks[4] == 1
