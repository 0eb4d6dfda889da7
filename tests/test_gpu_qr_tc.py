"""The blocked QR with tensor-core trailing updates (hc_qr_tc.cu) against the
unblocked FP64 QR (plan flag UNBLOCKED_QR) and the oracle.

The QR of the stacked factors (reference hcore_dgemm.c:123-124, :216-217)
runs as 16-column FP64 panels; between panels the columns on the right are
updated by the panel's reflectors through exact digit products on the tensor
cores.  Gates:
* ranks equal in both paths and to the oracle;
* the rebuilt factors within 1e-13 of the unblocked path's, relative to their
  norm (both FP64-accurate; the panel order changes the rounding only);
* products within the oracle's 1e-11 gate.
k covers one panel (20), two (21, 24, 25, 35), three (37, 40, 41, 48) and four
(53, 56, 57, 64) panels, and k above 64 (unblocked in both plans).
"""
import numpy as np
import pytest

from oracle import oracle as O
from test_gpu_rebuild_tc import _cases, _factors, _rel, _run

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-11
PATH_TOL = 1e-13


@pytest.mark.parametrize("M", [256, 1000, 2048])
def test_blocked_qr_matches_unblocked_and_oracle(hc, port, M):
    rng = np.random.default_rng(300 + M)
    ks = [20, 21, 24, 25, 35, 37, 40, 41, 48, 53, 56, 57, 64, 70]
    cases = _cases(rng, M, ks)
    _, keep_b, r_b, s_b = _run(hc, cases, 0)
    _, keep_u, r_u, s_u = _run(hc, cases, hc.UNBLOCKED_QR)
    assert (s_b == 0).all() and (s_u == 0).all()
    assert np.array_equal(r_b, r_u)
    for cs, r, (CUb, CVb), (CUu, CVu) in zip(cases, r_b, _factors(keep_b, r_b),
                                             _factors(keep_u, r_u)):
        k = cs["a"] + cs["c"]
        assert _rel(CUb @ CVb.T, CUu @ CVu.T) < PATH_TOL, (k, _rel(CUb @ CVb.T, CUu @ CVu.T))
        assert np.abs(CUb.T @ CUb - np.eye(int(r))).max() < PATH_TOL
        AU, AV, BU, BV, CU, CV = cs["arrays"]
        ref = port.gemm(M, -1.0, AU, AV, cs["a"], BU, BV, cs["b"], 1.0, CU, CV, cs["c"],
                        maxrk=k, acc=1e-8)
        assert int(r) == ref["rank"]
        assert O.rel_fro(CUb @ CVb.T, ref["CU"] @ ref["CV"].T) < FP64_TOL


def test_blocked_qr_graded_columns(hc, port):
    """Stacked columns of very different sizes (C's factor scaled by 1e-6,
    the B factor by 1e-120): the per-column scales of the trailing update keep
    each column's digits exact; rank and product against the oracle."""
    rng = np.random.default_rng(17)
    cases = _cases(rng, 512, [35, 48, 64])
    for cs in cases:
        AU, AV, BU, BV, CU, CV = cs["arrays"]
        cs["arrays"] = (AU, AV, BU * 1e-120, BV, CU * 1e-6, CV)
    acc = 1e-14   # C's singular values are 1e-6 .. 1e-14 (x 3 above), A B^T's below 1e-119
    _, keep_b, r_b, s_b = _run(hc, cases, 0, acc=acc)
    _, keep_u, r_u, s_u = _run(hc, cases, hc.UNBLOCKED_QR, acc=acc)
    assert (s_b == 0).all() and np.array_equal(r_b, r_u)
    for cs, r, (CUb, CVb), (CUu, CVu) in zip(cases, r_b, _factors(keep_b, r_b),
                                             _factors(keep_u, r_u)):
        assert _rel(CUb @ CVb.T, CUu @ CVu.T) < 1e-12
        AU, AV, BU, BV, CU, CV = cs["arrays"]
        k = cs["a"] + cs["c"]
        ref = port.gemm(512, -1.0, AU, AV, cs["a"], BU, BV, cs["b"], 1.0, CU, CV, cs["c"],
                        maxrk=k, acc=acc)
        assert int(r) == ref["rank"]
        assert O.rel_fro(CUb @ CVb.T, ref["CU"] @ ref["CV"].T) < FP64_TOL
