"""The stack phase's products F = AV^T BV and G = BU F^T on the tensor cores
(hc_stack_tc.cu, opt-in plan flag TC_STACK) against the FP64 stack kernel
(the default) and the oracle (reference hcore_dgemm.c:175-178, :199-205).

Tensor-core updates have 1 <= a <= 64 and 1 <= b <= 32; the others (b = 33,
40) keep the FP64 products in both plans.  Gates: ranks equal in both paths
and to the oracle, products within 1e-13 of the FP64 path's and within the
oracle's 1e-11.
"""
import numpy as np
import pytest

from oracle import oracle as O
from test_gpu_rebuild_tc import _factors, _rel, _run

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-11
PATH_TOL = 1e-13


def _abc_cases(rng, M, abcs, scales=(1.0, 1.0, 1.0, 1.0)):
    cases = []
    for a, b, c in abcs:
        AU, AV = O.graded_lowrank(rng, M, a)
        BU, BV = O.graded_lowrank(rng, M, b)
        CU, CV = O.graded_lowrank(rng, M, c)
        sa, sav, sbu, sbv = scales
        cases.append(dict(M=M, a=a, b=b, c=c,
                          arrays=(AU * sa, AV * sav, BU * sbu, BV * sbv, CU, CV)))
    return cases


def _check(hc, port, cases, acc=1e-8, path_tol=PATH_TOL):
    _, keep_t, r_t, s_t = _run(hc, cases, hc.TC_STACK, acc=acc)
    _, keep_d, r_d, s_d = _run(hc, cases, 0, acc=acc)
    assert (s_t == 0).all() and (s_d == 0).all()
    assert np.array_equal(r_t, r_d)
    for cs, r, (CUt, CVt), (CUd, CVd) in zip(cases, r_t, _factors(keep_t, r_t),
                                             _factors(keep_d, r_d)):
        P, Pd = CUt @ CVt.T, CUd @ CVd.T
        assert _rel(P, Pd) < path_tol, (cs["a"], cs["b"], cs["c"], _rel(P, Pd))
        AU, AV, BU, BV, CU, CV = cs["arrays"]
        k = cs["a"] + cs["c"]
        ref = port.gemm(cs["M"], -1.0, AU, AV, cs["a"], BU, BV, cs["b"], 1.0, CU, CV, cs["c"],
                        maxrk=k, acc=acc)
        assert int(r) == ref["rank"]
        assert O.rel_fro(P, ref["CU"] @ ref["CV"].T) < FP64_TOL


@pytest.mark.parametrize("M", [256, 1000, 2048])
def test_stack_tc_matches_dfma_and_oracle(hc, port, M):
    rng = np.random.default_rng(500 + M)
    abcs = [(1, 1, 4), (5, 3, 9), (16, 16, 16), (17, 31, 20), (32, 32, 30), (40, 8, 20),
            (64, 32, 1), (20, 33, 20), (30, 40, 25)]
    _check(hc, port, _abc_cases(rng, M, abcs))


def test_stack_tc_graded_factor_scales(hc, port):
    """AV scaled 1e-100, BV 1e+80 and BU 1e+20 (A B^T stays comparable to C,
    F is ~1e-20): the per-column and per-row scales of the digit products keep
    F and G FP64-accurate."""
    rng = np.random.default_rng(23)
    cases = _abc_cases(rng, 512, [(12, 20, 15), (30, 32, 24)],
                       scales=(1.0, 1e-100, 1e20, 1e80))
    _check(hc, port, cases, acc=1e-8)


def test_stack_tc_nonfinite_input_gives_noconv(hc):
    """A NaN in AV: the tensor-core products are NaN, as the FP64 ones would
    be, and the update ends with HCORE_GPU_S_NOCONV (6); the other update of
    the batch is unaffected."""
    rng = np.random.default_rng(29)
    cases = _abc_cases(rng, 256, [(10, 12, 8), (10, 12, 8)])
    AU, AV, BU, BV, CU, CV = cases[0]["arrays"]
    AV = AV.copy()
    AV[17, 3] = np.nan
    cases[0]["arrays"] = (AU, AV, BU, BV, CU, CV)
    _, _, ranks, status = _run(hc, cases, hc.TC_STACK)
    assert status[0] == 6 and status[1] == 0
