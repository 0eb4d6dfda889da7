"""The rebuild phase on the tensor cores (hc_rebuild_tc.cu) against the FP64
reflector kernel (plan flag DFMA_REBUILD) and the oracle.

The tensor-core rebuild forms Q [X0; 0] through the compact WY form with the
Gram matrix and the Y Z product as exact bf16 digit products; it takes the
updates with a + c <= 64 and leaves larger ones to the DFMA kernel.  Gates:
* ranks equal in both paths and to the oracle (the rebuild does not touch
  the rank);
* each rebuilt factor within 1e-13 of the DFMA kernel's, relative to the
  factor's norm (both are FP64-accurate: ~1e-15 apart in a CPU emulation);
* CU keeps orthonormal columns to 1e-13 (Q_A times orthonormal U_r);
* the product within the oracle's 1e-11 gate (reference hcore_dgemm.c:508-696).
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-11
PATH_TOL = 1e-13


def _cases(rng, M, ks):
    cases = []
    for k in ks:
        c = max(1, k // 2)
        a = k - c
        b = int(rng.integers(1, 41))
        AU, AV = O.graded_lowrank(rng, M, a)
        BU, BV = O.graded_lowrank(rng, M, b)
        CU, CV = O.graded_lowrank(rng, M, c)
        cases.append(dict(M=M, a=a, b=b, c=c, arrays=(AU, AV, BU, BV, CU, CV)))
    return cases


def _run(hc, cases, flags, acc=1e-8, maxrk=None, storage=None):
    import torch
    from hcore_gb300 import devmem

    keep, tasks = [], []
    for q, cs in enumerate(cases):
        AU, AV, BU, BV, CU, CV = cs["arrays"]
        M, a, b, c = cs["M"], cs["a"], cs["b"], cs["c"]
        k = a + c
        dA = [devmem.to_device(x) for x in (AU, AV, BU, BV)]
        dCU = devmem.to_device(CU, ncols=k)
        dCV = devmem.to_device(CV, ncols=k)
        oCU = torch.full_like(dCU, float("nan"))
        oCV = torch.full_like(dCV, float("nan"))
        keep.append((dA, dCU, dCV, oCU, oCV))
        tasks.append(hc.LrTask(M=M, a=a, b=b, c=c, rk=0, maxrk=maxrk or k, ld_newv=0,
                               storage_maxrank=(storage[q] if storage else 0), alpha=-1.0,
                               beta=1.0, acc=acc, AU=dA[0].data_ptr(), AV=dA[1].data_ptr(),
                               lda=M, BU=dA[2].data_ptr(), BV=dA[3].data_ptr(), ldb=M,
                               Bdense=None, CU=dCU.data_ptr(), CV=dCV.data_ptr(), ldc=M,
                               CUo=oCU.data_ptr(), CVo=oCV.data_ptr(), ldco=M))
    batch = hc.Batch(tasks, flags=flags)
    batch.execute()
    ranks, status = batch.results()
    return batch, keep, ranks, status


def _factors(keep, ranks):
    from hcore_gb300 import devmem

    return [(devmem.to_host(o[3], int(r)), devmem.to_host(o[4], int(r)))
            for o, r in zip(keep, ranks)]


def _rel(X, Y):
    return np.linalg.norm(X - Y) / max(np.linalg.norm(Y), 1e-300)


@pytest.mark.parametrize("M", [256, 1000, 2048])
def test_tc_rebuild_matches_dfma_and_oracle(hc, port, M):
    """k from 2 to 64 (all four kernel variants) plus k above 64 (DFMA in
    both plans); M a multiple of 128 or not."""
    rng = np.random.default_rng(100 + M)
    ks = [2, 9, 16, 17, 30, 32, 33, 47, 48, 49, 63, 64, 65, 80]
    ks = [k for k in ks if k <= M]
    cases = _cases(rng, M, ks)
    _, keep_t, r_t, s_t = _run(hc, cases, 0)
    _, keep_d, r_d, s_d = _run(hc, cases, hc.DFMA_REBUILD)
    assert (s_t == 0).all() and (s_d == 0).all()
    assert np.array_equal(r_t, r_d)
    ft, fd = _factors(keep_t, r_t), _factors(keep_d, r_d)
    for cs, r, (CUt, CVt), (CUd, CVd) in zip(cases, r_t, ft, fd):
        assert _rel(CUt, CUd) < PATH_TOL, (cs["a"] + cs["c"], _rel(CUt, CUd))
        assert _rel(CVt, CVd) < PATH_TOL, (cs["a"] + cs["c"], _rel(CVt, CVd))
        assert np.abs(CUt.T @ CUt - np.eye(int(r))).max() < PATH_TOL
        AU, AV, BU, BV, CU, CV = cs["arrays"]
        k = cs["a"] + cs["c"]
        ref = port.gemm(M, -1.0, AU, AV, cs["a"], BU, BV, cs["b"], 1.0, CU, CV, cs["c"],
                        maxrk=k, acc=1e-8)
        assert int(r) == ref["rank"]
        assert O.rel_fro(CUt @ CVt.T, ref["CU"] @ ref["CV"].T) < FP64_TOL


def test_tc_rebuild_keeps_all_columns(hc, port):
    """acc = 0 keeps every singular triplet (r = k = 64): the widest output
    tile (N = 64) and the largest Z."""
    rng = np.random.default_rng(7)
    cases = _cases(rng, 512, [64, 48, 31])
    _, keep_t, r_t, s_t = _run(hc, cases, 0, acc=0.0)
    _, keep_d, r_d, s_d = _run(hc, cases, hc.DFMA_REBUILD, acc=0.0)
    assert (s_t == 0).all() and np.array_equal(r_t, r_d)
    assert list(r_t) == [64, 48, 31]
    for (CUt, CVt), (CUd, CVd) in zip(_factors(keep_t, r_t), _factors(keep_d, r_d)):
        assert _rel(CUt, CUd) < PATH_TOL and _rel(CVt, CVd) < PATH_TOL


def test_tc_rebuild_of_storage_overflow(hc):
    """Updates whose rank exceeds their storage limit are rebuilt later from
    the workspace (hcore_gpu_plan_rebuild): the tensor-core path there too."""
    import torch
    from hcore_gb300 import devmem

    rng = np.random.default_rng(5)
    cases = _cases(rng, 384, [40, 56, 20])
    storage = [4, 4, 4]
    res = []
    for flags in (0, hc.DFMA_REBUILD):
        batch, keep, ranks, status = _run(hc, cases, flags, storage=storage)
        assert (status == 5).all()  # HCORE_GPU_S_STORAGE
        assert (ranks > 4).all()
        outs = [(torch.full((int(r), 384), float("nan"), dtype=torch.float64, device="cuda"),
                 torch.full((int(r), 384), float("nan"), dtype=torch.float64, device="cuda"))
                for r in ranks]
        batch.rebuild(list(range(3)), [o[0].data_ptr() for o in outs],
                      [o[1].data_ptr() for o in outs], [384] * 3)
        torch.cuda.synchronize()
        ranks2, status2 = batch.results()
        assert (status2 == 0).all() and np.array_equal(ranks2, ranks)
        res.append([(devmem.to_host(o[0], int(r)), devmem.to_host(o[1], int(r)))
                    for o, r in zip(outs, ranks)])
    for (CUt, CVt), (CUd, CVd) in zip(*res):
        assert np.isfinite(CUt).all() and np.isfinite(CVt).all()
        assert _rel(CUt, CUd) < PATH_TOL and _rel(CVt, CVd) < PATH_TOL


def test_tc_rebuild_small_magnitudes(hc):
    """Far-field sized factors (entries ~1e-150 and ~1e-280): the per-row and
    per-column scales keep the digits exact; results agree with the DFMA
    kernel relative to their own size."""
    rng = np.random.default_rng(9)
    for scale in (1e-150, 1e-280):
        cases = _cases(rng, 300, [24, 40])
        for cs in cases:
            AU, AV, BU, BV, CU, CV = cs["arrays"]
            cs["arrays"] = (AU * scale, AV, BU, BV, CU * scale, CV)
        _, keep_t, r_t, s_t = _run(hc, cases, 0, acc=1e-8 * scale)
        _, keep_d, r_d, s_d = _run(hc, cases, hc.DFMA_REBUILD, acc=1e-8 * scale)
        assert (s_t == 0).all() and np.array_equal(r_t, r_d)
        for (CUt, CVt), (CUd, CVd) in zip(_factors(keep_t, r_t), _factors(keep_d, r_d)):
            assert _rel(CUt, CUd) < PATH_TOL
            assert _rel(CVt, CVd) < 1e-12
