"""GPU parity: the CUDA path (through the C ABI) against the reference's
results (tests/golden/) and the oracle (oracle/, LAPACK restatement) on the
same seeded inputs.

Gates (written per test):
* rank: equal to the reference's / oracle's rank;
* FP64 product CU*CV^T: relative Frobenius distance to the reference's
  product <= 1e-11, and distance to the exact dense update no more than the
  reference's own truncation error + 1e-12 relative;
* FP32 (HCORE_sgemm): product within 5e-5 relative of the reference's.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-11
FP32_TOL = 5e-5


def _inputs(golden, name, dtype=np.float64):
    _, g = golden
    return [g[f"{name}_{f}"].astype(dtype) for f in ("AU", "AV", "BU", "BV", "CU", "CV")]


@pytest.mark.parametrize("i", range(11))
def test_dropin_matches_reference_golden(hc, golden, i):
    """HCORE_dgemm / HCORE_dgemm_fast / HCORE_sgemm drop-in calls on the
    reference's golden cases (host pointers: staged by the library)."""
    meta, g = golden
    case = meta["gemm"][i]
    kind, name = case["kind"], case["name"]
    dtype = np.float32 if kind == "sgemm" else np.float64
    AU, AV, BU, BV, CU, CV = _inputs(golden, name, dtype)
    fn = {"dgemm": hc.hcore_dgemm, "fast": hc.hcore_dgemm_fast, "sgemm": hc.hcore_sgemm}[kind]
    r, CUo, CVo, fl = fn(case["M"], case["alpha"], AU, AV, case["a"], BU, BV, case["b"],
                         case["beta"], CU, CV, case["c"], rk=case["rk"], maxrk=case["maxrk"],
                         acc=case["acc"])
    assert r == case["rank_out"]
    if case["flops"] is not None:
        assert fl == case["flops"]          # the reference's flop model, bit for bit
    P = CUo.astype(np.float64) @ CVo.T.astype(np.float64)
    P_ref = g[f"{name}_CUo"].astype(np.float64) @ g[f"{name}_CVo"].T.astype(np.float64)
    assert O.rel_fro(P, P_ref) < (FP32_TOL if dtype == np.float32 else FP64_TOL)


def test_dropin_known_answer_case(hc, golden):
    """testing_dgemm.c:250-392: rank 4 -> 6 and inf-norm error < 10*acc."""
    meta, g = golden
    M = 10
    r, CUo, CVo, fl = hc.hcore_dgemm(M, 1.0, g["kat_dgemm_AU"], g["kat_dgemm_AV"], 4,
                                     g["kat_dgemm_BU"], g["kat_dgemm_BV"], 4, 1.0,
                                     g["kat_dgemm_CU"], g["kat_dgemm_CV"], 4, maxrk=M, acc=1e-4)
    assert r == 6 and fl == meta["kat_dgemm"]["flops"]
    ref_C = g["kat_dgemm_C"] + g["kat_dgemm_A"] @ g["kat_dgemm_B"].T
    assert np.abs(CUo @ CVo.T - ref_C).sum(axis=1).max() < 10 * 1e-4


def test_dropin_config512(hc, port):
    """nb=512, ranks 32/32/32, sigma_i = 10^(-8i/32), acc 1e-8, maxrk 64."""
    rng = np.random.default_rng(2024)
    AU, AV = O.graded_lowrank(rng, 512, 32)
    BU, BV = O.graded_lowrank(rng, 512, 32)
    CU, CV = O.graded_lowrank(rng, 512, 32)
    ref = port.gemm(512, 1.0, AU, AV, 32, BU, BV, 32, 1.0, CU, CV, 32, maxrk=64, acc=1e-8)
    r, CUo, CVo, fl = hc.hcore_dgemm(512, 1.0, AU, AV, 32, BU, BV, 32, 1.0, CU, CV, 32, maxrk=64,
                                     acc=1e-8)
    assert r == ref["rank"] and fl == ref["flops"]
    P, P_ref = CUo @ CVo.T, ref["CU"] @ ref["CV"].T
    D = O.dense_update(1.0, AU, AV, BU, BV, 1.0, CU, CV)
    assert O.rel_fro(P, P_ref) < FP64_TOL
    assert O.rel_fro(P, D) <= O.rel_fro(P_ref, D) + 1e-12
    assert O.rel_fro(P, D) < 1e-8
    # U factor orthonormal, as Q_A U_r is in the reference
    assert np.abs(CUo.T @ CUo - np.eye(r)).max() < 1e-12


def _batch_case(rng, M, a, b, c, decades=8.0):
    AU, AV = O.graded_lowrank(rng, M, a, decades)
    BU, BV = O.graded_lowrank(rng, M, b, decades)
    CU, CV = O.graded_lowrank(rng, M, c, decades) if c else (np.zeros((M, 0)), np.zeros((M, 0)))
    return AU, AV, BU, BV, CU, CV


def _run_batch(hc, cases, dtype=np.float64, flags=0, precision=0, in_place=False, tuning=None):
    """cases: list of dict(M, a, b, c, alpha, beta, rk, maxrk, acc, arrays)."""
    import torch
    from hcore_gb300 import devmem

    keep, tasks = [], []
    for cs in cases:
        AU, AV, BU, BV, CU, CV = cs["arrays"]
        M, a, b, c = cs["M"], cs["a"], cs["b"], cs["c"]
        k = a + c
        dA = [devmem.to_device(x.astype(dtype)) for x in (AU, AV, BU, BV)]
        dCU = devmem.to_device(CU.astype(dtype), ncols=max(k, 1))
        dCV = devmem.to_device(CV.astype(dtype), ncols=max(k, 1))
        if in_place:
            oCU, oCV = dCU, dCV
        else:
            oCU = torch.full_like(dCU, float("nan"))
            oCV = torch.full_like(dCV, float("nan"))
        keep.append((dA, dCU, dCV, oCU, oCV))
        t = hc.LrTask(M=M, a=a, b=b, c=c, rk=cs.get("rk", 0), maxrk=cs["maxrk"], ld_newv=0,
                      storage_maxrank=cs.get("storage", 0), alpha=cs["alpha"], beta=cs["beta"],
                      acc=cs["acc"], AU=dA[0].data_ptr(), AV=dA[1].data_ptr(), lda=M,
                      BU=dA[2].data_ptr(), BV=dA[3].data_ptr(), ldb=M, Bdense=None,
                      CU=dCU.data_ptr(), CV=dCV.data_ptr(), ldc=M, CUo=oCU.data_ptr(),
                      CVo=oCV.data_ptr(), ldco=M)
        tasks.append(t)
    batch = hc.Batch(tasks, precision=precision, flags=flags, tuning=tuning)
    batch.execute()
    ranks, status = batch.results()
    outs = []
    for (dA, dCU, dCV, oCU, oCV), r in zip(keep, ranks):
        outs.append((devmem.to_host(oCU, int(r)), devmem.to_host(oCV, int(r))))
    return batch, ranks, status, outs


def test_batched_uneven_ranks_vs_oracle(hc, port):
    """A panel-like batch: 24 updates, M=256, ranks 1..40, alpha=-1 (Schur)."""
    rng = np.random.default_rng(11)
    cases = []
    for i in range(24):
        a, b, c = (int(x) for x in rng.integers(1, 41, size=3))
        cases.append(dict(M=256, a=a, b=b, c=c, alpha=-1.0, beta=1.0, maxrk=80, acc=1e-8,
                          arrays=_batch_case(rng, 256, a, b, c)))
    batch, ranks, status, outs = _run_batch(hc, cases)
    assert (status == 0).all()
    for cs, r, (CUo, CVo) in zip(cases, ranks, outs):
        AU, AV, BU, BV, CU, CV = cs["arrays"]
        ref = port.gemm(256, -1.0, AU, AV, cs["a"], BU, BV, cs["b"], 1.0, CU, CV, cs["c"],
                        maxrk=80, acc=1e-8)
        assert r == ref["rank"]
        assert O.rel_fro(CUo @ CVo.T, ref["CU"] @ ref["CV"].T) < FP64_TOL
        # singular values agree with LAPACK's dgesvd on the same core
        sig = batch.sigma(cases.index(cs))
        np.testing.assert_allclose(sig, ref["sigma"], rtol=0, atol=1e-13 * ref["sigma"][0])


def test_batched_equals_single_calls(hc):
    """The batched plan and the drop-in call run the same kernels: identical
    bits when the plan takes the single call's launch shape (four lanes per
    Jacobi column pair, eight-warp QR CTAs; the lanes set the SVD's
    reduction order)."""
    rng = np.random.default_rng(3)
    cases = [dict(M=192, a=12, b=9, c=15, alpha=-1.0, beta=1.0, maxrk=40, acc=1e-8,
                  arrays=_batch_case(rng, 192, 12, 9, 15)) for _ in range(4)]
    _, ranks, status, outs = _run_batch(hc, cases,
                                        tuning=hc.make_tuning(svd_lanes=[4, 4, 4], qr_warps=8))
    for cs, r, (CUo, CVo) in zip(cases, ranks, outs):
        AU, AV, BU, BV, CU, CV = cs["arrays"]
        r1, CU1, CV1, _ = hc.hcore_dgemm(192, -1.0, AU, AV, 12, BU, BV, 9, 1.0, CU, CV, 15,
                                         maxrk=40, acc=1e-8)
        assert r1 == r
        assert np.array_equal(CU1, CUo) and np.array_equal(CV1, CVo)


def test_batched_in_place_and_edge_cases(hc, port):
    """In-place outputs, c = 0 (split-API semantics), rank-1 inputs, fixed
    rank, acc = 0 (keep all k), k = M."""
    rng = np.random.default_rng(21)
    cases = [
        dict(M=64, a=10, b=7, c=0, alpha=1.0, beta=1.0, maxrk=16, acc=1e-8),
        dict(M=64, a=1, b=1, c=1, alpha=1.0, beta=1.0, maxrk=4, acc=1e-8),
        dict(M=96, a=9, b=9, c=9, alpha=1.0, beta=1.0, maxrk=18, acc=1e-8, rk=5),
        dict(M=96, a=6, b=6, c=6, alpha=2.0, beta=0.5, maxrk=12, acc=0.0),
        dict(M=32, a=16, b=12, c=16, alpha=1.0, beta=1.0, maxrk=32, acc=1e-10),
    ]
    for cs in cases:
        cs["arrays"] = _batch_case(rng, cs["M"], cs["a"], cs["b"], cs["c"])
    _, ranks, status, outs = _run_batch(hc, cases, in_place=True)
    assert (status == 0).all()
    for cs, r, (CUo, CVo) in zip(cases, ranks, outs):
        AU, AV, BU, BV, CU, CV = cs["arrays"]
        ref = port.gemm(cs["M"], cs["alpha"], AU, AV, cs["a"], BU, BV, cs["b"], cs["beta"], CU,
                        CV, cs["c"], rk=cs.get("rk", 0), maxrk=cs["maxrk"], acc=cs["acc"],
                        variant=2)
        assert ref["status"] == 0
        assert r == ref["rank"], (cs, r, ref["rank"])
        assert O.rel_fro(CUo @ CVo.T, ref["CU"] @ ref["CV"].T) < FP64_TOL


def test_batched_statuses_and_untouched_outputs(hc):
    """Per-task statuses instead of exit(-1); a rejected task leaves its outputs alone."""
    import torch
    from hcore_gb300 import devmem

    rng = np.random.default_rng(8)
    AU, AV, BU, BV, CU, CV = _batch_case(rng, 64, 8, 8, 8, decades=2.0)
    cases = [dict(M=64, a=8, b=8, c=8, alpha=1.0, beta=1.0, maxrk=8, acc=1e-12,
                  arrays=(AU, AV, BU, BV, CU, CV)),       # new rank 16 > maxrk 8
             dict(M=64, a=8, b=8, c=8, alpha=1.0, beta=1.0, maxrk=7, acc=1e-8,
                  arrays=(AU, AV, BU, BV, CU, CV)),       # a + c > 2*maxrk
             dict(M=8, a=8, b=8, c=8, alpha=1.0, beta=1.0, maxrk=8, acc=1e-8,
                  arrays=tuple(x[:8] for x in (AU, AV, BU, BV, CU, CV))),  # k > M
             dict(M=64, a=8, b=8, c=8, alpha=1.0, beta=1.0, maxrk=16, acc=1e-8,
                  arrays=(AU, AV, BU, BV, CU, CV))]
    _, ranks, status, outs = _run_batch(hc, cases)
    assert list(status) == [4, 2, 7, 0]
    assert np.isnan(outs[0][0]).all() if outs[0][0].size else True


def test_sgemm_batched_vs_oracle(hc, port):
    """HCORE_sgemm semantics, FP32 end to end, acc 1e-4."""
    rng = np.random.default_rng(17)
    cases = []
    for i in range(6):
        a, b, c = (int(x) for x in rng.integers(2, 20, size=3))
        cases.append(dict(M=128, a=a, b=b, c=c, alpha=-1.0, beta=1.0, maxrk=40, acc=1e-4,
                          arrays=_batch_case(rng, 128, a, b, c, decades=6.0)))
    _, ranks, status, outs = _run_batch(hc, cases, dtype=np.float32, precision=1)
    assert (status == 0).all()
    for cs, r, (CUo, CVo) in zip(cases, ranks, outs):
        AU, AV, BU, BV, CU, CV = (x.astype(np.float32) for x in cs["arrays"])
        ref = port.gemm(128, -1.0, AU, AV, cs["a"], BU, BV, cs["b"], 1.0, CU, CV, cs["c"],
                        maxrk=40, acc=1e-4, dtype=np.float32)
        assert r == ref["rank"]
        P = CUo.astype(np.float64) @ CVo.T.astype(np.float64)
        P_ref = ref["CU"].astype(np.float64) @ ref["CV"].T.astype(np.float64)
        assert O.rel_fro(P, P_ref) < FP32_TOL


def test_dsyrk_dgemmcd_dropin_vs_golden(hc, golden):
    meta, g = golden
    L = hc.lib()
    dp = C.POINTER(C.c_double)
    for c in meta["syrk"]:
        n = c["name"]
        AU, AV = (np.asfortranarray(g[f"{n}_{f}"]) for f in ("AU", "AV"))
        CD = np.asfortranarray(g[f"{n}_CD"]).copy(order="F")
        fc = hc.FlopCounter()
        L.HCORE_dsyrk(122, 111, c["M"], c["K"], c["alpha"], AU.ctypes.data_as(dp), AU.shape[0],
                      AV.ctypes.data_as(dp), AV.shape[0], 1.0, CD.ctypes.data_as(dp), CD.shape[0],
                      None, C.byref(fc))
        np.testing.assert_allclose(CD, g[f"{n}_CDo"], rtol=0, atol=1e-12 * np.abs(g[f"{n}_CDo"]).max())
        assert fc.syrk == c["flops"]
        assert np.all(np.triu(CD, 1) == 0)
    for c in meta["gemmcd"]:
        n = c["name"]
        Au, Av, Bu, Bv = (np.asfortranarray(g[f"{n}_{f}"]) for f in ("Au", "Av", "Bu", "Bv"))
        CD = np.asfortranarray(g[f"{n}_CD"]).copy(order="F")
        fc = hc.FlopCounter()
        L.HCORE_dgemmcd(111, 112, c["M"], -1.0, Au.ctypes.data_as(dp), Av.ctypes.data_as(dp),
                        c["a"], c["M"], Bu.ctypes.data_as(dp), Bv.ctypes.data_as(dp), c["b"],
                        c["M"], 1.0, CD.ctypes.data_as(dp), c["M"], max(c["a"], c["b"]), None,
                        C.byref(fc))
        np.testing.assert_allclose(CD, g[f"{n}_CDo"], rtol=0, atol=1e-12 * np.abs(g[f"{n}_CDo"]).max())


def test_dense_batched_sequential_semantics(hc, port):
    """63 syrk + gemmcd tasks on one tile in list order == the oracle applied in order."""
    import torch
    from hcore_gb300 import devmem

    rng = np.random.default_rng(33)
    M = 160
    CD0 = np.asfortranarray(np.tril(rng.standard_normal((M, M))))
    dCD = devmem.to_device(CD0)
    ref = CD0.copy(order="F")
    tasks, keep = [], []
    for i in range(12):
        kind = i % 3 == 2   # every third task is a gemmcd
        a, b = int(rng.integers(1, 24)), int(rng.integers(1, 24))
        Au, Av = (np.asfortranarray(rng.standard_normal((M, a)) * 0.1) for _ in range(2))
        Bu, Bv = (np.asfortranarray(rng.standard_normal((M, b)) * 0.1) for _ in range(2))
        d = [devmem.to_device(x) for x in (Au, Av, Bu, Bv)]
        keep.append(d)
        if kind:
            ref = port.dgemmcd(M, Au, Av, a, Bu, Bv, b, ref)
            tasks.append(hc.DenseTask(kind=1, M=M, a=a, b=b, alpha=-1.0, Au=d[0].data_ptr(),
                                      Av=d[1].data_ptr(), lda=M, Bu=d[2].data_ptr(),
                                      Bv=d[3].data_ptr(), ldb=M, CD=dCD.data_ptr(), ldcd=M))
        else:
            ref, _ = port.dsyrk(M, a, -1.0, Au, Av, ref)
            tasks.append(hc.DenseTask(kind=0, M=M, a=a, b=0, alpha=-1.0, Au=d[0].data_ptr(),
                                      Av=d[1].data_ptr(), lda=M, Bu=None, Bv=None, ldb=M,
                                      CD=dCD.data_ptr(), ldcd=M))
    hc.dense_batched(tasks)
    out = devmem.to_host(dCD, M)
    np.testing.assert_allclose(out, ref, rtol=0, atol=1e-12 * np.abs(ref).max())


def test_dgemm_dense_dropin(hc):
    rng = np.random.default_rng(4)
    L = hc.lib()
    dp = C.POINTER(C.c_double)
    for ta, tb in ((111, 111), (111, 112), (112, 111), (112, 112)):
        M, N, K = 70, 45, 33
        A = np.asfortranarray(rng.standard_normal((K, M) if ta == 112 else (M, K)))
        B = np.asfortranarray(rng.standard_normal((N, K) if tb == 112 else (K, N)))
        Cm = np.asfortranarray(rng.standard_normal((M, N)))
        ref = 0.7 * ((A.T if ta == 112 else A) @ (B.T if tb == 112 else B)) - 1.3 * Cm
        L.HCORE_dgemm_dense(ta, tb, M, N, K, 0.7, A.ctypes.data_as(dp), A.shape[0],
                            B.ctypes.data_as(dp), B.shape[0], -1.3, Cm.ctypes.data_as(dp), M)
        np.testing.assert_allclose(Cm, ref, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("pinned", [True, False])
def test_staged_host_inputs_equal_device_plan(hc, pinned):
    """HCORE_GPU_STAGE_INPUTS: host factors (pinned or pageable) in one arena,
    tiles shared between updates (copied once per execute) and one tile read
    by a single update (read in place when pinned, copied when pageable);
    results identical to the device plan's."""
    import torch
    from hcore_gb300 import devmem

    rng = np.random.default_rng(77)
    M, ranks = 128, [9, 12, 7, 15, 10, 11]
    facs = [O.graded_lowrank(rng, M, r) for r in ranks]
    arenaU = np.concatenate([u.T.reshape(-1) for u, _ in facs])
    arenaV = np.concatenate([v.T.reshape(-1) for _, v in facs])
    offs = np.concatenate([[0], np.cumsum([M * r for r in ranks])])
    hU, hV = torch.from_numpy(arenaU.copy()), torch.from_numpy(arenaV.copy())
    if pinned:
        hU, hV = hU.pin_memory(), hV.pin_memory()
    dU, dV = hU.cuda(), hV.cuda()
    pairs = [(0, 1, 2), (0, 3, 4), (1, 3, 2), (4, 0, 1), (3, 1, 5)]   # (A, B, C) slots; 5 private
    kmax = max(ranks[x] + ranks[z] for x, _, z in pairs)
    outs = {}
    for mode in ("device", "staged"):
        oU = torch.zeros(len(pairs) * M * kmax, dtype=torch.float64, device="cuda")
        oV = torch.zeros_like(oU)
        baseU, baseV = (dU, dV) if mode == "device" else (hU, hV)
        tasks = []
        for u, (x, y, z) in enumerate(pairs):
            e = 8
            tasks.append(hc.LrTask(
                M=M, a=ranks[x], b=ranks[y], c=ranks[z], rk=0, maxrk=kmax, ld_newv=0,
                storage_maxrank=0, alpha=-1.0, beta=1.0, acc=1e-8,
                AU=baseU.data_ptr() + e * int(offs[x]), AV=baseV.data_ptr() + e * int(offs[x]), lda=M,
                BU=baseU.data_ptr() + e * int(offs[y]), BV=baseV.data_ptr() + e * int(offs[y]), ldb=M,
                Bdense=None,
                CU=baseU.data_ptr() + e * int(offs[z]), CV=baseV.data_ptr() + e * int(offs[z]), ldc=M,
                CUo=oU.data_ptr() + e * u * M * kmax, CVo=oV.data_ptr() + e * u * M * kmax, ldco=M))
        b = hc.Batch(tasks, flags=hc.STAGE_INPUTS if mode == "staged" else 0)
        b.execute()
        rk, st = b.results()
        assert (st == 0).all()
        if mode == "staged":
            private = 2 * M * ranks[5] * 8
            assert b.staged_bytes + b.zero_copy_bytes == arenaU.nbytes + arenaV.nbytes
            assert b.zero_copy_bytes == (private if pinned else 0)
        outs[mode] = (rk.copy(), oU.cpu().numpy(), oV.cpu().numpy())
        b.close()
    assert np.array_equal(outs["device"][0], outs["staged"][0])
    assert np.array_equal(outs["device"][1], outs["staged"][1])
    assert np.array_equal(outs["device"][2], outs["staged"][2])


@pytest.mark.parametrize("acc", [1e-4, 1e-6])
def test_mixed_factors_vs_fp64_oracle(hc, port, acc):
    """HCORE_GPU_MIXED_FACTORS at loose accuracies: factor products and the
    rebuild in FP32, QR/SVD/truncation in FP64.  Same rank as the FP64
    oracle on cases without a singular value near acc; error against the
    exact update no more than the oracle's truncation error + 2e-6 relative
    (FP32 rounding of the products)."""
    rng = np.random.default_rng(91)
    cases = []
    for i in range(10):
        a, b, c = (int(x) for x in rng.integers(4, 30, size=3))
        cases.append(dict(M=256, a=a, b=b, c=c, alpha=-1.0, beta=1.0, maxrk=64, acc=acc,
                          arrays=_batch_case(rng, 256, a, b, c, decades=10.0)))
    _, ranks, status, outs = _run_batch(hc, cases, flags=hc.MIXED_FACTORS)
    assert (status == 0).all()
    for cs, r, (CUo, CVo) in zip(cases, ranks, outs):
        AU, AV, BU, BV, CU, CV = cs["arrays"]
        ref = port.gemm(256, -1.0, AU, AV, cs["a"], BU, BV, cs["b"], 1.0, CU, CV, cs["c"],
                        maxrk=64, acc=acc)
        sig = ref["sigma"]
        near = np.any(np.abs(sig - acc) < 1e-3 * acc)
        if not near:
            assert r == ref["rank"]
        D = O.dense_update(-1.0, AU, AV, BU, BV, 1.0, CU, CV)
        nd = np.linalg.norm(D)
        eg = np.linalg.norm(CUo @ CVo.T - D)
        er = np.linalg.norm(ref["CU"] @ ref["CV"].T - D)
        assert eg <= 1.01 * er + 2e-6 * nd


# Tiny-magnitude updates: far-field interactions whose factor products reach
# the subnormal range (FP32 tiles of a covariance kernel between distant
# clusters).  The QR takes the scaled-norm / dlarfg-rescaling paths and the
# SVD its power-of-two pre-scaling; the rank, the singular values and the
# product must still match the oracle (LAPACK scales the same way).
# (scale of every factor, acc, precision)
_TINY = [(1e-12, 1e-4, 1), (1e-12, 1e-28, 1), (3e-17, 1e-4, 1), (1e-20, 1e-4, 1),
         (1e-100, 1e-8, 0), (1e-100, 1e-208, 0), (1e-152, 1e-8, 0), (1e-160, 1e-8, 0)]


@pytest.mark.parametrize("scale,acc,precision", _TINY)
def test_tiny_magnitude_updates_vs_oracle(hc, port, scale, acc, precision):
    dtype = np.float32 if precision else np.float64
    rng = np.random.default_rng(5)
    M, a, b, c = 256, 12, 10, 14
    arrays = tuple(x * scale for x in _batch_case(rng, M, a, b, c, decades=6.0))
    cases = [dict(M=M, a=a, b=b, c=c, alpha=-1.0, beta=1.0, maxrk=64, acc=acc, arrays=arrays)]
    batch, ranks, status, outs = _run_batch(hc, cases, dtype=dtype, precision=precision)
    assert status[0] == 0
    AU, AV, BU, BV, CU, CV = (x.astype(dtype) for x in arrays)
    ref = port.gemm(M, -1.0, AU, AV, a, BU, BV, b, 1.0, CU, CV, c, maxrk=64, acc=acc, dtype=dtype)
    assert ranks[0] == ref["rank"]
    tol = FP32_TOL if precision else FP64_TOL
    tiny = float(np.finfo(dtype).smallest_subnormal)
    sig, sig_ref = batch.sigma(0), np.asarray(ref["sigma"], dtype=np.float64)
    smax = np.abs(sig_ref).max()
    # subnormal results carry fewer bits: allow a few units of the smallest subnormal
    assert np.abs(sig - sig_ref).max() <= tol * smax + 64 * tiny
    CUo, CVo = outs[0]
    P = CUo.astype(np.float64) @ CVo.T.astype(np.float64)
    P_ref = ref["CU"].astype(np.float64) @ ref["CV"].T.astype(np.float64)
    assert np.linalg.norm(P - P_ref) <= tol * np.linalg.norm(P_ref) + 64 * tiny * M


@pytest.mark.parametrize("precision", [0, 1])
def test_nonfinite_input_marks_update_noconv(hc, port, precision):
    """A NaN or Inf in an update's factors gives that update the NOCONV
    status (its outputs are not written); the other updates of the batch
    are unaffected."""
    dtype = np.float32 if precision else np.float64
    rng = np.random.default_rng(23)
    M, a, b, c = 128, 10, 9, 11
    good = _batch_case(rng, M, a, b, c, decades=6.0)
    with_nan = tuple(x.copy() for x in good)
    with_nan[0][5, 3] = np.nan
    with_inf = tuple(x.copy() for x in good)
    with_inf[3][7, 2] = np.inf
    cases = [dict(M=M, a=a, b=b, c=c, alpha=-1.0, beta=1.0, maxrk=40, acc=1e-4, arrays=arr)
             for arr in (with_nan, good, with_inf)]
    _, ranks, status, outs = _run_batch(hc, cases, dtype=dtype, precision=precision)
    assert list(status) == [6, 0, 6]
    AU, AV, BU, BV, CU, CV = (x.astype(dtype) for x in good)
    ref = port.gemm(M, -1.0, AU, AV, a, BU, BV, b, 1.0, CU, CV, c, maxrk=40, acc=1e-4, dtype=dtype)
    assert ranks[1] == ref["rank"]
    CUo, CVo = outs[1]
    P = CUo.astype(np.float64) @ CVo.T.astype(np.float64)
    P_ref = ref["CU"].astype(np.float64) @ ref["CV"].T.astype(np.float64)
    assert O.rel_fro(P, P_ref) < (FP32_TOL if precision else FP64_TOL)


@pytest.mark.parametrize("M,a,b,c,maxrk,acc", [
    (2048, 256, 200, 256, 512, 1e-7),    # k = 512: Jacobi matrices in global memory, 64 rows/lane
    (1024, 150, 100, 130, 300, 1e-8),    # k = 280
    (2048, 40, 30, 50, 128, 1e-7),       # M = 2048 with a small k (shared-memory Jacobi)
    (512, 60, 50, 70, 160, 1e-8),        # k = 130: R^T in shared memory, V_J in global memory
    (1024, 80, 70, 80, 200, 1e-8),       # k = 160: the same mode near its limit
    (1024, 90, 60, 90, 200, 1e-8)])      # k = 180: both in global memory again
def test_large_rank_updates_vs_oracle(hc, port, M, a, b, c, maxrk, acc):
    """The largest shapes a plan takes (a + c up to 512, M up to 2048), as in
    a 3D covariance matrix with nb = 2048 and tiles of rank up to 256."""
    rng = np.random.default_rng(M + a)
    arrays = _batch_case(rng, M, a, b, c, decades=10.0)
    cases = [dict(M=M, a=a, b=b, c=c, alpha=-1.0, beta=1.0, maxrk=maxrk, acc=acc, arrays=arrays)]
    _, ranks, status, outs = _run_batch(hc, cases)
    assert status[0] == 0
    AU, AV, BU, BV, CU, CV = arrays
    ref = port.gemm(M, -1.0, AU, AV, a, BU, BV, b, 1.0, CU, CV, c, maxrk=maxrk, acc=acc)
    assert ref["status"] == 0
    assert ranks[0] == ref["rank"]
    CUo, CVo = outs[0]
    assert O.rel_fro(CUo @ CVo.T, ref["CU"] @ ref["CV"].T) < FP64_TOL


def test_output_aliasing_another_tasks_input(hc, port):
    """Task 0 writes its result over the factors that task 1 reads as its A:
    task 1 must still see the original A (every input is read before any
    output is written), whichever stream group each task lands in."""
    import torch
    from hcore_gb300 import devmem

    rng = np.random.default_rng(91)
    M, a, b, c = 128, 10, 8, 12
    cases = [_batch_case(rng, M, a, b, c, decades=8.0) for _ in range(2)]
    AU1, AV1 = cases[1][0], cases[1][1]
    # task 1's A lives in a buffer wide enough to receive task 0's output
    width = a + c
    shared_U = devmem.to_device(AU1, ncols=width)
    shared_V = devmem.to_device(AV1, ncols=width)
    keep, tasks = [], []
    for u, (AU, AV, BU, BV, CU, CV) in enumerate(cases):
        d = [devmem.to_device(x) for x in (AU, AV, BU, BV, CU, CV)]
        keep.append(d)
        if u == 1:
            d[0], d[1] = shared_U, shared_V
        oU, oV = (shared_U, shared_V) if u == 0 else (torch.zeros((width, M), dtype=torch.float64,
                                                                   device="cuda"),) * 2
        if u == 1:
            oV = torch.zeros_like(oU)
        keep.append((oU, oV))
        tasks.append(hc.LrTask(M=M, a=a, b=b, c=c, rk=0, maxrk=width, ld_newv=0, storage_maxrank=0,
                               alpha=-1.0, beta=1.0, acc=1e-8, AU=d[0].data_ptr(), AV=d[1].data_ptr(),
                               lda=M, BU=d[2].data_ptr(), BV=d[3].data_ptr(), ldb=M, Bdense=None,
                               CU=d[4].data_ptr(), CV=d[5].data_ptr(), ldc=M, CUo=oU.data_ptr(),
                               CVo=oV.data_ptr(), ldco=M))
    batch = hc.Batch(tasks)
    batch.execute()
    ranks, status = batch.results()
    assert (status == 0).all()
    AU, AV, BU, BV, CU, CV = cases[1]
    ref = port.gemm(M, -1.0, AU, AV, a, BU, BV, b, 1.0, CU, CV, c, maxrk=width, acc=1e-8)
    oU1, oV1 = keep[3]
    r1 = int(ranks[1])
    assert r1 == ref["rank"]
    P = devmem.to_host(oU1, r1) @ devmem.to_host(oV1, r1).T
    assert O.rel_fro(P, ref["CU"] @ ref["CV"].T) < FP64_TOL
