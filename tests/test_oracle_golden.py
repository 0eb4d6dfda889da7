"""The oracle (C restatement, oracle/hcore_port_impl.h) against the reference.

The fixtures in tests/golden/ were produced by the reference HCORE compiled
from its own sources (tests/golden/make_golden.py); these tests pin the
restatement to them on whatever machine runs them.  CPU only.
"""
import numpy as np
import pytest

from oracle import oracle as O


def test_known_answer_programs_recorded(golden):
    """The reference's own four ctest programs passed when the fixtures were made."""
    meta, _ = golden
    ka = meta["known_answer"]
    assert ka["testing_dgemm"]["rc"] == 0 and ka["testing_dgemm"]["crank_out"] == 6
    assert ka["testing_dgemm"]["inf_norm_err"] < 10 * 1e-4          # testing_dgemm.c:378
    assert ka["testing_sgemm"]["rc"] == 0 and ka["testing_sgemm"]["crank_out"] == 6
    assert ka["testing_dsyrk"]["inf_norm_err"] < 1000 * 2.2e-16     # testing_dsyrk.c:205
    assert ka["testing_dgemmcd"]["inf_norm_err"] < 1000 * 2.2e-16


def test_port_reproduces_dgemm_known_answer(port, golden):
    """testing_dgemm.c:250-392 rebuilt: dlatms(iseed 0,0,0,1) -> compress -> update."""
    meta, g = golden
    kat = meta["kat_dgemm"]
    iseed = np.array([0, 0, 0, 1], dtype=np.int32)
    M = kat["M"]
    A, AU, AV, ar = O.generate_compress(port, M, iseed, 1e-4, 6)
    B, BU, BV, br = O.generate_compress(port, M, iseed, 1e-4, 6)
    Cd, CU, CV, cr = O.generate_compress(port, M, iseed, 1e-4, 6)
    assert [ar, br, cr] == kat["ranks"]
    np.testing.assert_allclose(A, g["kat_dgemm_A"], rtol=0, atol=1e-13)
    out = port.gemm(M, 1.0, AU, AV, ar, BU, BV, br, 1.0, CU, CV, cr, maxrk=M, acc=1e-4)
    assert out["status"] == 0 and out["rank"] == kat["rank_out"] == 6
    assert out["flops"] == kat["flops"]
    ref_C = Cd + A @ B.T
    err = np.abs(out["CU"] @ out["CV"].T - ref_C).sum(axis=1).max()   # inf norm
    assert err < 10 * 1e-4
    P_ref = g["kat_dgemm_CUo"] @ g["kat_dgemm_CVo"].T
    assert O.rel_fro(out["CU"] @ out["CV"].T, P_ref) < 1e-12


@pytest.mark.parametrize("i", range(11))
def test_port_matches_reference_cases(port, golden, i):
    meta, g = golden
    case = meta["gemm"][i]
    name, kind = case["name"], case["kind"]
    dtype = np.float32 if kind == "sgemm" else np.float64
    AU, AV, BU, BV, CU, CV = (g[f"{name}_{f}"] for f in ("AU", "AV", "BU", "BV", "CU", "CV"))
    out = port.gemm(case["M"], case["alpha"], AU, AV, case["a"], BU, BV, case["b"], case["beta"],
                    CU, CV, case["c"], rk=case["rk"], maxrk=case["maxrk"], acc=case["acc"],
                    variant=1 if kind == "fast" else 0, dtype=dtype)
    assert out["status"] == 0
    assert out["rank"] == case["rank_out"]
    if case["flops"] is not None:
        assert out["flops"] == case["flops"]
    P = out["CU"].astype(np.float64) @ out["CV"].T.astype(np.float64)
    P_ref = g[f"{name}_CUo"].astype(np.float64) @ g[f"{name}_CVo"].T.astype(np.float64)
    tol = 2e-5 if dtype == np.float32 else 1e-12
    assert O.rel_fro(P, P_ref) < tol


def test_port_config512_fingerprint(port, golden):
    """nb=512, ranks 32, sigma_i = 10^(-8i/32), acc 1e-8, maxrk 64."""
    meta, g = golden
    c = meta["cfg512"]
    rng = np.random.default_rng(c["seed"])
    AU, AV = O.graded_lowrank(rng, 512, 32)
    BU, BV = O.graded_lowrank(rng, 512, 32)
    CU, CV = O.graded_lowrank(rng, 512, 32)
    out = port.gemm(512, 1.0, AU, AV, 32, BU, BV, 32, 1.0, CU, CV, 32, maxrk=64, acc=1e-8)
    assert out["rank"] == c["rank_out"] and out["flops"] == c["flops"]
    omega = np.random.default_rng(c["omega_seed"]).standard_normal((512, 8))
    fp = (out["CU"] @ out["CV"].T) @ omega
    assert O.rel_fro(fp, g["cfg512_fingerprint"]) < 1e-10
    D = O.dense_update(1.0, AU, AV, BU, BV, 1.0, CU, CV)
    assert O.rel_fro(out["CU"] @ out["CV"].T, D) < 1e-8


@pytest.mark.parametrize("i", range(2))
def test_port_dsyrk_matches_reference(port, golden, i):
    meta, g = golden
    c = meta["syrk"][i]
    n = c["name"]
    CDo, fl = port.dsyrk(c["M"], c["K"], c["alpha"], g[f"{n}_AU"], g[f"{n}_AV"], g[f"{n}_CD"])
    np.testing.assert_allclose(CDo, g[f"{n}_CDo"], rtol=1e-12, atol=1e-12)
    assert fl == c["flops"]


@pytest.mark.parametrize("i", range(2))
def test_port_dgemmcd_matches_reference(port, golden, i):
    meta, g = golden
    c = meta["gemmcd"][i]
    n = c["name"]
    CDo = port.dgemmcd(c["M"], g[f"{n}_Au"], g[f"{n}_Av"], c["a"], g[f"{n}_Bu"], g[f"{n}_Bv"],
                       c["b"], g[f"{n}_CD"])
    np.testing.assert_allclose(CDo, g[f"{n}_CDo"], rtol=1e-12, atol=1e-12)


def test_port_error_statuses(port):
    """The reference's exit(-1) conditions become status codes in the oracle."""
    rng = np.random.default_rng(5)
    AU, AV = O.graded_lowrank(rng, 64, 8)
    out = port.gemm(64, 1.0, AU, AV, 8, AU, AV, 8, 1.0, AU, AV, 0, maxrk=16, acc=1e-8)
    assert out["status"] == 1                                   # zero rank (hcore_dgemm.c:743)
    out = port.gemm(64, 1.0, AU, AV, 8, AU, AV, 8, 1.0, AU, AV, 8, maxrk=7, acc=1e-8)
    assert out["status"] == 2                                   # a + c > 2*maxrk (:91)
    out = port.gemm(64, 1.0, AU, AV, 8, AU, AV, 8, 1.0, AU, AV, 8, maxrk=12, acc=1e-8)
    assert out["status"] == 3                                   # ld_newV < k (:924)
    out = port.gemm(64, 1.0, AU, AV, 8, AU, AV, 8, 1.0, AU, AV, 8, maxrk=16, acc=0.0)
    assert out["status"] == 0 and out["rank"] == 16
    out = port.gemm(64, 1.0, AU, AV, 8, AU, AV, 8, 1.0, AU, AV, 8, maxrk=16, acc=0.0, rk=20)
    assert out["rank"] == 16                                    # rk capped at k (:448-450)


def test_flop_model_matches_reference_formula(port):
    """flop_counts.c:3-70 restated; the total of one nb=512, ranks-32 update
    (new rank 47) is 2.7635e7."""
    M, a, b, c, r = 512, 32, 32, 32, 47
    k = a + c
    tot = (2 * port.flop_counts("q", M, k) + port.flop_counts("m", a, b, M) +
           port.flop_counts("m", M, a, b) + port.flop_counts("s", k) + r * k +
           port.flop_counts("o", M, r, k, 1) + port.flop_counts("o", r, M, k, 2))
    assert tot == 27634720


# ---- the tile steps around the update (golden_tlr.npz) ----

def _close(x, y, tol=1e-13):
    """Equal NaN pattern; finite entries within tol relative to max |y|."""
    x, y = np.asarray(x), np.asarray(y)
    assert np.array_equal(np.isnan(x), np.isnan(y))
    f = ~np.isnan(y)
    scale = max(np.abs(y[f]).max(), 1.0) if f.any() else 1.0
    assert np.abs(x[f] - y[f]).max(initial=0.0) <= tol * scale


def test_port_duncompress_matches_reference(port, golden_tlr):
    meta, g = golden_tlr
    for c in meta["uncompress"]:
        n = c["name"]
        out = port.duncompress(c["M"], c["N"], g[f"{n}_AU"], c["a"], g[f"{n}_BV"], g[f"{n}_CD"])
        _close(out, g[f"{n}_CDo"])


def test_port_dgemmbdcd_matches_reference(port, golden_tlr):
    meta, g = golden_tlr
    for c in meta["gemmbdcd"]:
        n = c["name"]
        out, fl = port.dgemmbdcd(c["transA"], c["M"], c["N"], c["alpha"], g[f"{n}_AU"],
                                 g[f"{n}_AV"], c["a"], g[f"{n}_BD"], c["beta"], g[f"{n}_CD"])
        _close(out, g[f"{n}_CDo"])
        assert fl == c["flops"]


def test_port_dtrsm_matches_reference(port, golden_tlr):
    """Every side/uplo/trans/diag; the unused triangle of A is NaN."""
    meta, g = golden_tlr
    assert len(meta["trsm"]) == 16
    for c in meta["trsm"]:
        n = c["name"]
        out, fl = port.dtrsm(c["side"], c["uplo"], c["trans"], c["diag"], c["M"], c["N"],
                             c["alpha"], g[f"{n}_A"], g[f"{n}_B"])
        _close(out, g[f"{n}_Bo"], 1e-12)
        assert fl == c["flops"]


def test_port_dpotrf_matches_reference(port, golden_tlr):
    """Both triangles, a failing pivot (info 11) and uplo = HCORE_Lower, which
    LAPACKE rejects (info -2): the reference passes uplo through as a char."""
    meta, g = golden_tlr
    infos = []
    for c in meta["potrf"]:
        n = c["name"]
        out, info, fl = port.dpotrf(c["uplo"], c["n"], g[f"{n}_A"])
        assert info == c["info"] and fl == c["flops"]
        _close(out, g[f"{n}_Ao"], 1e-12)
        infos.append(info)
    assert infos == [0, 0, 11, -2]


def test_port_compress_matches_reference(port, golden_compress):
    """The restated compressor against generate_compress: same rank (8, a cap
    at 10, 0, 5), same product U V^T."""
    meta, g = golden_compress
    assert [c["rank"] for c in meta] == [8, 10, 0, 5]
    for c in meta:
        n = c["name"]
        r, U, V, sig = port.dcompress(g[f"{n}_A"], c["acc"], c["maxrank"])
        assert r == c["rank"]
        if r:
            _close(U @ V.T, g[f"{n}_U"] @ g[f"{n}_V"].T, 1e-13)


def test_complex_restatement_matches_reference_zgemm(golden_zgemm):
    """The dense restatement of the complex update (plain transposes, the
    reference's rank rule) against HCORE_zgemm's fixtures: same rank, same
    product; the flop model of HCORE_dgemm applies unchanged."""
    from hcore_gb300.panel import update_flops

    meta, g = golden_zgemm
    for c in meta:
        n = c["name"]
        alpha, beta = complex(*c["alpha"]), complex(*c["beta"])
        r, P, _ = O.zgemm_dense_truncation(alpha, g[f"{n}_AU"], g[f"{n}_AV"], g[f"{n}_BU"],
                                           g[f"{n}_BV"], beta, g[f"{n}_CU"], g[f"{n}_CV"],
                                           rk=c["rk"], acc=c["acc"])
        assert r == c["rank"]
        Pref = g[f"{n}_CUo"] @ g[f"{n}_CVo"].T
        assert np.linalg.norm(P - Pref) <= 1e-12 * np.linalg.norm(Pref)
        assert update_flops(c["M"], c["a"], c["b"], c["c"], r) == c["flops"]


def test_port_zgemm_matches_reference(port, golden_zgemm):
    """The C restatement of HCORE_zgemm against its fixtures: rank, flops and
    the product (within 1e-12: the same LAPACK calls)."""
    meta, g = golden_zgemm
    for c in meta:
        n = c["name"]
        out = port.zgemm(c["M"], complex(*c["alpha"]), g[f"{n}_AU"], g[f"{n}_AV"], c["a"],
                         g[f"{n}_BU"], g[f"{n}_BV"], c["b"], complex(*c["beta"]), g[f"{n}_CU"],
                         g[f"{n}_CV"], c["c"], rk=c["rk"], maxrk=c["maxrk"], acc=c["acc"])
        assert out["status"] == 0 and out["rank"] == c["rank"] and out["flops"] == c["flops"]
        Pref = g[f"{n}_CUo"] @ g[f"{n}_CVo"].T
        assert np.linalg.norm(out["CU"] @ out["CV"].T - Pref) <= 1e-12 * np.linalg.norm(Pref)


def test_zuncompress_fixture_is_the_plain_transpose_product(golden_zgemm):
    _, g = golden_zgemm
    P = g["zunc_AU"] @ g["zunc_BV"].T
    assert np.abs(g["zunc_CDo"] - P).max() <= 1e-13 * np.abs(P).max()


@pytest.mark.parametrize("seed", range(3))
def test_complex_restatements_agree(port, seed):
    """The C restatement of HCORE_zgemm and the dense restatement on seeded
    complex updates with complex alpha and beta (rank and product)."""
    rng = np.random.default_rng(4000 + seed)
    M, a, b, c = 80, int(rng.integers(2, 12)), int(rng.integers(2, 12)), int(rng.integers(2, 12))

    def clr(k):
        U, _ = np.linalg.qr(rng.standard_normal((M, k)) + 1j * rng.standard_normal((M, k)))
        V, _ = np.linalg.qr(rng.standard_normal((M, k)) + 1j * rng.standard_normal((M, k)))
        return U * 10.0 ** (-6 * np.arange(k) / k), V

    (AU, AV), (BU, BV), (CU, CV) = clr(a), clr(b), clr(c)
    alpha = complex(rng.standard_normal(), rng.standard_normal())
    beta = complex(rng.standard_normal(), rng.standard_normal())
    out = port.zgemm(M, alpha, AU, AV, a, BU, BV, b, beta, CU, CV, c, maxrk=32, acc=1e-7)
    r, P, S = O.zgemm_dense_truncation(alpha, AU, AV, BU, BV, beta, CU, CV, acc=1e-7)
    assert out["status"] == 0 and out["rank"] == r
    assert np.linalg.norm(out["CU"] @ out["CV"].T - P) <= 1e-12 * np.linalg.norm(P)


def test_gemm_list_runs_the_same_calls(port):
    """The CPU baseline's C loop (port_dgemm_list) over a small panel: every
    update succeeds with the benchmark's limits, and every one is refused when
    maxrk is below the rank sums (the reference's exit condition as a status),
    so the loop really calls port_dgemm per update."""
    from hcore_gb300 import panel as pnl

    p = pnl.build_panel(n_points=4096, nb=256, device="cpu", workers=2)
    sa = [p.index[(i, 0)] for i, j in p.updates]
    sb = [p.index[(j, 0)] for i, j in p.updates]
    sc = [p.index[(i, j)] for i, j in p.updates]
    U, V = p.U.numpy(), p.V.numpy()
    assert port.gemm_list(p.nb, U, V, p.offset, sa, sb, sc, alpha=-1.0, beta=1.0,
                          maxrk=p.maxrank, acc=p.acc, variant=2) == 0
    assert port.gemm_list(p.nb, U, V, p.offset, sa, sb, sc, alpha=-1.0, beta=1.0, maxrk=1,
                          acc=p.acc, variant=2) == len(sa)
