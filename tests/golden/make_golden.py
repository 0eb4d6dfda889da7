"""Generate the golden fixtures in this folder from the reference HCORE.

Runs where the reference checkout exists: it compiles the reference from its
own sources (oracle/build.py -> oracle/_ref), runs the reference's four
known-answer programs (testing/testing_*.c) and calls the reference library
through ctypes on seeded inputs.  The outputs are committed as

* ``golden_meta.json`` — the known-answer programs' printed results, the
  case parameters, ranks and flop counts;
* ``golden_small.npz`` — inputs and reference outputs of the small cases
  (full matrices, a few hundred KB in total);
* config "nb=512, ranks 32" is stored by seed plus a fingerprint
  (rank, Frobenius norm, (CU CV^T) @ Omega for a seeded Omega), since its
  inputs regenerate from the seed.

* ``golden_tlr.npz`` / ``golden_tlr_meta.json`` — the same for the tile
  steps around the update: HCORE_duncompress, HCORE_dgemmbdcd, HCORE_dtrsm
  (every side/uplo/trans/diag) and HCORE_dpotrf (both triangles, a failing
  pivot, an invalid uplo).

* ``golden_compress.npz`` / ``golden_compress_meta.json`` — the reference
  tests' compressor (generate_compress) on dlatms tiles.

* ``golden_zgemm.npz`` / ``golden_zgemm_meta.json`` — the reference's
  HCORE_zgemm (complex) on seeded complex low-rank inputs.

Usage:  python tests/golden/make_golden.py [--tlr-only | --compress-only | --zgemm-only]
"""
from __future__ import annotations

import ctypes
import json
import os
import re
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import build as obuild  # noqa: E402
from oracle import oracle as O  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))

# (name, M, a, b, c, alpha, beta, rk, maxrk, acc, kind)
# kind: "dgemm" = HCORE_dgemm, "fast" = HCORE_dgemm_fast, "sgemm" = HCORE_sgemm
GEMM_CASES = [
    ("d_small_mixed", 64, 5, 7, 3, 1.0, 1.0, 0, 16, 1e-8, "dgemm"),
    ("d_schur", 96, 16, 12, 20, -1.0, 1.0, 0, 40, 1e-8, "dgemm"),
    ("d_acc1e6", 128, 24, 24, 24, 1.0, 1.0, 0, 48, 1e-6, "dgemm"),
    ("d_fixed_rank", 80, 10, 9, 11, 1.0, 1.0, 5, 24, 1e-8, "dgemm"),
    ("d_scaled", 72, 8, 8, 8, 0.5, 2.0, 0, 16, 1e-7, "dgemm"),
    ("d_k_eq_maxrk", 64, 12, 10, 20, 1.0, 1.0, 0, 32, 1e-8, "dgemm"),
    ("d_rank1", 48, 1, 1, 1, 1.0, 1.0, 0, 4, 1e-8, "dgemm"),
    ("fast_small", 64, 6, 9, 7, -1.0, 1.0, 0, 32, 1e-8, "fast"),
    ("fast_trunc2", 64, 3, 3, 3, 1.0, 1.0, 0, 16, 10.0, "fast"),
    ("s_small", 64, 6, 6, 6, 1.0, 1.0, 0, 16, 1e-4, "sgemm"),
    ("s_schur", 96, 12, 10, 14, -1.0, 1.0, 0, 32, 1e-4, "sgemm"),
]
SYRK_CASES = [("syrk_a", 64, 7, 1.0), ("syrk_b", 96, 12, -1.0)]
GEMMCD_CASES = [("gemmcd_a_gt_b", 64, 9, 6), ("gemmcd_a_le_b", 64, 5, 8)]


def run_known_answer_programs() -> dict:
    res = {}
    for t in obuild.REF_TESTS:
        exe = os.path.join(obuild.REF_OUT, t)
        p = subprocess.run([exe], capture_output=True, text=True,
                           env=dict(os.environ, OPENBLAS_NUM_THREADS="1"))
        out = p.stdout
        ent = {"rc": p.returncode}
        m = re.search(r"Crank: (\d+) -> (\d+)", out)
        if m:
            ent["crank_in"], ent["crank_out"] = int(m.group(1)), int(m.group(2))
        m = re.search(r"inf norm\(C - appC\):([0-9.e+-]+)", out)
        if m:
            ent["inf_norm_err"] = float(m.group(1))
        m = re.search(r"Infinity norm of \|reference_C - C\| = ([0-9.e+-]+)", out)
        if m:
            ent["inf_norm_err"] = float(m.group(1))
        ent["input_ranks"] = [int(x) for x in re.findall(r"Rank:(\d+)", out)]
        res[t] = ent
    return res


def seeded_inputs(seed, M, a, b, c, dtype=np.float64):
    rng = np.random.default_rng(seed)
    AU, AV = O.graded_lowrank(rng, M, a)
    BU, BV = O.graded_lowrank(rng, M, b)
    CU, CV = O.graded_lowrank(rng, M, c)
    return [x.astype(dtype) for x in (AU, AV, BU, BV, CU, CV)]


def libc_rand_matrices(nrows, ranks, fill_C_lower=True):
    """The reference dsyrk/dgemmcd tests draw from glibc rand() with its
    default seed (testing/testing_dsyrk.c:127-139)."""
    libc = ctypes.CDLL("libc.so.6")
    libc.srand(1)
    RM = 2147483647.0
    Cm = np.zeros((nrows, nrows), order="F")
    for i in range(nrows):
        for j in range(i + 1):
            Cm[i, j] = libc.rand() / RM
    mats = []
    facs = [np.zeros((nrows, r), order="F") for r in ranks for _ in range(2)]
    for i in range(nrows):
        for t, r in enumerate(ranks):
            for j in range(r):
                facs[2 * t][i, j] = libc.rand() / RM
                facs[2 * t + 1][i, j] = libc.rand() / RM
    mats.append(Cm)
    return Cm, facs


def main():
    ref = O.RefLib()
    port = O.Port()
    meta = {"known_answer": run_known_answer_programs(), "gemm": [], "syrk": [], "gemmcd": []}
    arrs = {}

    # -- the reference HCORE_dgemm known-answer case, rebuilt through dlatms --
    iseed = np.array([0, 0, 0, 1], dtype=np.int32)
    M = 10
    Ad, AU, AV, ar = O.generate_compress(port, M, iseed, 1e-4, 6)
    Bd, BU, BV, br = O.generate_compress(port, M, iseed, 1e-4, 6)
    Cd, CU, CV, cr = O.generate_compress(port, M, iseed, 1e-4, 6)
    out = ref.dgemm(M, 1.0, AU, AV, ar, BU, BV, br, 1.0, CU, CV, cr, maxrk=M, acc=1e-4)
    for nm, v in dict(A=Ad, B=Bd, C=Cd, AU=AU, AV=AV, BU=BU, BV=BV, CU=CU, CV=CV,
                      CUo=out["CU"], CVo=out["CV"]).items():
        arrs[f"kat_dgemm_{nm}"] = v
    meta["kat_dgemm"] = dict(M=M, ranks=[ar, br, cr], rank_out=out["rank"], flops=out["flops"],
                             maxrk=M, acc=1e-4)

    # -- seeded low-rank update cases --
    for i, (name, M, a, b, c, alpha, beta, rk, maxrk, acc, kind) in enumerate(GEMM_CASES):
        dtype = np.float32 if kind == "sgemm" else np.float64
        AU, AV, BU, BV, CU, CV = seeded_inputs(100 + i, M, a, b, c, dtype)
        out = ref.dgemm(M, alpha, AU, AV, a, BU, BV, b, beta, CU, CV, c, rk=rk, maxrk=maxrk,
                        acc=acc, fast=(kind == "fast"), dtype=dtype)
        for nm, v in dict(AU=AU, AV=AV, BU=BU, BV=BV, CU=CU, CV=CV, CUo=out["CU"],
                          CVo=out["CV"]).items():
            arrs[f"{name}_{nm}"] = v
        meta["gemm"].append(dict(name=name, M=M, a=a, b=b, c=c, alpha=alpha, beta=beta, rk=rk,
                                 maxrk=maxrk, acc=acc, kind=kind, rank_out=out["rank"],
                                 flops=out["flops"]))

    # -- config "nb=512, ranks 32, acc 1e-8, maxrk 64": seed + fingerprint --
    AU, AV, BU, BV, CU, CV = seeded_inputs(2024, 512, 32, 32, 32)
    out = ref.dgemm(512, 1.0, AU, AV, 32, BU, BV, 32, 1.0, CU, CV, 32, maxrk=64, acc=1e-8)
    P = out["CU"] @ out["CV"].T
    omega = np.random.default_rng(7).standard_normal((512, 8))
    D = O.dense_update(1.0, AU, AV, BU, BV, 1.0, CU, CV)
    arrs["cfg512_fingerprint"] = P @ omega
    meta["cfg512"] = dict(seed=2024, omega_seed=7, M=512, a=32, b=32, c=32, maxrk=64, acc=1e-8,
                          rank_out=out["rank"], flops=out["flops"], fro=float(np.linalg.norm(P)),
                          err_vs_dense=O.rel_fro(P, D))

    # -- HCORE_dsyrk / HCORE_dgemmcd --
    for i, (name, M, K, alpha) in enumerate(SYRK_CASES):
        rng = np.random.default_rng(300 + i)
        AU = np.asfortranarray(rng.standard_normal((M, K)))
        AV = np.asfortranarray(rng.standard_normal((M, K)))
        CD = np.asfortranarray(np.tril(rng.standard_normal((M, M))))
        CDo, fl = ref.dsyrk(M, K, alpha, AU, AV, CD)
        arrs.update({f"{name}_AU": AU, f"{name}_AV": AV, f"{name}_CD": CD, f"{name}_CDo": CDo})
        meta["syrk"].append(dict(name=name, M=M, K=K, alpha=alpha, flops=fl))
    for i, (name, M, ra, rb) in enumerate(GEMMCD_CASES):
        rng = np.random.default_rng(400 + i)
        Au, Av = (np.asfortranarray(rng.standard_normal((M, ra))) for _ in range(2))
        Bu, Bv = (np.asfortranarray(rng.standard_normal((M, rb))) for _ in range(2))
        CD = np.asfortranarray(rng.standard_normal((M, M)))
        CDo = ref.dgemmcd(M, Au, Av, ra, Bu, Bv, rb, CD, max(ra, rb))
        arrs.update({f"{name}_Au": Au, f"{name}_Av": Av, f"{name}_Bu": Bu, f"{name}_Bv": Bv,
                     f"{name}_CD": CD, f"{name}_CDo": CDo})
        meta["gemmcd"].append(dict(name=name, M=M, a=ra, b=rb))

    # the reference dsyrk/dgemmcd known-answer inputs (glibc rand, default seed)
    Cm, (AU7, AV7) = libc_rand_matrices(10, [7])
    CDo, fl = ref.dsyrk(10, 7, 1.0, AU7, AV7, Cm)
    arrs.update(kat_dsyrk_C=Cm, kat_dsyrk_AU=AU7, kat_dsyrk_AV=AV7, kat_dsyrk_CDo=CDo)
    meta["kat_dsyrk"] = dict(M=10, K=7, flops=fl)

    np.savez_compressed(os.path.join(OUT, "golden_small.npz"), **arrs)
    with open(os.path.join(OUT, "golden_meta.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)
    print(json.dumps(meta["known_answer"], indent=1))
    print("cases:", len(meta["gemm"]), "size:",
          os.path.getsize(os.path.join(OUT, "golden_small.npz")))


def tlr_spd(rng, n):
    """Seeded symmetric positive definite n x n (well conditioned)."""
    X = rng.standard_normal((n, n))
    return np.asfortranarray(X @ X.T / n + np.eye(n))


def tlr_triangle(rng, n, uplo):
    """Seeded triangular n x n, diagonal in [2, 3] with random signs, the
    unused triangle NaN (BLAS must not read it)."""
    T = rng.uniform(-0.5, 0.5, (n, n)) / np.sqrt(n)
    np.fill_diagonal(T, rng.uniform(2, 3, n) * rng.choice([-1.0, 1.0], n))
    keep = np.tril(np.ones((n, n), bool)) if uplo == 122 else np.triu(np.ones((n, n), bool))
    return np.asfortranarray(np.where(keep, T, np.nan))


def make_tlr():
    """Fixtures of HCORE_duncompress, HCORE_dgemmbdcd, HCORE_dtrsm and
    HCORE_dpotrf (golden_tlr.npz / golden_tlr_meta.json)."""
    ref = O.RefLib()
    meta = {"uncompress": [], "gemmbdcd": [], "trsm": [], "potrf": []}
    arrs = {}
    for i, (M, N, a) in enumerate([(64, 48, 6), (40, 40, 0)]):
        rng = np.random.default_rng(500 + i)
        AU = np.asfortranarray(rng.standard_normal((M, a)))
        BV = np.asfortranarray(rng.standard_normal((N, a)))
        CD = np.asfortranarray(rng.standard_normal((M, N)))
        name = f"unc{i}"
        arrs.update({f"{name}_AU": AU, f"{name}_BV": BV, f"{name}_CD": CD,
                     f"{name}_CDo": ref.duncompress(M, N, AU, a, BV, CD)})
        meta["uncompress"].append(dict(name=name, M=M, N=N, a=a))
    # (transA, M, N, a, LDA, LDB, LDC): LDB > M and LDA > M exercise the two
    # branches' row counts (hcore_dgemmbdcd.c:78-117)
    for i, (tr, M, N, a, lda, ldb, ldc) in enumerate([(111, 64, 40, 9, 64, 64, 64),
                                                      (112, 64, 40, 9, 64, 64, 64),
                                                      (111, 48, 33, 7, 60, 56, 50),
                                                      (112, 48, 33, 7, 52, 48, 52)]):
        rng = np.random.default_rng(600 + i)
        AU = np.asfortranarray(rng.standard_normal((lda, a)))
        AV = np.asfortranarray(rng.standard_normal((lda, a)))
        BD = np.asfortranarray(rng.standard_normal((ldb, N)))
        CD = np.asfortranarray(rng.standard_normal((ldc, N)))
        CDo, fl = ref.dgemmbdcd(tr, M, N, 0.7, AU, AV, a, BD, -1.3, CD)
        name = f"bdcd{i}"
        arrs.update({f"{name}_AU": AU, f"{name}_AV": AV, f"{name}_BD": BD, f"{name}_CD": CD,
                     f"{name}_CDo": CDo})
        meta["gemmbdcd"].append(dict(name=name, transA=tr, M=M, N=N, a=a, alpha=0.7, beta=-1.3,
                                     flops=fl))
    i = 0
    for side in (141, 142):
        for uplo in (121, 122):
            for tr in (111, 112):
                for dg in (131, 132):
                    rng = np.random.default_rng(700 + i)
                    M, N = 40, 7
                    na = M if side == 141 else N
                    A = tlr_triangle(rng, na, uplo)
                    B = np.asfortranarray(rng.standard_normal((M, N)))
                    Bo, fl = ref.dtrsm(side, uplo, tr, dg, M, N, 0.5, A, B)
                    name = f"trsm{i}"
                    arrs.update({f"{name}_A": A, f"{name}_B": B, f"{name}_Bo": Bo})
                    meta["trsm"].append(dict(name=name, side=side, uplo=uplo, trans=tr, diag=dg,
                                             M=M, N=N, alpha=0.5, flops=fl))
                    i += 1
    for i, (uplo, n, fail_at) in enumerate([(ord("L"), 100, None), (ord("U"), 70, None),
                                            (ord("L"), 40, 11), (122, 20, None)]):
        rng = np.random.default_rng(800 + i)
        S = tlr_spd(rng, n)
        if fail_at is not None:
            S[fail_at - 1, fail_at - 1] = -5.0
        # the triangle dpotrf must not read
        other = np.triu(np.ones((n, n), bool), 1) if uplo != ord("U") else np.tril(np.ones((n, n), bool), -1)
        S = np.asfortranarray(np.where(other, np.nan, S))
        So, info, fl = ref.dpotrf(uplo, n, S)
        name = f"potrf{i}"
        arrs.update({f"{name}_A": S, f"{name}_Ao": So})
        meta["potrf"].append(dict(name=name, uplo=uplo, n=n, info=info, flops=fl))
    np.savez_compressed(os.path.join(OUT, "golden_tlr.npz"), **arrs)
    with open(os.path.join(OUT, "golden_tlr_meta.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)
    print("tlr cases:", {k: len(v) for k, v in meta.items()}, "size:",
          os.path.getsize(os.path.join(OUT, "golden_tlr.npz")))


def make_compress():
    """Fixtures of the reference tests' compressor, generate_compress
    (testing/testing_dgemm.c:119-236): dlatms tiles with sigma_i = 10^-i from
    iseed {0,0,0,1}, compressed at thresholds between singular values (no
    ties), with a rank cap and a rank of 0 (golden_compress.npz / .json)."""
    ref = O.RefLib()
    meta, arrs = [], {}
    for i, (M, acc, maxrank) in enumerate([(64, 3e-8, 64), (100, 3e-13, 10), (48, 2.0, 8),
                                           (130, 5e-5, 130)]):
        A, r, U, V, _ = ref.generate_compress(M, acc, maxrank, [0, 0, 0, 1 + 2 * i])
        name = f"cmp{i}"
        arrs.update({f"{name}_A": A, f"{name}_U": U, f"{name}_V": V})
        meta.append(dict(name=name, M=M, acc=acc, maxrank=maxrank, rank=r))
    np.savez_compressed(os.path.join(OUT, "golden_compress.npz"), **arrs)
    with open(os.path.join(OUT, "golden_compress_meta.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)
    print("compress cases:", [(c["M"], c["rank"]) for c in meta])


def complex_lowrank(rng, M, k, decades):
    """U diag(sigma) and V with complex orthonormal U, V (QR of complex
    Gaussians), sigma_i = 10^(-decades*i/k) folded into U."""
    U, _ = np.linalg.qr(rng.standard_normal((M, k)) + 1j * rng.standard_normal((M, k)))
    V, _ = np.linalg.qr(rng.standard_normal((M, k)) + 1j * rng.standard_normal((M, k)))
    s = 10.0 ** (-decades * np.arange(k) / k)
    return np.asfortranarray(U * s), np.asfortranarray(V)


# (name, M, a, b, c, alpha, beta, rk, maxrk, acc)
ZGEMM_CASES = [
    ("z_small", 64, 6, 7, 5, 1 + 0.5j, 0.8 - 0.2j, 0, 16, 1e-8),
    ("z_schur", 96, 12, 10, 14, -1.0, 1.0, 0, 40, 1e-6),
    ("z_fixed", 80, 10, 9, 11, 1.0, 1.0, 5, 24, 1e-8),
    ("z_rank1", 48, 1, 1, 1, 0.5j, 1.0, 0, 4, 1e-8),
]


def make_zgemm():
    """Fixtures of the reference's HCORE_zgemm (golden_zgemm.npz / .json)."""
    ref = O.RefLib()
    meta, arrs = [], {}
    for i, (name, M, a, b, c, alpha, beta, rk, maxrk, acc) in enumerate(ZGEMM_CASES):
        rng = np.random.default_rng(900 + i)
        AU, AV = complex_lowrank(rng, M, a, 8)
        BU, BV = complex_lowrank(rng, M, b, 8)
        CU, CV = complex_lowrank(rng, M, c, 8)
        out = ref.zgemm(M, alpha, AU, AV, a, BU, BV, b, beta, CU, CV, c, rk=rk, maxrk=maxrk,
                        acc=acc)
        for nm, v in dict(AU=AU, AV=AV, BU=BU, BV=BV, CU=CU, CV=CV, CUo=out["CU"],
                          CVo=out["CV"]).items():
            arrs[f"{name}_{nm}"] = v
        meta.append(dict(name=name, M=M, a=a, b=b, c=c,
                         alpha=[complex(alpha).real, complex(alpha).imag],
                         beta=[complex(beta).real, complex(beta).imag], rk=rk, maxrk=maxrk,
                         acc=acc, rank=out["rank"], flops=out["flops"]))
    # HCORE_zuncompress: CD = AU BV^T (M x N), plain transpose
    rng = np.random.default_rng(950)
    M, N, r = 50, 40, 5
    AU = np.asfortranarray(rng.standard_normal((M, r)) + 1j * rng.standard_normal((M, r)))
    BV = np.asfortranarray(rng.standard_normal((N, r)) + 1j * rng.standard_normal((N, r)))
    CD = np.asfortranarray(rng.standard_normal((M, N)) + 0j)
    arrs.update(zunc_AU=AU, zunc_BV=BV, zunc_CDo=ref.zuncompress(M, N, AU, r, BV, CD))
    np.savez_compressed(os.path.join(OUT, "golden_zgemm.npz"), **arrs)
    with open(os.path.join(OUT, "golden_zgemm_meta.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)
    print("zgemm cases:", [(c["name"], c["rank"]) for c in meta])


if __name__ == "__main__":
    only = [a for a in sys.argv[1:] if a.endswith("-only")]
    if not only:
        main()
    if not only or "--tlr-only" in only:
        make_tlr()
    if not only or "--compress-only" in only:
        make_compress()
    if not only or "--zgemm-only" in only:
        make_zgemm()
