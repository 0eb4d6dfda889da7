"""The C boundary from a compiled C caller.

tests/capi_caller.c includes the library's public headers (include/hcore_d.h,
include/hcore_s.h), defines `use_scratch` as the reference's test programs do,
and calls HCORE_dgemm, HCORE_sgemm, HCORE_dsyrk and HCORE_dgemmcd.  Compiling
it with gcc and linking -lhcore_gb300 checks the prototypes against a C
compiler and linker, not only through hand-written ctypes argtypes.  The
outputs are compared with the reference's golden results, with the gates of
the reference's own known-answer programs (testing/testing_dgemm.c:250-392:
rank 4 -> 6, inf-norm error < 10 acc; testing_dsyrk.c, testing_dgemmcd.c:
1000 eps) and of the other parity tests (FP64 product within 1e-11, FP32
within 5e-5, dense tiles within 1e-12 of the largest entry, flop counts equal
bit for bit).
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _write(d, name, field, x, dtype=np.float64):
    np.asfortranarray(np.asarray(x, dtype=dtype)).T.tofile(os.path.join(d, f"{name}_{field}.bin"))


def _read(d, name, field, M, cols, dtype=np.float64):
    x = np.fromfile(os.path.join(d, f"{name}_{field}.bin"), dtype=dtype)
    return x.reshape(cols, M).T


def test_compiled_c_caller_matches_reference(hc, golden, tmp_path):
    from hcore_gb300 import build as hbuild

    gcc = shutil.which("gcc") or shutil.which("cc")
    assert gcc, "a C compiler is needed for this test"
    exe = str(tmp_path / "capi_caller")
    libdir = os.path.dirname(hbuild.LIB)
    cmd = [gcc, "-std=c99", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "capi_caller.c"), "-o", exe, f"-L{libdir}", "-lhcore_gb300",
           f"-Wl,-rpath,{libdir}", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr

    meta, g = golden
    d = str(tmp_path)
    lines = []
    for c in meta["gemm"]:
        if c["kind"] == "fast":
            continue
        n, dt = c["name"], (np.float32 if c["kind"] == "sgemm" else np.float64)
        for f in ("AU", "AV", "BU", "BV", "CU", "CV"):
            _write(d, n, f, g[f"{n}_{f}"], dt)
        lines.append(f"{c['kind']} {n} {c['M']} {c['a']} {c['b']} {c['c']} {c['alpha']!r} "
                     f"{c['beta']!r} {c['acc']!r} {c['maxrk']} {c['rk']}")
    for c in meta["syrk"]:
        n = c["name"]
        for f in ("AU", "AV", "CD"):
            _write(d, n, f, g[f"{n}_{f}"])
        lines.append(f"dsyrk {n} {c['M']} {c['K']} {c['alpha']!r}")
    for c in meta["gemmcd"]:
        n = c["name"]
        for f in ("Au", "Av", "Bu", "Bv", "CD"):
            _write(d, n, f, g[f"{n}_{f}"])
        lines.append(f"dgemmcd {n} {c['M']} {c['a']} {c['b']}")
    for f in ("A", "B", "C", "AU", "AV", "BU", "BV", "CU", "CV"):
        _write(d, "kat_dgemm", f, g[f"kat_dgemm_{f}"])
    lines.append("kat kat_dgemm 10 4 4 4 0.0001")
    with open(os.path.join(d, "cases.txt"), "w") as fh:
        fh.write("\n".join(lines) + "\n")

    r = subprocess.run([exe, d], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    out = {}
    for ln in r.stdout.splitlines():
        parts = ln.split()
        out[parts[0]] = dict(p.split("=", 1) for p in parts[1:] if "=" in p)
        out[parts[0]]["verdict"] = parts[-1]

    for c in meta["gemm"]:
        if c["kind"] == "fast":
            continue
        n, dt = c["name"], (np.float32 if c["kind"] == "sgemm" else np.float64)
        rk = int(out[n]["rank"])
        assert rk == c["rank_out"], n
        if c["flops"] is not None:
            assert int(out[n]["flops"]) == c["flops"], n
        P = _read(d, n, "CUo", c["M"], rk, dt).astype(np.float64) @ \
            _read(d, n, "CVo", c["M"], rk, dt).T.astype(np.float64)
        P_ref = g[f"{n}_CUo"].astype(np.float64) @ g[f"{n}_CVo"].T.astype(np.float64)
        assert O.rel_fro(P, P_ref) < (5e-5 if dt == np.float32 else 1e-11), n
    for c in meta["syrk"] + meta["gemmcd"]:
        n = c["name"]
        CD = _read(d, n, "CDo", c["M"], c["M"])
        ref = g[f"{n}_CDo"]
        np.testing.assert_allclose(CD, ref, rtol=0, atol=1e-12 * np.abs(ref).max())
        if "flops" in c:
            assert int(out[n]["flops"]) == c["flops"]
    kat = out["kat_dgemm"]
    assert int(kat["rank"]) == 6 and kat["verdict"] == "PASS"
    assert int(kat["flops"]) == meta["kat_dgemm"]["flops"]
