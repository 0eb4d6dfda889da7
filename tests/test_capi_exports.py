"""The C-ABI library loads without a GPU and exports every symbol that
include/*.h declares (functions and globals).  CPU only: nothing is called."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    funcs, globs = set(), set()
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"//[^\n]*", "", src)
        for m in re.finditer(r"\b(HCORE_\w+|hcore_gpu_\w+)\s*\(", src):
            if not src[:m.start()].rstrip().endswith("define"):
                funcs.add(m.group(1))
        for m in re.finditer(r"\bextern\s+int\s+(\w+)\s*;", src):
            globs.add(m.group(1))
    return funcs, globs


@pytest.fixture(scope="module")
def so():
    from hcore_gb300 import build

    path = build.build()
    return ctypes.CDLL(path)


def test_headers_declare_the_reference_entry_points():
    funcs, globs = declared_symbols()
    for f in ("HCORE_dgemm", "HCORE_sgemm", "HCORE_dgemm_fast", "HCORE_dsyrk", "HCORE_dgemmcd",
              "HCORE_dgemm_qr_svd", "HCORE_dgemm_qr_svd_b_dense", "HCORE_dgemm_ormqr",
              "HCORE_sgemm_qr_svd", "HCORE_sgemm_ormqr", "HCORE_dgemm_dense", "HCORE_dtrsm",
              "HCORE_dpotrf", "HCORE_duncompress", "HCORE_dgemmbdcd"):
        assert f in funcs
    for g in ("use_trmm", "gemm_print_index", "gemm_print_mat", "hc_nelm_limit",
              "sgemm_use_trmm", "syrk_print_index", "gemmcd_print_index", "gemmbdcd_print_index"):
        assert g in globs
    assert "use_scratch" not in globs   # the caller's, as in the reference


def test_library_exports_every_declared_symbol(so):
    funcs, globs = declared_symbols()
    missing = [s for s in sorted(funcs | globs) if not hasattr(so, s)]
    assert not missing, missing


def test_globals_have_reference_defaults(so):
    assert ctypes.c_int.in_dll(so, "use_trmm").value == 0
    assert ctypes.c_int.in_dll(so, "hc_nelm_limit").value == 512
    assert ctypes.c_int.in_dll(so, "gemm_print_index").value == 0


def test_c_caller_compiles_and_links_against_the_headers(so, tmp_path):
    """tests/capi_caller.c (the compiled caller the GPU test runs) builds with
    -Wall -Werror against include/*.h and links -lhcore_gb300 with no
    unresolved symbol: the prototypes agree with a C compiler and linker."""
    import shutil
    import subprocess

    from hcore_gb300 import build

    gcc = shutil.which("gcc") or shutil.which("cc")
    if not gcc:
        pytest.skip("no C compiler")
    libdir = os.path.dirname(build.LIB)
    exe = str(tmp_path / "capi_caller")
    r = subprocess.run([gcc, "-std=c99", "-O2", "-Wall", "-Werror", "-I",
                        os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "capi_caller.c"),
                        "-o", exe, f"-L{libdir}", "-lhcore_gb300", f"-Wl,-rpath,{libdir}",
                        "-Wl,--no-undefined", "-lm"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
