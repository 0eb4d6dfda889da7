"""ORACLE build recipe (test infrastructure only).

Two products, both git-ignored:

* ``oracle/_build/libhcore_port.so`` — the C restatement in ``hcore_port.c``,
  built on whichever machine runs the tests against the OpenBLAS that SciPy
  bundles.  This is the checker the GPU tests and the CPU baseline use.
* ``oracle/_ref/`` — the reference HCORE itself, compiled unmodified from its
  own sources where they lie (``src/compute/*.c``, ``src/misc/descutil/
  flop_counts.c``) plus its four ctest programs (``testing/testing_*.c``).
  Only built where the reference checkout exists; it is used to pin the
  restatement (tests/golden/make_golden.py) and is never shipped.

The reference's CMake build cannot run here (its ECRC CMake submodule is
empty), so this recipe calls gcc on the few source files directly, with the
compatibility headers in ``oracle/compat`` standing in for cblas.h/lapacke.h.
"""
from __future__ import annotations

import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
REFERENCE_ROOT = os.environ.get("HCORE_REFERENCE_ROOT", "/root/reference")

# reference sources of the low-rank update path (file names within the project)
REF_SOURCES = [
    "src/compute/hcore_dgemm.c",
    "src/compute/hcore_sgemm.c",
    "src/compute/hcore_dgemm_fast.c",
    "src/compute/hcore_dsyrk.c",
    "src/compute/hcore_dgemmcd.c",
    "src/compute/hcore_dgemmbdcd.c",
    "src/compute/hcore_dpotrf.c",
    "src/compute/hcore_dtrsm.c",
    "src/compute/hcore_duncompress.c",
    "src/compute/hcore_zgemm.c",
    "src/compute/hcore_zuncompress.c",
    "src/misc/descutil/flop_counts.c",
]
REF_TESTS = ["testing_dgemm", "testing_sgemm", "testing_dsyrk", "testing_dgemmcd"]


def openblas_lib() -> str:
    """Path of the OpenBLAS shared library bundled with the installed SciPy."""
    import scipy

    libdir = os.path.join(os.path.dirname(os.path.dirname(scipy.__file__)), "scipy.libs")
    cands = sorted(glob.glob(os.path.join(libdir, "libscipy_openblas*.so*")))
    if not cands:
        raise RuntimeError(f"no SciPy-bundled OpenBLAS under {libdir}")
    return cands[0]


def _link_flags() -> list[str]:
    lib = openblas_lib()
    d = os.path.dirname(lib)
    return [f"-L{d}", f"-l:{os.path.basename(lib)}", f"-Wl,-rpath,{d}", "-lm"]


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def port_path() -> str:
    return os.path.join(BUILD, "libhcore_port.so")


def build_port(force: bool = False) -> str:
    """Compile the C restatement; returns the .so path."""
    os.makedirs(BUILD, exist_ok=True)
    out = port_path()
    srcs = [os.path.join(HERE, f) for f in ("hcore_port.c", "hcore_port_impl.h", "hcore_port.h")]
    if not force and os.path.exists(out) and all(
        os.path.getmtime(out) >= os.path.getmtime(s) for s in srcs
    ):
        return out
    tmp = out + f".tmp{os.getpid()}"
    _run(["gcc", "-O2", "-std=gnu99", "-fPIC", "-shared", "-I", HERE,
          os.path.join(HERE, "hcore_port.c"), "-o", tmp] + _link_flags())
    os.replace(tmp, out)
    return out


def reference_available() -> bool:
    return os.path.isdir(os.path.join(REFERENCE_ROOT, "src", "compute"))


def ref_lib_path() -> str:
    return os.path.join(REF_OUT, "libhcore_ref.so")


def ref_test_lib_path() -> str:
    return os.path.join(REF_OUT, "libhcore_reftest.so")


def build_ref(force: bool = False) -> str | None:
    """Compile the reference HCORE from its own sources (only where present)."""
    if not reference_available():
        return None
    os.makedirs(REF_OUT, exist_ok=True)
    out = ref_lib_path()
    if os.path.exists(out) and os.path.exists(ref_test_lib_path()) and not force:
        return out
    inc = ["-I", os.path.join(HERE, "compat"),
           "-I", os.path.join(REFERENCE_ROOT, "src", "include"),
           "-I", os.path.join(REFERENCE_ROOT, "src", "misc", "include")]
    cflags = ["gcc", "-O2", "-std=gnu99", "-fcommon", "-fPIC", "-w"] + inc
    objs = []
    for s in REF_SOURCES:
        o = os.path.join(REF_OUT, os.path.basename(s).replace(".c", ".o"))
        _run(cflags + ["-c", os.path.join(REFERENCE_ROOT, s), "-o", o])
        objs.append(o)
    # (hcore_duncompress.c:23-24 declares gemmfrk_print_index/_mat extern;
    # hcore_zuncompress.c defines them)
    # the library leaves use_scratch to its caller (hcore_dgemm.c:38); the
    # ctypes-loaded copy gets it from this one-line definition
    glob_c = os.path.join(REF_OUT, "use_scratch.c")
    with open(glob_c, "w") as f:
        f.write("int use_scratch = 0;\n")
    _run(cflags + ["-c", glob_c, "-o", os.path.join(REF_OUT, "use_scratch.o")])
    _run(["gcc", "-shared", "-o", out] + objs + [os.path.join(REF_OUT, "use_scratch.o")]
         + _link_flags())
    # testing_dgemm.c as a library (its main renamed) for its compressor,
    # generate_compress (:119-236), which the reference has nowhere else
    t_o = os.path.join(REF_OUT, "testing_dgemm_lib.o")
    _run(cflags + ["-Dmain=hcore_testing_dgemm_main", "-c",
                   os.path.join(REFERENCE_ROOT, "testing", "testing_dgemm.c"), "-o", t_o])
    _run(["gcc", "-shared", "-o", ref_test_lib_path(), t_o] + objs + _link_flags())
    # the reference's four known-answer test programs, linked statically
    # against the same objects (each defines its own use_scratch)
    for t in REF_TESTS:
        exe = os.path.join(REF_OUT, t)
        _run(cflags + [os.path.join(REFERENCE_ROOT, "testing", t + ".c"), "-o", exe] + objs
             + _link_flags())
    return out


if __name__ == "__main__":
    print(build_port(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
