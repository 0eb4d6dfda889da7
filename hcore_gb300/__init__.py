"""hcore-gb300: HCORE's tile low-rank kernels on one GB300 GPU.

The product is the C-ABI library ``libhcore_gb300.so`` (include/hcore_d.h,
include/hcore_s.h, include/hcore_gb300.h).  This package is its Python host
side: it loads the library with ctypes and mirrors the reference's operator
interface so tests and benchmarks read like the reference's own:

* :func:`hcore_dgemm` / :func:`hcore_sgemm` — one update with the signature
  and semantics of HCORE_dgemm / HCORE_sgemm (src/compute/hcore_dgemm.c:703),
  on numpy arrays, through the drop-in C entry points;
* :class:`Batch` — many independent updates in one plan (device tensors),
  executed by the batched GPU kernels and capturable in a CUDA graph;
* :func:`dense_batched` — HCORE_dsyrk / HCORE_dgemmcd / HCORE_duncompress /
  HCORE_dgemmbdcd tile operations;
* :func:`trsm_batched` / :func:`potrf_batched` — HCORE_dtrsm on many factors
  and HCORE_dpotrf on dense tiles, the steps either side of the update in a
  TLR Cholesky;
* :func:`compress_batched` — dense tiles to U, V factors (the reference
  tests' compressor semantics) on the GPU;
* :func:`hcore_zgemm` — the complex update (HCORE_zgemm) through its drop-in
  entry point;
* :class:`RankMLP` — the rank predictor's network, trained and run by the
  library's own CUDA kernels (see :mod:`hcore_gb300.predictor`).

There is no CPU fallback: importing works without a GPU, but every call into
the library needs the compiled extension and a CUDA device, and raises
otherwise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .build import LIB as _LIB_PATH

__all__ = ["lib", "LrTask", "DenseTask", "Batch", "DensePlan", "hcore_dgemm", "hcore_sgemm", "hcore_dgemm_fast",
           "dense_batched", "TrsmTask", "PotrfTask", "trsm_batched", "potrf_batched",
           "CompressTask", "compress_batched", "hcore_zgemm", "ZlrTask", "zgemm_batched", "HcoreError", "STATUS", "FlopCounter", "RankMLP", "Tuning",
           "make_tuning", "autotune"]

F64, F32 = 0, 1
FAST_RULES = 0x1
STAGE_INPUTS = 0x2
MIXED_FACTORS = 0x4
DFMA_REBUILD = 0x8
UNBLOCKED_QR = 0x10
TC_STACK = 0x20
STATUS = {0: "ok", 1: "zero rank", 2: "rank sum > 2*maxrk", 3: "rank sum > ld_newV",
          4: "new rank > maxrk", 5: "new rank > storage maxrank", 6: "Jacobi did not converge",
          7: "bad shape", 8: "tensor-core wait timed out"}


class HcoreError(RuntimeError):
    pass


class LrTask(C.Structure):
    """Mirror of hcore_lr_task (include/hcore_gb300.h)."""

    _fields_ = [("M", C.c_int), ("a", C.c_int), ("b", C.c_int), ("c", C.c_int), ("rk", C.c_int),
                ("maxrk", C.c_int), ("ld_newv", C.c_int), ("storage_maxrank", C.c_int),
                ("alpha", C.c_double), ("beta", C.c_double), ("acc", C.c_double),
                ("AU", C.c_void_p), ("AV", C.c_void_p), ("lda", C.c_int),
                ("BU", C.c_void_p), ("BV", C.c_void_p), ("ldb", C.c_int),
                ("Bdense", C.c_void_p),
                ("CU", C.c_void_p), ("CV", C.c_void_p), ("ldc", C.c_int),
                ("CUo", C.c_void_p), ("CVo", C.c_void_p), ("ldco", C.c_int)]


class DenseTask(C.Structure):
    """Mirror of hcore_dense_task (include/hcore_gb300.h)."""

    _fields_ = [("kind", C.c_int), ("M", C.c_int), ("a", C.c_int), ("b", C.c_int),
                ("alpha", C.c_double), ("Au", C.c_void_p), ("Av", C.c_void_p), ("lda", C.c_int),
                ("Bu", C.c_void_p), ("Bv", C.c_void_p), ("ldb", C.c_int), ("CD", C.c_void_p),
                ("ldcd", C.c_int), ("N", C.c_int), ("beta", C.c_double), ("kdim", C.c_int),
                ("Bd", C.c_void_p)]


class TrsmTask(C.Structure):
    """Mirror of hcore_trsm_task (include/hcore_gb300.h)."""

    _fields_ = [("side", C.c_int), ("uplo", C.c_int), ("trans", C.c_int), ("diag", C.c_int),
                ("M", C.c_int), ("N", C.c_int), ("alpha", C.c_double), ("A", C.c_void_p),
                ("lda", C.c_int), ("B", C.c_void_p), ("ldb", C.c_int)]


class PotrfTask(C.Structure):
    """Mirror of hcore_potrf_task (include/hcore_gb300.h); uplo is 'L' or 'U'."""

    _fields_ = [("uplo", C.c_int), ("n", C.c_int), ("A", C.c_void_p), ("lda", C.c_int)]


class TlrMatrix(C.Structure):
    """Mirror of hcore_tlr_matrix (include/hcore_gb300.h): D, U, V are
    addresses of pointer arrays (nt and nt*nt entries), rank the address of
    an nt*nt int array."""

    _fields_ = [("nt", C.c_int), ("nb", C.c_int), ("D", C.c_void_p), ("ldd", C.c_int),
                ("U", C.c_void_p), ("V", C.c_void_p), ("rank", C.c_void_p), ("maxrank", C.c_int)]


class CompressTask(C.Structure):
    """Mirror of hcore_compress_task (include/hcore_gb300.h)."""

    _fields_ = [("M", C.c_int), ("D", C.c_void_p), ("ldd", C.c_int), ("acc", C.c_double),
                ("relative", C.c_int), ("maxrank", C.c_int), ("U", C.c_void_p), ("V", C.c_void_p),
                ("ldo", C.c_int)]


class DComplex(C.Structure):
    """double _Complex by value (hcore_dcomplex in include/hcore_z.h)."""

    _fields_ = [("re", C.c_double), ("im", C.c_double)]


class ZlrTask(C.Structure):
    """Mirror of hcore_zlr_task (include/hcore_z.h)."""

    _fields_ = [("M", C.c_int), ("a", C.c_int), ("b", C.c_int), ("c", C.c_int),
                ("rk", C.c_int), ("maxrk", C.c_int), ("alpha", DComplex), ("beta", DComplex),
                ("acc", C.c_double), ("AU", C.c_void_p), ("AV", C.c_void_p), ("lda", C.c_int),
                ("BU", C.c_void_p), ("BV", C.c_void_p), ("ldb", C.c_int), ("CU", C.c_void_p),
                ("CV", C.c_void_p), ("ldc", C.c_int)]


class Tuning(C.Structure):
    """Mirror of hcore_gpu_tuning (include/hcore_gb300.h)."""

    _fields_ = [("stream_groups", C.c_int), ("svd_lanes", C.c_int * 3), ("bucket_width", C.c_int),
                ("phase_sync", C.c_int), ("qr_warps", C.c_int)]

    def as_dict(self) -> dict:
        return {"stream_groups": self.stream_groups, "svd_lanes": list(self.svd_lanes),
                "bucket_width": self.bucket_width, "phase_sync": self.phase_sync,
                "qr_warps": self.qr_warps}


class FlopCounter(C.Structure):
    """Mirror of flop_counter (include/flop_util_structs.h)."""

    _fields_ = [("__pad1", C.c_ulong), ("__pad2", C.c_ulong), ("copy", C.c_ulong),
                ("flop", C.c_ulong), ("tid", C.c_int), ("potrf", C.c_ulong),
                ("trsm", C.c_ulong), ("syrk", C.c_ulong), ("update", C.c_ulong)] + [
        (n, C.c_ulong) for n in (
            "geqrfu", "geqrfv", "geqrfv_gemm", "gesvd", "gesvd_gemm", "gesvd_lasetu",
            "gesvd_lasetv", "gesvd_lacpyu", "gesvd_lacpyv", "gesvd_dscal", "ormqru",
            "ormqru_laset", "ormqru_lacpy", "ormqrv", "ormqrv_laset", "ormqrv_lacpy",
            "omatcopy")] + [("numthreads", C.c_int), ("__pad3", C.c_ulong),
                            ("__pad4", C.c_ulong)]


_lib = None
_dp, _fp, _ip = C.POINTER(C.c_double), C.POINTER(C.c_float), C.POINTER(C.c_int)


def lib_path() -> str:
    return _LIB_PATH


def lib() -> C.CDLL:
    """Load libhcore_gb300.so (built by hcore_gb300/build.py); raises if absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB_PATH):
        raise HcoreError(f"{_LIB_PATH} is missing: run `python -m hcore_gb300.build` first")
    L = C.CDLL(_LIB_PATH)
    vp = C.c_void_p
    L.hcore_gpu_plan_create.argtypes = [C.POINTER(vp), C.c_int, C.c_int, C.POINTER(LrTask), C.c_uint]
    L.hcore_gpu_plan_execute.argtypes = [vp, vp]
    L.hcore_gpu_plan_create_tuned.argtypes = [C.POINTER(vp), C.c_int, C.c_int, C.POINTER(LrTask),
                                              C.c_uint, C.POINTER(Tuning)]
    L.hcore_gpu_tuning_default.argtypes = [C.POINTER(Tuning)]
    L.hcore_gpu_autotune.argtypes = [C.c_int, C.c_int, C.POINTER(LrTask), C.c_uint, C.c_int, vp,
                                     C.POINTER(Tuning), C.POINTER(C.c_double)]
    L.hcore_gpu_plan_results.argtypes = [vp, _ip, _ip, vp]
    L.hcore_gpu_plan_sigma.argtypes = [vp, C.c_int, _dp, _ip, vp]
    L.hcore_gpu_plan_destroy.argtypes = [vp]
    L.hcore_gpu_plan_sweeps.argtypes = [vp, _ip, vp]
    L.hcore_gpu_plan_execute_phases.argtypes = [vp, vp, C.c_uint]
    L.hcore_gpu_plan_rebuild.argtypes = [vp, C.c_int, _ip, C.POINTER(vp), C.POINTER(vp), _ip, _ip,
                                         vp]
    L.hcore_gpu_fp64_peak.argtypes = [vp]
    L.hcore_gpu_fp64_peak.restype = C.c_double
    L.hcore_gpu_fp64_probe.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, vp, _dp, _dp]
    L.hcore_gpu_plan_device_ranks.argtypes = [vp]
    L.hcore_gpu_plan_device_ranks.restype = vp
    L.hcore_gpu_plan_device_status.argtypes = [vp]
    L.hcore_gpu_plan_device_status.restype = vp
    L.hcore_gpu_plan_launches.argtypes = [vp]
    L.hcore_gpu_plan_workspace_bytes.argtypes = [vp]
    L.hcore_gpu_plan_workspace_bytes.restype = C.c_size_t
    L.hcore_gpu_plan_staged_bytes.argtypes = [vp]
    L.hcore_gpu_plan_staged_bytes.restype = C.c_size_t
    L.hcore_gpu_plan_zero_copy_bytes.argtypes = [vp]
    L.hcore_gpu_plan_zero_copy_bytes.restype = C.c_size_t
    L.hcore_gpu_dgemm_batched.argtypes = [C.c_int, C.POINTER(LrTask), _ip, _ip, vp]
    L.hcore_gpu_sgemm_batched.argtypes = [C.c_int, C.POINTER(LrTask), _ip, _ip, vp]
    L.hcore_gpu_dense_batched.argtypes = [C.c_int, C.POINTER(DenseTask), vp]
    L.hcore_gpu_dense_plan_create.argtypes = [C.POINTER(vp), C.c_int, C.POINTER(DenseTask)]
    L.hcore_gpu_dense_plan_execute.argtypes = [vp, vp]
    L.hcore_gpu_dense_plan_destroy.argtypes = [vp]
    L.hcore_gpu_trsm_batched.argtypes = [C.c_int, C.POINTER(TrsmTask), vp]
    L.hcore_gpu_compress_batched.argtypes = [C.c_int, C.POINTER(CompressTask),
                                             C.POINTER(C.c_int), C.POINTER(C.c_int), vp]
    L.hcore_gpu_potrf_batched.argtypes = [C.c_int, C.POINTER(PotrfTask), C.POINTER(C.c_int), vp]
    L.hcore_gpu_tlr_panel_step.argtypes = [C.POINTER(TlrMatrix), C.c_int, C.c_double, C.c_int,
                                           C.POINTER(C.c_int), C.POINTER(C.c_int), vp]
    L.hcore_gpu_mlp_create.argtypes = [C.POINTER(vp), C.c_ulonglong]
    L.hcore_gpu_mlp_params.argtypes = [vp, _fp, C.c_int]
    L.hcore_gpu_mlp_gradient.argtypes = [vp, vp, vp, C.c_int, _fp, _fp, vp]
    L.hcore_gpu_mlp_train.argtypes = [vp, vp, vp, C.c_int, C.c_int, C.c_int, C.c_float,
                                      C.c_ulonglong, _fp, vp]
    L.hcore_gpu_mlp_predict.argtypes = [vp, vp, C.c_int, vp, vp]
    L.hcore_gpu_mlp_destroy.argtypes = [vp]
    L.hcore_gpu_last_error.restype = C.c_char_p
    L.hcore_gpu_thread_stream.restype = vp
    for name, rp, real in (("HCORE_dgemm", _dp, C.c_double), ("HCORE_sgemm", _fp, C.c_float)):
        f = getattr(L, name)
        f.restype = None
        f.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, real, rp, rp, rp, C.c_int, rp, rp, rp,
                      C.c_int, real, rp, rp, rp, C.c_int, C.c_int, C.c_int, real, rp,
                      C.POINTER(FlopCounter)]
    L.HCORE_dgemm_fast.restype = None
    L.HCORE_dgemm_fast.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, _dp, _dp, _dp,
                                   C.c_int, _dp, _dp, _dp, C.c_int, C.c_double, _dp, _dp, _dp,
                                   C.c_int, C.c_int, C.c_int, C.c_double, _dp]
    L.HCORE_dsyrk.restype = None
    L.HCORE_dsyrk.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, _dp, C.c_int, _dp,
                              C.c_int, C.c_double, _dp, C.c_int, _dp, C.POINTER(FlopCounter)]
    L.HCORE_dgemmcd.restype = None
    L.HCORE_dgemmcd.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, _dp, _dp, C.c_int, C.c_int,
                                _dp, _dp, C.c_int, C.c_int, C.c_double, _dp, C.c_int, C.c_int, _dp,
                                C.POINTER(FlopCounter)]
    L.HCORE_zgemm.restype = None
    L.HCORE_zgemm.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, DComplex, vp, vp, _dp, C.c_int,
                              vp, vp, _dp, C.c_int, DComplex, vp, vp, _dp, C.c_int, C.c_int,
                              C.c_int, C.c_double, vp, C.POINTER(FlopCounter)]
    L.hcore_gpu_zgemm_batched.argtypes = [C.c_int, C.POINTER(ZlrTask), C.POINTER(C.c_int),
                                          C.POINTER(C.c_int), vp]
    L.HCORE_zuncompress.restype = None
    L.HCORE_zuncompress.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, DComplex, vp, _dp, C.c_int,
                                    vp, _dp, C.c_int, DComplex, vp, C.c_int]
    L.HCORE_duncompress.restype = None
    L.HCORE_duncompress.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, _dp, _dp,
                                    C.c_int, _dp, _dp, C.c_int, C.c_double, _dp, C.c_int]
    L.HCORE_dgemmbdcd.restype = None
    L.HCORE_dgemmbdcd.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, _dp, _dp, _dp,
                                  C.c_int, _dp, C.c_int, C.c_double, _dp, C.c_int, _dp,
                                  C.POINTER(FlopCounter)]
    L.HCORE_dtrsm.restype = None
    L.HCORE_dtrsm.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                              _dp, C.c_int, _dp, C.c_int, C.POINTER(FlopCounter)]
    L.HCORE_dpotrf.restype = None
    L.HCORE_dpotrf.argtypes = [C.c_int, C.c_int, _dp, C.c_int, C.POINTER(C.c_int),
                               C.POINTER(FlopCounter)]
    for name, rp, real in (("HCORE_dgemm_dense", _dp, C.c_double),
                           ("HCORE_sgemm_dense", _fp, C.c_float)):
        f = getattr(L, name)
        f.restype = None
        f.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, real, rp, C.c_int, rp, C.c_int,
                      real, rp, C.c_int]
    _lib = L
    return L


def last_error() -> str:
    return lib().hcore_gpu_last_error().decode()


def _check(rc: int, what: str) -> None:
    if rc != 0 and rc != -4:
        raise HcoreError(f"{what} failed ({rc}): {last_error()}")


def _fortran(a, dtype):
    return np.asfortranarray(np.asarray(a, dtype=dtype))


def _lr_update(name, M, alpha, AU, AV, a, BU, BV, b, beta, CU, CV, c, rk, maxrk, acc, dtype,
               fast=False):
    """Call the drop-in entry point on host arrays; returns (rank, CU, CV, flops)."""
    L = lib()
    rp = _fp if dtype == np.float32 else _dp
    AU, AV, BU, BV = (_fortran(x, dtype) for x in (AU, AV, BU, BV))
    ldc = CU.shape[0]
    ncol = max(a + c, c, 1)
    CUo = np.zeros((ldc, ncol), dtype=dtype, order="F")
    CVo = np.zeros((ldc, ncol), dtype=dtype, order="F")
    CUo[:, :c] = CU[:, :c]
    CVo[:, :c] = CV[:, :c]
    ra, rb, rc = (np.array([v], dtype=dtype) for v in (a, b, c))
    p = lambda x: x.ctypes.data_as(rp)  # noqa: E731
    if fast:
        L.HCORE_dgemm_fast(111, 112, M, M, alpha, p(AU), p(AV), p(ra), AU.shape[0], p(BU), p(BV),
                           p(rb), BV.shape[0], beta, p(CUo), p(CVo), p(rc), ldc, rk, maxrk, acc,
                           None)
        fl = None
    else:
        fc = FlopCounter()
        getattr(L, name)(111, 112, M, M, alpha, p(AU), p(AV), p(ra), AU.shape[0], p(BU), p(BV),
                         p(rb), BV.shape[0], beta, p(CUo), p(CVo), p(rc), ldc, rk, maxrk, acc,
                         None, C.byref(fc))
        fl = fc.update
    r = int(rc[0])
    return r, CUo[:, :r].copy(order="F"), CVo[:, :r].copy(order="F"), fl


def hcore_dgemm(M, alpha, AU, AV, a, BU, BV, b, beta, CU, CV, c, *, rk=0, maxrk, acc):
    """HCORE_dgemm on host arrays (drop-in path). Returns (rank, CU, CV, flops)."""
    return _lr_update("HCORE_dgemm", M, alpha, AU, AV, a, BU, BV, b, beta, CU, CV, c, rk, maxrk,
                      acc, np.float64)


def hcore_sgemm(M, alpha, AU, AV, a, BU, BV, b, beta, CU, CV, c, *, rk=0, maxrk, acc):
    """HCORE_sgemm on host arrays (drop-in path). Returns (rank, CU, CV, flops)."""
    return _lr_update("HCORE_sgemm", M, alpha, AU, AV, a, BU, BV, b, beta, CU, CV, c, rk, maxrk,
                      acc, np.float32)


def hcore_zgemm(M, alpha, AU, AV, a, BU, BV, b, beta, CU, CV, c, *, rk=0, maxrk, acc):
    """HCORE_zgemm (src/compute/hcore_zgemm.c:663) on complex128 arrays
    through the drop-in entry point; returns (rank, CU, CV, flops)."""
    z = lambda x: np.asfortranarray(np.asarray(x, dtype=np.complex128))  # noqa: E731
    AU, AV, BU, BV = (z(x) for x in (AU, AV, BU, BV))
    ldc = CU.shape[0]
    ncol = max(a + c, c, 1)
    CUo = np.zeros((ldc, ncol), dtype=np.complex128, order="F")
    CVo = np.zeros((ldc, ncol), dtype=np.complex128, order="F")
    CUo[:, :c] = CU[:, :c]
    CVo[:, :c] = CV[:, :c]
    ra, rb, rc = (np.array([v], dtype=np.float64) for v in (a, b, c))
    fc = FlopCounter()
    p = lambda x: x.ctypes.data  # noqa: E731
    lib().HCORE_zgemm(111, 112, M, M, DComplex(complex(alpha).real, complex(alpha).imag), p(AU),
                      p(AV), ra.ctypes.data_as(_dp), AU.shape[0], p(BU), p(BV),
                      rb.ctypes.data_as(_dp), BV.shape[0],
                      DComplex(complex(beta).real, complex(beta).imag), p(CUo), p(CVo),
                      rc.ctypes.data_as(_dp), ldc, rk, maxrk, acc, None, C.byref(fc))
    r = int(rc[0])
    return r, CUo[:, :r], CVo[:, :r], fc.update


def zgemm_batched(tasks, stream=None):
    """Run ZlrTask list (complex updates, CU/CV in place); returns (ranks,
    status) arrays."""
    arr = (ZlrTask * max(len(tasks), 1))(*tasks)
    r = (C.c_int * max(len(tasks), 1))()
    st = (C.c_int * max(len(tasks), 1))()
    _check(lib().hcore_gpu_zgemm_batched(len(tasks), arr, r, st, stream or None),
           "hcore_gpu_zgemm_batched")
    return (np.array(r[:len(tasks)], dtype=np.int32), np.array(st[:len(tasks)], dtype=np.int32))


def hcore_dgemm_fast(M, alpha, AU, AV, a, BU, BV, b, beta, CU, CV, c, *, rk=0, maxrk, acc):
    """HCORE_dgemm_fast on host arrays. Returns (rank, CU, CV, None)."""
    return _lr_update("HCORE_dgemm_fast", M, alpha, AU, AV, a, BU, BV, b, beta, CU, CV, c, rk,
                      maxrk, acc, np.float64, fast=True)


class Batch:
    """A plan over many independent low-rank updates (device pointers).

    ``tasks`` is a sequence of :class:`LrTask` whose pointers are device (or
    pinned host) addresses, e.g. ``tensor.data_ptr()`` of column-major torch
    tensors.  The plan allocates its workspace once; :meth:`execute` only
    launches kernels (no allocation, no host synchronisation) and may be
    captured in a CUDA graph.
    """

    def __init__(self, tasks, precision=F64, flags=0, tuning=None):
        L = lib()
        self.n = len(tasks)
        self._tasks = (LrTask * max(self.n, 1))(*tasks)
        self._plan = C.c_void_p()
        if tuning is None:
            _check(L.hcore_gpu_plan_create(C.byref(self._plan), precision, self.n, self._tasks,
                                           flags), "hcore_gpu_plan_create")
        else:
            t = tuning if isinstance(tuning, Tuning) else make_tuning(**tuning)
            _check(L.hcore_gpu_plan_create_tuned(C.byref(self._plan), precision, self.n,
                                                 self._tasks, flags, C.byref(t)),
                   "hcore_gpu_plan_create_tuned")

    def execute(self, stream=None):
        _check(lib().hcore_gpu_plan_execute(self._plan, stream or None), "hcore_gpu_plan_execute")

    def results(self, stream=None):
        ranks = np.zeros(max(self.n, 1), dtype=np.int32)
        status = np.zeros(max(self.n, 1), dtype=np.int32)
        _check(lib().hcore_gpu_plan_results(self._plan, ranks.ctypes.data_as(_ip),
                                            status.ctypes.data_as(_ip), stream or None),
               "hcore_gpu_plan_results")
        return ranks[:self.n], status[:self.n]

    def sigma(self, i, stream=None):
        """Task i's k singular values, descending (hcore_gpu_plan_sigma).  In
        FP64 the values below the SVD's deflation bound
        min(1e-13 acc, 1e-16 ||R_A R_B^T||_F) are 0."""
        k = C.c_int(0)
        lib().hcore_gpu_plan_sigma(self._plan, i, None, C.byref(k), stream or None)
        out = np.zeros(max(k.value, 1))
        _check(lib().hcore_gpu_plan_sigma(self._plan, i, out.ctypes.data_as(_dp), C.byref(k),
                                          stream or None), "hcore_gpu_plan_sigma")
        return out[:k.value]

    def sweeps(self, stream=None):
        out = np.zeros(max(self.n, 1), dtype=np.int32)
        _check(lib().hcore_gpu_plan_sweeps(self._plan, out.ctypes.data_as(_ip), stream or None),
               "hcore_gpu_plan_sweeps")
        return out[:self.n]

    def rebuild(self, idx, CUo, CVo, ldco, max_rank=None, stream=None):
        """Rebuild STORAGE-status tasks idx[q] into CUo[q]/CVo[q] (pointers,
        leading dimension ldco[q]) from the last execute's workspace; with
        max_rank, truncate each to at most max_rank[q] columns."""
        n = len(idx)
        if n == 0:
            return
        ia = (C.c_int * n)(*[int(i) for i in idx])
        cu = (C.c_void_p * n)(*[int(x) for x in CUo])
        cv = (C.c_void_p * n)(*[int(x) for x in CVo])
        ld = (C.c_int * n)(*[int(x) for x in ldco])
        mr = (C.c_int * n)(*[int(x) for x in max_rank]) if max_rank is not None else None
        _check(lib().hcore_gpu_plan_rebuild(self._plan, n, ia, cu, cv, ld, mr, stream or None),
               "hcore_gpu_plan_rebuild")

    def execute_phases(self, phases, stream=None):
        _check(lib().hcore_gpu_plan_execute_phases(self._plan, stream or None, phases),
               "hcore_gpu_plan_execute_phases")

    @property
    def device_ranks_ptr(self) -> int:
        return lib().hcore_gpu_plan_device_ranks(self._plan)

    @property
    def device_status_ptr(self) -> int:
        return lib().hcore_gpu_plan_device_status(self._plan)

    @property
    def zero_copy_bytes(self) -> int:
        """Pinned host input bytes read in place (not staged) by every execute."""
        return int(lib().hcore_gpu_plan_zero_copy_bytes(self._plan))

    @property
    def staged_bytes(self) -> int:
        return int(lib().hcore_gpu_plan_staged_bytes(self._plan))

    @property
    def launches(self) -> int:
        """Kernel launches of one execute."""
        return int(lib().hcore_gpu_plan_launches(self._plan))

    @property
    def workspace_bytes(self) -> int:
        return int(lib().hcore_gpu_plan_workspace_bytes(self._plan))

    def close(self):
        if self._plan:
            lib().hcore_gpu_plan_destroy(self._plan)
            self._plan = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DensePlan:
    """HCORE_dsyrk / HCORE_dgemmcd tasks (device pointers) as a reusable plan."""

    def __init__(self, tasks):
        self.n = len(tasks)
        self._tasks = (DenseTask * max(self.n, 1))(*tasks)
        self._plan = C.c_void_p()
        _check(lib().hcore_gpu_dense_plan_create(C.byref(self._plan), self.n, self._tasks),
               "hcore_gpu_dense_plan_create")

    def execute(self, stream=None):
        _check(lib().hcore_gpu_dense_plan_execute(self._plan, stream or None),
               "hcore_gpu_dense_plan_execute")

    def close(self):
        if self._plan:
            lib().hcore_gpu_dense_plan_destroy(self._plan)
            self._plan = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def dense_batched(tasks, stream=None):
    """Run HCORE_dsyrk / HCORE_dgemmcd tasks (device pointers) in one batch."""
    arr = (DenseTask * max(len(tasks), 1))(*tasks)
    _check(lib().hcore_gpu_dense_batched(len(tasks), arr, stream or None), "hcore_gpu_dense_batched")


def trsm_batched(tasks, stream=None):
    """Run TrsmTask list (device or pinned pointers); returns when done."""
    arr = (TrsmTask * max(len(tasks), 1))(*tasks)
    _check(lib().hcore_gpu_trsm_batched(len(tasks), arr, stream or None), "hcore_gpu_trsm_batched")


def potrf_batched(tasks, stream=None) -> np.ndarray:
    """Factor PotrfTask tiles in place; returns each task's LAPACK info."""
    arr = (PotrfTask * max(len(tasks), 1))(*tasks)
    info = (C.c_int * max(len(tasks), 1))()
    _check(lib().hcore_gpu_potrf_batched(len(tasks), arr, info, stream or None),
           "hcore_gpu_potrf_batched")
    return np.array(info[:len(tasks)], dtype=np.int32)


def compress_batched(tasks, stream=None):
    """Compress dense tiles (CompressTask list, device or pinned pointers);
    returns (ranks, status) arrays.  A non-zero status (NOCONV, RANK_MAX) is
    reported per tile, not raised."""
    arr = (CompressTask * max(len(tasks), 1))(*tasks)
    r = (C.c_int * max(len(tasks), 1))()
    st = (C.c_int * max(len(tasks), 1))()
    _check(lib().hcore_gpu_compress_batched(len(tasks), arr, r, st, stream or None),
           "hcore_gpu_compress_batched")
    return (np.array(r[:len(tasks)], dtype=np.int32), np.array(st[:len(tasks)], dtype=np.int32))


class RankMLP:
    """The rank predictor's 6 -> 64 -> 64 -> 1 MLP (FP32 weights, BF16
    activations) held on the GPU by the library (hcore_gpu_mlp_*).  Inputs
    are (n, 6) float32 CUDA tensors, targets and outputs (n,) float32."""

    NPARAMS = 6 * 64 + 64 + 64 * 64 + 64 + 64 + 1

    def __init__(self, seed: int = 0):
        self._m = C.c_void_p()
        _check(lib().hcore_gpu_mlp_create(C.byref(self._m), seed), "hcore_gpu_mlp_create")

    def get_params(self) -> np.ndarray:
        out = np.zeros(self.NPARAMS, dtype=np.float32)
        _check(lib().hcore_gpu_mlp_params(self._m, out.ctypes.data_as(_fp), 0), "hcore_gpu_mlp_params")
        return out

    def set_params(self, p) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.NPARAMS
        _check(lib().hcore_gpu_mlp_params(self._m, p.ctypes.data_as(_fp), 1), "hcore_gpu_mlp_params")

    def gradient(self, X, T, stream=None):
        g = np.zeros(self.NPARAMS, dtype=np.float32)
        loss = C.c_float(0)
        _check(lib().hcore_gpu_mlp_gradient(self._m, X.data_ptr(), T.data_ptr(), X.shape[0],
                                            g.ctypes.data_as(_fp), C.byref(loss), stream),
               "hcore_gpu_mlp_gradient")
        return float(loss.value), g

    def train(self, X, T, epochs: int, batch: int, lr: float, seed: int = 0, stream=None):
        losses = np.zeros(epochs, dtype=np.float32)
        _check(lib().hcore_gpu_mlp_train(self._m, X.data_ptr(), T.data_ptr(), X.shape[0], epochs,
                                         batch, lr, seed, losses.ctypes.data_as(_fp), stream),
               "hcore_gpu_mlp_train")
        return losses

    def predict(self, X, out=None, stream=None):
        import torch

        if out is None:
            out = torch.empty(X.shape[0], dtype=torch.float32, device=X.device)
        _check(lib().hcore_gpu_mlp_predict(self._m, X.data_ptr(), X.shape[0], out.data_ptr(), stream),
               "hcore_gpu_mlp_predict")
        return out

    def close(self) -> None:
        if self._m:
            lib().hcore_gpu_mlp_destroy(self._m)
            self._m = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def make_tuning(stream_groups=None, svd_lanes=None, bucket_width=None, phase_sync=None,
                qr_warps=None) -> Tuning:
    """A Tuning from the library default with the given fields replaced."""
    t = Tuning()
    _check(lib().hcore_gpu_tuning_default(C.byref(t)), "hcore_gpu_tuning_default")
    if stream_groups is not None:
        t.stream_groups = int(stream_groups)
    if svd_lanes is not None:
        for q in range(3):
            t.svd_lanes[q] = int(svd_lanes[q])
    if bucket_width is not None:
        t.bucket_width = int(bucket_width)
    if phase_sync is not None:
        t.phase_sync = int(phase_sync)
    if qr_warps is not None:
        t.qr_warps = int(qr_warps)
    return t


def autotune(tasks, precision=F64, flags=0, reps=5, stream=None):
    """Search the plan's launch-shape parameters on these tasks (the batch runs
    several times; outputs must not alias inputs).  Returns (Tuning, ms)."""
    n = len(tasks)
    arr = (LrTask * max(n, 1))(*tasks)
    best = Tuning()
    ms = C.c_double(0)
    _check(lib().hcore_gpu_autotune(precision, n, arr, flags, reps, stream or None, C.byref(best),
                                    C.byref(ms)), "hcore_gpu_autotune")
    return best, float(ms.value)
