"""ORACLE — Python face of the CPU restatement (test infrastructure only).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg may import this module; the GPU product never does.

* :class:`Port` wraps ``oracle/_build/libhcore_port.so`` (the C restatement of
  the reference path, hcore_port_impl.h) with numpy arrays.
* :class:`RefLib` wraps ``oracle/_ref/libhcore_ref.so`` (the reference compiled
  from its own sources) — available only where the reference checkout is.
* Generators for the seeded inputs: Haar-random factors (configuration
  "nb=512, ranks 32, sigma_i = 10^(-8i/32)"), the reference tests'
  ``generate_compress`` (testing/testing_dgemm.c:119-236) and dense helpers.

All matrices are column-major numpy arrays of shape (ld, ncols) (Fortran
order), matching the reference's storage.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int)
_ulp = C.POINTER(C.c_ulong)

PORT_STATUS = {0: "ok", 1: "zero rank", 2: "rank sum > 2*maxrk", 3: "ld_newV < k",
               4: "rank > maxrk", 5: "rank > storage maxrank", 6: "LAPACK info", 7: "k > M"}


def _ptr(a, t=_dp):
    return None if a is None else a.ctypes.data_as(t)


def fortran(a, dtype=np.float64):
    return np.asfortranarray(np.asarray(a, dtype=dtype))


class FlopCounter(C.Structure):
    """Layout of flop_counter (src/misc/include/flop_util_structs.h:5-36)."""

    _fields_ = [("__pad1", C.c_ulong), ("__pad2", C.c_ulong), ("copy", C.c_ulong),
                ("flop", C.c_ulong), ("tid", C.c_int), ("potrf", C.c_ulong),
                ("trsm", C.c_ulong), ("syrk", C.c_ulong), ("update", C.c_ulong)] + [
        (n, C.c_ulong) for n in (
            "geqrfu", "geqrfv", "geqrfv_gemm", "gesvd", "gesvd_gemm", "gesvd_lasetu",
            "gesvd_lasetv", "gesvd_lacpyu", "gesvd_lacpyv", "gesvd_dscal", "ormqru",
            "ormqru_laset", "ormqru_lacpy", "ormqrv", "ormqrv_laset", "ormqrv_lacpy",
            "omatcopy")] + [("numthreads", C.c_int), ("__pad3", C.c_ulong),
                            ("__pad4", C.c_ulong)]


class DComplex(C.Structure):
    """double _Complex passed by value (two doubles, real first)."""

    _fields_ = [("re", C.c_double), ("im", C.c_double)]

    @classmethod
    def of(cls, z):
        z = complex(z)
        return cls(z.real, z.imag)


class Port:
    """ctypes wrapper of the C restatement."""

    _lib = None

    def __init__(self):
        if Port._lib is None:
            path = _build.build_port()
            lib = C.CDLL(path)
            lib.port_flop_counts.restype = C.c_ulong
            lib.port_flop_counts.argtypes = [C.c_char, C.c_ulong, C.c_ulong, C.c_ulong, C.c_ulong]
            for name, rp, real in (("port_dgemm", _dp, C.c_double), ("port_sgemm", _fp, C.c_float)):
                f = getattr(lib, name)
                f.restype = C.c_int
                f.argtypes = [C.c_int, real, rp, rp, C.c_int, C.c_int, rp, rp, C.c_int, C.c_int, rp,
                              real, rp, rp, _ip, C.c_int, C.c_int, C.c_int, C.c_int, real, C.c_int,
                              rp, _ulp]
            lib.port_dsyrk.argtypes = [C.c_int, C.c_int, C.c_double, _dp, C.c_int, _dp, _dp, C.c_int, _ulp]
            lib.port_dgemmcd.argtypes = [C.c_int, _dp, _dp, C.c_int, _dp, _dp, C.c_int, _dp]
            lib.port_duncompress.restype = None
            lib.port_duncompress.argtypes = [C.c_int, C.c_int, _dp, C.c_int, C.c_int, _dp, C.c_int,
                                             _dp, C.c_int]
            lib.port_dgemmbdcd.restype = None
            lib.port_dgemmbdcd.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, _dp, _dp, C.c_int,
                                           C.c_int, _dp, C.c_int, C.c_double, _dp, C.c_int, _ulp]
            lib.port_dtrsm.restype = None
            lib.port_dtrsm.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                       C.c_double, _dp, C.c_int, _dp, C.c_int, _ulp]
            lib.port_dpotrf.restype = C.c_int
            lib.port_dpotrf.argtypes = [C.c_int, C.c_int, _dp, C.c_int, _ulp]
            lib.port_zgemm.restype = C.c_int
            lib.port_zgemm.argtypes = [C.c_int, DComplex, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                       C.c_void_p, C.c_void_p, C.c_int, C.c_int, DComplex,
                                       C.c_void_p, C.c_void_p, _ip, C.c_int, C.c_int, C.c_int,
                                       C.c_double, _ulp]
            lib.port_dcompress.restype = C.c_int
            lib.port_dcompress.argtypes = [C.c_int, C.c_int, _dp, C.c_int, C.c_double, C.c_int,
                                           C.c_int, _dp, _dp, C.c_int, _ip, _dp]
            lib.port_dlatms.argtypes = [C.c_int, C.c_int, C.c_char, _ip, C.c_char, _dp, C.c_int,
                                        C.c_double, C.c_double, C.c_int, C.c_int, C.c_char, _dp,
                                        C.c_int]
            lib.port_set_threads.argtypes = [C.c_int]
            lib.port_dgemm_list.restype = C.c_int
            lib.port_dgemm_list.argtypes = [C.c_int, _dp, _dp, C.c_void_p, C.c_int, _ip, _ip, _ip,
                                            C.c_double, C.c_double, C.c_int, C.c_double, C.c_int]
            Port._lib = lib
        self.lib = Port._lib

    def set_threads(self, n: int) -> None:
        self.lib.port_set_threads(n)

    def gemm_list(self, nb, U, V, off, sa, sb, sc, *, alpha, beta, maxrk, acc, variant=0):
        """port_dgemm over a list of updates whose factors live in two flat
        FP64 arenas U, V (tile t: column-major nb x rank block at off[t]);
        the loop runs in C.  Returns the count of updates that failed."""
        U = np.ascontiguousarray(U, dtype=np.float64)
        V = np.ascontiguousarray(V, dtype=np.float64)
        off = np.ascontiguousarray(off, dtype=np.int64)
        sa, sb, sc = (np.ascontiguousarray(x, dtype=np.int32) for x in (sa, sb, sc))
        return int(self.lib.port_dgemm_list(nb, _ptr(U), _ptr(V), off.ctypes.data, len(sa),
                                            _ptr(sa, _ip), _ptr(sb, _ip), _ptr(sc, _ip), alpha,
                                            beta, maxrk, acc, variant))

    def flop_counts(self, op: str, a: int, b: int = 0, c: int = 0, d: int = 0) -> int:
        return int(self.lib.port_flop_counts(op.encode(), a, b, c, d))

    def gemm(self, M, alpha, AU, AV, a, BU, BV, b, beta, CU, CV, c, *, rk=0, maxrk, acc,
             variant=0, storage_maxrank=None, dense_B=None, dtype=np.float64):
        """One update C <- beta*C + alpha*A*B^T; returns a dict.

        CU/CV are copied (not modified); their storage must hold the new rank
        (the result is written into copies with at least max(c, k) columns).
        """
        single = dtype == np.float32
        rp = _fp if single else _dp
        AU, AV = fortran(AU, dtype), fortran(AV, dtype)
        BU = fortran(BU, dtype) if BU is not None else None
        BV = fortran(BV, dtype)
        lda, ldb = AU.shape[0], BV.shape[0]
        ldc = CU.shape[0]
        k = a + c
        ncol = max(k, c, 1)
        CUo = np.zeros((ldc, ncol), dtype=dtype, order="F")
        CVo = np.zeros((ldc, ncol), dtype=dtype, order="F")
        CUo[:, :c] = CU[:, :c]
        CVo[:, :c] = CV[:, :c]
        crk = C.c_int(c)
        sig = np.zeros(max(k, 1), dtype=dtype)
        fl = C.c_ulong(0)
        dB = fortran(dense_B, dtype) if dense_B is not None else None
        fn = self.lib.port_sgemm if single else self.lib.port_dgemm
        st = fn(M, alpha, _ptr(AU, rp), _ptr(AV, rp), a, lda,
                _ptr(BU, rp) if BU is not None else None, _ptr(BV, rp), b, ldb, _ptr(dB, rp),
                beta, _ptr(CUo, rp), _ptr(CVo, rp), C.byref(crk), ldc, rk, maxrk,
                storage_maxrank if storage_maxrank is not None else maxrk, acc, variant,
                _ptr(sig, rp), C.byref(fl))
        r = crk.value
        return dict(status=st, rank=r, CU=CUo[:, :r], CV=CVo[:, :r], sigma=sig[:k],
                    flops=fl.value)

    def dsyrk(self, M, K, alpha, AU, AV, CD):
        AU, AV = fortran(AU), fortran(AV)
        CDo = fortran(CD).copy(order="F")
        fl = C.c_ulong(0)
        self.lib.port_dsyrk(M, K, alpha, _ptr(AU), AU.shape[0], _ptr(AV), _ptr(CDo), CDo.shape[0],
                            C.byref(fl))
        return CDo, fl.value

    def dgemmcd(self, M, Au, Av, Arank, Bu, Bv, Brank, CD):
        Au, Av, Bu, Bv = (fortran(x) for x in (Au, Av, Bu, Bv))
        CDo = fortran(CD).copy(order="F")
        self.lib.port_dgemmcd(M, _ptr(Au), _ptr(Av), Arank, _ptr(Bu), _ptr(Bv), Brank, _ptr(CDo))
        return CDo

    def duncompress(self, M, N, AU, a, BV, CD):
        AU, BV = fortran(AU), fortran(BV)
        CDo = fortran(CD).copy(order="F")
        self.lib.port_duncompress(M, N, _ptr(AU), a, AU.shape[0], _ptr(BV), BV.shape[0], _ptr(CDo),
                                  CDo.shape[0])
        return CDo

    def dgemmbdcd(self, transA, M, N, alpha, AU, AV, a, BD, beta, CD):
        """AU and AV share one leading dimension (their row count)."""
        AU, AV, BD = fortran(AU), fortran(AV), fortran(BD)
        assert AU.shape[0] == AV.shape[0]
        CDo = fortran(CD).copy(order="F")
        fl = C.c_ulong(0)
        self.lib.port_dgemmbdcd(transA, M, N, alpha, _ptr(AU), _ptr(AV), a, AU.shape[0], _ptr(BD),
                                BD.shape[0], beta, _ptr(CDo), CDo.shape[0], C.byref(fl))
        return CDo, fl.value

    def dtrsm(self, side, uplo, trans, diag, M, N, alpha, A, B):
        A = fortran(A)
        Bo = fortran(B).copy(order="F")
        fl = C.c_ulong(0)
        self.lib.port_dtrsm(side, uplo, trans, diag, M, N, alpha, _ptr(A), A.shape[0], _ptr(Bo),
                            Bo.shape[0], C.byref(fl))
        return Bo, fl.value

    def dpotrf(self, uplo, N, A):
        Ao = fortran(A).copy(order="F")
        fl = C.c_ulong(0)
        info = self.lib.port_dpotrf(uplo, N, _ptr(Ao), Ao.shape[0], C.byref(fl))
        return Ao, info, fl.value

    def zgemm(self, M, alpha, AU, AV, a, BU, BV, b, beta, CU, CV, c, *, rk=0, maxrk, acc):
        """The restated HCORE_zgemm on complex128 arrays: dict(status, rank, CU,
        CV, flops)."""
        AU, AV, BU, BV = (np.asfortranarray(x, dtype=np.complex128) for x in (AU, AV, BU, BV))
        ldc = CU.shape[0]
        ncol = max(a + c, c, 1)
        CUo = np.zeros((ldc, ncol), dtype=np.complex128, order="F")
        CVo = np.zeros((ldc, ncol), dtype=np.complex128, order="F")
        CUo[:, :c] = CU[:, :c]
        CVo[:, :c] = CV[:, :c]
        crk = C.c_int(c)
        fl = C.c_ulong(0)
        p = lambda x: x.ctypes.data_as(C.c_void_p)  # noqa: E731
        st = self.lib.port_zgemm(M, DComplex.of(alpha), p(AU), p(AV), a, AU.shape[0], p(BU),
                                 p(BV), b, BV.shape[0], DComplex.of(beta), p(CUo), p(CVo),
                                 C.byref(crk), ldc, rk, maxrk, acc, C.byref(fl))
        r = crk.value
        return dict(status=st, rank=r, CU=CUo[:, :r], CV=CVo[:, :r], flops=fl.value)

    def dcompress(self, D, acc, maxrank, relative=False):
        """generate_compress's SVD truncation of a dense tile: returns
        (rank, U, V, sigma) with U, V of shape (M, rank)."""
        D = fortran(D)
        M, N = D.shape
        U = np.zeros((M, max(min(M, N), 1)), order="F")
        V = np.zeros((M, max(min(M, N), 1)), order="F")
        sig = np.zeros(max(min(M, N), 1))
        r = C.c_int(0)
        st = self.lib.port_dcompress(M, N, _ptr(D), M, acc, int(relative), maxrank, _ptr(U),
                                     _ptr(V), M, C.byref(r), _ptr(sig))
        if st != 0:
            raise RuntimeError(f"dgesvd failed ({st})")
        return r.value, U[:, :r.value], V[:, :r.value], sig[:min(M, N)]

    def dlatms(self, m, n, iseed, d, ld):
        """LAPACKE_dlatms(m, n, 'U', iseed, 'N', d, mode=0, cond=-1, dmax=-1,
        kl=m-1, ku=n-1, 'N') as called at testing/testing_dgemm.c:159."""
        a = np.zeros((ld, n), order="F")
        dd = np.array(d, dtype=np.float64)
        st = self.lib.port_dlatms(m, n, b"U", iseed.ctypes.data_as(_ip), b"N", _ptr(dd), 0, -1.0,
                                  -1.0, m - 1, n - 1, b"N", _ptr(a), ld)
        if st != 0:
            raise RuntimeError(f"dlatms info={st}")
        return a


class RefLib:
    """ctypes wrapper of the reference HCORE compiled from source (oracle/_ref).

    The reference calls exit(-1) on invalid input, so only valid inputs may be
    passed through this wrapper.
    """

    _lib = None

    @staticmethod
    def available() -> bool:
        return _build.reference_available()

    def __init__(self):
        if RefLib._lib is None:
            path = _build.build_ref()
            if path is None:
                raise RuntimeError("reference checkout not present")
            lib = C.CDLL(path)
            for name, rp, real in (("HCORE_dgemm", _dp, C.c_double), ("HCORE_sgemm", _fp, C.c_float)):
                f = getattr(lib, name)
                f.restype = None
                f.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, real, rp, rp, rp, C.c_int, rp, rp,
                              rp, C.c_int, real, rp, rp, rp, C.c_int, C.c_int, C.c_int, real, rp,
                              C.POINTER(FlopCounter)]
            lib.HCORE_dgemm_fast.restype = None
            lib.HCORE_dgemm_fast.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, _dp,
                                             _dp, _dp, C.c_int, _dp, _dp, _dp, C.c_int, C.c_double,
                                             _dp, _dp, _dp, C.c_int, C.c_int, C.c_int, C.c_double,
                                             _dp]
            lib.HCORE_dsyrk.restype = None
            lib.HCORE_dsyrk.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, _dp,
                                        C.c_int, _dp, C.c_int, C.c_double, _dp, C.c_int, _dp,
                                        C.POINTER(FlopCounter)]
            lib.HCORE_dgemmcd.restype = None
            lib.HCORE_dgemmcd.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, _dp, _dp, C.c_int,
                                          C.c_int, _dp, _dp, C.c_int, C.c_int, C.c_double, _dp,
                                          C.c_int, C.c_int, _dp, C.POINTER(FlopCounter)]
            lib.HCORE_duncompress.restype = None
            lib.HCORE_duncompress.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, _dp,
                                              _dp, C.c_int, _dp, _dp, C.c_int, C.c_double, _dp,
                                              C.c_int]
            lib.HCORE_dgemmbdcd.restype = None
            lib.HCORE_dgemmbdcd.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, _dp,
                                            _dp, _dp, C.c_int, _dp, C.c_int, C.c_double, _dp,
                                            C.c_int, _dp, C.POINTER(FlopCounter)]
            lib.HCORE_dtrsm.restype = None
            lib.HCORE_dtrsm.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                        C.c_double, _dp, C.c_int, _dp, C.c_int,
                                        C.POINTER(FlopCounter)]
            lib.HCORE_dpotrf.restype = None
            lib.HCORE_dpotrf.argtypes = [C.c_int, C.c_int, _dp, C.c_int, _ip,
                                         C.POINTER(FlopCounter)]
            lib.HCORE_zgemm.restype = None
            lib.HCORE_zgemm.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, DComplex, C.c_void_p,
                                        C.c_void_p, _dp, C.c_int, C.c_void_p, C.c_void_p, _dp,
                                        C.c_int, DComplex, C.c_void_p, C.c_void_p, _dp, C.c_int,
                                        C.c_int, C.c_int, C.c_double, C.c_void_p,
                                        C.POINTER(FlopCounter)]
            lib.HCORE_zuncompress.restype = None
            lib.HCORE_zuncompress.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, DComplex,
                                              C.c_void_p, _dp, C.c_int, C.c_void_p, _dp, C.c_int,
                                              DComplex, C.c_void_p, C.c_int]
            RefLib._lib = lib
        self.lib = RefLib._lib

    def set_int(self, name: str, value: int) -> None:
        C.c_int.in_dll(self.lib, name).value = value

    def dgemm(self, M, alpha, AU, AV, a, BU, BV, b, beta, CU, CV, c, *, rk=0, maxrk, acc,
              fast=False, dtype=np.float64):
        single = dtype == np.float32
        rp, real = (_fp, C.c_float) if single else (_dp, C.c_double)
        AU, AV, BU, BV = (fortran(x, dtype) for x in (AU, AV, BU, BV))
        ldc = CU.shape[0]
        ncol = max(a + c, c)
        CUo = np.zeros((ldc, ncol), dtype=dtype, order="F")
        CVo = np.zeros((ldc, ncol), dtype=dtype, order="F")
        CUo[:, :c] = CU[:, :c]
        CVo[:, :c] = CV[:, :c]
        ra, rb, rc = (np.array([v], dtype=dtype) for v in (a, b, c))
        if fast:
            self.set_int("use_trmm", 1)
            self.set_int("use_scratch", 1)
            work = np.zeros(64 * M * max(maxrk, ncol) + 64 * ncol * ncol + 4096)
            self.lib.HCORE_dgemm_fast(111, 112, M, M, alpha, _ptr(AU), _ptr(AV), _ptr(ra),
                                      AU.shape[0], _ptr(BU), _ptr(BV), _ptr(rb), BV.shape[0], beta,
                                      _ptr(CUo), _ptr(CVo), _ptr(rc), ldc, rk, maxrk, acc,
                                      _ptr(work))
            self.set_int("use_trmm", 0)
            self.set_int("use_scratch", 0)
            fl = None
        else:
            fc = FlopCounter()
            fn = self.lib.HCORE_sgemm if single else self.lib.HCORE_dgemm
            fn(111, 112, M, M, alpha, _ptr(AU, rp), _ptr(AV, rp), _ptr(ra, rp), AU.shape[0],
               _ptr(BU, rp), _ptr(BV, rp), _ptr(rb, rp), BV.shape[0], beta, _ptr(CUo, rp),
               _ptr(CVo, rp), _ptr(rc, rp), ldc, rk, maxrk, acc, None, C.byref(fc))
            fl = fc.update
        r = int(rc[0])
        return dict(rank=r, CU=CUo[:, :r].copy(order="F"), CV=CVo[:, :r].copy(order="F"),
                    flops=fl)

    def dsyrk(self, M, K, alpha, AU, AV, CD):
        AU, AV = fortran(AU), fortran(AV)
        CDo = fortran(CD).copy(order="F")
        fc = FlopCounter()
        self.lib.HCORE_dsyrk(122, 111, M, K, alpha, _ptr(AU), AU.shape[0], _ptr(AV), AV.shape[0],
                             1.0, _ptr(CDo), CDo.shape[0], None, C.byref(fc))
        return CDo, fc.syrk

    def dgemmcd(self, M, Au, Av, Arank, Bu, Bv, Brank, CD, maxrank):
        Au, Av, Bu, Bv = (fortran(x) for x in (Au, Av, Bu, Bv))
        CDo = fortran(CD).copy(order="F")
        fc = FlopCounter()
        self.lib.HCORE_dgemmcd(111, 112, M, -1.0, _ptr(Au), _ptr(Av), Arank, M, _ptr(Bu),
                               _ptr(Bv), Brank, M, 1.0, _ptr(CDo), M, maxrank, None, C.byref(fc))
        return CDo

    def zgemm(self, M, alpha, AU, AV, a, BU, BV, b, beta, CU, CV, c, *, rk=0, maxrk, acc):
        """HCORE_zgemm (src/compute/hcore_zgemm.c:663) on complex128 arrays;
        returns dict(rank, CU, CV, flops)."""
        AU, AV, BU, BV = (np.asfortranarray(x, dtype=np.complex128) for x in (AU, AV, BU, BV))
        ldc = CU.shape[0]
        ncol = max(a + c, c)
        CUo = np.zeros((ldc, ncol), dtype=np.complex128, order="F")
        CVo = np.zeros((ldc, ncol), dtype=np.complex128, order="F")
        CUo[:, :c] = CU[:, :c]
        CVo[:, :c] = CV[:, :c]
        ra, rb, rc = (np.array([v], dtype=np.float64) for v in (a, b, c))
        fc = FlopCounter()
        p = lambda x: x.ctypes.data_as(C.c_void_p)  # noqa: E731
        self.lib.HCORE_zgemm(111, 112, M, M, DComplex.of(alpha), p(AU), p(AV), _ptr(ra),
                             AU.shape[0], p(BU), p(BV), _ptr(rb), BV.shape[0],
                             DComplex.of(beta), p(CUo), p(CVo), _ptr(rc), ldc, rk, maxrk, acc,
                             None, C.byref(fc))
        r = int(rc[0])
        return dict(rank=r, CU=CUo[:, :r].copy(order="F"), CV=CVo[:, :r].copy(order="F"),
                    flops=fc.update)

    def zuncompress(self, M, N, AU, a, BV, CD):
        AU, BV = (np.asfortranarray(x, dtype=np.complex128) for x in (AU, BV))
        CDo = np.asfortranarray(CD, dtype=np.complex128).copy(order="F")
        ra = np.array([a], dtype=np.float64)
        p = lambda x: x.ctypes.data_as(C.c_void_p)  # noqa: E731
        self.lib.HCORE_zuncompress(111, 112, M, N, DComplex.of(1.0), p(AU), _ptr(ra), AU.shape[0],
                                   p(BV), _ptr(ra), BV.shape[0], DComplex.of(0.0), p(CDo),
                                   CDo.shape[0])
        return CDo

    _test_lib = None

    def generate_compress(self, M, acc, maxrank, iseed):
        """The reference tests' generate_compress (testing/testing_dgemm.c:119-236),
        called as that file's main calls it (ld = M, maxMNK = M): returns the
        generated tile, its rank and U, V (M x rank), and the advanced iseed."""
        if RefLib._test_lib is None:
            lib = C.CDLL(_build.ref_test_lib_path())
            lib.generate_compress.restype = C.c_int
            lib.generate_compress.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, C.c_int,
                                              C.c_int, C.c_double, _ip, _ip]
            RefLib._test_lib = lib
        A = np.zeros((M, M), order="F")
        U = np.zeros((M, M), order="F")
        V = np.zeros((M, M), order="F")
        seed = np.array(iseed, dtype=np.int32)
        r = C.c_int(0)
        st = RefLib._test_lib.generate_compress(M, M, M, _ptr(A), _ptr(U), _ptr(V), maxrank, M, acc,
                                                seed.ctypes.data_as(_ip), C.byref(r))
        if st != 0:
            raise RuntimeError("generate_compress failed")
        return A, r.value, U[:, :r.value].copy(order="F"), V[:, :r.value].copy(order="F"), seed

    def duncompress(self, M, N, AU, a, BV, CD):
        AU, BV = fortran(AU), fortran(BV)
        CDo = fortran(CD).copy(order="F")
        ra = np.array([a], dtype=np.float64)
        self.lib.HCORE_duncompress(111, 112, M, N, 1.0, _ptr(AU), _ptr(ra), AU.shape[0], _ptr(BV),
                                   _ptr(ra), BV.shape[0], 0.0, _ptr(CDo), CDo.shape[0])
        return CDo

    def dgemmbdcd(self, transA, M, N, alpha, AU, AV, a, BD, beta, CD):
        AU, AV, BD = fortran(AU), fortran(AV), fortran(BD)
        CDo = fortran(CD).copy(order="F")
        ra = np.array([a], dtype=np.float64)
        fc = FlopCounter()
        self.lib.HCORE_dgemmbdcd(transA, 111, M, N, alpha, _ptr(AU), _ptr(AV), _ptr(ra), AU.shape[0],
                                 _ptr(BD), BD.shape[0], beta, _ptr(CDo), CDo.shape[0], None,
                                 C.byref(fc))
        return CDo, fc.update

    def dtrsm(self, side, uplo, trans, diag, M, N, alpha, A, B):
        A = fortran(A)
        Bo = fortran(B).copy(order="F")
        fc = FlopCounter()
        self.lib.HCORE_dtrsm(side, uplo, trans, diag, M, N, alpha, _ptr(A), A.shape[0], _ptr(Bo),
                             Bo.shape[0], C.byref(fc))
        return Bo, fc.trsm

    def dpotrf(self, uplo, N, A):
        Ao = fortran(A).copy(order="F")
        info = C.c_int(0)
        fc = FlopCounter()
        self.lib.HCORE_dpotrf(uplo, N, _ptr(Ao), Ao.shape[0], C.byref(info), C.byref(fc))
        return Ao, info.value, fc.potrf


def zgemm_dense_truncation(alpha, AU, AV, BU, BV, beta, CU, CV, *, rk=0, acc):
    """The complex update's mathematics restated densely (numpy, small cases):
    C = beta CU CV^T + alpha AU AV^T (BU BV^T)^T with plain transposes
    (hcore_zgemm.c:138-220), its singular values, and the truncation of
    hcore_zgemm.c's rank rule (the first i >= 1 with sigma_i < acc, or
    min(rk, k)).  Returns (rank, truncated product, sigma)."""
    Cd = beta * (CU @ CV.T) + alpha * (AU @ AV.T) @ (BU @ BV.T).T
    k = AU.shape[1] + CU.shape[1]
    U, S, Vh = np.linalg.svd(Cd)
    if rk:
        r = min(rk, k)
    else:
        r = k
        for i in range(1, k):
            if S[i] < acc:
                r = i
                break
    return r, (U[:, :r] * S[:r]) @ Vh[:r], S[:k]


def tlr_panel_step(port: Port, D, U, V, rank, k, acc, maxrk, maxrank):
    """Panel step k of a TLR Cholesky on the CPU, the sequence of HiCMA's
    per-tile calls restated with the reference's kernels as the oracle has
    them: HCORE_dpotrf of D[k] (src/compute/hcore_dpotrf.c:23-34, lower),
    HCORE_dtrsm of every panel V factor (hcore_dtrsm.c:24-48: Left, Lower,
    NoTrans, NonUnit), HCORE_dsyrk of every later diagonal tile
    (hcore_dsyrk.c:47-189, alpha = -1) and the recompressed Schur updates
    A_ij -= A_ik A_jk^T (hcore_dgemm.c:703, the split API's rank rules:
    a + c <= 2 maxrk, new rank <= maxrk and <= maxrank).  Tiles of rank 0 take
    no call.  D (list of nb x nb), U, V (dicts (i, j) -> nb x rank) and rank
    (dict) are updated in place.  Returns (potrf info, {(i, j): status})."""
    nt = len(D)
    nb = D[0].shape[0]
    Lk, info, _ = port.dpotrf(ord("L"), nb, D[k])
    D[k] = Lk
    if info != 0:
        return info, {}
    for i in range(k + 1, nt):
        if rank[(i, k)] > 0:
            V[(i, k)], _ = port.dtrsm(141, 122, 111, 131, nb, rank[(i, k)], 1.0, Lk, V[(i, k)])
    for i in range(k + 1, nt):
        if rank[(i, k)] > 0:
            D[i], _ = port.dsyrk(nb, rank[(i, k)], -1.0, U[(i, k)], V[(i, k)], D[i])
    status = {}
    for j in range(k + 1, nt):
        for i in range(j + 1, nt):
            a, b, c = rank[(i, k)], rank[(j, k)], rank[(i, j)]
            if a == 0 or b == 0:
                continue
            CU = U[(i, j)] if c > 0 else np.zeros((nb, 0))
            CV = V[(i, j)] if c > 0 else np.zeros((nb, 0))
            ref = port.gemm(nb, -1.0, U[(i, k)], V[(i, k)], a, U[(j, k)], V[(j, k)], b, 1.0,
                            CU, CV, c, maxrk=maxrk, acc=acc, variant=2, storage_maxrank=maxrank)
            status[(i, j)] = ref["status"]
            if ref["status"] == 0:
                U[(i, j)], V[(i, j)], rank[(i, j)] = ref["CU"], ref["CV"], ref["rank"]
    return 0, status


# --------------------------------------------------------------------------
# seeded generators
# --------------------------------------------------------------------------

def haar(rng: np.random.Generator, m: int, k: int) -> np.ndarray:
    """m x k with orthonormal columns, Haar distributed (QR of a Gaussian with
    the sign of R's diagonal folded into Q)."""
    g = rng.standard_normal((m, k))
    q, r = np.linalg.qr(g)
    q = q * np.sign(np.diag(r))[None, :]
    return np.asfortranarray(q)


def graded_lowrank(rng, m: int, k: int, decades: float = 8.0, ld: int | None = None,
                   cols: int | None = None):
    """U diag(sigma) V^T with Haar U, V and sigma_i = 10^(-decades*i/k), the
    singular values folded into U (configuration "nb=512, ranks 32")."""
    ld = ld or m
    cols = cols or k
    s = 10.0 ** (-decades * np.arange(k) / k)
    U = np.zeros((ld, cols), order="F")
    V = np.zeros((ld, cols), order="F")
    U[:m, :k] = haar(rng, m, k) * s[None, :]
    V[:m, :k] = haar(rng, m, k)
    return U, V


def generate_compress(port: Port, m: int, iseed: np.ndarray, acc: float, storage_maxrank: int):
    """Restatement of the reference tests' generator/compressor
    (testing/testing_dgemm.c:119-236): dlatms with sigma_i = 10^-i, full
    dgesvd, keep sigma >= acc (absolute, :195), cap at storage_maxrank, U = left
    vectors, V = (S V^T)^T.  Advances ``iseed`` in place like dlatms does."""
    import scipy.linalg as sl

    d = 10.0 ** (-np.arange(m, dtype=np.float64))
    dense = port.dlatms(m, m, iseed, d, m)
    u, s, vt = sl.svd(dense, lapack_driver="gesvd")
    rank = 0
    while rank < m and s[rank] >= acc:
        rank += 1
    rank = min(rank, storage_maxrank)
    U = np.asfortranarray(u[:, :rank])
    V = np.asfortranarray((s[:rank, None] * vt[:rank, :]).T)
    return dense, U, V, rank


def dense_update(alpha, AU, AV, BU, BV, beta, CU, CV):
    """Exact-arithmetic target beta*CU CV^T + alpha*(AU AV^T)(BU BV^T)^T."""
    return beta * (CU @ CV.T) + alpha * (AU @ (AV.T @ BV) @ BU.T)


def rel_fro(X, Y) -> float:
    n = np.linalg.norm(Y)
    return float(np.linalg.norm(X - Y) / (n if n > 0 else 1.0))
