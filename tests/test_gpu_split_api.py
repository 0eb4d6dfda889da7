"""GPU parity of the two-phase API (src/compute/hcore_dgemm.c:1022-1699):
HCORE_dgemm_qr_svd / HCORE_dgemm_qr_svd_b_dense decide the rank and return
their state in host buffers; the caller then calls HCORE_dgemm_ormqr, which
rebuilds the factors into _CU_save/_CV_save and sets Crk.  Checked against
the oracle's split-API restatement (variant 2: ld_newV = 2*maxrk,
storage_maxrank) on the same inputs."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu
vp, ip = C.c_void_p, C.POINTER(C.c_int)


def _bind(L, hc, prefix, real):
    q = getattr(L, f"HCORE_{prefix}gemm_qr_svd")
    qd = getattr(L, f"HCORE_{prefix}gemm_qr_svd_b_dense")
    o = getattr(L, f"HCORE_{prefix}gemm_ormqr")
    fc = C.POINTER(hc.FlopCounter)
    outs = [C.POINTER(vp), C.POINTER(vp), C.POINTER(vp), ip, ip, C.POINTER(vp), ip, C.POINTER(vp),
            ip, C.POINTER(vp), ip, C.POINTER(vp), ip, C.POINTER(vp), ip, C.POINTER(vp),
            C.POINTER(vp), ip, C.POINTER(vp)]
    q.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, real, vp, vp, ip, C.c_int, vp, vp, ip,
                  C.c_int, real, vp, vp, ip, C.c_int, C.c_int, C.c_int, C.c_int, real, vp, fc] + outs
    qd.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, real, vp, vp, ip, C.c_int, vp, C.c_int,
                   real, vp, vp, ip, C.c_int, C.c_int, C.c_int, C.c_int, real, vp, fc] + outs
    o.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, real, vp, vp, ip, C.c_int, real, vp, vp, ip,
                  C.c_int, C.c_int, C.c_int, C.c_int, real, vp, fc, vp, vp, C.c_int, C.c_int, vp,
                  C.c_int, vp, C.c_int, vp, C.c_int, vp, C.c_int, vp, C.c_int, vp, vp, C.c_int, vp]
    q.restype = qd.restype = o.restype = None
    return q, qd, o


def _two_phase(hc, prefix, dtype, M, alpha, AU, AV, a, BU, BV, b, Bd, beta, CU, CV, c, maxrk,
               storage, acc):
    L = hc.lib()
    real = C.c_float if dtype == np.float32 else C.c_double
    q, qd, o = _bind(L, hc, prefix, real)
    f = lambda x: np.asfortranarray(x, dtype=dtype)  # noqa: E731
    AU, AV = f(AU), f(AV)
    ncol = max(storage, c)
    CUs = np.zeros((M, ncol), dtype=dtype, order="F")
    CVs = np.zeros((M, ncol), dtype=dtype, order="F")
    CUs[:, :c] = CU
    CVs[:, :c] = CV
    ra, rb, rc = C.c_int(a), C.c_int(b), C.c_int(c)
    st = [vp(), vp(), vp(), C.c_int(), C.c_int(), vp(), C.c_int(), vp(), C.c_int(), vp(),
          C.c_int(), vp(), C.c_int(), vp(), C.c_int(), vp(), vp(), C.c_int(), vp()]
    fl = hc.FlopCounter()
    ptr = lambda x: x.ctypes.data_as(vp)  # noqa: E731
    if Bd is None:
        BU, BV = f(BU), f(BV)
        q(111, 112, M, M, alpha, ptr(AU), ptr(AV), C.byref(ra), M, ptr(BU), ptr(BV), C.byref(rb),
          M, beta, ptr(CUs), ptr(CVs), C.byref(rc), M, 0, storage, maxrk, acc, None, C.byref(fl),
          *[C.byref(x) for x in st])
    else:
        Bd = f(Bd)
        qd(111, 112, M, M, alpha, ptr(AU), ptr(AV), C.byref(ra), M, ptr(Bd), M, beta, ptr(CUs),
           ptr(CVs), C.byref(rc), M, 0, storage, maxrk, acc, None, C.byref(fl),
           *[C.byref(x) for x in st])
    (work_new, _CU, _CV, CU_ncols, new_rk, newU, ld_newU, tauA, CV_ncols, newV, ld_newV, tauB,
     use_clone, CUclone, ld_CUclone, CU_save, CVclone, ld_CVclone, CV_save) = st
    assert CU_ncols.value == a + c and CV_ncols.value == a + c
    assert ld_newU.value == M and ld_newV.value == 2 * maxrk      # hcore_dgemm.c:1479-1480
    assert CU_save.value == CUs.ctypes.data
    r = new_rk.value
    fl1 = fl.update
    o(111, 112, M, M, alpha, ptr(AU), ptr(AV), C.byref(ra), M, beta, ptr(CUs), ptr(CVs),
      C.byref(rc), M, 0, storage, maxrk, acc, None, C.byref(fl), _CU, _CV, CU_ncols.value, r,
      newU, ld_newU.value, tauA, CV_ncols.value, newV, ld_newV.value, tauB, use_clone.value,
      CUclone, ld_CUclone.value, CU_save, CVclone, ld_CVclone.value, CV_save)
    assert rc.value == r                                           # Crk[0] set by ormqr
    return r, CUs[:, :r], CVs[:, :r], fl1, fl.update


@pytest.mark.parametrize("prefix,dtype,tol", [("d", np.float64, 1e-11), ("s", np.float32, 5e-5)])
def test_split_api_matches_oracle(hc, port, prefix, dtype, tol):
    rng = np.random.default_rng(61)
    # compmaxrank 24: a + c = 44 <= 2*maxrk = ld_newV; the new rank must stay
    # <= maxrk and <= storage_maxrank, or the reference exits (hcore_dgemm.c:465)
    M, a, b, c, maxrk, storage = 160, 14, 11, 20, 24, 24
    AU, AV = O.graded_lowrank(rng, M, a, 12.0)
    BU, BV = O.graded_lowrank(rng, M, b, 12.0)
    CU, CV = O.graded_lowrank(rng, M, c, 12.0)
    acc = 1e-4 if dtype == np.float32 else 1e-8
    ref = port.gemm(M, -1.0, AU, AV, a, BU, BV, b, 1.0, CU, CV, c, maxrk=maxrk,
                    storage_maxrank=storage, acc=acc, variant=2, dtype=dtype)
    assert ref["status"] == 0, "case must be valid for the reference (it would exit)"
    r, CUo, CVo, fl1, fl = _two_phase(hc, prefix, dtype, M, -1.0, AU, AV, a, BU, BV, b, None,
                                      1.0, CU, CV, c, maxrk, storage, acc)
    assert r == ref["rank"]
    assert fl == ref["flops"]                    # both phases together: the reference model
    P = CUo.astype(np.float64) @ CVo.T.astype(np.float64)
    Pr = ref["CU"].astype(np.float64) @ ref["CV"].T.astype(np.float64)
    assert O.rel_fro(P, Pr) < tol


def test_split_api_dense_b_matches_oracle(hc, port):
    """HCORE_dgemm_qr_svd_b_dense: B is a dense M x M tile, G = B * AV."""
    rng = np.random.default_rng(62)
    M, a, c, maxrk, storage = 128, 12, 16, 32, 32
    AU, AV = O.graded_lowrank(rng, M, a, 4.0)
    CU, CV = O.graded_lowrank(rng, M, c, 4.0)
    XU, XV = O.graded_lowrank(rng, M, 40, 10.0)
    Bd = np.asfortranarray(XU @ XV.T)
    ref = port.gemm(M, -1.0, AU, AV, a, None, np.zeros((M, 1)), 0, 1.0, CU, CV, c, maxrk=maxrk,
                    storage_maxrank=storage, acc=1e-8, variant=2, dense_B=Bd)
    assert ref["status"] == 0, "case must be valid for the reference (it would exit)"
    r, CUo, CVo, fl1, fl = _two_phase(hc, "d", np.float64, M, -1.0, AU, AV, a, None, None, 0, Bd,
                                      1.0, CU, CV, c, maxrk, storage, 1e-8)
    assert r == ref["rank"]
    assert fl == ref["flops"]
    D = 1.0 * (CU @ CV.T) - (AU @ AV.T) @ Bd.T
    assert O.rel_fro(CUo @ CVo.T, ref["CU"] @ ref["CV"].T) < 1e-11
    assert O.rel_fro(CUo @ CVo.T, D) <= O.rel_fro(ref["CU"] @ ref["CV"].T, D) + 1e-12
