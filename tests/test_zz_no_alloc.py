"""hcore_gpu_dgemm_noalloc: the update entry point for callers that cannot
allocate device memory (task-runtime workers that must not stall the other
workers' streams, runtimes that reserved all their device memory up front).
Its workspace is a fixed device array inside the library.

Checked through the C ABI against the existing plan entry point
(hcore_gpu_plan_*) on the same inputs, two calls in a row (the second call
reuses the array the first one left behind), with the tolerance of the other
parity tests: equal rank, product within 1e-11 relative Frobenius.  This file
is collected last so that a run stopping at the first failure has already
run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-11


def _bind(L):
    dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int)
    f = L.hcore_gpu_dgemm_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_int, C.c_double, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                  C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_void_p, C.c_void_p, C.c_int,
                  C.c_int, C.c_int, C.c_int, C.c_double, ip, ip, C.c_void_p]
    return f


def _case(seed, M, a, b, c):
    rng = np.random.default_rng(seed)
    AU, AV = O.graded_lowrank(rng, M, a)
    BU, BV = O.graded_lowrank(rng, M, b)
    CU, CV = O.graded_lowrank(rng, M, c)
    return AU, AV, BU, BV, CU, CV


def _via_plan(hc, devmem, M, arrays, a, b, c, maxrk, acc):
    AU, AV, BU, BV, CU, CV = arrays
    d = [devmem.to_device(x) for x in (AU, AV, BU, BV)]
    dCU, dCV = devmem.to_device(CU, a + c), devmem.to_device(CV, a + c)
    t = hc.LrTask(M=M, a=a, b=b, c=c, rk=0, maxrk=maxrk, ld_newv=maxrk, storage_maxrank=0,
                  alpha=-1.0, beta=1.0, acc=acc, AU=d[0].data_ptr(), AV=d[1].data_ptr(), lda=M,
                  BU=d[2].data_ptr(), BV=d[3].data_ptr(), ldb=M, Bdense=None,
                  CU=dCU.data_ptr(), CV=dCV.data_ptr(), ldc=M, CUo=dCU.data_ptr(),
                  CVo=dCV.data_ptr(), ldco=M)
    batch = hc.Batch([t])
    batch.execute()
    ranks, status = batch.results()
    assert status[0] == 0
    r = int(ranks[0])
    return r, devmem.to_host(dCU, r), devmem.to_host(dCV, r)


# capacity of the fixed array in doubles, and the workspace one update needs
# (the library's per-update layout: two M x k stacks, three k-vectors, a x b,
# four k x k blocks, each region rounded up to 32 doubles)
NOALLOC_WS_ELEMS = 393216


def _ws_need(M, a, b, k):
    o = 0
    for size in (M * k, M * k, k, k, k, a * b, k * k, k * k, k * k, k * k):
        o = (o + size + 31) & ~31
    return o


def _call(f, hc, M, a, b, c, maxrk, arrays):
    from hcore_gb300 import devmem

    AU, AV, BU, BV, CU, CV = arrays
    d = [devmem.to_device(x) for x in (AU, AV, BU, BV)]
    dCU, dCV = devmem.to_device(CU, a + c), devmem.to_device(CV, a + c)
    r, st = C.c_int(-1), C.c_int(-1)
    rc = f(M, -1.0, d[0].data_ptr(), d[1].data_ptr(), a, M, d[2].data_ptr(),
           d[3].data_ptr(), b, M, 1.0, dCU.data_ptr(), dCV.data_ptr(), c, M, 0, maxrk, 1e-8,
           C.byref(r), C.byref(st), None)
    assert rc == 0, hc.last_error()
    assert st.value == 0
    return r.value, devmem.to_host(dCU, r.value), devmem.to_host(dCV, r.value)


def _check_against_plan(f, hc, seed, M, a, b, c, maxrk):
    from hcore_gb300 import devmem

    arrays = _case(seed, M, a, b, c)
    r, gU, gV = _call(f, hc, M, a, b, c, maxrk, arrays)
    r_ref, CU_ref, CV_ref = _via_plan(hc, devmem, M, arrays, a, b, c, maxrk, 1e-8)
    assert r == r_ref
    assert O.rel_fro(gU @ gV.T, CU_ref @ CV_ref.T) < FP64_TOL


def test_noalloc_matches_plan_entry_point_twice(hc):
    f = _bind(hc.lib())
    # two calls in a row on the shared array (the second finds the first's
    # contents there)
    for seed, M, a, b, c, maxrk in [(41, 512, 20, 18, 24, 64), (42, 1024, 30, 26, 34, 128)]:
        _check_against_plan(f, hc, seed, M, a, b, c, maxrk)


def test_noalloc_at_its_documented_and_exact_limits(hc):
    """M = 1024 with a + c = 128 (the documented capacity), then the largest
    rank sum whose workspace still fits the array (a + c = 146, where the SVD
    keeps only R^T in shared memory); one more column is refused."""
    f = _bind(hc.lib())
    assert _ws_need(1024, 64, 64, 128) <= NOALLOC_WS_ELEMS
    _check_against_plan(f, hc, 43, 1024, 64, 64, 64, 128)
    assert _ws_need(1024, 73, 73, 146) <= NOALLOC_WS_ELEMS < _ws_need(1024, 73, 73, 147)
    _check_against_plan(f, hc, 44, 1024, 73, 73, 73, 146)
    arrays = _case(45, 1024, 73, 73, 74)
    from hcore_gb300 import devmem

    d = [devmem.to_device(x) for x in arrays]
    r, st = C.c_int(-1), C.c_int(-1)
    rc = f(1024, -1.0, d[0].data_ptr(), d[1].data_ptr(), 73, 1024, d[2].data_ptr(),
           d[3].data_ptr(), 73, 1024, 1.0, d[4].data_ptr(), d[5].data_ptr(), 74, 1024, 0, 147,
           1e-8, C.byref(r), C.byref(st), None)
    assert rc == -1
    assert "scratch" in hc.last_error()


def test_noalloc_rejects_updates_beyond_its_scratch(hc):
    """M = 2048 with a + c = 128 needs more than the fixed array: refused on
    the host with a message, before any launch."""
    import torch

    f = _bind(hc.lib())
    M, a, b, c = 2048, 64, 64, 64
    x = torch.zeros((a, M), dtype=torch.float64, device="cuda")
    r, st = C.c_int(-1), C.c_int(-1)
    rc = f(M, -1.0, x.data_ptr(), x.data_ptr(), a, M, x.data_ptr(), x.data_ptr(), b, M, 1.0,
           x.data_ptr(), x.data_ptr(), c, M, 0, 128, 1e-8, C.byref(r), C.byref(st), None)
    assert rc == -1
    assert "scratch" in hc.last_error()
