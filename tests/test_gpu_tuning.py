"""Launch-shape tuning of a plan and the autotuner (hcore_gpu_tuning,
hcore_gpu_plan_create_tuned, hcore_gpu_autotune): any valid tuning gives the
default plan's ranks and statuses and its products to rounding (1e-12
relative: only the SVD's reduction order follows the lanes per pair); the
autotuner returns a valid tuning; invalid tunings are refused."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _tasks(hc, rng, n=60, M=256):
    import torch
    from hcore_gb300 import devmem

    keep, tasks = [], []
    for _ in range(n):
        a, b, c = (int(x) for x in rng.integers(1, 41, size=3))
        arr = [O.graded_lowrank(rng, M, r, 8.0) for r in (a, b, c)]
        d = [devmem.to_device(x) for pair in arr for x in pair]
        oU = torch.zeros((a + c, M), dtype=torch.float64, device="cuda")
        oV = torch.zeros_like(oU)
        keep.append((d, oU, oV))
        tasks.append(hc.LrTask(M=M, a=a, b=b, c=c, rk=0, maxrk=a + c, ld_newv=0, storage_maxrank=0,
                               alpha=-1.0, beta=1.0, acc=1e-8, AU=d[0].data_ptr(), AV=d[1].data_ptr(),
                               lda=M, BU=d[2].data_ptr(), BV=d[3].data_ptr(), ldb=M, Bdense=None,
                               CU=d[4].data_ptr(), CV=d[5].data_ptr(), ldc=M, CUo=oU.data_ptr(),
                               CVo=oV.data_ptr(), ldco=M))
    return keep, tasks


def _run(hc, tasks, keep, tuning):
    from hcore_gb300 import devmem

    b = hc.Batch(tasks, tuning=tuning)
    b.execute()
    r, st = b.results()
    b.close()
    prods = [devmem.to_host(oU, int(ri)) @ devmem.to_host(oV, int(ri)).T
             for (d, oU, oV), ri in zip(keep, r)]
    return r.copy(), st.copy(), prods


def test_tunings_give_the_same_results(hc):
    rng = np.random.default_rng(71)
    keep, tasks = _tasks(hc, rng)
    r0, s0, p0 = _run(hc, tasks, keep, None)
    assert (s0 == 0).all()
    for tun in ({"stream_groups": 1}, {"stream_groups": 3, "bucket_width": 16},
                {"svd_lanes": (2, 8, 4)}, {"stream_groups": 64, "svd_lanes": (1, 2, 1)},
                {"svd_lanes": (2, 2, 2)}, {"svd_lanes": (4, 4, 4), "qr_warps": 8},
                {"stream_groups": 8, "phase_sync": 1}, {"qr_warps": 4}, {"qr_warps": 2}):
        r, st, p = _run(hc, tasks, keep, tun)
        assert np.array_equal(r, r0) and np.array_equal(st, s0), tun
        for a, b in zip(p, p0):
            assert O.rel_fro(a, b) < 1e-12, tun


def test_autotune_returns_a_valid_tuning(hc):
    rng = np.random.default_rng(72)
    keep, tasks = _tasks(hc, rng, n=40)
    best, ms = hc.autotune(tasks, reps=2)
    t = best.as_dict()
    assert ms > 0
    assert 1 <= t["stream_groups"] <= 64 and t["bucket_width"] in (8, 16)
    assert t["phase_sync"] in (0, 1) and t["qr_warps"] in (2, 4, 8)
    assert all(x in (0, 1, 2, 4, 8, 16, 32) for x in t["svd_lanes"])   # 0: fill the warps
    r, st, _ = _run(hc, tasks, keep, best)
    assert (st == 0).all()


def test_invalid_tuning_is_refused(hc):
    rng = np.random.default_rng(73)
    keep, tasks = _tasks(hc, rng, n=4)
    for bad in ({"stream_groups": 0}, {"svd_lanes": (3, 4, 2)}, {"svd_lanes": (-1, 2, 2)},
                {"bucket_width": 12},
                {"phase_sync": 2}, {"qr_warps": 6}):
        with pytest.raises(hc.HcoreError):
            hc.Batch(tasks, tuning=bad)
