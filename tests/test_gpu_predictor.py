"""What the rank predictor gains, and that it changes no result.

A small TLR matrix (8192 seeded 2D points, nb = 256, 32 x 32 tiles, kernel
exp(-|x-y|/0.2), tiles compressed to 1e-7 relative, maxrank 64) gives the
Schur updates of panels 0 and 1 (acc 1e-5, maxrk 96; new ranks 5..66).  The
library MLP is trained on the GPU on panel 0's recompression logs (the ranks
the method produced) and sizes panel 1's output slots:

* results equal the pad-to-maxrank batch: every rank and status, products
  within 1e-12 relative (the same kernels decide every rank);
* the output slots take less than half the pad batch's memory, with at most
  10% of the updates rebuilt into overflow slots;
* an untrained network (same architecture, random weights) sized by the
  same policy loses what the trained one gains;
* with every capacity forced to 1, all updates overflow and their rebuild
  from the workspace still reproduces the pad batch.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

NB, T, MAXRK, ACC = 256, 32, 96, 1e-5


@pytest.fixture(scope="module")
def tlr():
    from hcore_gb300 import panel as pnl

    pts = pnl.morton_points(NB * T, 2, 3)
    tiles = [(i, j) for i in range(T) for j in range(i)]
    return pnl.TileStore.build(pts, NB, tiles, "exp", 0.2, 1e-7, 64, seed=0)


def _updates(k):
    return [(i, j) for j in range(k + 1, T) for i in range(j + 1, T)]


def _feats(store, ups, k):
    from hcore_gb300 import predictor as P

    cen, diam = P.cluster_geometry(store.points, NB)
    a = [store.tiles[(i, k)][3] for i, j in ups]
    b = [store.tiles[(j, k)][3] for i, j in ups]
    c = [store.tiles[(i, j)][3] for i, j in ups]
    nA = [store.norm[(i, k)] for i, j in ups]
    nB = [store.norm[(j, k)] for i, j in ups]
    nC = [store.norm[(i, j)] for i, j in ups]
    d = [np.linalg.norm(cen[i] - cen[j]) for i, j in ups]
    dm = [(diam[i] + diam[j]) / 2 for i, j in ups]
    return P.features(a, b, c, nA, nB, nC, d, dm, ACC)


def _task_maker(hc, store, ups, k):
    def make(u, storage, oU, oV):
        i, j = ups[u]
        au, av, a = store.ptrs((i, k))
        bu, bv, b = store.ptrs((j, k))
        cu, cv, c = store.ptrs((i, j))
        return hc.LrTask(M=NB, a=a, b=b, c=c, rk=0, maxrk=MAXRK, ld_newv=0,
                         storage_maxrank=storage, alpha=-1.0, beta=1.0, acc=ACC, AU=au, AV=av,
                         lda=NB, BU=bu, BV=bv, ldb=NB, Bdense=None, CU=cu, CV=cv, ldc=NB,
                         CUo=oU, CVo=oV, ldco=NB)
    return make


def _product(res, u, r):
    U, V, o = res["where"][u]
    n = NB * r
    Uu = U[o:o + n].cpu().numpy().reshape(r, NB).T
    Vv = V[o:o + n].cpu().numpy().reshape(r, NB).T
    return Uu @ Vv.T


def test_predictor_sizes_outputs_without_changing_results(hc, tlr):
    from hcore_gb300 import predictor as P

    ups0, ups1 = _updates(0), _updates(1)
    pad = np.full(len(ups0), MAXRK)
    log0 = P.run_capacity_batch(hc, _task_maker(hc, tlr, ups0, 0), len(ups0), NB, pad, MAXRK)
    assert (log0["status"] == 0).all()
    F0, F1 = _feats(tlr, ups0, 0), _feats(tlr, ups1, 1)
    pred_net = P.RankPredictor(seed=1)
    losses = pred_net.fit(F0, log0["ranks"], epochs=300, batch=128, lr=3e-3, seed=2)
    assert losses[-1] < 0.2 * losses[0]
    policy = P.CapacityPolicy.fit(pred_net.predict(F0), log0["ranks"], target_overflow=0.02)

    make1 = _task_maker(hc, tlr, ups1, 1)
    ref = P.run_capacity_batch(hc, make1, len(ups1), NB, np.full(len(ups1), MAXRK), MAXRK)
    caps = policy(pred_net.predict(F1), MAXRK)
    got = P.run_capacity_batch(hc, make1, len(ups1), NB, caps, MAXRK)
    assert (ref["status"] == 0).all() and (got["status"] == 0).all()
    assert np.array_equal(got["ranks"], ref["ranks"])
    for u in range(0, len(ups1), 7):
        r = int(ref["ranks"][u])
        assert O.rel_fro(_product(got, u, r), _product(ref, u, r)) < 1e-12
    # the gain: output memory, at a small overflow rate
    assert got["overflow"] <= 0.10 * len(ups1)
    assert got["arena_bytes"] < 0.5 * ref["arena_bytes"]

    # the same policy on an untrained network of the same shape
    raw = P.RankPredictor(seed=1)
    raw.mu, raw.sd = pred_net.mu, pred_net.sd
    caps_raw = policy(raw.predict(F1), MAXRK)
    untrained = P.run_capacity_batch(hc, make1, len(ups1), NB, caps_raw, MAXRK)
    assert np.array_equal(untrained["ranks"], ref["ranks"])
    assert (untrained["overflow"] > 2 * got["overflow"] + 5 or
            untrained["arena_bytes"] > 1.5 * got["arena_bytes"])


def test_every_update_overflowing_still_matches(hc, tlr):
    from hcore_gb300 import predictor as P

    ups = _updates(1)[:60]
    make = _task_maker(hc, tlr, ups, 1)
    ref = P.run_capacity_batch(hc, make, len(ups), NB, np.full(len(ups), MAXRK), MAXRK)
    got = P.run_capacity_batch(hc, make, len(ups), NB, np.ones(len(ups), np.int64), MAXRK)
    overflowed = int((ref["ranks"] > 1).sum())
    assert got["overflow"] == overflowed
    assert np.array_equal(got["ranks"], ref["ranks"]) and (got["status"] == 0).all()
    for u in range(len(ups)):
        r = int(ref["ranks"][u])
        assert O.rel_fro(_product(got, u, r), _product(ref, u, r)) < 1e-12


def test_rebuild_with_rank_cap_equals_fixed_rank_update(hc, port):
    """An update whose rank exceeds its storage is rebuilt truncated to
    max_rank: the result is HCORE_dgemm's fixed-rank update (rk = max_rank)."""
    import torch
    from hcore_gb300 import devmem

    rng = np.random.default_rng(31)
    M, a, b, c, cap = 256, 20, 18, 24, 10
    AU, AV = O.graded_lowrank(rng, M, a, 10.0)
    BU, BV = O.graded_lowrank(rng, M, b, 10.0)
    CU, CV = O.graded_lowrank(rng, M, c, 10.0)
    d = [devmem.to_device(x) for x in (AU, AV, BU, BV, CU, CV)]
    oU = torch.zeros((cap, M), dtype=torch.float64, device="cuda")
    oV = torch.zeros_like(oU)
    t = hc.LrTask(M=M, a=a, b=b, c=c, rk=0, maxrk=64, ld_newv=0, storage_maxrank=cap,
                  alpha=-1.0, beta=1.0, acc=1e-12, AU=d[0].data_ptr(), AV=d[1].data_ptr(), lda=M,
                  BU=d[2].data_ptr(), BV=d[3].data_ptr(), ldb=M, Bdense=None, CU=d[4].data_ptr(),
                  CV=d[5].data_ptr(), ldc=M, CUo=oU.data_ptr(), CVo=oV.data_ptr(), ldco=M)
    batch = hc.Batch([t])
    batch.execute()
    r, st = batch.results()
    assert st[0] == 5 and r[0] > cap                      # STORAGE, outputs untouched
    assert float(oU.abs().max()) == 0.0
    batch.rebuild([0], [oU.data_ptr()], [oV.data_ptr()], [M], max_rank=[cap])
    r, st = batch.results()
    assert st[0] == 0 and r[0] == cap
    ref = port.gemm(M, -1.0, AU, AV, a, BU, BV, b, 1.0, CU, CV, c, rk=cap, maxrk=64, acc=1e-12)
    assert ref["status"] == 0 and ref["rank"] == cap
    P = devmem.to_host(oU, cap) @ devmem.to_host(oV, cap).T
    assert O.rel_fro(P, ref["CU"] @ ref["CV"].T) < 1e-11
