"""GPU parity on the benchmark's own tiles and at the truncation threshold.

* A slice of the 65,536-point panel workload (the first 64 of its 1953
  Schur updates C_ij -= A_i0 A_j0^T, tiles built by hcore_gb300.panel exactly
  as the benchmark builds them) through the batched plan, every update
  against the oracle (the reference's LAPACK sequence restated,
  src/compute/hcore_dgemm.c:703-1012): equal rank, product within 1e-11
  relative Frobenius, and error against the exact update C - A B^T no more
  than the oracle's own truncation error + 1e-14 relative.
* The rank rule (hcore_dgemm.c:446-463: first i with sigma_i < acc, absolute
  and strict) with one singular value of the updated tile placed at
  acc (1 + 1e-9) or at acc (1 - 1e-9), i.e. outside the 1e-12 relative band
  where any FP64 SVD may flip the rank.  The tile's largest
  singular value is kept at or below 1e-4 so that the SVD's absolute error
  (a few eps sigma_max) stays far below the 1e-17 gap to the threshold.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _lr_norm(X, Y) -> float:
    """||X Y^T||_F by QR of both factors (no dense product)."""
    if X.shape[1] == 0:
        return 0.0
    return float(np.linalg.norm(np.linalg.qr(X, mode="r") @ np.linalg.qr(Y, mode="r").T))


def test_panel_slice_against_oracle(hc, port):
    import torch

    from hcore_gb300 import panel as pnl

    pnl_ = pnl.build_panel(device="cuda", max_updates=64)
    nb, n = pnl_.nb, len(pnl_.updates)
    assert n == 64
    off = np.arange(n + 1, dtype=np.int64) * nb * pnl_.maxrank
    oU = torch.zeros(int(off[-1]), dtype=torch.float64, device="cuda")
    oV = torch.zeros_like(oU)
    e = 8
    tasks = []

    def ptrs(s_):
        o = int(pnl_.offset[s_])
        return pnl_.U.data_ptr() + e * o, pnl_.V.data_ptr() + e * o, int(pnl_.rank[s_])

    for u, (i, j) in enumerate(pnl_.updates):
        au, av, a = ptrs(pnl_.index[(i, 0)])
        bu, bv, b = ptrs(pnl_.index[(j, 0)])
        cu, cv, c = ptrs(pnl_.index[(i, j)])
        tasks.append(hc.LrTask(M=nb, a=a, b=b, c=c, rk=0, maxrk=pnl_.maxrank, ld_newv=0,
                               storage_maxrank=pnl_.maxrank, alpha=-1.0, beta=1.0, acc=pnl_.acc,
                               AU=au, AV=av, lda=nb, BU=bu, BV=bv, ldb=nb, Bdense=None, CU=cu,
                               CV=cv, ldc=nb, CUo=oU.data_ptr() + e * int(off[u]),
                               CVo=oV.data_ptr() + e * int(off[u]), ldco=nb))
    batch = hc.Batch(tasks)
    batch.execute()
    ranks, status = batch.results()
    assert (status == 0).all()
    U, V = pnl_.U.cpu().numpy(), pnl_.V.cpu().numpy()

    def fac(s_):
        o0, o1 = int(pnl_.offset[s_]), int(pnl_.offset[s_ + 1])
        r = (o1 - o0) // nb
        return (np.asfortranarray(U[o0:o1].reshape(r, nb).T),
                np.asfortranarray(V[o0:o1].reshape(r, nb).T), r)

    gU_all, gV_all = oU.cpu().numpy(), oV.cpu().numpy()
    e2g = e2r = d2 = 0.0
    for u, (i, j) in enumerate(pnl_.updates):
        AU, AV, a = fac(pnl_.index[(i, 0)])
        BU, BV, b = fac(pnl_.index[(j, 0)])
        CU, CV, c = fac(pnl_.index[(i, j)])
        r = int(ranks[u])
        gU = gU_all[int(off[u]):int(off[u]) + nb * r].reshape(r, nb).T
        gV = gV_all[int(off[u]):int(off[u]) + nb * r].reshape(r, nb).T
        ref = port.gemm(nb, -1.0, AU, AV, a, BU, BV, b, 1.0, CU, CV, c, maxrk=pnl_.maxrank,
                        acc=pnl_.acc)
        assert r == ref["rank"], (u, r, ref["rank"])
        diff = _lr_norm(np.hstack([gU, ref["CU"]]), np.hstack([gV, -ref["CV"]]))
        assert diff <= 1e-11 * _lr_norm(ref["CU"], ref["CV"]), u
        AF = AU @ (AV.T @ BV)                    # exact update D = [CU | AF] [CV | -BU]^T
        eg = _lr_norm(np.hstack([gU, CU, AF]), np.hstack([gV, -CV, BU]))
        er = _lr_norm(np.hstack([ref["CU"], CU, AF]), np.hstack([ref["CV"], -CV, BU]))
        nd = _lr_norm(np.hstack([CU, AF]), np.hstack([CV, -BU]))
        assert eg <= 1.01 * er + 1e-14 * nd, u
        e2g, e2r, d2 = e2g + eg * eg, e2r + er * er, d2 + nd * nd
    assert np.sqrt(e2g / d2) <= pnl_.acc                 # panel-level relative error <= acc
    assert np.sqrt(e2g / d2) <= 1.01 * np.sqrt(e2r / d2) + 1e-14
    batch.close()


def _threshold_case(rng, M, smax, acc, above):
    """C = U1 diag(s1) V1^T and A B^T = U2 diag(s2) V2^T with U1 _|_ U2 and
    V1 _|_ V2, so C + A B^T has exactly the singular values s1 and s2.  One of
    them is acc (1 + 1e-9) (above) or acc (1 - 1e-9); the others lie at least
    40% away from it, so the truncated product is well conditioned."""
    x = acc * (1 + 1e-9) if above else acc * (1 - 1e-9)
    s1 = np.array([smax, smax / 3, x, 0.4 * acc, 0.1 * acc, 0.01 * acc])
    s2 = np.array([smax / 2, smax / 10, 0.6 * acc, 0.5 * acc, 0.05 * acc, 0.005 * acc])
    k = len(s1)
    Q = O.haar(rng, M, 3 * k)
    P = O.haar(rng, M, 2 * k)
    U1, U2, W = Q[:, :k], Q[:, k:2 * k], Q[:, 2 * k:]
    V1, V2 = P[:, :k], P[:, k:]
    CU, CV = np.asfortranarray(U1 * s1), np.asfortranarray(V1)
    AU, AV = np.asfortranarray(U2 * s2), np.asfortranarray(W)   # A = U2 S2 W^T
    BU, BV = np.asfortranarray(V2), np.asfortranarray(W)        # B = V2 W^T, A B^T = U2 S2 V2^T
    exact = int((np.concatenate([s1, s2]) >= acc).sum())
    return AU, AV, BU, BV, CU, CV, k, exact


@pytest.mark.parametrize("smax", [1e-6, 1e-5, 1e-4])
@pytest.mark.parametrize("above", [True, False])
def test_rank_just_outside_the_threshold_band(hc, port, smax, above):
    from hcore_gb300 import devmem

    acc, M = 1e-8, 512
    rng = np.random.default_rng(int(smax * 1e9) + above)
    AU, AV, BU, BV, CU, CV, k, exact = _threshold_case(rng, M, smax, acc, above)
    assert exact == (5 if above else 4)
    d = [devmem.to_device(x) for x in (AU, AV, BU, BV)]
    dCU, dCV = devmem.to_device(CU, 2 * k), devmem.to_device(CV, 2 * k)
    t = hc.LrTask(M=M, a=k, b=k, c=k, rk=0, maxrk=2 * k, ld_newv=0, storage_maxrank=0,
                  alpha=1.0, beta=1.0, acc=acc, AU=d[0].data_ptr(), AV=d[1].data_ptr(), lda=M,
                  BU=d[2].data_ptr(), BV=d[3].data_ptr(), ldb=M, Bdense=None, CU=dCU.data_ptr(),
                  CV=dCV.data_ptr(), ldc=M, CUo=dCU.data_ptr(), CVo=dCV.data_ptr(), ldco=M)
    batch = hc.Batch([t])
    batch.execute()
    ranks, status = batch.results()
    sig = batch.sigma(0)
    batch.close()
    assert status[0] == 0
    ref = port.gemm(M, 1.0, AU, AV, k, BU, BV, k, 1.0, CU, CV, k, maxrk=2 * k, acc=acc)
    assert ref["rank"] == exact                       # LAPACK resolves the gap
    assert int(ranks[0]) == exact                     # and so does the GPU path
    assert sig[exact - 1] >= acc > sig[exact]
    r = int(ranks[0])
    P = devmem.to_host(dCU, r) @ devmem.to_host(dCV, r).T
    assert O.rel_fro(P, ref["CU"] @ ref["CV"].T) < 1e-11
