"""Tile compression on the GPU (hcore_gpu_compress_batched) against the
reference tests' compressor (generate_compress fixtures) and the oracle.

The GPU finds each tile's range with a truncated pivoted QR (remaining
Frobenius norm below 1e-3 of the threshold), then runs the recompression
plan's QR, Jacobi SVD and rebuild on it.  So ranks equal the reference's
whenever no singular value lies within that margin of the threshold (the
cases here are checked to have none), and products agree with the full-SVD
truncation to 1e-12 of the tile's norm plus the margin.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _run(hc, tiles, acc, maxrank, relative=False):
    import torch
    from hcore_gb300 import devmem

    dD = [devmem.to_device(np.asfortranarray(D)) for D in tiles]
    outs, tasks = [], []
    for D, d in zip(tiles, dD):
        M = D.shape[0]
        U = torch.full((M, M), np.nan, dtype=torch.float64, device="cuda")
        V = torch.full((M, M), np.nan, dtype=torch.float64, device="cuda")
        outs.append((U, V))
        tasks.append(hc.CompressTask(M=M, D=d.data_ptr(), ldd=M, acc=acc, relative=int(relative),
                                     maxrank=maxrank, U=U.data_ptr(), V=V.data_ptr(), ldo=M))
    ranks, status = hc.compress_batched(tasks)
    res = []
    for (U, V), r in zip(outs, ranks):
        r = int(r)
        res.append((devmem.to_host(U, r) if r else None, devmem.to_host(V, r) if r else None))
    del dD, torch
    return ranks, status, res


def test_compress_matches_reference_fixtures(hc, golden_compress):
    meta, g = golden_compress
    for c in meta:
        n = c["name"]
        A = g[f"{n}_A"]
        ranks, status, res = _run(hc, [A], c["acc"], c["maxrank"])
        assert status[0] == 0 and ranks[0] == c["rank"], (n, ranks, status)
        if c["rank"]:
            U, V = res[0]
            P, Pref = U @ V.T, g[f"{n}_U"] @ g[f"{n}_V"].T
            assert np.abs(P - Pref).max() <= 1e-12 * np.abs(A).max() + 1e-3 * c["acc"]
            # U has orthonormal columns, V's columns are orthogonal with the
            # singular values as norms (sigma_i = 10^-i from dlatms)
            assert np.abs(U.T @ U - np.eye(c["rank"])).max() < 1e-12
            sv = np.linalg.norm(V, axis=0)
            assert np.allclose(sv, 10.0 ** -np.arange(c["rank"]), rtol=1e-9, atol=1e-14)


def _kernel_tiles(rng, M, count):
    """Off-diagonal covariance tiles exp(-|x-y|^2/0.01) of 2D point clusters."""
    tiles = []
    for q in range(count):
        X = rng.uniform(0, 0.25, (M, 2))
        Y = rng.uniform(0, 0.25, (M, 2)) + np.array([0.2 + 0.1 * q, 0.1])
        d2 = ((X[:, None, :] - Y[None, :, :]) ** 2).sum(-1)
        tiles.append(np.asfortranarray(np.exp(-d2 / 0.01)))
    return tiles


def _margin_ok(sig, thr, r):
    """No singular value within the GPU's margin of the threshold."""
    return np.all(np.abs(sig - thr) > 2e-3 * thr)


def test_compress_kernel_tiles_relative_rule(hc, port):
    """Batched tiles of sizes 1, 33, 256, 1024 and 2048 with the relative rule
    (1e-8 sigma_max, the TLR workloads' compression) and a rank cap."""
    rng = np.random.default_rng(81)
    tiles = [np.full((1, 1), 3.0)] + _kernel_tiles(rng, 33, 1) + _kernel_tiles(rng, 256, 2) + \
        _kernel_tiles(rng, 1024, 2) + _kernel_tiles(rng, 2048, 1)
    for maxrank in (128, 12):
        ranks, status, res = _run(hc, tiles, 1e-8, maxrank, relative=True)
        assert (status == 0).all(), status
        for D, r, (U, V) in zip(tiles, ranks, res):
            rr, Ur, Vr, sig = port.dcompress(D, 1e-8, maxrank, relative=True)
            assert _margin_ok(sig, 1e-8 * sig[0], rr)
            assert r == rr, (D.shape, r, rr)
            if r:
                assert np.abs(U @ V.T - Ur @ Vr.T).max() <= 1e-10 * sig[0]


def test_compress_edge_cases(hc, port):
    """A zero tile (rank 0), a tile below the threshold (rank 0), a NaN tile
    (NOCONV, the others unaffected), maxrank 0, and a full-rank 64 x 64 tile
    (range of all 64 columns)."""
    rng = np.random.default_rng(82)
    Z = np.zeros((40, 40), order="F")
    small = np.asfortranarray(1e-9 * rng.standard_normal((50, 50)))
    bad = np.asfortranarray(rng.standard_normal((30, 30)))
    bad[3, 4] = np.nan
    Q, _ = np.linalg.qr(rng.standard_normal((64, 64)))
    full = np.asfortranarray(Q @ np.diag(np.linspace(1.0, 2.0, 64)) @ Q.T)
    ranks, status, res = _run(hc, [Z, small, bad, full], 1e-6, 64)
    assert list(status) == [0, 0, 6, 0]
    assert list(ranks[:2]) == [0, 0] and ranks[3] == 64
    U, V = res[3]
    assert np.abs(U @ V.T - full).max() < 1e-12
    ranks, status, _ = _run(hc, [full], 1e-6, 0)
    assert status[0] == 0 and ranks[0] == 0
