"""Synthetic TLR Cholesky panel: the Schur updates of one panel as a batch.

The reference leaves tile generation to its caller (HiCMA); its only
compressor is the test helper generate_compress (testing/testing_dgemm.c:119-
236: SVD, keep sigma >= acc, U = left vectors, V = (S V^T)^T).  This module
builds the workload the batched path is measured on:

* n seeded uniform points in [0,1]^dim, sorted along a Morton (Z-order)
  curve so that tile (i, j) couples nearby point clusters;
* covariance tiles K_ij = k(x_p, y_q) of size nb x nb, kernel
  ``sqexp`` exp(-|x-y|^2 / ell) or ``exp`` (Matern 1/2) exp(-|x-y| / ell);
* every tile compressed to U_ij V_ij^T with the same U/V convention as the
  reference's generate_compress, truncated at sigma >= acc * sigma_max
  (relative: with the reference's absolute rule most far tiles of this kernel
  would have rank 0, which HCORE_dgemm rejects) and capped at ``maxrank``;
* the panel-0 update list C_ij <- C_ij - A_i0 A_j0^T for 1 <= j < i < T.

Compression of the input tiles is set-up work, not the measured path: it
runs once, on the host cores (randomized range finder + small SVD, LAPACK).
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field

import numpy as np


def _spread_bits(x: np.ndarray, dim: int, bits: int) -> np.ndarray:
    out = np.zeros_like(x, dtype=np.uint64)
    for b in range(bits):
        out |= ((x >> np.uint64(b)) & np.uint64(1)) << np.uint64(b * dim)
    return out


def morton_points(n: int, dim: int, seed: int) -> np.ndarray:
    """n uniform points in [0,1]^dim, Morton-sorted (deterministic)."""
    rng = np.random.default_rng(seed)
    P = rng.random((n, dim))
    bits = 63 // dim if dim > 1 else 62
    bits = min(bits, 21)
    q = np.minimum((P * (1 << bits)).astype(np.uint64), np.uint64((1 << bits) - 1))
    code = np.zeros(n, dtype=np.uint64)
    for d in range(dim):
        code |= _spread_bits(q[:, d], dim, bits) << np.uint64(d)
    return P[np.argsort(code, kind="stable")]


@dataclass
class Panel:
    """Compressed tiles of a TLR matrix and the update list of panel 0.

    Factors live in two device arenas (one column-major block per factor,
    ld = nb): ``U[t]``/``V[t]`` for every tile t in ``tiles`` (a list of
    (i, j) pairs).  ``rank[t]`` is the tile's rank."""

    nb: int
    ntiles: int
    acc: float
    maxrank: int
    tiles: list
    rank: np.ndarray
    offset: np.ndarray           # element offset of tile t's factors in the arena
    U: "object" = None           # torch tensor (flat, fp64)
    V: "object" = None
    updates: list = field(default_factory=list)  # (i, j) pairs, panel k = 0
    index: dict = field(default_factory=dict)    # (i, j) -> tile slot


def _kernel_np(X: np.ndarray, Y: np.ndarray, kind: str, ell: float) -> np.ndarray:
    d2 = (X * X).sum(-1)[:, None] + (Y * Y).sum(-1)[None, :] - 2.0 * X @ Y.T
    np.maximum(d2, 0.0, out=d2)
    if kind == "sqexp":
        return np.exp(-d2 / ell)
    if kind == "exp":
        return np.exp(-np.sqrt(d2) / ell)
    raise ValueError(kind)


def compress_tile(K: np.ndarray, acc: float, maxrank: int, seed: int, oversample: int = 32):
    """Randomized compression of one nb x nb tile (host, LAPACK): range
    finder with p = maxrank + oversample Gaussian vectors, QR, small SVD.
    Returns (U, V, rank) with U orthonormal and V = (S V^T)^T, truncated at
    sigma >= acc * sigma_max and capped at maxrank."""
    import scipy.linalg as sl

    nb = K.shape[0]
    p = min(nb, maxrank + oversample)
    omega = np.random.default_rng(seed).standard_normal((nb, p))
    Q, _ = sl.qr(K @ omega, mode="economic")
    Ub, S, Vh = sl.svd(Q.T @ K, full_matrices=False, lapack_driver="gesvd")
    r = int(min(maxrank, (S >= acc * S[0]).sum())) if S[0] > 0 else 1
    r = max(r, 1)
    U = Q @ Ub[:, :r]
    V = (S[:r, None] * Vh[:r]).T
    return U, V, r


def _compress_job(args):
    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    folder, slots, nb, kind, ell, acc, maxrank, seed = args
    P = np.load(os.path.join(folder, "points.npy"), mmap_mode="r")
    out = []
    for s, i, j in slots:
        K = _kernel_np(np.asarray(P[i * nb:(i + 1) * nb]), np.asarray(P[j * nb:(j + 1) * nb]),
                       kind, ell)
        U, V, r = compress_tile(K, acc, maxrank, seed * 100003 + s)
        out.append((s, np.ascontiguousarray(U.T), np.ascontiguousarray(V.T), r))
    return out


def panel_layout(n_points: int = 65536, dim: int = 2, nb: int = 1024, seed: int = 0,
                 max_updates: int | None = None):
    """Points, tile count per dimension, the tiles panel 0 touches and its
    update list.  Tile slot s (its index in the returned list) seeds that
    tile's compression, so any subset of tiles compresses to the same factors
    as the full panel."""
    T = n_points // nb
    P = morton_points(n_points, dim, seed)
    tiles = [(i, 0) for i in range(1, T)]
    updates = [(i, j) for j in range(1, T) for i in range(j + 1, T)]
    if max_updates is not None:
        updates = updates[:max_updates]
    tiles += sorted(set(updates))
    return P, T, tiles, updates


def compress_slots(P: np.ndarray, nb: int, tiles: list, slots, kernel: str = "sqexp",
                   ell: float = 0.01, acc: float = 1e-8, maxrank: int = 128, seed: int = 0,
                   workers: int | None = None) -> dict:
    """Compress the tiles at the given slots of `tiles` on the host cores (one
    single-threaded LAPACK process per core, spawn start method so a CUDA
    context in the parent is safe).  Returns slot -> (U^T, V^T, rank)."""
    import multiprocessing as mp
    import tempfile

    slots = list(slots)
    workers = max(1, min(workers or os.cpu_count() or 1, len(slots) or 1))
    jobs = [(s, tiles[s][0], tiles[s][1]) for s in slots]
    out = {}
    if not jobs:
        return out
    with tempfile.TemporaryDirectory() as folder:
        np.save(os.path.join(folder, "points.npy"), P)
        chunks = [jobs[w::workers] for w in range(workers)]
        chunks = [c for c in chunks if c]
        args = [(folder, c, nb, kernel, ell, acc, maxrank, seed) for c in chunks]
        if len(chunks) == 1:
            parts = [_compress_job(args[0])]
        else:
            # children inherit the environment: one BLAS thread per process
            saved = {v: os.environ.get(v) for v in ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS")}
            os.environ.update(OPENBLAS_NUM_THREADS="1", OMP_NUM_THREADS="1")
            try:
                with mp.get_context("spawn").Pool(len(chunks)) as pool:
                    parts = pool.map(_compress_job, args)
            finally:
                for v, old in saved.items():
                    if old is None:
                        os.environ.pop(v, None)
                    else:
                        os.environ[v] = old
    for part in parts:
        for s, Ut, Vt, r in part:
            out[s] = (Ut, Vt, r)
    return out


def assemble_panel(nb: int, T: int, acc: float, maxrank: int, tiles: list, updates: list,
                   factors: dict, device: str = "cuda") -> Panel:
    """A Panel over the given tiles (in that order) from tile -> (U^T, V^T,
    rank); factors are uploaded to ``device`` (kept on the host for "cpu")."""
    import torch

    ranks = np.array([factors[t][2] for t in tiles], dtype=np.int32)
    offset = np.zeros(len(tiles) + 1, dtype=np.int64)
    offset[1:] = np.cumsum(ranks.astype(np.int64) * nb)
    Uflat = np.concatenate([factors[t][0].reshape(-1) for t in tiles])
    Vflat = np.concatenate([factors[t][1].reshape(-1) for t in tiles])
    Ut = torch.from_numpy(Uflat)
    Vt = torch.from_numpy(Vflat)
    if device != "cpu":
        Ut, Vt = Ut.to(device), Vt.to(device)
    index = {t: s for s, t in enumerate(tiles)}
    return Panel(nb=nb, ntiles=T, acc=acc, maxrank=maxrank, tiles=list(tiles), rank=ranks,
                 offset=offset, U=Ut, V=Vt, updates=list(updates), index=index)


def build_panel(n_points: int = 65536, dim: int = 2, nb: int = 1024, kernel: str = "sqexp",
                ell: float = 0.01, acc: float = 1e-8, maxrank: int = 128, seed: int = 0,
                device: str = "cuda", max_updates: int | None = None,
                workers: int | None = None) -> Panel:
    """Generate and compress the tiles that panel 0's Schur updates touch.

    Compression runs on the host cores (compress_slots); the factors are then
    uploaded to ``device`` (or kept on the host when device is "cpu")."""
    P, T, tiles, updates = panel_layout(n_points, dim, nb, seed, max_updates)
    comp = compress_slots(P, nb, tiles, range(len(tiles)), kernel, ell, acc, maxrank, seed,
                          workers)
    factors = {tiles[s]: v for s, v in comp.items()}
    return assemble_panel(nb, T, acc, maxrank, tiles, updates, factors, device)


def build_panel_share(rank: int, world: int, all_sum, n_points: int = 65536, dim: int = 2,
                      nb: int = 1024, kernel: str = "sqexp", ell: float = 0.01,
                      acc: float = 1e-8, maxrank: int = 128, seed: int = 0,
                      device: str = "cuda", max_updates: int | None = None,
                      workers: int | None = None):
    """One rank's share of panel 0 for a multi-GPU run, holding only the tiles
    its updates read.

    1. Tile ranks: this rank compresses every world-th tile; `all_sum` (a
       set-up reduction over ranks of an integer numpy vector, e.g. an
       all_reduce) gives every rank all tile ranks.
    2. The updates are partitioned by longest processing time first on the
       per-update cost model (hcore_gb300.shard), the same on every rank.
    3. This rank compresses the tiles its share reads that step 1 did not
       already give it, and keeps only those.
    Returns (Panel of the share, the partition as update-index lists, the
    share's imbalance)."""
    from . import shard as sh

    P, T, tiles, updates = panel_layout(n_points, dim, nb, seed, max_updates)
    own = compress_slots(P, nb, tiles, range(rank, len(tiles), world), kernel, ell, acc,
                         maxrank, seed, workers)
    rk = np.zeros(len(tiles), dtype=np.int64)
    for s, (_, _, r) in own.items():
        rk[s] = r
    rk = np.asarray(all_sum(rk), dtype=np.int64)
    slot = {t: s for s, t in enumerate(tiles)}
    costs = [sh.update_cost(nb, int(rk[slot[(i, 0)]]), int(rk[slot[(j, 0)]]),
                            int(rk[slot[(i, j)]])) for i, j in updates]
    parts = sh.lpt_partition(costs, world)
    mine = [updates[u] for u in parts[rank]]
    need = sh.tiles_read(mine)
    mine_tiles = [t for t in tiles if t in need]
    more = compress_slots(P, nb, tiles, [slot[t] for t in mine_tiles if slot[t] not in own],
                          kernel, ell, acc, maxrank, seed, workers)
    factors = {tiles[s]: v for s, v in own.items() if tiles[s] in need}
    factors.update({tiles[s]: v for s, v in more.items()})
    pnl = assemble_panel(nb, T, acc, maxrank, mine_tiles, mine, factors, device)
    return pnl, parts, sh.imbalance(costs, parts)


def compress_tiles(points: np.ndarray, nb: int, tiles: list, kernel: str, ell: float, acc: float,
                   maxrank: int, seed: int = 0, workers: int | None = None) -> list:
    """Compress the covariance tiles (i, j) of `points` (host spawn pool, one
    single-threaded LAPACK process per core).  Returns, per tile, (U^T, V^T,
    rank) with U^T, V^T of shape (rank, nb) (column-major factors)."""
    import multiprocessing as mp
    import tempfile

    workers = workers or os.cpu_count() or 1
    jobs = [(s, i, j) for s, (i, j) in enumerate(tiles)]
    results = [None] * len(tiles)
    with tempfile.TemporaryDirectory() as folder:
        np.save(os.path.join(folder, "points.npy"), points)
        chunks = [c for c in (jobs[w::workers] for w in range(workers)) if c]
        args = [(folder, c, nb, kernel, ell, acc, maxrank, seed) for c in chunks]
        if len(chunks) <= 1:
            parts = [_compress_job(a) for a in args]
        else:
            saved = {v: os.environ.get(v) for v in ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS")}
            os.environ.update(OPENBLAS_NUM_THREADS="1", OMP_NUM_THREADS="1")
            try:
                with mp.get_context("spawn").Pool(len(chunks)) as pool:
                    parts = pool.map(_compress_job, args)
            finally:
                for v, old in saved.items():
                    if old is None:
                        os.environ.pop(v, None)
                    else:
                        os.environ[v] = old
    for part in parts:
        for s_, Ut, Vt, r in part:
            results[s_] = (Ut, Vt, r)
    return results


class TileStore:
    """Low-rank tiles of a TLR matrix on the device: tile (i, j) -> its
    factors as (U arena, V arena, element offset, rank), column-major nb x
    rank blocks with ld = nb.  Updates replace a tile's entry with the slot
    their new factors were written to."""

    def __init__(self, nb: int, points: np.ndarray, dtype=None, device: str = "cuda"):
        self.nb, self.points, self.device = nb, points, device
        self.dtype = dtype
        self.tiles = {}
        self.norm = {}

    @staticmethod
    def build(points: np.ndarray, nb: int, tiles: list, kernel: str, ell: float, acc: float,
              maxrank: int, seed: int = 0, device: str = "cuda") -> "TileStore":
        import torch

        comp = compress_tiles(points, nb, tiles, kernel, ell, acc, maxrank, seed)
        ranks = np.array([r for _, _, r in comp], dtype=np.int64)
        off = np.zeros(len(tiles) + 1, dtype=np.int64)
        off[1:] = np.cumsum(ranks * nb)
        U = torch.from_numpy(np.concatenate([u.reshape(-1) for u, _, _ in comp]))
        V = torch.from_numpy(np.concatenate([v.reshape(-1) for _, v, _ in comp]))
        if device != "cpu":
            U, V = U.to(device), V.to(device)
        st = TileStore(nb, points, dtype=U.dtype, device=device)
        for s_, t in enumerate(tiles):
            st.tiles[t] = (U, V, int(off[s_]), int(ranks[s_]))
            st.norm[t] = float(np.linalg.norm(comp[s_][1]))   # ||U V^T||_F = ||V||_F
        return st

    def ptrs(self, t):
        U, V, o, r = self.tiles[t]
        e = U.element_size()
        return U.data_ptr() + e * o, V.data_ptr() + e * o, r

    def factors(self, t):
        """(U, V) of tile t as host Fortran arrays (nb x rank)."""
        U, V, o, r = self.tiles[t]
        n = self.nb * r
        u = U[o:o + n].cpu().numpy().reshape(r, self.nb).T
        v = V[o:o + n].cpu().numpy().reshape(r, self.nb).T
        return np.asfortranarray(u), np.asfortranarray(v)


def update_flops(M: int, a: int, b: int, c: int, r: int) -> int:
    """Reference flop model of one HCORE_dgemm update (flop_counts.c:3-70 as
    accumulated at hcore_dgemm.c:125,179,208,224,434,493,595,666)."""
    k = a + c

    def q(m, n):
        return 2 * m * n * n - int(np.float32(2 * n * n * n) / np.float32(3.0)) + 2 * m * n + \
            int(np.float32(17 * n) / np.float32(3.0))

    o1 = 4 * r * M * k - 2 * r * k * k + 3 * r * k
    o2 = 4 * M * r * k - 2 * r * k * k + 2 * r * k + M * k - k * k // 2 + k // 2
    return 2 * q(M, k) + 2 * a * b * M + 2 * M * a * b + 22 * k ** 3 + r * k + o1 + o2


def phase_flops(M: int, a: int, b: int, c: int, r: int) -> dict:
    """The same model split by the four GPU phases."""
    k = a + c

    def q(m, n):
        return 2 * m * n * n - int(np.float32(2 * n * n * n) / np.float32(3.0)) + 2 * m * n + \
            int(np.float32(17 * n) / np.float32(3.0))

    o1 = 4 * r * M * k - 2 * r * k * k + 3 * r * k
    o2 = 4 * M * r * k - 2 * r * k * k + 2 * r * k + M * k - k * k // 2 + k // 2
    return {"stack": 4 * a * b * M, "qr": 2 * q(M, k), "svd": 22 * k ** 3 + r * k,
            "rebuild": o1 + o2}
