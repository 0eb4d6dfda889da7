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
runs once, on the GPU through torch (randomized range finder + small SVD).
"""
from __future__ import annotations

import math
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


def _kernel(X, Y, kind: str, ell: float):
    import torch

    d2 = (X * X).sum(-1)[..., :, None] + (Y * Y).sum(-1)[..., None, :] - 2.0 * X @ Y.transpose(-1, -2)
    d2 = torch.clamp(d2, min=0.0)
    if kind == "sqexp":
        return torch.exp(-d2 / ell)
    if kind == "exp":
        return torch.exp(-torch.sqrt(d2) / ell)
    raise ValueError(kind)


def compress_tiles(K, acc: float, maxrank: int, seed: int, oversample: int = 32):
    """Randomized compression of a batch of nb x nb tiles (torch, fp64, GPU).

    Returns (U, V, ranks) with U, V of shape (batch, nb, p) whose first
    ranks[t] columns are the factors (U orthonormal, V = (S V^T)^T)."""
    import torch

    T, nb, _ = K.shape
    p = min(nb, maxrank + oversample)
    g = torch.Generator(device=K.device)
    g.manual_seed(seed)
    omega = torch.randn((nb, p), generator=g, dtype=K.dtype, device=K.device)
    Y = K @ omega
    Q, _ = torch.linalg.qr(Y)
    B = Q.transpose(-1, -2) @ K
    Ub, S, Vh = torch.linalg.svd(B, full_matrices=False)
    U = Q @ Ub
    thr = acc * S[:, :1]
    ranks = torch.clamp((S >= thr).sum(-1), max=maxrank)
    V = (S[:, :, None] * Vh).transpose(-1, -2)
    return U, V, ranks


def build_panel(n_points: int = 65536, dim: int = 2, nb: int = 1024, kernel: str = "sqexp",
                ell: float = 0.01, acc: float = 1e-8, maxrank: int = 128, seed: int = 0,
                device: str = "cuda", batch: int = 32, max_updates: int | None = None) -> Panel:
    """Generate and compress the tiles that panel 0's Schur updates touch."""
    import torch

    T = n_points // nb
    P = torch.from_numpy(morton_points(n_points, dim, seed)).to(device)
    tiles = [(i, 0) for i in range(1, T)]
    updates = [(i, j) for j in range(1, T) for i in range(j + 1, T)]
    if max_updates is not None:
        updates = updates[:max_updates]
    need_c = sorted({u for u in updates})
    tiles += need_c
    index = {t: s for s, t in enumerate(tiles)}
    ranks = np.zeros(len(tiles), dtype=np.int32)
    Us, Vs = [], []
    for s0 in range(0, len(tiles), batch):
        chunk = tiles[s0:s0 + batch]
        X = torch.stack([P[i * nb:(i + 1) * nb] for i, _ in chunk])
        Yp = torch.stack([P[j * nb:(j + 1) * nb] for _, j in chunk])
        K = _kernel(X, Yp, kernel, ell)
        U, V, r = compress_tiles(K, acc, maxrank, seed + s0)
        r = r.cpu().numpy()
        ranks[s0:s0 + len(chunk)] = r
        for t in range(len(chunk)):
            Us.append(U[t, :, :r[t]].transpose(0, 1).contiguous())   # (r, nb): column-major
            Vs.append(V[t, :, :r[t]].transpose(0, 1).contiguous())
        del K, U, V
    offset = np.zeros(len(tiles) + 1, dtype=np.int64)
    offset[1:] = np.cumsum(ranks.astype(np.int64) * nb)
    Uflat = torch.cat([u.reshape(-1) for u in Us]) if Us else torch.zeros(1, device=device)
    Vflat = torch.cat([v.reshape(-1) for v in Vs]) if Vs else torch.zeros(1, device=device)
    return Panel(nb=nb, ntiles=T, acc=acc, maxrank=maxrank, tiles=tiles, rank=ranks,
                 offset=offset, U=Uflat, V=Vflat, updates=updates, index=index)


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
