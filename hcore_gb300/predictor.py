"""Learned output-rank predictor for batched recompression.

Before a batch of Schur updates C_ij <- C_ij - A_ik A_jk^T runs, each
update's new rank is unknown: it is decided by the SVD inside the batch.  A
batch that must hold its outputs (new tiles written to plan-owned slots,
workspace, launch shape) without knowing them pads every update to maxrank.
This module predicts each rank from cheap features with the library's MLP
(hcore_gpu_mlp_*, trained by the library's own CUDA kernels on ranks the
method itself produced), sizes every update's output slot to the predicted
capacity, and passes that capacity to the plan as the task's
storage_maxrank (the plan then also sizes its rebuild grid by the largest
capacity).  The SVD still decides every rank: an update whose rank exceeds its
capacity is reported with HCORE_GPU_S_STORAGE (its slot untouched) and is
rebuilt from the plan's workspace into an overflow slot of exactly its rank
(only the rebuild phase runs again).

Features of update (i, j) of panel k, with A = tile (i, k), B = (j, k),
C = (i, j) and tile norms ||X||_F = ||V_X||_F (U orthonormal):
  log2(1 + a), log2(1 + b), log2(1 + c),
  log10(||A|| ||B|| / acc), log10(||C|| / acc),
  log2(1 + dist(cluster i, cluster j) / cluster diameter)
Target: log2(1 + new rank).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

NFEAT = 6


def cluster_geometry(points: np.ndarray, nb: int):
    """Centre and diameter (bounding-box diagonal) of each block of nb points."""
    T = points.shape[0] // nb
    P = points[:T * nb].reshape(T, nb, -1)
    lo, hi = P.min(1), P.max(1)
    return (lo + hi) / 2, np.linalg.norm(hi - lo, axis=1)


def features(a, b, c, normA, normB, normC, dist, diam, acc) -> np.ndarray:
    """(n, 6) float32 feature matrix; all arguments are arrays of length n
    (acc may be a scalar)."""
    a, b, c = (np.asarray(x, dtype=np.float64) for x in (a, b, c))
    tiny = 1e-300
    acc = np.broadcast_to(np.asarray(acc, dtype=np.float64), a.shape)
    F = np.stack([np.log2(1 + a), np.log2(1 + b), np.log2(1 + c),
                  np.log10(np.maximum(np.asarray(normA) * np.asarray(normB), tiny) / acc),
                  np.log10(np.maximum(np.asarray(normC), tiny) / acc),
                  np.log2(1 + np.asarray(dist) / np.maximum(np.asarray(diam), tiny))], axis=1)
    return F.astype(np.float32)


def rank_target(r) -> np.ndarray:
    return np.log2(1 + np.asarray(r, dtype=np.float64)).astype(np.float32)


def rank_from_output(y) -> np.ndarray:
    return np.exp2(np.asarray(y, dtype=np.float64)) - 1


@dataclass
class CapacityPolicy:
    """capacity = clip(ceil(pred * (1 + margin)) + slack, 1, maxrank)."""

    margin: float = 0.15
    slack: int = 4

    def __call__(self, pred: np.ndarray, maxrank: int) -> np.ndarray:
        cap = np.ceil(np.maximum(pred, 0) * (1 + self.margin)) + self.slack
        return np.clip(cap, 1, maxrank).astype(np.int64)

    @staticmethod
    def fit(pred: np.ndarray, actual: np.ndarray, target_overflow: float = 0.02,
            slack: int = 4) -> "CapacityPolicy":
        """Smallest margin (on a grid) whose overflow rate on (pred, actual)
        is at most target_overflow."""
        pred, actual = np.asarray(pred, float), np.asarray(actual, float)
        for m in np.arange(0.0, 3.01, 0.05):
            cap = np.ceil(np.maximum(pred, 0) * (1 + m)) + slack
            if np.mean(actual > cap) <= target_overflow:
                return CapacityPolicy(margin=float(m), slack=slack)
        return CapacityPolicy(margin=3.0, slack=slack)


class RankPredictor:
    """Feature standardisation + the library MLP (trained on the GPU)."""

    def __init__(self, seed: int = 0):
        import hcore_gb300 as hc

        self.net = hc.RankMLP(seed=seed)
        self.mu = np.zeros(NFEAT, np.float32)
        self.sd = np.ones(NFEAT, np.float32)

    def _x(self, F):
        import torch

        Z = ((np.asarray(F, np.float32) - self.mu) / self.sd).astype(np.float32)
        return torch.from_numpy(np.ascontiguousarray(Z)).cuda()

    def fit(self, F, ranks, epochs: int = 200, batch: int = 256, lr: float = 2e-3, seed: int = 0):
        import torch

        F = np.asarray(F, np.float32)
        self.mu = F.mean(0)
        self.sd = np.maximum(F.std(0), 1e-3).astype(np.float32)
        T = torch.from_numpy(rank_target(ranks)).cuda()
        return self.net.train(self._x(F), T, epochs=epochs, batch=batch, lr=lr, seed=seed)

    def predict(self, F) -> np.ndarray:
        if len(F) == 0:
            return np.zeros(0)
        return rank_from_output(self.net.predict(self._x(F)).cpu().numpy())

    def state(self) -> dict:
        return {"params": self.net.get_params(), "mu": self.mu, "sd": self.sd}

    def load(self, st: dict) -> None:
        self.net.set_params(st["params"])
        self.mu, self.sd = np.asarray(st["mu"], np.float32), np.asarray(st["sd"], np.float32)


def slot_offsets(cols: np.ndarray, nb: int) -> np.ndarray:
    """Element offsets of consecutive output slots of nb x cols[u] each."""
    off = np.zeros(len(cols) + 1, dtype=np.int64)
    off[1:] = np.cumsum(np.asarray(cols, np.int64) * nb)
    return off


def run_capacity_batch(hc, make_task, n: int, nb: int, caps: np.ndarray, maxrank: int,
                       dtype=None, device="cuda", precision=0, flags=0):
    """Run n updates with per-update output capacities `caps`; updates whose
    new rank exceeds their capacity (but not maxrank) are then rebuilt from
    the plan's workspace into overflow slots of exactly their rank
    (hcore_gpu_plan_rebuild: the rebuild phase only, no recompression).

    make_task(u, storage, CUo_ptr, CVo_ptr) -> LrTask for update u.
    Returns dict(ranks, status, where) where where[u] = (U arena, V arena,
    element offset) of update u's new factors, plus bytes and counts."""
    import torch

    dtype = dtype or torch.float64
    caps = np.asarray(caps, np.int64)
    off = slot_offsets(caps, nb)
    oU = torch.empty(int(off[-1]) + 1, dtype=dtype, device=device)
    oV = torch.empty_like(oU)
    esz = oU.element_size()
    tasks = [make_task(u, int(caps[u]), oU.data_ptr() + esz * int(off[u]),
                       oV.data_ptr() + esz * int(off[u])) for u in range(n)]
    batch = hc.Batch(tasks, precision=precision, flags=flags)
    batch.execute()
    ranks, status = batch.results()
    where = [(oU, oV, int(off[u])) for u in range(n)]
    over = np.nonzero((status == 5) & (ranks <= maxrank) & (caps < maxrank))[0]   # STORAGE
    arena_bytes = 2 * oU.numel() * esz
    if len(over):
        off2 = slot_offsets(ranks[over], nb)
        xU = torch.empty(int(off2[-1]) + 1, dtype=dtype, device=device)
        xV = torch.empty_like(xU)
        batch.rebuild(over, [xU.data_ptr() + esz * int(off2[q]) for q in range(len(over))],
                      [xV.data_ptr() + esz * int(off2[q]) for q in range(len(over))],
                      [nb] * len(over))
        ranks, status = batch.results()
        for q, u in enumerate(over):
            where[u] = (xU, xV, int(off2[q]))
        arena_bytes += 2 * xU.numel() * esz
    ws_bytes = batch.workspace_bytes
    batch.close()
    return dict(ranks=ranks, status=status, where=where, overflow=len(over),
                arena_bytes=arena_bytes, workspace_bytes=ws_bytes)
