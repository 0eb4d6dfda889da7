"""Column-major device buffers for the C ABI, held in torch CUDA tensors.

torch supplies device memory and streams only; all arithmetic runs in the
library's own kernels.  A column-major (ld x ncols) matrix is stored as a
row-major torch tensor of shape (ncols, ld), so ``tensor.data_ptr()`` is the
address the C ABI expects and column j is ``tensor[j]``.
"""
from __future__ import annotations

import numpy as np


def to_device(a: np.ndarray, ncols: int | None = None, device="cuda"):
    """Copy a column-major numpy matrix (ld x n) to a (ncols x ld) CUDA tensor
    (ncols >= n; extra columns are zero)."""
    import torch

    a = np.asarray(a)
    ld, n = a.shape
    ncols = max(ncols or n, 1)
    t = torch.zeros((ncols, ld), dtype=torch.float64 if a.dtype == np.float64 else torch.float32,
                    device=device)
    if n:
        t[:n] = torch.from_numpy(np.ascontiguousarray(a.T)).to(device)
    return t


def to_host(t, ncols: int) -> np.ndarray:
    """First ncols columns of a device matrix as a Fortran-ordered numpy array."""
    return np.asfortranarray(t[:ncols].cpu().numpy().T)
