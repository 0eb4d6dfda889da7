"""CPU oracle of the rank-predictor MLP (test infrastructure only).

The reference has no learned component; this restates the network that the
library's CUDA kernels train and run (hcore_gb300/csrc/hc_mlp.cu), so that
their forward pass, gradients and Adam steps can be checked on the CPU:

* 6 -> 64 -> 64 -> 1, ReLU, FP32 parameters in one array
  (W1[6][64] in x out, b1[64], W2[64][64], b2[64], w3[64], b3);
* activations h1, h2 rounded to BF16 (round to nearest even);
* every forward sum taken in input order with separately rounded FP32
  products and additions, as the kernels do, so ``forward`` is bit-exact;
* loss mean(0.5 (y - t)^2); the backward treats the BF16 rounding as the
  identity (straight-through), as the kernels do;
* Adam with beta1 0.9, beta2 0.999, eps 1e-8.

``grad`` accumulates in FP64 from the FP32 forward values: the GPU's FP32
sums (in another order, with atomics across CTAs) are compared to it with a
tolerance.  With ``bf16=False, dtype=np.float64`` the same code is a plain
FP64 network, which the tests check against finite differences.
"""
from __future__ import annotations

import numpy as np

IN, HID = 6, 64
_SHAPES = [("W1", (IN, HID)), ("b1", (HID,)), ("W2", (HID, HID)), ("b2", (HID,)),
           ("w3", (HID,)), ("b3", (1,))]
OFFSETS = {}
_o = 0
for _name, _shape in _SHAPES:
    OFFSETS[_name] = (_o, _shape)
    _o += int(np.prod(_shape))
NPARAMS = _o   # 4673


def unpack(p: np.ndarray) -> dict:
    return {k: p[o:o + int(np.prod(s))].reshape(s) for k, (o, s) in OFFSETS.items()}


def bf16_round(x: np.ndarray) -> np.ndarray:
    """FP32 -> BF16 -> FP32, round to nearest even (finite inputs)."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def forward(p: np.ndarray, X: np.ndarray, bf16: bool = True, dtype=np.float32):
    """Returns y (n,) and the intermediates (z1, h1, z2, h2)."""
    P = {k: v.astype(dtype) for k, v in unpack(np.asarray(p)).items()}
    X = np.asarray(X, dtype=dtype)
    n = X.shape[0]
    rnd = bf16_round if bf16 else (lambda a: a)
    z1 = np.broadcast_to(P["b1"], (n, HID)).copy()
    for i in range(IN):                       # input order, no fused multiply-add
        z1 = z1 + X[:, i:i + 1] * P["W1"][i]
    h1 = rnd(np.maximum(z1, 0))
    z2 = np.broadcast_to(P["b2"], (n, HID)).copy()
    for i in range(HID):
        z2 = z2 + h1[:, i:i + 1] * P["W2"][i]
    h2 = rnd(np.maximum(z2, 0))
    y = np.full(n, P["b3"][0], dtype=dtype)
    for j in range(HID):
        y = y + h2[:, j] * P["w3"][j]
    return y, (z1, h1, z2, h2)


def loss_and_grad(p: np.ndarray, X: np.ndarray, T: np.ndarray, bf16: bool = True,
                  dtype=np.float32):
    """Mean loss 0.5 (y - t)^2 and its gradient (FP64, NPARAMS)."""
    y, (z1, h1, z2, h2) = forward(p, X, bf16, dtype)
    P = {k: v.astype(np.float64) for k, v in unpack(np.asarray(p)).items()}
    X64, h1, h2 = (np.asarray(a, dtype=np.float64) for a in (X, h1, h2))
    n = X64.shape[0]
    e = y.astype(np.float64) - np.asarray(T, dtype=np.float64)
    loss = 0.5 * float(np.mean(e * e))
    dy = e / n
    g = {}
    g["w3"] = h2.T @ dy
    g["b3"] = np.array([dy.sum()])
    dz2 = (dy[:, None] * P["w3"][None, :]) * (z2 > 0)
    g["W2"] = h1.T @ dz2
    g["b2"] = dz2.sum(0)
    dz1 = (dz2 @ P["W2"].T) * (z1 > 0)
    g["W1"] = X64.T @ dz1
    g["b1"] = dz1.sum(0)
    out = np.zeros(NPARAMS)
    for k, (o, s) in OFFSETS.items():
        out[o:o + int(np.prod(s))] = g[k].reshape(-1)
    return loss, out


def adam_step(p, g, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam update (step counts from 1); returns new (p, m, v) in FP32."""
    p, g, m, v = (np.asarray(a, dtype=np.float32) for a in (p, g, m, v))
    m = np.float32(b1) * m + np.float32(1 - b1) * g
    v = np.float32(b2) * v + np.float32(1 - b2) * g * g
    c1 = np.float32(1.0 / (1.0 - b1 ** step))
    c2 = np.float32(1.0 / (1.0 - b2 ** step))
    p = p - np.float32(lr) * (m * c1) / (np.sqrt(v * c2) + np.float32(eps))
    return p, m, v
