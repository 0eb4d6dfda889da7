"""GPU checks of the rank-predictor MLP kernels (hcore_gpu_mlp_*) against
the CPU oracle (oracle/mlp.py) on the same parameters and samples:

* forward (hcore_gpu_mlp_predict): bit-exact (same FP32 operation order,
  same BF16 rounding);
* gradient: FP32 sums with atomics vs the oracle's FP64 sums of the same
  activations, relative error per parameter block <= 1e-4;
* one full-batch Adam step: parameters within 1e-5 (relative) of the
  oracle's Adam step taken from the GPU gradient;
* training on a smooth synthetic target lowers the loss 10x.
"""
import numpy as np
import pytest

from oracle import mlp as M

pytestmark = pytest.mark.gpu


def _data(rng, n):
    X = rng.standard_normal((n, M.IN)).astype(np.float32)
    T = (np.sin(X[:, 0]) + 0.5 * X[:, 1] * X[:, 2] - 0.3 * np.abs(X[:, 3])).astype(np.float32)
    return X, T


def _dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_forward_bit_exact(hc):
    rng = np.random.default_rng(3)
    net = hc.RankMLP(seed=7)
    X, _ = _data(rng, 1000)
    y = net.predict(_dev(X)).cpu().numpy()
    y_ref, _ = M.forward(net.get_params(), X)
    assert np.array_equal(y, y_ref)


@pytest.mark.parametrize("n", [1, 127, 1000])
def test_gradient_vs_oracle(hc, n):
    rng = np.random.default_rng(4 + n)
    net = hc.RankMLP(seed=11)
    X, T = _data(rng, n)
    loss, g = net.gradient(_dev(X), _dev(T))
    loss_ref, g_ref = M.loss_and_grad(net.get_params(), X, T)
    assert abs(loss - loss_ref) <= 1e-5 * max(loss_ref, 1e-30)
    for name, (o, shape) in M.OFFSETS.items():
        sz = int(np.prod(shape))
        a, b = g[o:o + sz], g_ref[o:o + sz]
        assert np.linalg.norm(a - b) <= 1e-4 * max(np.linalg.norm(b), 1e-30), name


def test_adam_step_vs_oracle(hc):
    rng = np.random.default_rng(5)
    net = hc.RankMLP(seed=13)
    X, T = _data(rng, 512)
    p0 = net.get_params()
    _, g = net.gradient(_dev(X), _dev(T))
    net.train(_dev(X), _dev(T), epochs=1, batch=512, lr=1e-3)   # one full-batch step
    p_ref, _, _ = M.adam_step(p0, g, np.zeros_like(p0), np.zeros_like(p0), 1, 1e-3)
    p1 = net.get_params()
    assert np.abs(p1 - p_ref).max() <= 1e-5 * max(np.abs(p_ref).max(), 1.0)


def test_training_lowers_loss(hc):
    rng = np.random.default_rng(6)
    net = hc.RankMLP(seed=17)
    X, T = _data(rng, 8192)
    Xd, Td = _dev(X), _dev(T)
    l0, _ = net.gradient(Xd, Td)
    losses = net.train(Xd, Td, epochs=60, batch=256, lr=2e-3, seed=1)
    l1, _ = net.gradient(Xd, Td)
    assert losses[-1] < losses[0]
    assert l1 < 0.1 * l0
    y = net.predict(Xd).cpu().numpy()
    y_ref, _ = M.forward(net.get_params(), X)
    assert np.array_equal(y, y_ref)
