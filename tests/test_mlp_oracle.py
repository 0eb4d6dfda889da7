"""CPU checks of the rank-predictor MLP's oracle (oracle/mlp.py): its
backward against central finite differences of its own forward (FP64, no
BF16 rounding), the BF16 rounding rule, and the parameter layout against the
C header."""
import re

import numpy as np

from oracle import mlp as M


def _rand_params(rng, scale=0.3):
    return (rng.standard_normal(M.NPARAMS) * scale).astype(np.float64)


def test_parameter_count_matches_header():
    src = open("include/hcore_gb300.h").read()
    m = re.search(r"#define HCORE_MLP_PARAMS \(([^)]*)\)", src)
    assert m and eval(m.group(1)) == M.NPARAMS == 4673


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = _rand_params(rng)
    X = rng.standard_normal((37, M.IN))
    T = rng.standard_normal(37)
    loss, g = M.loss_and_grad(p, X, T, bf16=False, dtype=np.float64)
    idx = np.concatenate([rng.choice(M.NPARAMS, 60, replace=False),
                          [M.OFFSETS["b3"][0], M.OFFSETS["W1"][0], M.OFFSETS["w3"][0] + 5]])
    h = 1e-6
    for i in idx:
        e = np.zeros(M.NPARAMS)
        e[i] = h
        lp, _ = M.loss_and_grad(p + e, X, T, bf16=False, dtype=np.float64)
        lm, _ = M.loss_and_grad(p - e, X, T, bf16=False, dtype=np.float64)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])


def test_bf16_round_to_nearest_even():
    # exactly representable values stay, halfway cases go to the even neighbour
    x = np.array([1.0, -2.5, 2.0 ** 127, 1.0 + 2 ** -7], dtype=np.float32)
    assert np.array_equal(M.bf16_round(x), x)
    half_up = np.float32(1.0 + 2 ** -8)            # halfway between 1 and 1 + 2^-7
    assert M.bf16_round(np.array([half_up]))[0] == np.float32(1.0)
    half_odd = np.float32(1.0 + 3 * 2 ** -8)       # halfway between 1+2^-7 (odd) and 1+2^-6
    assert M.bf16_round(np.array([half_odd]))[0] == np.float32(1.0 + 2 ** -6)
    r = M.bf16_round(np.random.default_rng(1).standard_normal(1000).astype(np.float32))
    assert np.all((r.view(np.uint32) & 0xFFFF) == 0)


def test_adam_first_step_moves_by_lr():
    # first step: m_hat = g, v_hat = g^2, so each parameter moves by ~lr * sign(g)
    rng = np.random.default_rng(2)
    p = rng.standard_normal(50).astype(np.float32)
    g = rng.standard_normal(50).astype(np.float32)
    p2, m, v = M.adam_step(p, g, np.zeros(50), np.zeros(50), 1, 1e-3)
    assert np.allclose(p - p2, 1e-3 * np.sign(g), rtol=1e-4)
