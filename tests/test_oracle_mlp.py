"""The network oracle on the CPU: backward formulas against finite differences, BF16 rounding
against torch's conversion."""

import numpy as np
import torch

from oracle import mlp_oracle as MO


def _params(rng, n_in, n_h):
    return {"W1": rng.normal(size=(n_h, n_in)) * 0.5, "b1": rng.normal(size=n_h) * 0.1,
            "W2": rng.normal(size=(n_h, n_h)) * 0.5, "b2": rng.normal(size=n_h) * 0.1,
            "w3": rng.normal(size=n_h) * 0.5, "b3": np.array([0.3])}


def test_float64_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    p = _params(rng, 12, 7)
    X = (rng.random((9, 12)) < 0.4).astype(float)
    t = rng.normal(size=9)
    g = MO.float64_grads(X, t, p)
    h = 1e-6
    for name in p:
        flat = p[name].reshape(-1)
        for k in range(flat.size):
            old = flat[k]
            flat[k] = old + h
            lp = MO.float64_loss(X, t, p)
            flat[k] = old - h
            lm = MO.float64_loss(X, t, p)
            flat[k] = old
            assert abs((lp - lm) / (2 * h) - g[name].reshape(-1)[k]) < 1e-6 * (1 + abs(g[name].reshape(-1)[k]))


def test_bf16_rounding_matches_torch():
    rng = np.random.default_rng(1)
    x = np.concatenate([rng.normal(size=5000) * 10.0 ** rng.integers(-6, 6, size=5000), [0.0, -0.0, 1.0, -3.5]])
    ref = torch.from_numpy(x.astype(np.float32)).to(torch.bfloat16).to(torch.float64).numpy()
    assert np.array_equal(MO.bf16(x), ref)


def test_bits_layout():
    w = np.array([[np.uint64(1) << np.uint64(63), np.uint64(1)]], dtype=np.uint64)
    b = MO.bits(w, 130)
    assert b[0, 0] == 1 and b[0, 127] == 1 and b.sum() == 2
