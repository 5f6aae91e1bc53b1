"""CPU oracle of the basis-pruning network (test infrastructure only; never imported by the
product).  The network has no upstream counterpart: upstream impurityModel keeps every state
of a basis expansion (impurityModel/ed/finite.py:1696-1803).

It mirrors the device arithmetic: BF16 operands (input bits, weights, hidden activations and
their gradients rounded to BF16 at the same points as the device kernels), sums in float64
(the device accumulates in FP32), ReLU hidden layers, a linear output and a mean-squared-error
loss.  ``float64_grads`` is the same network without any rounding, used to pin the
backward formulas against finite differences.
"""

import numpy as np


def bf16(x):
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    f = np.asarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return (u.astype(np.uint32)).view(np.float32).astype(np.float64)


def bits(states_words, n_in):
    """[B, W] uint64 words -> [B, n_in] occupations (spin-orbital i at bit 63 - i%64 of word i/64)."""
    w = np.asarray(states_words, dtype=np.uint64)
    out = np.zeros((w.shape[0], n_in))
    for i in range(n_in):
        q = i // 64
        if q < w.shape[1]:
            out[:, i] = ((w[:, q] >> np.uint64(63 - i % 64)) & np.uint64(1)).astype(np.float64)
    return out


def forward(X, p):
    """y and the cached activations, rounding as the device kernels do."""
    W1b, W2b = bf16(p["W1"]), bf16(p["W2"])
    H1 = bf16(np.maximum(X @ W1b.T + p["b1"], 0.0))
    H2 = bf16(np.maximum(H1 @ W2b.T + p["b2"], 0.0))
    y = H2 @ p["w3"] + p["b3"][0]
    return y, (W1b, W2b, H1, H2)


def grads(X, t, p):
    """Loss and gradients of the mean squared error, BF16 rounding of the deltas as on the device."""
    y, (W1b, W2b, H1, H2) = forward(X, p)
    B = X.shape[0]
    dy = 2.0 * (y - t) / B
    dH2 = bf16(dy[:, None] * p["w3"][None, :] * (H2 > 0))
    dH1 = bf16((dH2 @ W2b) * (H1 > 0))
    g = {
        "w3": H2.T @ dy,
        "b3": np.array([dy.sum()]),
        "W2": dH2.T @ H1,
        "b2": dH2.sum(0),
        "W1": dH1.T @ X,
        "b1": dH1.sum(0),
    }
    return float(np.mean((y - t) ** 2)), g


def float64_loss(X, t, p):
    H1 = np.maximum(X @ p["W1"].T + p["b1"], 0.0)
    H2 = np.maximum(H1 @ p["W2"].T + p["b2"], 0.0)
    y = H2 @ p["w3"] + p["b3"][0]
    return float(np.mean((y - t) ** 2))


def float64_grads(X, t, p):
    """Exact gradients of float64_loss (the formulas of ``grads`` without rounding)."""
    H1 = np.maximum(X @ p["W1"].T + p["b1"], 0.0)
    H2 = np.maximum(H1 @ p["W2"].T + p["b2"], 0.0)
    y = H2 @ p["w3"] + p["b3"][0]
    B = X.shape[0]
    dy = 2.0 * (y - t) / B
    dH2 = dy[:, None] * p["w3"][None, :] * (H2 > 0)
    dH1 = (dH2 @ p["W2"]) * (H1 > 0)
    return {"w3": H2.T @ dy, "b3": np.array([dy.sum()]), "W2": dH2.T @ H1, "b2": dH2.sum(0), "W1": dH1.T @ X,
            "b1": dH1.sum(0)}
