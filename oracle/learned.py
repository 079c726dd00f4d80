"""CPU oracle of the learned index (test infrastructure only: the tests compare the GPU kernels
with it; nothing in the product calls it).

The learned index has no counterpart in the reference; what is restated here is its
mathematics, in float64, so that the GPU kernels can be checked against it:

* ``mlp_forward`` / ``mlp_backward`` -- the per-segment network y = b2 + sum_j w2_j relu(w1_j x +
  b1_j) and the gradient of sum_i dy_i y_i with respect to (w1, b1, w2, b2), written from the
  chain rule; ``finite_difference`` pins the analytic gradient numerically.
* ``row_keys`` / ``distinct_keys`` -- the 16-base key of every suffix-array row (2 bits a base,
  A=0..T=3, first base in the top bits, bases past the end of the read = 0) and the first row of
  each distinct key, from the reads and a suffix array (the reference's text: the reads, or every
  read reversed, src/index.c:558-585).
"""
from __future__ import annotations

import numpy as np

HIDDEN = 64
STRIDE = 196
KEY_BASES = 16


def unpack(params: np.ndarray):
    p = np.asarray(params, np.float64)
    H = HIDDEN
    return p[:H], p[H:2 * H], p[2 * H:3 * H], p[3 * H]


def mlp_forward(params: np.ndarray, x: np.ndarray) -> np.ndarray:
    w1, b1, w2, b2 = unpack(params)
    a = np.outer(np.asarray(x, np.float64), w1) + b1
    return np.maximum(a, 0.0) @ w2 + b2


def mlp_backward(params: np.ndarray, x: np.ndarray, dy: np.ndarray) -> np.ndarray:
    """d/d(w1, b1, w2, b2) of sum_i dy_i * y_i, 193 values."""
    w1, b1, w2, _ = unpack(params)
    x = np.asarray(x, np.float64)
    dy = np.asarray(dy, np.float64)
    a = np.outer(x, w1) + b1
    h = np.maximum(a, 0.0)
    on = (a > 0.0).astype(np.float64)
    dz = (dy[:, None] * w2[None, :]) * on            # d/da
    g_w2 = h.T @ dy
    g_w1 = dz.T @ x
    g_b1 = dz.sum(0)
    g_b2 = dy.sum()
    return np.concatenate([g_w1, g_b1, g_w2, [g_b2]])


def adam_step(params: np.ndarray, m1: np.ndarray, m2: np.ndarray, x: np.ndarray, target: np.ndarray,
              step: int, lr: float):
    """One step of the learned index's joint training phase in float64: gradient of the mean squared
    error sum_i (mlp(x_i) - target_i)^2 / n, then Adam (beta1 0.9, beta2 0.999, eps 1e-8, bias
    correction for step number `step`) on the 193 parameters.  Returns (params, m1, m2)."""
    p = np.asarray(params, np.float64).copy()
    n = len(x)
    y = mlp_forward(p, x)
    dy = 2.0 * (y - np.asarray(target, np.float64)) / n
    g = mlp_backward(p, x, dy)
    k = 3 * HIDDEN + 1
    a = 0.9 * np.asarray(m1, np.float64)[:k] + 0.1 * g
    b = 0.999 * np.asarray(m2, np.float64)[:k] + 0.001 * g * g
    mh = a / (1.0 - 0.9 ** step)
    vh = b / (1.0 - 0.999 ** step)
    p[:k] -= lr * mh / (np.sqrt(vh) + 1e-8)
    return p, a, b


def finite_difference(params: np.ndarray, x: np.ndarray, dy: np.ndarray, eps: float = 1e-6) -> np.ndarray:
    """Central differences of sum_i dy_i * mlp(x_i) with respect to the 193 parameters."""
    p = np.asarray(params, np.float64).copy()
    g = np.empty(3 * HIDDEN + 1)
    dy = np.asarray(dy, np.float64)
    for k in range(3 * HIDDEN + 1):
        old = p[k]
        p[k] = old + eps
        fp = float(dy @ mlp_forward(p, x))
        p[k] = old - eps
        fm = float(dy @ mlp_forward(p, x))
        p[k] = old
        g[k] = (fp - fm) / (2 * eps)
    return g


def text_of(reads: np.ndarray, direction: int) -> np.ndarray:
    """The indexed text of one direction: the reads (0) or every read reversed (1), codes 1..4."""
    r = np.asarray(reads, np.uint8)
    return (r if direction == 0 else r[:, ::-1]).reshape(-1)


def row_keys(reads: np.ndarray, sa: np.ndarray, direction: int) -> np.ndarray:
    """key16 of every suffix-array row."""
    L = reads.shape[1]
    text = text_of(reads, direction).astype(np.int64)
    n = len(text)
    p = np.asarray(sa, np.int64)
    m = L - p % L                                        # bases to the end of the read
    key = np.zeros(len(p), np.uint64)
    for j in range(KEY_BASES):
        c = np.where(j < m, text[np.minimum(p + j, n - 1)] - 1, 0).astype(np.uint64)
        key = (key << np.uint64(2)) | c
    return key.astype(np.uint32)


def distinct_keys(reads: np.ndarray, sa: np.ndarray, direction: int):
    """(distinct keys, first row of each) in suffix-array order."""
    k = row_keys(reads, sa, direction)
    head = np.ones(len(k), bool)
    head[1:] = k[1:] != k[:-1]
    rows = np.nonzero(head)[0]
    return k[rows], rows
