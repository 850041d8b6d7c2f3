"""CPU oracle of the subgrid-stress network (test infrastructure only).

The reference has no closure, so there is no reference function to follow:
this is the network's own definition (10 -> 64 -> 64 -> 64 -> 6, SiLU,
mean-squared loss in normalised units, Adam) in numpy FP64, with the BF16
roundings of the tensor-core path made at the same points when
``bf16=True``: the normalised inputs, the weights, every hidden activation
and every backward operand are rounded to BF16 (round to nearest even)
before they enter a product; products and sums are exact FP64 here and FP32
on the GPU.  ``bf16=False`` is the plain FP64 network, against which the
finite-difference check of the gradient runs.

Parameter vector: the order of include/chgpu_closure.h (W1[64][16] with the
bias in column 10, W2, b2, W3, b3, W4[6][64], b4).  Used only by tests/.
"""
from __future__ import annotations

import numpy as np

NIN, NH, NOUT = 10, 64, 6
OFF_W1, OFF_W2, OFF_B2, OFF_W3, OFF_B3, OFF_W4, OFF_B4 = 0, 1024, 5120, 5184, 9280, 9344, 9728
NPARAMS = 9734


def bf16(x) -> np.ndarray:
    """Round to the nearest BF16 (ties to even), returned as float64."""
    b = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(theta: np.ndarray):
    t = np.asarray(theta, dtype=np.float64)
    W1 = t[OFF_W1:OFF_W1 + 1024].reshape(64, 16)
    W2 = t[OFF_W2:OFF_W2 + 4096].reshape(64, 64)
    b2 = t[OFF_B2:OFF_B2 + 64]
    W3 = t[OFF_W3:OFF_W3 + 4096].reshape(64, 64)
    b3 = t[OFF_B3:OFF_B3 + 64]
    W4 = t[OFF_W4:OFF_W4 + 384].reshape(6, 64)
    b4 = t[OFF_B4:OFF_B4 + 6]
    return W1, W2, b2, W3, b3, W4, b4


def pack(W1, W2, b2, W3, b3, W4, b4) -> np.ndarray:
    return np.concatenate([np.ravel(W1), np.ravel(W2), b2, np.ravel(W3), b3, np.ravel(W4), b4])


def init(seed: int = 0) -> np.ndarray:
    """A random parameter vector (numpy generator; not the library's)."""
    rng = np.random.default_rng(seed)
    W1 = np.zeros((64, 16))
    W1[:, :NIN] = rng.uniform(-1, 1, (64, NIN)) * np.sqrt(6 / NIN)
    W1[:, NIN] = rng.uniform(-0.1, 0.1, 64)
    W2 = rng.uniform(-1, 1, (64, 64)) * np.sqrt(6 / 64)
    W3 = rng.uniform(-1, 1, (64, 64)) * np.sqrt(6 / 64)
    W4 = rng.uniform(-1, 1, (6, 64)) * np.sqrt(3 / 64)
    return pack(W1, W2, rng.uniform(-0.1, 0.1, 64), W3, rng.uniform(-0.1, 0.1, 64), W4, rng.uniform(-0.1, 0.1, 6))


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def _normalise(feat, norm):
    mu_in, sd_in = np.asarray(norm["mu_in"], np.float64), np.asarray(norm["sd_in"], np.float64)
    return (np.asarray(feat, np.float64).T - mu_in) / sd_in  # (n, 10)


def forward(theta, feat, norm, bf16_=True):
    """Outputs in physical units, shape (6, n), from feat (10, n)."""
    r = bf16 if bf16_ else (lambda a: np.asarray(a, np.float64))
    W1, W2, b2, W3, b3, W4, b4 = (r(w) if w.ndim == 2 else w for w in unpack(theta))
    x = _normalise(feat, norm)
    X = np.concatenate([x, np.ones((x.shape[0], 1)), np.zeros((x.shape[0], 5))], axis=1)
    h = r(silu(r(X) @ W1.T))
    h = r(silu(h @ W2.T + b2))
    h = r(silu(h @ W3.T + b3))
    y = h @ W4.T + b4
    return (y * np.asarray(norm["sd_out"]) + np.asarray(norm["mu_out"])).T


def loss_and_grad(theta, feat, targ, norm, bf16_=True):
    """Mean of (y - t)^2 over points and outputs (normalised units) and its
    gradient with respect to theta, with the GPU's rounding points."""
    r = bf16 if bf16_ else (lambda a: np.asarray(a, np.float64))
    W1, W2, b2, W3, b3, W4, b4 = unpack(theta)
    W1b, W2b, W3b, W4b = r(W1), r(W2), r(W3), r(W4)
    x = _normalise(feat, norm)
    n = x.shape[0]
    X = r(np.concatenate([x, np.ones((n, 1)), np.zeros((n, 5))], axis=1))
    t = (np.asarray(targ, np.float64).T - np.asarray(norm["mu_out"])) / np.asarray(norm["sd_out"])
    z1 = X @ W1b.T
    h1 = r(silu(z1))
    z2 = h1 @ W2b.T + b2
    h2 = r(silu(z2))
    z3 = h2 @ W3b.T + b3
    h3 = r(silu(z3))
    y = h3 @ W4b.T + b4
    d = y - t
    loss = float(np.mean(d * d))
    dy = r(d * (2.0 / (n * NOUT)))
    gW4, gb4 = dy.T @ h3, dy.sum(0)
    dz3 = r((dy @ W4b) * dsilu(z3))
    gW3, gb3 = dz3.T @ h2, dz3.sum(0)
    dz2 = r((dz3 @ W3b) * dsilu(z2))
    gW2, gb2 = dz2.T @ h1, dz2.sum(0)
    dz1 = r((dz2 @ W2b) * dsilu(z1))
    gW1 = dz1.T @ X
    gW1[:, NIN + 1:] = 0.0
    return loss, pack(gW1, gW2, gb2, gW3, gb3, gW4, gb4)


class Adam:
    """Adam with the library's constants (beta1 0.9, beta2 0.999, eps 1e-8)."""

    def __init__(self, n: int):
        self.m = np.zeros(n)
        self.v = np.zeros(n)
        self.t = 0

    def step(self, theta, g, lr):
        self.t += 1
        self.m = 0.9 * self.m + 0.1 * g
        self.v = 0.999 * self.v + 0.001 * g * g
        mh = self.m / (1 - 0.9 ** self.t)
        vh = self.v / (1 - 0.999 ** self.t)
        return theta - lr * mh / (np.sqrt(vh) + 1e-8)
