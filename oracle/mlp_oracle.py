"""Test infrastructure: FP64 NumPy restatement of the warm-start network and
its descriptors (pysic_gb300/csrc/mlp.cu), for gradient and parity checks.

Parameter layout: W1 (h1 x n_in, row-major), b1, W2 (h2 x h1), b2, w3 (h2), b3.
The engine's forward pass reads BF16 weights and rounds its inputs and its
first-layer activations to BF16 (the operands of its tensor-core products):
``bf16`` rounds FP32 values to the nearest BF16 (ties to even) so that the
oracle computes the same function in FP64.
"""
import numpy as np


def split(p, n_in, h1, h2):
    p = np.asarray(p, dtype=np.float64)
    o = 0
    W1 = p[o:o + h1 * n_in].reshape(h1, n_in); o += h1 * n_in
    b1 = p[o:o + h1]; o += h1
    W2 = p[o:o + h2 * h1].reshape(h2, h1); o += h2 * h1
    b2 = p[o:o + h2]; o += h2
    w3 = p[o:o + h2]; o += h2
    b3 = p[o]
    return W1, b1, W2, b2, w3, b3


def bf16(p):
    u = np.asarray(p, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def _r(a, exact=False):
    return np.asarray(a, dtype=np.float64) if exact else bf16(a).astype(np.float64)


def forward(p, x, n_in, h1, h2, exact=False):
    """Output, first-layer activations (before rounding) and second-layer
    activations of x~ -> tanh(W1 x~ + b1) = a1 -> tanh(W2 a1~ + b2) -> w3 . a2 + b3;
    exact: without the BF16 rounding of x and a1 (for derivative checks)."""
    W1, b1, W2, b2, w3, b3 = split(p, n_in, h1, h2)
    a1 = np.tanh(_r(x, exact) @ W1.T + b1)
    a2 = np.tanh(_r(a1, exact) @ W2.T + b2)
    return a2 @ w3 + b3, a1, a2


def loss_and_grad(p, x, y, n_in, h1, h2, tensor_core=False, exact=False):
    """Mean squared error and its gradient with respect to p, the roundings
    passed through unchanged.  tensor_core: the layer errors dz2 and dz1
    rounded to BF16 where they enter a matrix product, as the engine's
    tensor-core training step does; exact: no rounding at all."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    W1, b1, W2, b2, w3, b3 = split(p, n_in, h1, h2)
    out, a1, a2 = forward(p, x, n_in, h1, h2, exact)
    n = len(y)
    err = out - y
    dy = 2.0 * err / n
    dz2 = dy[:, None] * w3[None, :] * (1.0 - a2 ** 2)
    if tensor_core:
        dz2 = _r(dz2)
    dz1 = (dz2 @ W2) * (1.0 - a1 ** 2)
    if tensor_core:
        dz1 = _r(dz1)
    g = np.concatenate([(dz1.T @ _r(x, exact)).ravel(), dz1.sum(0), (dz2.T @ _r(a1, exact)).ravel(), dz2.sum(0),
                        a2.T @ dy, [dy.sum()]])
    return float(np.mean(err ** 2)), g


def descriptors(positions, cell, types, n_types, counts, idx, off, n_gauss, r0, r1, width, cutoff):
    """Radial features per atom over the given neighbour lists (CSR)."""
    pos = np.asarray(positions, dtype=np.float64)
    cell = np.asarray(cell, dtype=np.float64)
    n = len(pos)
    mu = np.linspace(r0, r1, n_gauss) if n_gauss > 1 else np.array([r0])
    out = np.zeros((n, n_types * n_gauss))
    start = np.concatenate([[0], np.cumsum(counts)])
    for i in range(n):
        for e in range(start[i], start[i + 1]):
            j = idx[e]
            r = np.linalg.norm(pos[j] - pos[i] + np.asarray(off[e]) @ cell)
            if r >= cutoff:
                continue
            f = np.exp(-(r - mu) ** 2 / (2 * width * width)) * 0.5 * (1 + np.cos(np.pi * r / cutoff))
            t = types[j]
            out[i, t * n_gauss:(t + 1) * n_gauss] += f
    return out
