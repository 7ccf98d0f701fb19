"""CPU oracle of the scheduler's work MLP -- test infrastructure only.

Float64 numpy restatement of the network the engine's CUDA kernels evaluate
and train (cudancorr_gb300/csrc/sched.cu): 28 inputs -> 64 ReLU -> 64 ReLU
-> 1, parameter vector [W1 (28 x 64, row-major by input), b1 (64),
W2 (64 x 64, row-major by hidden input), b2 (64), w3 (64), b3]. The loss is
the mean squared error over the samples. The reference has no learned part;
this oracle is pinned by a finite-difference check of its own gradient
(tests/test_oracle_mlp.py), and the GPU gradient is checked against it.
"""
from __future__ import annotations

import numpy as np

N_IN, N_HID = 28, 64
OFF_W1 = 0
OFF_B1 = OFF_W1 + N_IN * N_HID
OFF_W2 = OFF_B1 + N_HID
OFF_B2 = OFF_W2 + N_HID * N_HID
OFF_W3 = OFF_B2 + N_HID
OFF_B3 = OFF_W3 + N_HID
N_PARAMS = OFF_B3 + 1


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    w1 = p[OFF_W1:OFF_B1].reshape(N_IN, N_HID)
    b1 = p[OFF_B1:OFF_W2]
    w2 = p[OFF_W2:OFF_B2].reshape(N_HID, N_HID)
    b2 = p[OFF_B2:OFF_W3]
    w3 = p[OFF_W3:OFF_B3]
    b3 = p[OFF_B3]
    return w1, b1, w2, b2, w3, b3


def bf16(a):
    """Round float32 values to bfloat16 (nearest, ties to even), as float64."""
    b = np.ascontiguousarray(np.asarray(a, dtype=np.float32)).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def forward(p, x, bf16_forward=False):
    """Predictions for the rows of x (n x 28). bf16_forward: the BF16 forward
    pass of the engine's kernels -- weights, inputs and hidden activations
    rounded to bfloat16, biases not, sums in (here) float64."""
    w1, b1, w2, b2, w3, b3 = unpack(p)
    x = np.asarray(x, dtype=np.float64)
    r = bf16 if bf16_forward else (lambda a: np.asarray(a, dtype=np.float64))
    if bf16_forward:
        w1, w2, w3 = r(w1), r(w2), r(w3)
    h1 = r(np.maximum(r(x) @ w1 + b1, 0.0))
    h2 = r(np.maximum(h1 @ w2 + b2, 0.0))
    return h2 @ w3 + b3


def loss_and_grad(p, x, t, bf16_forward=False):
    """(sum of squared errors, gradient of the mean squared error).
    bf16_forward: the forward pass rounds weights, inputs and activations to
    bfloat16 and the backward pass uses the rounded values."""
    w1, b1, w2, b2, w3, b3 = unpack(p)
    x = np.asarray(x, dtype=np.float64)
    t = np.asarray(t, dtype=np.float64)
    r = bf16 if bf16_forward else (lambda a: a)
    if bf16_forward:
        w1, w2, w3, x = r(w1), r(w2), r(w3), r(x)
    n = x.shape[0]
    z1 = x @ w1 + b1
    h1 = r(np.maximum(z1, 0.0))
    z2 = h1 @ w2 + b2
    h2 = r(np.maximum(z2, 0.0))
    y = h2 @ w3 + b3
    r = y - t
    dy = 2.0 * r / n
    g = np.zeros(N_PARAMS)
    g[OFF_W3:OFF_B3] = h2.T @ dy
    g[OFF_B3] = dy.sum()
    d2 = np.outer(dy, w3) * (z2 > 0)
    g[OFF_W2:OFF_B2] = (h1.T @ d2).reshape(-1)
    g[OFF_B2:OFF_W3] = d2.sum(axis=0)
    d1 = (d2 @ w2.T) * (z1 > 0)
    g[OFF_W1:OFF_B1] = (x.T @ d1).reshape(-1)
    g[OFF_B1:OFF_W2] = d1.sum(axis=0)
    return float(r @ r), g
