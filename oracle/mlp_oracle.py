"""CPU oracle of the warm-start perceptron (test infrastructure only).

Restates, in float64 numpy, the forward pass, the mean-squared-error
gradient and one Adam step of the library's network
(pdos_gb300/csrc/mlp.cu), rounding to bfloat16 at exactly the points where
the GPU stores bfloat16: the inputs, the weight copies, the hidden
activations and the backward-pass signals.  Everything else is float64, so
the GPU result differs from this one only by its float32 accumulation.
The network is not part of the reference (it has no learned component);
its published algorithms are the perceptron with ReLU and Adam (Kingma &
Ba, 2015).
"""
import numpy as np


def bf16(a):
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def forward(params, x):
    """params: [(W1, b1), (W2, b2), (W3, b3)], W of shape (out, in)."""
    (w1, b1), (w2, b2), (w3, b3) = params
    x0 = bf16(x)
    h1 = bf16(np.maximum(x0 @ bf16(w1).T + b1, 0.0))
    h2 = bf16(np.maximum(h1 @ bf16(w2).T + b2, 0.0))
    y = h2 @ bf16(w3).T + b3
    return x0, h1, h2, y


def loss_and_grads(params, x, t):
    """Loss (before the step) and gradients as the GPU computes them."""
    (w1, _), (w2, _), (w3, _) = params
    x0, h1, h2, y = forward(params, x)
    B, N = t.shape
    diff = y - t
    loss = float(np.sum(diff * diff) / (B * N))
    dy = bf16(2.0 * diff / (B * N))
    gw3, gb3 = dy.T @ h2, dy.sum(axis=0)
    dz2 = bf16((dy @ bf16(w3)) * (h2 > 0))
    gw2, gb2 = dz2.T @ h1, dz2.sum(axis=0)
    dz1 = bf16((dz2 @ bf16(w2)) * (h1 > 0))
    gw1, gb1 = dz1.T @ x0, dz1.sum(axis=0)
    return loss, y, [(gw1, gb1), (gw2, gb2), (gw3, gb3)]


def adam_step(w, g, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam update (bias-corrected), returns (w, m, v)."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    c1, c2 = 1 - b1 ** step, 1 - b2 ** step
    return w - lr * (m / c1) / (np.sqrt(v / c2) + eps), m, v
