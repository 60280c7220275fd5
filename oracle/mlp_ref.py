"""CPU reference of the learned planner's network -- TEST INFRASTRUCTURE ONLY.

NumPy float64 restatement of the library's MLP (omr-ntt_gb300/csrc/mlp.cu):
features -> Linear -> ReLU -> Linear -> ReLU -> Linear, parameters packed as
W1 [h x in], b1 [h], W2 [h x h], b2 [h], W3 [out x h], b3 [out]; loss = masked
mean squared error sum(mask * (y - t)^2) / sum(mask).  Used by the tests to
check the GPU forward pass and gradients, and to evaluate a trained network on
stored timings without a GPU.  The reference crate has no learned planner;
this is the checker of new work.
"""
from __future__ import annotations

import numpy as np


def unpack(p, n_in, n_h, n_out):
    p = np.asarray(p, dtype=np.float64)
    o = 0
    W1 = p[o:o + n_h * n_in].reshape(n_h, n_in); o += n_h * n_in
    b1 = p[o:o + n_h]; o += n_h
    W2 = p[o:o + n_h * n_h].reshape(n_h, n_h); o += n_h * n_h
    b2 = p[o:o + n_h]; o += n_h
    W3 = p[o:o + n_out * n_h].reshape(n_out, n_h); o += n_out * n_h
    b3 = p[o:o + n_out]; o += n_out
    assert o == p.size
    return W1, b1, W2, b2, W3, b3


def forward(p, x, n_in, n_h, n_out):
    W1, b1, W2, b2, W3, b3 = unpack(p, n_in, n_h, n_out)
    x = np.asarray(x, dtype=np.float64)
    h1 = np.maximum(x @ W1.T + b1, 0.0)
    h2 = np.maximum(h1 @ W2.T + b2, 0.0)
    return h2 @ W3.T + b3


def loss_and_grad(p, x, t, m, n_in, n_h, n_out):
    W1, b1, W2, b2, W3, b3 = unpack(p, n_in, n_h, n_out)
    x = np.asarray(x, dtype=np.float64)
    t = np.asarray(t, dtype=np.float64)
    m = np.asarray(m, dtype=np.float64)
    z1 = x @ W1.T + b1
    h1 = np.maximum(z1, 0.0)
    z2 = h1 @ W2.T + b2
    h2 = np.maximum(z2, 0.0)
    y = h2 @ W3.T + b3
    denom = max(m.sum(), 1.0)
    d = m * (y - t)
    loss = float((d * d).sum() / denom)
    dy = 2.0 * d / denom
    gW3 = dy.T @ h2
    gb3 = dy.sum(0)
    dh2 = (dy @ W3) * (h2 > 0)
    gW2 = dh2.T @ h1
    gb2 = dh2.sum(0)
    dh1 = (dh2 @ W2) * (h1 > 0)
    gW1 = dh1.T @ x
    gb1 = dh1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return loss, g
