"""The learned selector's network on the GPU: forward pass and gradients
match the CPU reference (oracle/mlp_ref.py), training lowers the loss, and an
installed network drives the planner."""
import ctypes

import numpy as np
import pytest

from omr_ntt import _lib
from omr_ntt import planner as P

pytestmark = pytest.mark.gpu


def _data(rows, k, seed):
    rng = np.random.default_rng(seed)
    X = rng.random((rows, P.N_FEATURES), dtype=np.float32)
    Y = rng.normal(size=(rows, k)).astype(np.float32)
    M = (rng.random((rows, k)) < 0.6).astype(np.float32)
    return X, Y, M


def test_forward_and_gradients_match_cpu_reference():
    from oracle import mlp_ref

    k = P.n_classes()
    mlp = P.Mlp(seed=3)
    p = mlp.params().astype(np.float64)
    X, Y, M = _data(37, k, 1)
    y_gpu = mlp.forward(X)
    y_cpu = mlp_ref.forward(p, X, P.N_FEATURES, P.N_HIDDEN, k)
    assert np.allclose(y_gpu, y_cpu, rtol=1e-4, atol=1e-5)
    loss_gpu, g_gpu = mlp.gradients(X, Y, M)
    loss_cpu, g_cpu = mlp_ref.loss_and_grad(p, X, Y, M, P.N_FEATURES, P.N_HIDDEN, k)
    assert abs(loss_gpu - loss_cpu) <= 1e-4 * max(1.0, abs(loss_cpu))
    # fp32 kernels vs float64 reference: per-entry tolerance scaled to the gradient's size
    scale = np.abs(g_cpu).max()
    assert np.allclose(g_gpu, g_cpu, rtol=1e-3, atol=1e-4 * scale)


def test_fit_lowers_loss_deterministically():
    k = P.n_classes()
    X, _, M = _data(256, k, 2)
    Y = np.tanh(X @ np.random.default_rng(3).normal(size=(P.N_FEATURES, k))).astype(np.float32)
    a, b = P.Mlp(seed=5), P.Mlp(seed=5)
    ha = a.fit(X, Y, M, epochs=40, batch=32, lr=3e-3, seed=9)
    hb = b.fit(X, Y, M, epochs=40, batch=32, lr=3e-3, seed=9)
    assert ha[-1] < 0.5 * ha[0]
    assert np.array_equal(ha, hb) and np.array_equal(a.params(), b.params())


def test_installed_network_drives_the_planner():
    import omr_ntt
    from omr_ntt import NttDomain
    from omr_ntt.fields import BabyBear
    from oracle import oracle

    L = _lib.lib()
    k = P.n_classes()
    mlp = P.Mlp(seed=1)
    # bias the output layer so that the gather class of the balanced tile
    # plan (class 28) is the cheapest: the planner must then gather
    p = mlp.params()
    p[-k:] = 10.0
    p[-k + 28] = -10.0
    mlp.set_params(p)
    mlp.install()
    try:
        d = NttDomain(BabyBear, 1 << 14)
        x = omr_ntt.gen_input_seeded(BabyBear, 1 << 14, 4)
        got = omr_ntt.partial(d, x, omr_ntt.PREFIX, 64)
        assert np.array_equal(got, oracle.forward(0, x)[:64])
    finally:
        L.omr_ntt_mlp_install(None)
