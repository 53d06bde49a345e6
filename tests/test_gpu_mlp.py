"""The surrogate network's device kernels (BF16 products, FP32 accumulation, FP32 master weights, Adam) against a
float64 NumPy MLP: the gradients of every parameter, and a fit that converges."""
import numpy as np
import pytest
from scipy.special import erf

pytestmark = pytest.mark.gpu

D, H = 42, 256


def _bf(x):
    """Round to BF16 (nearest even) and back."""
    f = np.ascontiguousarray(x, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = (((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


def _gelu(z):
    return 0.5 * z * (1 + erf(z / np.sqrt(2)))


def _dgelu(z):
    return 0.5 * (1 + erf(z / np.sqrt(2))) + z * np.exp(-0.5 * z * z) / np.sqrt(2 * np.pi)


def _split(p):
    sizes = [H * D, H, H * H, H, H * H, H, H, 1]
    out, o = [], 0
    for s in sizes:
        out.append(np.asarray(p[o:o + s], np.float64))
        o += s
    W1, b1, W2, b2, W3, b3, w4, b4 = out
    return W1.reshape(H, D), b1, W2.reshape(H, H), b2, W3.reshape(H, H), b3, w4, b4


def _reference(p, x, t, rounded):
    """Loss and gradients in float64; rounded=True applies BF16 rounding where the kernels store BF16 (inputs,
    weights, activations, the pre-activation gradients fed to the products)."""
    R = _bf if rounded else (lambda v: np.asarray(v, np.float64))
    W1, b1, W2, b2, W3, b3, w4, b4 = _split(p)
    X = R(x)
    z1 = X @ R(W1).T + b1
    a1 = R(_gelu(z1))
    z2 = a1 @ R(W2).T + b2
    a2 = R(_gelu(z2))
    z3 = a2 @ R(W3).T + b3
    a3 = R(_gelu(z3))
    y = a3 @ R(w4) + b4[0]
    n = len(x)
    r = y - t
    dy = 2 * r / n
    g = {}
    g["w4"], g["b4"] = a3.T @ dy, np.array([dy.sum()])
    dz3 = dy[:, None] * R(w4)[None, :] * _dgelu(z3)
    g["W3"], g["b3"] = R(dz3).T @ a2, dz3.sum(0)
    dz2 = (R(dz3) @ R(W3)) * _dgelu(z2)
    g["W2"], g["b2"] = R(dz2).T @ a1, dz2.sum(0)
    dz1 = (R(dz2) @ R(W2)) * _dgelu(z1)
    g["W1"], g["b1"] = R(dz1).T @ X, dz1.sum(0)
    flat = np.concatenate([g["W1"].ravel(), g["b1"], g["W2"].ravel(), g["b2"], g["W3"].ravel(), g["b3"], g["w4"],
                           g["b4"]])
    return float((r * r).mean()), flat, y


def test_mlp_gradients_against_float64(gpu_lib):
    from bbarolo2_gb300.surrogate import MLP
    net = MLP(D, H, seed=1)
    rng = np.random.default_rng(0)
    x = rng.standard_normal((300, D)).astype(np.float32)
    t = (np.sin(x[:, 0]) + 0.5 * x[:, 1] * x[:, 2]).astype(np.float32)
    p = net.params()
    g, loss = net.gradients(x, t)
    y = net.predict(x)
    # the kernels' rounding points emulated in float64: the same gradients to the FP32 accumulation order
    loss_r, g_r, y_r = _reference(p, x, t, rounded=True)
    assert abs(loss - loss_r) <= 1e-4 * loss_r
    # (an activation on a BF16 rounding boundary rounds differently from float64 GELU to float32 erff: 1e-3)
    np.testing.assert_allclose(y, y_r, rtol=0, atol=1e-3 * np.abs(y_r).max())
    sizes = [H * D, H, H * H, H, H * H, H, H, 1]
    o = 0
    for s in sizes:
        np.testing.assert_allclose(g[o:o + s], g_r[o:o + s], rtol=0, atol=5e-3 * np.abs(g_r[o:o + s]).max())
        o += s
    # against the plain float64 network: the BF16 rounding moves the gradient by about a percent
    loss_f, g_f, _ = _reference(p, x, t, rounded=False)
    assert abs(loss - loss_f) <= 2e-2 * loss_f
    assert np.linalg.norm(g - g_f) <= 5e-2 * np.linalg.norm(g_f)
    assert float(g @ g_f) / (np.linalg.norm(g) * np.linalg.norm(g_f)) > 0.999


def test_mlp_training_converges(gpu_lib):
    from bbarolo2_gb300.surrogate import MLP
    net = MLP(D, H, seed=2)
    rng = np.random.default_rng(1)
    x = rng.standard_normal((4096, D)).astype(np.float32)
    w = rng.standard_normal(D) / np.sqrt(D)
    t = (x @ w + 0.3 * (x[:, :5] ** 2).sum(1)).astype(np.float32)
    t = (t - t.mean()) / t.std()
    first = None
    for step in range(600):
        idx = rng.integers(0, len(x), 512)
        loss = net.train_step(x[idx], t[idx], 1e-3)
        first = loss if first is None else first
    y = net.predict(x)
    assert float(np.mean((y - t) ** 2)) < 0.05 * first, (first, float(np.mean((y - t) ** 2)))


def test_mlp_train_on_device_minibatches(gpu_lib):
    """bbgpu_mlp_train (the minibatches drawn on the device, one call): the same fit as the host loop, repeatable for a
    seed, and a one-row minibatch of a one-row set is exactly train_step on that row."""
    from bbarolo2_gb300.surrogate import MLP
    rng = np.random.default_rng(1)
    x = rng.standard_normal((4096, D)).astype(np.float32)
    w = rng.standard_normal(D) / np.sqrt(D)
    t = (x @ w + 0.3 * (x[:, :5] ** 2).sum(1)).astype(np.float32)
    t = (t - t.mean()) / t.std()
    a, b = MLP(D, H, seed=2), MLP(D, H, seed=2)
    la = a.train(x, t, 600, 512, 1e-3, seed=5)
    lb = b.train(x, t, 600, 512, 1e-3, seed=5)
    assert abs(la - lb) <= 1e-5 * abs(la)          # (the reported loss is summed with atomics; the weights are not)
    np.testing.assert_array_equal(a.params(), b.params())
    y = a.predict(x)
    assert float(np.mean((y - t) ** 2)) < 0.05, float(np.mean((y - t) ** 2))
    c, d = MLP(D, H, seed=3), MLP(D, H, seed=3)
    c.train(x[:1], t[:1], 3, 1, 1e-3, seed=9)
    for _ in range(3):
        d.train_step(x[:1], t[:1], 1e-3)
    np.testing.assert_array_equal(c.params(), d.params())


def test_mlp_rejects_bad_arguments(gpu_lib):
    import ctypes as C
    from bbarolo2_gb300 import _lib
    L = _lib.load()
    h = C.c_void_p()
    assert L.bbgpu_mlp_create(C.byref(h), 0, 0, 256, 1) == _lib.ERR_ARG
    assert L.bbgpu_mlp_create(C.byref(h), 0, 42, 4, 1) == _lib.ERR_ARG
