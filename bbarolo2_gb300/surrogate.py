"""A learned surrogate of the log-likelihood, trained online on the evaluations a sampler makes.

The network (``libbbgpu.so``, ``bbgpu_mlp_*``) is a multilayer perceptron d -> 256 -> 256 -> 256 -> 1 with GELU
activations, trained on the device by the library's own BF16 forward and backward kernels with FP32 master weights
and Adam. Inputs are the sampler's unit-cube coordinates, standardised by the mean and spread of the points it was
last fitted on (the region of the live points, which shrinks as a nested sampler converges); targets are the
log-likelihoods relative to the sampler's current threshold, clipped to a window of a few tens of nats about it (the
screen only has to tell points above the threshold from points below it, not how far below).

The reference has no counterpart: its nested sampler (``bbarolo/bayesian/nautilus``) trains numba networks as
bounds of the live region (``nautilus/mlp.py:18-118``, ``bounds/neural.py``), not as surrogates of the likelihood.
"""

import ctypes as C

import numpy as np

from . import _lib


class MLP:
    """The device network: ``predict``, ``gradients`` and ``train_step`` on float32 host arrays."""

    def __init__(self, d_in, hidden=256, seed=0, device=0):
        self.L = _lib.load()
        h = C.c_void_p()
        rc = self.L.bbgpu_mlp_create(C.byref(h), int(device), int(d_in), int(hidden), int(seed) & (2 ** 64 - 1))
        if rc != _lib.OK:
            raise _lib.DeviceError(rc, "bbgpu_mlp_create failed (no CUDA device visible?)")
        self.h, self.d, self.hidden = h, int(d_in), int(hidden)
        self.nparams = int(self.L.bbgpu_mlp_nparams(h))

    def _check(self, rc, what):
        if rc != _lib.OK:
            raise _lib.DeviceError(rc, what)

    def params(self):
        p = np.empty(self.nparams, np.float32)
        self._check(self.L.bbgpu_mlp_get_params(self.h, _lib.ptr(p)), "bbgpu_mlp_get_params")
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.nparams
        self._check(self.L.bbgpu_mlp_set_params(self.h, _lib.ptr(p)), "bbgpu_mlp_set_params")

    def predict(self, x):
        x = np.ascontiguousarray(x, np.float32)
        y = np.empty(len(x), np.float32)
        self._check(self.L.bbgpu_mlp_predict(self.h, _lib.ptr(x), len(x), _lib.ptr(y)), "bbgpu_mlp_predict")
        return y

    def gradients(self, x, t):
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        g = np.empty(self.nparams, np.float32)
        loss = C.c_float(0)
        self._check(self.L.bbgpu_mlp_gradients(self.h, _lib.ptr(x), _lib.ptr(t), len(x), _lib.ptr(g),
                                                 C.byref(loss)), "bbgpu_mlp_gradients")
        return g, float(loss.value)

    def train(self, x, t, steps, batch, lr=1e-3, seed=0):
        """`steps` Adam steps on minibatches of `batch` rows drawn on the device from the set (x, t); returns the
        last minibatch's loss."""
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        loss = C.c_float(0)
        self._check(self.L.bbgpu_mlp_train(self.h, _lib.ptr(x), _lib.ptr(t), len(x), int(steps), int(batch),
                                           C.c_float(lr), int(seed) & (2 ** 64 - 1), C.byref(loss)),
                    "bbgpu_mlp_train")
        return float(loss.value)

    def train_step(self, x, t, lr=1e-3):
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        loss = C.c_float(0)
        self._check(self.L.bbgpu_mlp_train_step(self.h, _lib.ptr(x), _lib.ptr(t), len(x), C.c_float(lr),
                                                  C.byref(loss)), "bbgpu_mlp_train_step")
        return float(loss.value)

    def close(self):
        if getattr(self, "h", None):
            self.L.bbgpu_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Surrogate:
    """log L(u) on the unit cube of a sampler, learned from its evaluations (u, log L).

    ``fit(u, logl, center)`` trains on the pairs for ``steps`` Adam steps of minibatches (``steps_warm`` after the
    first fit); ``predict(u)`` returns
    log L (within the fitted window about the center); ``rmse(u, logl)`` the error on pairs it was not fitted on."""

    def __init__(self, ndim, hidden=256, seed=0, device=0, lr=1e-3, steps=150, batch=1024, steps_warm=150):
        self.net = MLP(ndim, hidden, seed, device)
        self.lr, self.steps, self.batch = float(lr), int(steps), int(batch)
        self.steps_warm = int(steps_warm)
        self.rng = np.random.default_rng(seed)
        self.mu = np.zeros(ndim)
        self.sd = np.ones(ndim)
        self.ymu, self.ysd = 0.0, 1.0
        self.trained = False
        self.last_rmse = np.inf

    def _x(self, u):
        return ((np.asarray(u, float) - self.mu) / self.sd).astype(np.float32)

    def fit(self, u, logl, center, scale=8.0, region=None):
        """Trains (warm-started) on the pairs (u, logl): targets (logl - center) / scale clipped to [-1, 1] (the shape
        of log L within `scale` of `center`, a sampler's threshold); inputs standardised by the points `region`
        (default u), redone at every fit as the live region shrinks."""
        u = np.asarray(u, float)
        ref = u if region is None else np.asarray(region, float)
        self.mu = ref.mean(axis=0)
        self.sd = np.maximum(ref.std(axis=0), 1e-12)
        self.ymu, self.ysd = float(center), float(scale)
        x = self._x(u)
        t = np.clip((np.asarray(logl, float) - self.ymu) / self.ysd, -1.0, 1.0).astype(np.float32)
        # the minibatches are drawn on the device: one call for all the steps (fewer once warm: the network starts
        # from the last fit, whose window moved by a fraction of its width since)
        steps = self.steps_warm if self.trained else self.steps
        loss = self.net.train(x, t, steps, min(self.batch, len(x)), self.lr, int(self.rng.integers(2 ** 62)))
        self.trained = True
        return loss * self.ysd ** 2

    def predict(self, u):
        return self.net.predict(self._x(u)).astype(float) * self.ysd + self.ymu

    def rmse(self, u, logl):
        y = np.asarray(logl, float)
        if len(y) == 0:
            return np.inf
        return float(np.sqrt(np.mean((self.predict(u) - y) ** 2)))
