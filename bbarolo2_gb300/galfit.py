"""The CLASSIC 3DFIT kernels on the device, with the reference's signatures.

``_conv_sparse(model, kern, scale)`` mirrors ``bbarolo/galmod.py:974-1037`` and ``_norm(model, data, mask, ...)``
mirrors ``bbarolo/galfit.py:39-188`` (the model is scaled in place, as the reference; the work array ``P`` is
accepted and ignored: the device keeps its own running sums). Both run on the GPU through ``libbbgpu.so``:
the reference's float64 arithmetic, ``_conv_sparse`` bit-exact, ``_norm`` with the same ring footprint, factors
and blank counts and its residual sum reduced in a fixed tree (rounding differences only). The fit that calls them,
ring by ring, is ``bbarolo2_gb300.classic``.
"""

import threading

import numpy as np

from . import _lib

_ctx = {}
_mu = threading.Lock()


def context(device=0):
    """The module's device context for ``device`` (one per host thread: a context owns one stream)."""
    key = (device, threading.get_ident())
    with _mu:
        c = _ctx.get(key)
        if c is None:
            c = _ctx[key] = _lib.Context(device)
    return c


def _conv_sparse(model, kern, scale, ctx=None):
    """'Same' 2D convolution of each channel of a (ny, nx, nz) model, values < 1e-12 set to zero, x scale."""
    c = ctx or context()
    m = np.ascontiguousarray(model, np.float64)
    k = np.ascontiguousarray(kern, np.float64)
    out = np.zeros_like(m)
    c.check(c.L.bbgpu_conv_sparse(c.h, _lib.ptr(m), _lib.ptr(out), *m.shape, _lib.ptr(k), k.shape[0], k.shape[1],
                                  float(scale)))
    return out


def _norm(model, data, mask, blo0, blo1, x0, y0, phi, inc, r1, r2, wpow, side, ftype, chan_noise, data_noise,
          bweight, normtype, pre, ilo, ihi, thr, P, foot, hmax, ctx=None):
    """The CLASSIC residual of a single-ring model (normalised in place); np.inf when no voxel counts."""
    c = ctx or context()
    if not (isinstance(model, np.ndarray) and model.dtype == np.float64 and model.flags.c_contiguous):
        raise TypeError("model must be a C-contiguous float64 array (it is normalised in place)")
    bsy, bsx, nz = model.shape
    d = np.ascontiguousarray(data, np.float32)
    k = np.ascontiguousarray(mask, dtype=bool).view(np.uint8)
    dny, dnx = d.shape[:2]
    trunc = pre is not None and np.asarray(pre).size > 0
    pre_ = np.ascontiguousarray(pre, np.float64) if trunc else None
    ilo_ = np.ascontiguousarray(ilo, np.int64) if trunc else None
    ihi_ = np.ascontiguousarray(ihi, np.int64) if trunc else None
    thr_ = np.ascontiguousarray(thr, np.float64) if trunc else None
    cn = np.ascontiguousarray(chan_noise, np.float64)
    out = np.zeros(1)
    c.check(c.L.bbgpu_norm(c.h, _lib.ptr(model), bsy, bsx, nz, _lib.ptr(d), _lib.ptr(k), dny, dnx, int(blo0),
                           int(blo1), float(x0), float(y0), float(phi), float(inc), float(r1), float(r2), float(wpow),
                           int(side), int(ftype), _lib.ptr(cn), float(data_noise), float(bweight), int(normtype),
                           _lib.ptr(pre_), _lib.ptr(ilo_), _lib.ptr(ihi_), int(ilo_.size) if trunc else 0,
                           _lib.ptr(thr_), int(foot), float(hmax), _lib.ptr(out)))
    return float(out[0])
