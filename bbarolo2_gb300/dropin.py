"""Drop-in replacements of the reference's numba kernels of the model path, with their signatures.

Each function below has the name (without the leading underscore), the arguments and the side effects of the
reference kernel it replaces, and runs on the GPU through ``libbbgpu.so``:

=====================  ==================================================  ==========================================
here                   reference                                           side effect
=====================  ==================================================  ==========================================
``galmod_mc``          ``bbarolo/galmod.py:92`` ``_galmod_mc``              out (by, bx, nz) += the MC model
``galmod_analytic``    ``bbarolo/galmod.py:326`` ``_galmod_analytic``       out += the ANALYTIC model
``ring_maps_analytic`` ``bbarolo/galmod.py:468`` ``_ring_maps_analytic``    out (nr, by, bx) += the ring maps
``conv_sparse``        ``bbarolo/galmod.py:974`` ``_conv_sparse``           returns the convolved model
``norm``               ``bbarolo/galfit.py:39`` ``_norm``                   model normalised in place; the residual
``sumsq_residuals``    ``bbarolo/bayesian/likelihood.py:22``                returns the sum of squares
``residuals_fracerr``  ``bbarolo/bayesian/likelihood.py:48``                returns (sum r^2 / v, sum log(v / s^2))
``FFTConvolver_call``  ``bbarolo/smooth.py:145`` ``FFTConvolver.__call__``  the "same" convolution of the planes
``galmod_wind``        ``bbarolo/galmod.py:539`` ``_galmod_wind``           out (by, bx, nz) += the wind's clouds
=====================  ==================================================  ==========================================

and the classes of the wind models (``bbarolo/windmodel.py``: ``WindModel``, ``WindCells``, ``WindPars``,
``Boxes``) by those of ``bbarolo2_gb300.wind``, in ``bbarolo.windmodel`` and in ``bbarolo.bayesian.wind`` (which
imports them by name), so that WINDFIT's likelihood builds its columns and normal equations on the device.

``install()`` binds them in place of the reference's functions in its modules (``bbarolo.galmod``,
``bbarolo.galfit``, ``bbarolo.bayesian.likelihood``, ``bbarolo.smooth``, ``bbarolo.galwind``, which imports
``_galmod_wind`` by name), so that ``GalmodSetup._build``,
``DiskModel.array/convolve/ring_maps``, ``Galfit._norm_value`` and ``LikelihoodMixin._calculate_residuals`` take
the device path unchanged; ``uninstall()`` restores them. The device contexts are cached by the scalars of the grid
each call passes (one context per distinct grid, one per host thread).
"""

import sys
import threading

import numpy as np

from . import _lib

_tls = threading.local()


def _ctxs():
    d = getattr(_tls, "ctxs", None)
    if d is None:
        d = _tls.ctxs = {}
    return d


def _grid_ctx(nx, ny, nz, radsep, cdens, cmode, pixarea, cdelt0, cdelt1, crota2, ltype, sig_instr, axtyp, velsys,
              lfreq0, crval3, cdelt3, crpix3, relint, cd2i, chwidth=0., zstep=0.25, vedges=None, device=0):
    """The device context of a grid (set_grid done), cached by its scalars and tables."""
    lf = np.ascontiguousarray(lfreq0, np.float64).ravel()
    ri = np.ascontiguousarray(relint, np.float64).ravel()
    cd = np.ascontiguousarray(cd2i, np.float64).ravel()
    ve = None if vedges is None else np.ascontiguousarray(vedges, np.float64)
    key = (int(nx), int(ny), int(nz), float(radsep), float(cdens), int(cmode), float(pixarea), float(cdelt0),
           float(cdelt1), float(crota2), int(ltype), float(sig_instr), int(axtyp), int(velsys), lf.tobytes(),
           float(crval3), float(cdelt3), float(crpix3), ri.tobytes(), cd.tobytes(), float(chwidth), float(zstep),
           None if ve is None else ve.tobytes(), int(device))
    d = _ctxs()
    c = d.get(key)
    if c is not None:
        return c
    if len(d) > 16:
        for old in d.values():
            old.close()
        d.clear()
    c = _lib.Context(device)
    g = _lib.Grid()
    g.nx, g.ny, g.nz, g.nlines = int(nx), int(ny), int(nz), int(lf.size)
    g.axtyp, g.velsys, g.ltype, g.cmode = int(axtyp), int(velsys), int(ltype), int(cmode)
    g.radsep, g.cdens, g.pixarea = float(radsep), float(cdens), float(pixarea)
    g.cdelt0, g.cdelt1, g.crota2 = float(cdelt0), float(cdelt1), float(crota2)
    g.sig_instr, g.crval3, g.cdelt3, g.crpix3 = float(sig_instr), float(crval3), float(cdelt3), float(crpix3)
    g.chwidth, g.zstep, g.scalefactor = float(chwidth), float(zstep), 1.0
    c.check(c.L.bbgpu_set_grid(c.h, g, _lib.ptr(cd), _lib.ptr(lf), _lib.ptr(ri), _lib.ptr(ve)))
    d[key] = c
    return c


def _out64(out):
    if not (isinstance(out, np.ndarray) and out.dtype == np.float64 and out.flags.c_contiguous):
        raise TypeError("out must be a C-contiguous float64 array (the kernels accumulate into it)")
    return out


def galmod_mc(out, sr, ring_lo, ring_hi, seed, radsep, nv, cdens, cmode, pixarea, cdelt0, cdelt1, crota2, blo0,
              blo1, bhi0, bhi1, ltype, sig_instr, axtyp, velsys, lfreq0, crval3, cdelt3, crpix3, relint, cd2i):
    """``_galmod_mc`` on the device: out (bhi1 - blo1, bhi0 - blo0, nz) += the Monte-Carlo model."""
    _out64(out)
    nz = out.shape[2]
    c = _grid_ctx(bhi0, bhi1, nz, radsep, cdens, cmode, pixarea, cdelt0, cdelt1, crota2, ltype, sig_instr, axtyp,
                  velsys, lfreq0, crval3, cdelt3, crpix3, relint, cd2i)
    sr = np.ascontiguousarray(sr, np.float64)
    nv = np.ascontiguousarray(nv, np.int64)
    c.check(c.L.bbgpu_galmod_mc(c.h, _lib.ptr(out), _lib.ptr(sr), sr.shape[1], int(ring_lo), int(ring_hi),
                                int(seed) & 0xFFFFFFFFFFFFFFFF, _lib.ptr(nv), int(blo0), int(blo1), int(bhi0),
                                int(bhi1)))
    return out


def galmod_analytic(out, sr, ring_lo, ring_hi, radsep, cdens, pixarea, cdelt0, cdelt1, crota2, blo0, blo1, bhi0,
                    bhi1, ltype, sig_instr, vedges, relint, cd2i, nzq, axtyp, velsys, lfreq0, crval3, cdelt3, crpix3,
                    chwidth, ptab, zstep):
    """``_galmod_analytic`` on the device (ptab: the reference's table of the normal CDF; the device has its own,
    computed with the same formula)."""
    _out64(out)
    nz = out.shape[2]
    c = _grid_ctx(bhi0, bhi1, nz, radsep, cdens, 1, pixarea, cdelt0, cdelt1, crota2, ltype, sig_instr, axtyp,
                  velsys, lfreq0, crval3, cdelt3, crpix3, relint, cd2i, chwidth, zstep, vedges)
    sr = np.ascontiguousarray(sr, np.float64)
    c.check(c.L.bbgpu_galmod_analytic(c.h, _lib.ptr(out), _lib.ptr(sr), sr.shape[1], int(ring_lo), int(ring_hi),
                                      int(nzq), int(blo0), int(blo1), int(bhi0), int(bhi1)))
    return out


def ring_maps_analytic(out, sr, widx, wval, radsep, pixarea, cdelt0, cdelt1, crota2, blo0, blo1, bhi0, bhi1, ltype,
                       nzq, sig_instr, chwidth, zstep):
    """``_ring_maps_analytic`` on the device: out (nr, by, bx) += the maps of the rings."""
    _out64(out)
    c = _grid_ctx(bhi0, bhi1, 1, radsep, 0., 1, pixarea, cdelt0, cdelt1, crota2, ltype, sig_instr, 4, 1, [0.], 0.,
                  1., 1., [1.], [1.], chwidth, zstep)
    sr = np.ascontiguousarray(sr, np.float64)
    widx = np.ascontiguousarray(widx, np.int64)
    wval = np.ascontiguousarray(wval, np.float64)
    c.check(c.L.bbgpu_ring_maps_analytic(c.h, _lib.ptr(out), out.shape[0], _lib.ptr(sr), sr.shape[1], _lib.ptr(widx),
                                         _lib.ptr(wval), int(nzq), int(blo0), int(blo1), int(bhi0), int(bhi1)))
    return out


def galmod_wind(out, sr, ring_lo, ring_hi, seed, sep, nv, cdens, cmode, pixarea, cdelt0, cdelt1, crota2, blo0, blo1,
                bhi0, bhi1, sig_instr, axtyp, velsys, lfreq0, crval3, cdelt3, crpix3, relint, cd2i):
    """``_galmod_wind`` on the device (GALWIND WTYPE 1): out (bhi1 - blo1, bhi0 - blo0, nz) += the clouds of the
    shells [ring_lo, ring_hi) of sr (11, nsub)."""
    _out64(out)
    nz = out.shape[2]
    c = _grid_ctx(bhi0, bhi1, nz, sep, cdens, cmode, pixarea, cdelt0, cdelt1, crota2, 1, sig_instr, axtyp, velsys,
                  lfreq0, crval3, cdelt3, crpix3, relint, cd2i)
    sr = np.ascontiguousarray(sr, np.float64)
    nv = np.ascontiguousarray(nv, np.int64)
    c.check(c.L.bbgpu_galmod_wind(c.h, _lib.ptr(out), _lib.ptr(sr), sr.shape[1], int(ring_lo), int(ring_hi),
                                  int(seed) & 0xFFFFFFFFFFFFFFFF, float(sep), _lib.ptr(nv), int(blo0), int(blo1),
                                  int(bhi0), int(bhi1)))
    return out


def _plain_ctx():
    d = _ctxs()
    c = d.get("plain")
    if c is None:
        c = d["plain"] = _lib.Context(0)
    return c


def conv_sparse(model, kern, scale):
    """``_conv_sparse`` on the device (bit-exact)."""
    from .galfit import _conv_sparse
    return _conv_sparse(model, kern, scale, ctx=_plain_ctx())


def norm(model, data, mask, blo0, blo1, x0, y0, phi, inc, r1, r2, wpow, side, ftype, chan_noise, data_noise, bweight,
         normtype, pre, ilo, ihi, thr, P, foot, hmax):
    """``_norm`` on the device (the model normalised in place)."""
    from .galfit import _norm
    return _norm(model, data, mask, blo0, blo1, x0, y0, phi, inc, r1, r2, wpow, side, ftype, chan_noise, data_noise,
                 bweight, normtype, pre, ilo, ihi, thr, P, foot, hmax, ctx=_plain_ctx())


def _resid(model, data, mask, maskmode, region, sigma2, eps2):
    c = _plain_ctx()
    m = np.ascontiguousarray(model, np.float64)
    d = np.ascontiguousarray(data, np.float32)
    k = np.ascontiguousarray(mask if mask is not None else d, dtype=bool).view(np.uint8)
    nz, ny, nx = m.shape
    r = None if region is None or np.asarray(region).size == 0 else np.ascontiguousarray(region, dtype=bool).view(np.uint8)
    if eps2 > 0:
        out = np.zeros(2)
        c.check(c.L.bbgpu_residuals_fracerr(c.h, _lib.ptr(m), _lib.ptr(d), _lib.ptr(k), int(maskmode), _lib.ptr(r), nz,
                                            ny, nx, float(sigma2), float(eps2), _lib.ptr(out)))
        return float(out[0]), float(out[1])
    out = np.zeros(1)
    c.check(c.L.bbgpu_sumsq_residuals(c.h, _lib.ptr(m), _lib.ptr(d), _lib.ptr(k), int(maskmode), _lib.ptr(r), nz, ny,
                                      nx, _lib.ptr(out)))
    return float(out[0])


def sumsq_residuals(model, data, mask, maskmode, region):
    """``_sumsq_residuals`` on the device (float64 sums)."""
    return _resid(model, data, mask, maskmode, region, 1.0, 0.0)


def residuals_fracerr(model, data, mask, maskmode, region, sigma2, eps2):
    """``_residuals_fracerr`` on the device: (sum r^2 / v, sum log(v / sigma^2))."""
    return _resid(model, data, mask, maskmode, region, sigma2, eps2)


def FFTConvolver_call(self, data, workers=None):
    """``FFTConvolver.__call__`` on the device: the "same" convolution of each plane of data ((n,) ny, nx) with the
    convolver's kernel (float32 accumulation, within 1e-6 of the peak of the float64 result)."""
    kern = np.ascontiguousarray(getattr(self, "kernel", getattr(self, "k", None)), np.float64)
    a = np.ascontiguousarray(data, np.float64)
    if a.ndim == 2:
        return FFTConvolver_call(self, a[None], workers)[0]
    nz, ny, nx = a.shape
    c = _plain_ctx()
    key = ("kern", kern.tobytes(), kern.shape, ny, nx)
    if getattr(c, "_kern_key", None) != key:
        g = _lib.Grid()
        g.nx, g.ny, g.nz, g.nlines = nx, ny, max(nz, 1), 1
        g.axtyp, g.velsys, g.ltype, g.cmode = 4, 1, 1, 1
        g.radsep, g.cdens, g.pixarea, g.cdelt0, g.cdelt1, g.cdelt3 = 1., 1., 1., 1., 1., 1.
        one = np.ones(max(nz, 1))
        c.check(c.L.bbgpu_set_grid(c.h, g, _lib.ptr(one), _lib.ptr(np.zeros(1)), _lib.ptr(np.ones(1)), None))
        c.check(c.L.bbgpu_set_kernel(c.h, _lib.ptr(kern), kern.shape[0], kern.shape[1]))
        c._kern_key = key
    out = np.empty_like(a)
    c.check(c.L.bbgpu_convolve(c.h, _lib.ptr(a), _lib.ptr(out), nz, ny, nx, 1.0, 0))
    return out


# the reference functions each replacement takes the place of: (module, attribute, replacement)
SEAMS = (("bbarolo.galmod", "_galmod_mc", galmod_mc),
         ("bbarolo.galmod", "_galmod_analytic", galmod_analytic),
         ("bbarolo.galmod", "_ring_maps_analytic", ring_maps_analytic),
         ("bbarolo.galmod", "_conv_sparse", conv_sparse),
         ("bbarolo.galfit", "_norm", norm),
         ("bbarolo.bayesian.likelihood", "_sumsq_residuals", sumsq_residuals),
         ("bbarolo.bayesian.likelihood", "_residuals_fracerr", residuals_fracerr),
         ("bbarolo.galmod", "_galmod_wind", galmod_wind),
         ("bbarolo.galwind", "_galmod_wind", galmod_wind))


def _wind_classes():
    from . import wind
    return {"WindModel": wind.WindModel, "WindCells": wind.WindCells, "WindPars": wind.WindPars, "Boxes": wind.Boxes}


WIND_MODULES = ("bbarolo.windmodel", "bbarolo.bayesian.wind")

_saved = {}


def install(modules=None):
    """Bind the device kernels in place of the reference's (in ``sys.modules`` or the given {name: module}),
    and ``FFTConvolver.__call__`` of ``bbarolo.smooth``. Returns the list of (module, attribute) replaced."""
    mods = sys.modules if modules is None else modules
    done = []
    for mname, attr, fn in SEAMS:
        m = mods.get(mname)
        if m is None or not hasattr(m, attr):
            continue
        _saved.setdefault((mname, attr), getattr(m, attr))
        setattr(m, attr, fn)
        done.append((mname, attr))
    sm = mods.get("bbarolo.smooth")
    if sm is not None and hasattr(sm, "FFTConvolver"):
        cls = sm.FFTConvolver
        _saved.setdefault(("bbarolo.smooth", "FFTConvolver.__call__"), cls.__call__)
        cls.__call__ = FFTConvolver_call
        done.append(("bbarolo.smooth", "FFTConvolver.__call__"))
    for mname in WIND_MODULES:
        m = mods.get(mname)
        if m is None:
            continue
        for attr, cls in _wind_classes().items():
            if hasattr(m, attr):
                _saved.setdefault((mname, attr), getattr(m, attr))
                setattr(m, attr, cls)
                done.append((mname, attr))
    return done


def uninstall(modules=None):
    """Restore the reference's functions replaced by ``install``."""
    mods = sys.modules if modules is None else modules
    for (mname, attr), fn in list(_saved.items()):
        m = mods.get(mname)
        if m is None:
            continue
        if attr == "FFTConvolver.__call__":
            m.FFTConvolver.__call__ = fn
        else:
            setattr(m, attr, fn)
        del _saved[(mname, attr)]
