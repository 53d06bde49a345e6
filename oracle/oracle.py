"""Python access to the CPU oracle (``oracle/bbref.c``): the reference kernels restated in plain C.

TEST INFRASTRUCTURE. Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` use
this module, as the checker of the GPU path. The product (``bbarolo2_gb300``) never imports it.

Each wrapper takes numpy arrays with the reference's layouts and argument meaning
(``bbarolo/galmod.py``, ``bbarolo/galfit.py``, ``bbarolo/bayesian/likelihood.py``) and returns what the
reference kernel returns.
"""

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
_lib = None

_d = C.c_double
_i = C.c_int
_i64 = C.c_int64
_u64 = C.c_uint64
_p = C.c_void_p


def build(force=False):
    """Compiles the oracle library (make in oracle/)."""
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(os.path.join(HERE, "bbref.c")):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        L.ref_rng_next.restype = _u64
        L.ref_rng_uniform.restype = _d
        L.ref_rng_normal.restype = _d
        L.ref_sumsq_residuals.restype = _d
        L.ref_norm.restype = _d
        L.ref_zgrid.restype = _i
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(_p) if a is not None else None


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class RNG:
    """The reference's xoroshiro128+ / ziggurat stream (``bbarolo/_rng.py``)."""

    def __init__(self, seed):
        self.s = np.zeros(2, np.uint64)
        lib().ref_rng_init(_u64(int(seed) & 0xFFFFFFFFFFFFFFFF), _ptr(self.s))

    def next(self):
        return int(lib().ref_rng_next(_ptr(self.s)))

    def uniform(self):
        return float(lib().ref_rng_uniform(_ptr(self.s)))

    def normal(self):
        return float(lib().ref_rng_normal(_ptr(self.s)))


def zig_tables():
    kn = np.zeros(128, np.int64)
    wn = np.zeros(128)
    fn = np.zeros(128)
    lib().ref_zig_tables(_ptr(kn), _ptr(wn), _ptr(fn))
    return kn, wn, fn


def phi_table():
    t = np.zeros(6146)
    lib().ref_phi_table(_ptr(t))
    return t


def galmod_mc(out, sr, ring_lo, ring_hi, seed, radsep, nv, cdens, cmode, pixarea, cdelt0, cdelt1, crota2,
              blo0, blo1, bhi0, bhi1, ltype, sig_instr, axtyp, velsys, lfreq0, crval3, cdelt3, crpix3, relint,
              cd2i):
    """``bbarolo/galmod.py:92-171`` with the same arguments; out (ny, nx, nz) float64 is accumulated."""
    assert out.dtype == np.float64 and out.flags.c_contiguous
    sr = _f64(sr)
    nv = np.ascontiguousarray(nv, np.int64)
    lf, ri, cd = _f64(lfreq0), _f64(relint), _f64(cd2i)
    ny, nx, nz = out.shape
    lib().ref_galmod_mc(_ptr(out), _i(ny), _i(nx), _i(nz), _ptr(sr), _i(sr.shape[1]), _i(ring_lo), _i(ring_hi),
                        _u64(int(seed)), _d(radsep), _ptr(nv), _d(cdens), _i(int(cmode)), _d(pixarea), _d(cdelt0),
                        _d(cdelt1), _d(crota2), _i64(blo0), _i64(blo1), _i64(bhi0), _i64(bhi1), _i(int(ltype)),
                        _d(sig_instr), _i(int(axtyp)), _i(int(velsys)), _i(lf.size), _ptr(lf), _d(crval3),
                        _d(cdelt3), _d(crpix3), _ptr(ri), _ptr(cd))
    return out


def galmod_analytic(out, sr, ring_lo, ring_hi, radsep, cdens, pixarea, cdelt0, cdelt1, crota2, blo0, blo1, bhi0,
                    bhi1, ltype, sig_instr, vedges, relint, cd2i, nzq, axtyp, velsys, lfreq0, crval3, cdelt3,
                    crpix3, chwidth, ptab=None, zstep=0.25):
    """``bbarolo/galmod.py:326-465`` with the same arguments (ptab: the oracle's own table)."""
    assert out.dtype == np.float64 and out.flags.c_contiguous
    sr = _f64(sr)
    ve = _f64(vedges)
    lf, ri, cd = _f64(lfreq0), _f64(relint), _f64(cd2i)
    ny, nx, nz = out.shape
    lib().ref_galmod_analytic(_ptr(out), _i(ny), _i(nx), _i(nz), _ptr(sr), _i(sr.shape[1]), _i(ring_lo),
                              _i(ring_hi), _d(radsep), _d(cdens), _d(pixarea), _d(cdelt0), _d(cdelt1), _d(crota2),
                              _i64(blo0), _i64(blo1), _i64(bhi0), _i64(bhi1), _i(int(ltype)), _d(sig_instr),
                              _ptr(ve), _ptr(ri), _ptr(cd), _i(int(nzq)), _i(int(axtyp)), _i(int(velsys)),
                              _i(lf.size), _ptr(lf), _d(crval3), _d(cdelt3), _d(crpix3), _d(chwidth), _d(zstep))
    return out


def ring_maps_analytic(out, sr, widx, wval, radsep, pixarea, cdelt0, cdelt1, crota2, blo0, blo1, bhi0, bhi1, ltype,
                       nzq, sig_instr, chwidth, zstep):
    """``bbarolo/galmod.py:468-536``; out (nr, ny, nx) float64 accumulated."""
    assert out.dtype == np.float64 and out.flags.c_contiguous
    sr = _f64(sr)
    widx = np.ascontiguousarray(widx, np.int64)
    wval = _f64(wval)
    nr, ny, nx = out.shape
    lib().ref_ring_maps_analytic(_ptr(out), _i(nr), _i(ny), _i(nx), _ptr(sr), _i(sr.shape[1]), _ptr(widx),
                                 _ptr(wval), _d(radsep), _d(pixarea), _d(cdelt0), _d(cdelt1), _d(crota2),
                                 _i64(blo0), _i64(blo1), _i64(bhi0), _i64(bhi1), _i(int(ltype)), _i(int(nzq)),
                                 _d(sig_instr), _d(chwidth), _d(zstep))
    return out


def conv_same(a, kernel, scale=1.0, threshold=True):
    """FP64 "same" convolution of each plane of a (nz, ny, nx) array (the FFT convolution of the reference
    computed directly), then values < 1e-12 set to zero and the scale factor (``DiskModel.convolve``)."""
    a = _f64(a)
    k = _f64(kernel)
    if a.ndim == 2:
        return conv_same(a[None], k, scale, threshold)[0]
    out = np.empty_like(a)
    nz, ny, nx = a.shape
    lib().ref_conv_same(_ptr(a), _ptr(out), _i(nz), _i(ny), _i(nx), _ptr(k), _i(k.shape[0]), _i(k.shape[1]),
                        _d(scale), _i(1 if threshold else 0))
    return out


def conv_sparse(model, kern, scale):
    """``bbarolo/galmod.py:974-1037``: model (ny, nx, nz) -> convolved (ny, nx, nz)."""
    m = _f64(model)
    k = _f64(kern)
    out = np.zeros_like(m)
    ny, nx, nz = m.shape
    lib().ref_conv_sparse(_ptr(m), _ptr(out), _i(ny), _i(nx), _i(nz), _ptr(k), _i(k.shape[0]), _i(k.shape[1]),
                          _d(scale))
    return out


def _region_arg(region, shape):
    if region is None or np.asarray(region).size == 0:
        return None
    r = np.ascontiguousarray(region, np.uint8)
    assert r.shape == shape
    return r


def sumsq_residuals(model, data, mask, maskmode, region):
    """``bbarolo/bayesian/likelihood.py:22-45``."""
    m = _f64(model)
    d = np.ascontiguousarray(data, np.float32)
    k = np.ascontiguousarray(mask if mask is not None else d, dtype=bool).view(np.uint8)
    nz, ny, nx = m.shape
    r = _region_arg(region, (ny, nx))
    return float(lib().ref_sumsq_residuals(_ptr(m), _ptr(d), _ptr(k), _i(int(maskmode)), _ptr(r), _i(nz), _i(ny),
                                           _i(nx)))


def residuals_fracerr(model, data, mask, maskmode, region, sigma2, eps2):
    """``bbarolo/bayesian/likelihood.py:48-77``: (sum r^2/v, sum log(v/sigma^2))."""
    m = _f64(model)
    d = np.ascontiguousarray(data, np.float32)
    k = np.ascontiguousarray(mask if mask is not None else d, dtype=bool).view(np.uint8)
    nz, ny, nx = m.shape
    r = _region_arg(region, (ny, nx))
    out = np.zeros(2)
    lib().ref_residuals_fracerr(_ptr(m), _ptr(d), _ptr(k), _i(int(maskmode)), _ptr(r), _i(nz), _i(ny), _i(nx),
                                _d(sigma2), _d(eps2), _ptr(out))
    return float(out[0]), float(out[1])


def norm(model, data, mask, blo0, blo1, x0, y0, phi, inc, r1, r2, wpow, side, ftype, chan_noise, data_noise,
         bweight, normtype, pre, ilo, ihi, thr, P, foot, hmax):
    """``bbarolo/galfit.py:39-188`` (model modified in place, as the reference); P is ignored (own buffer)."""
    assert model.dtype == np.float64 and model.flags.c_contiguous
    d = np.ascontiguousarray(data, np.float32)
    k = np.ascontiguousarray(mask, dtype=bool).view(np.uint8)
    bsy, bsx, nz = model.shape
    dny, dnx, _ = d.shape
    pre_ = None if pre is None or np.asarray(pre).size == 0 else _f64(pre)
    ilo = np.ascontiguousarray(ilo, np.int64)
    ihi = np.ascontiguousarray(ihi, np.int64)
    thr = _f64(thr) if np.asarray(thr).size else np.zeros(max(nz, 1))
    cn = _f64(chan_noise)
    return float(lib().ref_norm(_ptr(model), _i(bsy), _i(bsx), _i(nz), _ptr(d), _ptr(k), _i(dny), _i(dnx),
                                _i64(blo0), _i64(blo1), _d(x0), _d(y0), _d(phi), _d(inc), _d(r1), _d(r2), _d(wpow),
                                _i(int(side)), _i(int(ftype)), _ptr(cn), _d(data_noise), _d(bweight),
                                _i(int(normtype)), _ptr(pre_), _ptr(ilo), _ptr(ihi), _i(ilo.size), _ptr(thr),
                                _i(int(foot)), _d(hmax)))


# ---------------------------------------------------------------------------------------------- wind models
def _ai64(a):
    return np.ascontiguousarray(a, dtype=np.int64)


def wind_points(cells, qn, qoff, radii, vw, vd, vr, x0, y0, vsys, sinc, cinc, spa, cpa, cd0, cd1, th_in, th_out,
                rmax, sig_instr):
    """``bbarolo/windmodel.py:225-288``: a dict of gx, gy, vel, sig, w, r (per point) and vol, rbar (per cell)."""
    cells, qn, qoff = _f64(cells), _ai64(qn), _ai64(qoff)
    rs = [_f64(a) for a in (radii, vw, vd, vr)]
    n, m = int(qoff[-1]), cells.shape[0]
    out = {k: np.empty(n) for k in ("gx", "gy", "vel", "sig", "w", "r")}
    out.update(vol=np.empty(m), rbar=np.empty(m))
    lib().ref_wind_points(_ptr(cells), _ptr(qn), _ptr(qoff), _i(m), *[_ptr(a) for a in rs], _i(rs[0].size),
                          *[_d(v) for v in (x0, y0, vsys, sinc, cinc, spa, cpa, cd0, cd1, th_in, th_out, rmax,
                                            sig_instr)],
                          *[_ptr(out[k]) for k in ("gx", "gy", "vel", "sig", "w", "r", "vol", "rbar")])
    return out


def _spec_args(chmin, axtyp, velsys, lfreq0, crval3, cdelt3, crpix3):
    lf = _f64(lfreq0)
    return lf, [_d(chmin), _i(int(axtyp)), _i(int(velsys)), _i(lf.size), _ptr(lf), _d(crval3), _d(cdelt3),
                _d(crpix3)]


def wind_raw_boxes(qoff, gx, gy, vel, sig, w, lim, chmin, axtyp, velsys, lfreq0, crval3, cdelt3, crpix3):
    """``bbarolo/windmodel.py:291-319``: the raw boxes (ncell, 6) of the points within lim."""
    qoff = _ai64(qoff)
    pts = [_f64(a) for a in (gx, gy, vel, sig, w)]
    lim = _ai64(lim)
    out = np.empty((qoff.size - 1, 6), dtype=np.int64)
    lf, spec = _spec_args(chmin, axtyp, velsys, lfreq0, crval3, cdelt3, crpix3)
    lib().ref_wind_raw_boxes(_ptr(qoff), _i(qoff.size - 1), *[_ptr(a) for a in pts], _ptr(lim), *spec, _ptr(out))
    return out


def wind_deposit_raw(rbuf, roffs, rboxes, qoff, gx, gy, vel, sig, w, vedges, relint, cd2i, chmin, axtyp, velsys,
                     lfreq0, crval3, cdelt3, crpix3, nz):
    """``bbarolo/windmodel.py:322-366``: rbuf (float64) accumulated."""
    assert rbuf.dtype == np.float64 and rbuf.flags.c_contiguous
    roffs, rboxes, qoff = _ai64(roffs), _ai64(rboxes), _ai64(qoff)
    pts = [_f64(a) for a in (gx, gy, vel, sig, w)]
    ve, ri, cd = _f64(vedges), _f64(relint), _f64(cd2i)
    lf, spec = _spec_args(chmin, axtyp, velsys, lfreq0, crval3, cdelt3, crpix3)
    lib().ref_wind_deposit_raw(_ptr(rbuf), _ptr(roffs), _ptr(rboxes), _ptr(qoff), _i(qoff.size - 1),
                               *[_ptr(a) for a in pts], _ptr(ve), _ptr(ri), _ptr(cd), *spec, _i(int(nz)))
    return rbuf


def wind_convolve_boxes(rbuf, roffs, rboxes, kern, kx, ky, separable, buf, offs, boxes):
    """``bbarolo/windmodel.py:369-423``: buf (float64) accumulated."""
    assert buf.dtype == np.float64 and buf.flags.c_contiguous
    kern = _f64(kern)
    hy, hx = kern.shape[0] // 2, kern.shape[1] // 2
    lib().ref_wind_convolve_boxes(_ptr(_f64(rbuf)), _ptr(_ai64(roffs)), _ptr(_ai64(rboxes)), _i(len(roffs) - 1),
                                  _ptr(kern), _i(hy), _i(hx), _ptr(_f64(kx)), _ptr(_f64(ky)), _i(int(bool(separable))),
                                  _ptr(buf), _ptr(_ai64(offs)), _ptr(_ai64(boxes)))
    return buf


def wind_normal(buf, offs, boxes, wd, wm, lim, rel=0.):
    """``bbarolo/windmodel.py:477-554`` (voxel lists, then the normal equations): (G, b)."""
    wd, wm = _f64(wd), _f64(wm)
    n = len(offs) - 1
    G, b = np.empty((n, n)), np.empty(n)
    lib().ref_wind_normal(_ptr(_f64(buf)), _ptr(_ai64(offs)), _ptr(_ai64(boxes)), _i(n), _ptr(wd), _ptr(wm),
                          _i(wm.shape[1]), _i(wm.shape[2]), _ptr(_ai64(lim)), _d(rel), _ptr(G), _ptr(b))
    return G, b


def wind_scatter(shape, buf, offs, boxes, amp):
    """``bbarolo/windmodel.py:584-602``: the model (nz, ny, nx) of the columns with amplitudes amp."""
    out = np.zeros(shape)
    lib().ref_wind_scatter(_ptr(out), _i(shape[1]), _i(shape[2]), _ptr(_f64(buf)), _ptr(_ai64(offs)),
                           _ptr(_ai64(boxes)), _i(len(offs) - 1), _ptr(_f64(amp)))
    return out


def _offsets(boxes):
    size = (boxes[:, 1] - boxes[:, 0]) * (boxes[:, 3] - boxes[:, 2]) * (boxes[:, 5] - boxes[:, 4])
    return np.concatenate([[0], np.cumsum(np.maximum(size, 0))]).astype(np.int64)


def wind_boxes(pts, w, lim, shape, kern, kx, ky, separable, spec, vedges, relint, qoff):
    """The columns of the points (``WindModel.boxes``, ``bbarolo/windmodel.py:829-859``): the raw boxes within lim
    grown by the beam, the bilinear deposit, then the boxes grown by the beam and clipped to lim and the convolution.
    spec: dict of chmin, axtyp, velsys, lfreq0, crval3, cdelt3, crpix3. Returns (buf, offs, boxes)."""
    lim = _ai64(lim)
    hy, hx = kern.shape[0] // 2, kern.shape[1] // 2
    rlim = lim + np.array([-hx, hx, -hy, hy, 0, 0])
    sp = (spec["chmin"], spec["axtyp"], spec["velsys"], spec["lfreq0"], spec["crval3"], spec["cdelt3"],
          spec["crpix3"])
    rboxes = wind_raw_boxes(qoff, pts["gx"], pts["gy"], pts["vel"], pts["sig"], w, rlim, *sp)
    roffs = _offsets(rboxes)
    rbuf = np.zeros(int(roffs[-1]))
    wind_deposit_raw(rbuf, roffs, rboxes, qoff, pts["gx"], pts["gy"], pts["vel"], pts["sig"], w, vedges, relint,
                     np.ones(shape[0]), *sp, shape[0])
    if hx == 0 and hy == 0:
        return rbuf, roffs, np.clip(rboxes, np.repeat(lim[::2], 2), np.repeat(lim[1::2], 2))
    boxes = rboxes + np.array([-hx, hx, -hy, hy, 0, 0])
    boxes[:, 0:2] = np.clip(boxes[:, 0:2], lim[0], lim[1])
    boxes[:, 2:4] = np.clip(boxes[:, 2:4], lim[2], lim[3])
    empty = (rboxes[:, 1] <= rboxes[:, 0]) | (boxes[:, 1] <= boxes[:, 0]) | (boxes[:, 3] <= boxes[:, 2])
    boxes[empty] = (lim[0], lim[0], lim[2], lim[2], lim[4], lim[4])
    offs = _offsets(boxes)
    buf = np.zeros(int(offs[-1]))
    wind_convolve_boxes(rbuf, roffs, rboxes, kern, kx, ky, separable, buf, offs, boxes)
    return buf, offs, boxes


def galmod_wind(out, sr, ring_lo, ring_hi, seed, sep, nv, cdens, cmode, pixarea, cdelt0, cdelt1, crota2, blo0,
                blo1, bhi0, bhi1, sig_instr, axtyp, velsys, lfreq0, crval3, cdelt3, crpix3, relint, cd2i):
    """``bbarolo/galmod.py:539-590`` with the same arguments; out (ny, nx, nz) float64 is accumulated."""
    assert out.dtype == np.float64 and out.flags.c_contiguous
    sr = _f64(sr)
    nv = np.ascontiguousarray(nv, np.int64)
    lf, ri, cd = _f64(lfreq0), _f64(relint), _f64(cd2i)
    ny, nx, nz = out.shape
    lib().ref_galmod_wind(_ptr(out), _i(ny), _i(nx), _i(nz), _ptr(sr), _i(sr.shape[1]), _i(ring_lo), _i(ring_hi),
                          _u64(int(seed)), _d(sep), _ptr(nv), _d(cdens), _i(int(cmode)), _d(pixarea), _d(cdelt0),
                          _d(cdelt1), _d(crota2), _i64(blo0), _i64(blo1), _i64(bhi0), _i64(bhi1), _d(sig_instr),
                          _i(int(axtyp)), _i(int(velsys)), _i(lf.size), _ptr(lf), _d(crval3), _d(cdelt3), _d(crpix3),
                          _ptr(ri), _ptr(cd))
    return out
