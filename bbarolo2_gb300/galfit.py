"""The CLASSIC 3DFIT kernels on the device, with the reference's signatures.

``_conv_sparse(model, kern, scale)`` mirrors ``bbarolo/galmod.py:974-1037`` and ``_norm(model, data, mask, ...)``
mirrors ``bbarolo/galfit.py:39-188`` (the model is scaled in place, as the reference; the work array ``P`` is
accepted and ignored: the device keeps its own running sums). Both run on the GPU through ``libbbgpu.so``:
the reference's float64 arithmetic, ``_conv_sparse`` bit-exact, ``_norm`` with the same ring footprint, factors
and blank counts and its residual sum reduced in a fixed tree (rounding differences only).
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


# ------------------------------------------------------------------------------------------- CLASSIC driver
VROT, VDISP, DENS, Z0, INC, PA, XPOS, YPOS, VSYS, VRAD, MAXPAR = range(11)
NORMCODE = {"LOCAL": 0, "AZIM": 1, "NONE": 2}
SIDECODE = {"R": 1, "A": 2}


def _count_ring_pixels(mask2D, blo0, blo1, bhi0, bhi1, x0, y0, phi, inc, r1, r2):
    """(pixels of the ring's annulus in the box [blo, bhi] inclusive, those with mask), as
    ``bbarolo/galfit.py:198-216`` (the same float64 expressions, elementwise)."""
    import math
    F = math.pi / 180.
    sphi, cphi, cinc = math.sin(F * phi), math.cos(F * phi), math.cos(F * inc)
    y, x = np.mgrid[blo1:bhi1 + 1, blo0:bhi0 + 1]
    xx = (x - blo0).astype(np.float64)
    yy = (y - blo1).astype(np.float64)
    xr = -(xx - x0) * sphi + (yy - y0) * cphi
    yr = (-(xx - x0) * cphi - (yy - y0) * sphi) / cinc
    r = np.sqrt(xr * xr + yr * yr)
    ring = (r >= r1) & (r <= r2)
    ny, nx = mask2D.shape
    inside = (y < ny) & (x < nx)
    m = np.zeros(ring.shape, bool)
    m[inside] = mask2D[y[inside], x[inside]] > 0
    return int(ring.sum()), int((ring & m).sum())


class Galfit:
    """The CLASSIC 3DFIT of single rings (``bbarolo/galfit.py:455-1238``): each ring fitted alone by the downhill
    simplex of the reference (``minimize``, ``_mtry``, ``func3D`` with its bounds and seeded redraws), its model
    built and convolved on the device (``DiskModel.array(final=False)``: MC GALMOD and ``_conv_sparse``) and
    normalised against the data by ``_norm`` on the device. One stage with one thread (the rings in order): the
    REVERSE passes, the second stage, the errors and the outputs of the reference are outside this path.

    cube: a ``Cube`` (data array and header); inrings: the initial ``Rings``; par: the 3DFIT parameters (FREE,
    DELTAVROT, DELTAINC, DELTAPHI, MINVDISP, MAXVDISP, TOL, FTYPE, WFUNC, SIDE, BWEIGHT, NORM, NORMALCUBE,
    STARTRAD and the GALMOD ones); data_noise: the noise of the data (the reference's cube statistics);
    mask (nz, ny, nx) bool; chan_noise (nz) (default ones)."""

    CS_NONE, CS_OK, CS_FAILED = 0, 1, 2

    def __init__(self, cube, inrings, par, data_noise, mask, chan_noise=None, device=0):
        import threading
        from .engine import DiskModel
        from .galmod import arcsconv
        self.cin = cube
        self.par = par
        self.inr = inrings.copy()
        self.verb = 0
        h = cube.Head()
        self.arcconv = arcsconv(h.Cunit(0))
        nz = cube.DimZ()
        self.chan_noise = np.ones(nz) if chan_noise is None else np.asarray(chan_noise, np.float64)
        self.data_noise = float(data_noise)
        self.wpow = par.WFUNC
        self.setFree()
        self.mask = np.asarray(mask, bool)
        self.mask_T = np.ascontiguousarray(self.mask.transpose(1, 2, 0))
        self.mask2D = self.mask.sum(axis=0).astype(np.int32)
        norms = ["AZIM" if n == "AZIMUTHAL" else n for n in par.NORM.split()]
        if len(norms) == 1:
            norms.append(norms[0])
        for i in range(2):
            if norms[i] not in ("NONE", "AZIM", "LOCAL"):
                norms[i] = "LOCAL"
        if len(norms) == 2:
            norms.append(norms[1])
        self.norms = norms
        inr = self.inr
        self.maxs, self.mins = np.zeros(MAXPAR), np.zeros(MAXPAR)
        self.maxs[VROT] = inr.vrot.max() + par.DELTAVROT
        self.mins[VROT] = inr.vrot.min() - par.DELTAVROT
        self.maxs[VDISP], self.mins[VDISP] = par.MAXVDISP, par.MINVDISP
        self.maxs[Z0], self.mins[Z0] = 1000, 0.
        self.maxs[INC] = inr.inc.max() + par.DELTAINC
        self.mins[INC] = inr.inc.min() - par.DELTAINC
        self.maxs[PA] = inr.phi.max() + par.DELTAPHI
        self.mins[PA] = inr.phi.min() - par.DELTAPHI
        self.mins[VROT] = max(self.mins[VROT], 0)
        self.maxs[INC] = min(self.maxs[INC], 90)
        self.mins[INC] = max(self.mins[INC], 0)
        self.maxs[PA] = min(self.maxs[PA], 360)
        self.mins[PA] = max(self.mins[PA], -360)
        self.maxs[XPOS] = min(inr.xpos.max() + 10, cube.DimX())
        self.mins[XPOS] = max(inr.xpos.min() - 10, 0)
        self.maxs[YPOS] = min(inr.ypos.max() + 10, cube.DimY())
        self.mins[YPOS] = max(inr.ypos.min() - 10, 0)
        self.maxs[VRAD], self.mins[VRAD] = 500, -500
        self.model = DiskModel(cube, par=par, densflux=True, device=device)
        self.ctx = self.model.ctx
        self.outr = self.inr.copy()
        self.pixScale = ((abs(h.Cdelt(0)) * self.arcconv) + (abs(h.Cdelt(1)) * self.arcconv)) / 2.
        self.data_T = np.ascontiguousarray(np.asarray(cube.array, np.float32).transpose(1, 2, 0))
        self.n_galfit = 0
        self._pass = 0
        self._rngs, self._tls, self._lock = {}, threading.local(), threading.Lock()
        self._ringstat = {}
        self.nfunc = 0

    def setFree(self):
        f = self.par.FREE.lower()
        m = [False] * MAXPAR
        for key, idx in (("vrot", VROT), ("disp", VDISP), ("z0", Z0), ("inc", INC), ("xpos", XPOS), ("ypos", YPOS),
                         ("vsys", VSYS), ("vrad", VRAD)):
            if key in f:
                m[idx] = True
        if "pa" in f or "phi" in f:
            m[PA] = True
        if "all" in f:
            m = [True] * MAXPAR
        if not any(m):
            raise ValueError(" 3DFIT ERROR: NO free parameters!")
        self.mpar = m
        self.nfree = sum(m)

    # ---------------------------------------------------------------------------------- model and residual
    def _make_dring(self, ir, rings=None):
        """The ring ir as fitted (``bbarolo/galfit.py:978-1000``): the annulus halfway to its neighbours."""
        from .rings import Rings
        inr = self.inr
        vr = inr if rings is None else rings
        if inr.nr == 1:
            w1 = w2 = inr.radsep / 2. if inr.radsep > 0 else inr.radii[0] / 2.
        elif ir == 0:
            w1 = w2 = (inr.radii[1] - inr.radii[0]) / 2.
        elif ir == inr.nr - 1:
            w1 = w2 = (inr.radii[ir] - inr.radii[ir - 1]) / 2.
        else:
            w1 = (inr.radii[ir] - inr.radii[ir - 1]) / 2.
            w2 = (inr.radii[ir + 1] - inr.radii[ir]) / 2.
        w1, w2 = np.float32(w1), np.float32(w2)
        drads = [max(float(np.float32(inr.radii[ir] - w1)), 0.), max(float(np.float32(inr.radii[ir] + w2)), 0.)]
        d = Rings()
        d.setRings(radii=drads, xpos=vr.xpos[ir], ypos=vr.ypos[ir], vsys=vr.vsys[ir], vrot=vr.vrot[ir],
                   vdisp=vr.vdisp[ir], vrad=vr.vrad[ir], vvert=vr.vvert[ir], dvdz=vr.dvdz[ir], zcyl=vr.zcyl[ir],
                   dens=vr.dens[ir], z0=vr.z0[ir], inc=vr.inc[ir], phi=vr.phi[ir], z0thick=vr.z0thick[ir],
                   fthick=vr.fthick[ir], vdispthick=vr.vdispthick[ir])
        d.twolayer = vr.thick()
        d.radsep = drads[1] - drads[0]
        d.id = ir
        return d

    def _norm_value(self, dring, model, blo, foot=0, hmax=0.):
        """``Galfit._norm_value`` (``bbarolo/galfit.py:726-734``) with the device ``_norm``."""
        par = self.par
        ps = self.pixScale
        normtype = NORMCODE[self.norms[self.n_galfit - 1]] if self.n_galfit else 0
        return _norm(model, self.data_T, self.mask_T, blo[0], blo[1], dring.xpos[-1] - blo[0],
                     dring.ypos[-1] - blo[1], dring.phi[-1], dring.inc[-1], dring.radii[0] / ps,
                     dring.radii[-1] / ps, float(self.wpow), SIDECODE.get(par.SIDE, 0), par.FTYPE, self.chan_noise,
                     float(self.data_noise), float(par.BWEIGHT), normtype, None, None, None, None, None, foot,
                     float(hmax), ctx=self.ctx)

    def getFuncValue(self, dring):
        """The residual of the model of the ring (convolved with the beam) in its annulus
        (``bbarolo/galfit.py:736-749``, the fit of single rings)."""
        blo, bhi = self.model.box(dring)
        mod = self.model.array(dring, blo, bhi, final=False, layout="yxz")
        self.nfunc += 1
        return self._norm_value(dring, np.ascontiguousarray(mod, np.float64), blo)

    # ---------------------------------------------------------------------------------- minimisation
    def _rng(self):
        import threading
        r = getattr(self._tls, "rng", None)
        if r is not None:
            return r
        tid = threading.get_ident()
        with self._lock:
            r = self._rngs.get(tid)
            if r is None:
                r = np.random.default_rng([12345, len(self._rngs)])
                self._rngs[tid] = r
        return r

    def func3D(self, dring, zpar):
        """The parameters zpar kept within their bounds (redrawn at random inside them, as the reference,
        ``bbarolo/galfit.py:832-886``) set into the ring, then its residual."""
        par, inr, mins, maxs = self.par, self.inr, self.mins, self.maxs
        w = dring.id
        fran = self._rng().random
        vals = dict(vrot=dring.vrot[0], vdisp=dring.vdisp[0], dens=dring.dens[0], z0=dring.z0[0],
                    inc=dring.inc[0], phi=dring.phi[0], xpos=dring.xpos[0], ypos=dring.ypos[0],
                    vsys=dring.vsys[0], vrad=dring.vrad[0])
        np_ = 0
        m = self.mpar
        if m[VROT]:
            minv = max(inr.vrot[w] - par.DELTAVROT, mins[VROT])
            maxv = min(inr.vrot[w] + par.DELTAVROT, maxs[VROT])
            z = zpar[np_]
            if z > maxv:
                v = maxv - fran() * par.DELTAVROT
            elif z < minv:
                v = minv + fran() * par.DELTAVROT
            else:
                v = z
            vals["vrot"] = v
            zpar[np_] = v
            np_ += 1
        if m[VDISP]:
            z = zpar[np_]
            span = min(inr.vdisp[w], maxs[VDISP] - mins[VDISP])
            if z > maxs[VDISP]:
                v = maxs[VDISP] - fran() * span
            elif z < mins[VDISP]:
                v = mins[VDISP] + fran() * span
            else:
                v = z
            vals["vdisp"] = v
            zpar[np_] = v
            np_ += 1
        if m[DENS]:
            z = zpar[np_]
            v = inr.dens[w] if z < 0 else z
            vals["dens"] = v
            zpar[np_] = v
            np_ += 1
        if m[Z0]:
            z = zpar[np_]
            v = inr.z0[w] if (z < mins[Z0] or z > maxs[Z0]) else z
            vals["z0"] = v
            zpar[np_] = v
            np_ += 1
        if m[INC]:
            mini = max(inr.inc[w] - par.DELTAINC, mins[INC])
            maxi = min(inr.inc[w] + par.DELTAINC, maxs[INC])
            z = zpar[np_]
            v = maxi if z > maxi else (mini if z < mini else z)
            vals["inc"] = v
            zpar[np_] = v
            np_ += 1
        if m[PA]:
            minp = max(inr.phi[w] - par.DELTAPHI, mins[PA])
            maxp = min(inr.phi[w] + par.DELTAPHI, maxs[PA])
            z = zpar[np_]
            v = maxp if z > maxp else (minp if z < minp else z)
            vals["phi"] = v
            zpar[np_] = v
            np_ += 1
        for idx, key in ((XPOS, "xpos"), (YPOS, "ypos"), (VSYS, "vsys"), (VRAD, "vrad")):
            if m[idx]:
                z = zpar[np_]
                v = getattr(inr, key)[w] if (z < mins[idx] or z > maxs[idx]) else z
                vals[key] = v
                zpar[np_] = v
                np_ += 1
        for k, v in vals.items():
            getattr(dring, k)[:] = v
        return self.getFuncValue(dring)

    def minimize(self, dring):
        """The downhill simplex of the reference (Nelder & Mead, NR, ``bbarolo/galfit.py:888-962``):
        (converged, minimum, parameters)."""
        TINY = 1.0e-10
        tol = self.par.TOL
        ndim = self.nfree
        NMAX = 200 * ndim
        mpts = ndim + 1
        m = self.mpar
        point, dels = [], []
        if m[VROT]:
            dels.append(30. if dring.vrot[0] > 40 else 5)
            point.append(dring.vrot[0])
        if m[VDISP]:
            v = dring.vdisp[0]
            dels.append(20. if v > 80 else (10. if 20. < v <= 80. else (0.2 if v <= 2 else 5)))
            point.append(v)
        if m[DENS]:
            dels.append(0.2 * dring.dens[0])
            point.append(dring.dens[0])
        if m[Z0]:
            dels.append(0.2 * dring.z0[0])
            point.append(dring.z0[0])
        if m[INC]:
            dels.append(5.)
            point.append(dring.inc[0])
        if m[PA]:
            dels.append(10.)
            point.append(dring.phi[0])
        if m[XPOS]:
            dels.append((self.maxs[XPOS] - self.mins[XPOS]) / 4.)
            point.append(dring.xpos[0])
        if m[YPOS]:
            dels.append((self.maxs[YPOS] - self.mins[YPOS]) / 4.)
            point.append(dring.ypos[0])
        if m[VSYS]:
            dels.append((self.maxs[VSYS] - self.mins[VSYS]) / 4.)
            point.append(dring.vsys[0])
        if m[VRAD]:
            dels.append(25)
            point.append(dring.vrad[0])
        p = np.tile(np.array(point, float), (mpts, 1))
        for i in range(1, mpts):
            p[i, i - 1] += dels[i - 1]
        y = np.empty(mpts)
        for i in range(mpts):
            x = p[i].copy()
            y[i] = self.func3D(dring, x)
        nfunc = 0
        psum = p.sum(axis=0)
        while True:
            ilo = 0
            if y[0] > y[1]:
                ihi, inhi = 0, 1
            else:
                ihi, inhi = 1, 0
            for i in range(mpts):
                if y[i] <= y[ilo]:
                    ilo = i
                if y[i] > y[ihi]:
                    inhi = ihi
                    ihi = i
                elif y[i] > y[inhi] and i != ihi:
                    inhi = i
            rtol = 2.0 * abs(y[ihi] - y[ilo]) / (abs(y[ihi]) + abs(y[ilo]) + TINY)
            if rtol < tol:
                y[0], y[ilo] = y[ilo], y[0]
                p[[0, ilo]] = p[[ilo, 0]]
                return True, float(y[0]), p[0].copy()
            if nfunc >= NMAX:
                return False, float(y[ilo]), p[ilo].copy()
            nfunc += 2
            ytry = self._mtry(dring, p, y, psum, ihi, -1.0)
            if ytry <= y[ilo]:
                ytry = self._mtry(dring, p, y, psum, ihi, 2.0)
            elif ytry >= y[inhi]:
                ysave = y[ihi]
                ytry = self._mtry(dring, p, y, psum, ihi, 0.5)
                if ytry >= ysave:
                    for i in range(mpts):
                        if i != ilo:
                            p[i] = 0.5 * (p[i] + p[ilo])
                            ps_ = p[i].copy()
                            y[i] = self.func3D(dring, ps_)
                    nfunc += ndim
                    psum = p.sum(axis=0)
            else:
                nfunc -= 1

    def _mtry(self, dring, p, y, psum, ihi, fac):
        ndim = self.nfree
        fac1 = (1.0 - fac) / ndim
        fac2 = fac1 - fac
        ptry = psum * fac1 - p[ihi] * fac2
        ytry = self.func3D(dring, ptry)
        if ytry < y[ihi]:
            y[ihi] = ytry
            psum += ptry - p[ihi]
            p[ihi] = ptry
        return ytry

    # ---------------------------------------------------------------------------------- the ring loop
    def _store(self, ir, pmin):
        k = 0
        o = self.outr
        for idx, key in ((VROT, "vrot"), (VDISP, "vdisp"), (DENS, "dens"), (Z0, "z0"), (INC, "inc"),
                         (PA, "phi"), (XPOS, "xpos"), (YPOS, "ypos"), (VSYS, "vsys"), (VRAD, "vrad")):
            if self.mpar[idx]:
                getattr(o, key)[ir] = pmin[k]
                k += 1

    def _max_vrot(self, ir):
        """The largest VROT whose projection still falls in the spectral band (``bbarolo/galfit.py:1066-1074``;
        the band from the channel edges of the model's velocity grid)."""
        import math
        st = self.model.setup
        ve = np.asarray(st._vedges_lines[0], float) / 1000.           # (km/s)
        o = self.outr
        maxv = abs(ve[-1] - o.vsys[ir])
        minv = abs(ve[0] - o.vsys[ir])
        sini = math.sin(o.inc[ir] * math.pi / 180.)
        return max(maxv / sini, minv / sini) if sini != 0 else np.inf

    def _check_vrot(self, ir):
        return self.outr.vrot[ir] <= self._max_vrot(ir)

    def _fit_ring(self, ir, fitok):
        """The fit of ring ir (``bbarolo/galfit.py:1099-1160``) with its seeded generator."""
        seed = [12345, self.n_galfit, ir] + ([self._pass] if self._pass else [])
        self._tls.rng = np.random.default_rng(seed)
        try:
            self._fit_one_ring(ir, fitok)
        finally:
            self._tls.rng = None

    def _fit_one_ring(self, ir, fitok):
        dring = self._make_dring(ir)
        self._cstat[ir] = self.CS_NONE
        blo, bhi = self.model.box(dring)
        ps = self.pixScale
        nTot, nIn = _count_ring_pixels(self.mask2D, blo[0], blo[1], bhi[0], bhi[1], dring.xpos[-1] - blo[0],
                                       dring.ypos[-1] - blo[1], dring.phi[-1], dring.inc[-1], dring.radii[0] / ps,
                                       dring.radii[-1] / ps)
        if nIn < 20 and (nIn == 0 or nIn < 0.7 * nTot):
            self._ringstat[ir] = ("skipped: few pixels in the mask", None)
            fitok[ir] = False
            return
        ok, minimum, pmin = self.minimize(dring)
        fitok[ir] = ok
        self._cstat[ir] = self.CS_OK if ok else self.CS_FAILED
        if not ok:
            self._ringstat[ir] = ("not converged", minimum)
            return
        self._store(ir, pmin)
        if not self._check_vrot(ir):
            self._ringstat[ir] = ("rejected: VROT beyond the band", minimum)
            fitok[ir] = False
            self._cstat[ir] = self.CS_FAILED
            return
        self._ringstat[ir] = ("ok", minimum)

    def galfit(self, rings=None):
        """One fitting stage (``bbarolo/galfit.py:1162-1238``) with one thread and no REVERSE passes: the rings
        in order (or those given), the data normalised to a peak of 10 (NORMALCUBE) during the fit."""
        self.n_galfit = 2 if self.n_galfit == 1 else 1
        c = self.cin
        self.outr = self.inr.copy()
        dn_orig, dT_orig = self.data_noise, self.data_T
        if getattr(self.par, "NORMALCUBE", True):
            arr = np.asarray(c.array)
            scaling = 10. / float(np.nanmax(arr))
            self.data_T = np.ascontiguousarray((arr * scaling).astype(arr.dtype).transpose(1, 2, 0))
            self.data_noise = self.data_noise * scaling
        nr = self.inr.nr
        fitok = [False] * nr
        self._ringstat = {}
        self._cstat = np.full(nr, self.CS_NONE)
        self._pass = 0
        start = self.par.STARTRAD if self.par.STARTRAD < nr else 0
        try:
            for ir in (range(start, nr) if rings is None else rings):
                self._fit_ring(ir, fitok)
        finally:
            self.data_noise, self.data_T = dn_orig, dT_orig
        self.fitok = fitok
        return self.outr, fitok
