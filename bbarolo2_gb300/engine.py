"""The device model engine: ``DiskModel`` (``bbarolo/galmod.py:1147-1377``) with its models built, convolved and
compared with the data on the GPU.

``DiskModel(cube, par=None, ringmode=None, densflux=None, galmodtype=None, smooth=None)`` has the reference's
constructor and methods (``box``, ``array``, ``convolve``, ``ring_maps``), with the header-derived constants
(``GalmodSetup``) and the beam kernel computed on the host as the reference, and every model evaluation on the
device through ``libbbgpu.so``. ``BatchLikelihood`` evaluates the Gaussian log-likelihood of
``LikelihoodMixin._log_likelihood`` (``bbarolo/bayesian/likelihood.py:567-619``) for a batch of ring sets in
one device pass.
"""

import math

import numpy as np

from . import _lib
from .beam import BeamKernel
from .galmod import (GalmodSetup, ZSTEP_BEAM, ZSTEP_COARSE, ZSTEP_FINE, ZSAMPLES_MAX, arcsconv, model_rings, model_rows,
                     outer_edge, ringmode_name, seed32, subrings_batch)
from .rings import RING_KEYS


def grid_struct(st, scalefactor):
    """The ``bbgpu_grid`` of a GalmodSetup."""
    g = _lib.Grid()
    g.nx, g.ny, g.nz = st.dimx, st.dimy, st.nsubs
    g.nlines = int(st.lfreq0.size)
    g.axtyp, g.velsys, g.ltype, g.cmode = int(st.axtyp), int(st.velsys), int(st.ltype), int(st.cmode)
    g.radsep, g.cdens, g.pixarea = st.radsep, st.cdens, st.pixarea
    g.cdelt0, g.cdelt1, g.crota2 = st.cdelt[0], st.cdelt[1], st.crota2
    g.sig_instr, g.crval3, g.cdelt3, g.crpix3 = st.sig_instr, st.crval3, st.cdelt3, st.crpix3
    g.chwidth, g.zstep, g.scalefactor = st._chmin, st.zstep, float(scalefactor)
    return g


class DiskModel:
    """Models of a rotating disk on the grid of a cube, built on the GPU (see the module docstring)."""

    def __init__(self, cube, par=None, ringmode=None, densflux=None, galmodtype=None, smooth=None, device=0):
        p = cube.pars()
        self.cin = cube
        self.par = p.gf if par is None else par
        self.setup = GalmodSetup(cube, gmpar=self.par, galmodtype=galmodtype,
                                 densflux=self.par.DENSFLUX if densflux is None else densflux)
        self.ringmode = ringmode_name(getattr(p, "ringmode", "CENTRED") if ringmode is None else ringmode)
        self.arcconv = arcsconv(cube.Head().Cunit(0))
        self.cfield = None
        self.scalefactor = 1.
        self.smooth = bool(self.par.SM if smooth is None else smooth)
        if self.smooth:
            bk = BeamKernel.from_cube(cube)
            if bk.kernel is None:
                self.smooth = False
            else:
                self.cfield = bk.kernel
                self.scalefactor = 1.0 if self.setup.densIsFlux else bk.scalefac
        self.setup.zstep = self.zstep
        self.ctx = _lib.Context(device)
        st = self.setup
        self.ctx.check(self.ctx.L.bbgpu_set_grid(self.ctx.h, self._grid(), _lib.ptr(st.cd2i), _lib.ptr(st.lfreq0),
                                                 _lib.ptr(st.relint), _lib.ptr(st._vedges_lines)))
        if self.cfield is not None:
            k = np.ascontiguousarray(self.cfield, np.float64)
            self.ctx.check(self.ctx.L.bbgpu_set_kernel(self.ctx.h, _lib.ptr(k), k.shape[0], k.shape[1]))
        self._data_set = False

    def _grid(self):
        return grid_struct(self.setup, self.scalefactor)

    @property
    def conv(self):
        return self.cfield

    @property
    def zstep(self):
        """ZSTEP_COARSE for a beam whose minor axis is at least ZSTEP_BEAM pixels (``galmod.py:1193-1203``)."""
        if self.cfield is None:
            return ZSTEP_FINE
        h = self.cin.Head()
        pix = max(self.setup.pixsize) / 60.
        bmin = min(abs(h.Bmaj()), abs(h.Bmin()))
        return ZSTEP_COARSE if pix > 0 and bmin / pix >= ZSTEP_BEAM else ZSTEP_FINE

    # ------------------------------------------------------------------------------------------ geometry
    def box(self, rings, final=False):
        """Box [blo, bhi) of the cube containing the model (``bbarolo/galmod.py:1224-1240``)."""
        h = self.cin.Head()
        ext = rings.radii[-1] + rings.radsep / 2.
        if final:
            ext = max(ext, outer_edge(rings, self.ringmode))
        ext = ext + 3 * float(rings.layer_height()[-1])
        xdis = int(math.ceil(ext / (abs(h.Cdelt(0)) * self.arcconv)))
        ydis = int(math.ceil(ext / (abs(h.Cdelt(1)) * self.arcconv)))
        xpos = int(math.ceil(rings.xpos[-1]))
        ypos = int(math.ceil(rings.ypos[-1]))
        blo = [max(xpos - xdis, 0), max(ypos - ydis, 0)]
        bhi = [min(xpos + xdis + 1, self.cin.DimX()), min(ypos + ydis + 1, self.cin.DimY())]
        return blo, bhi

    # ------------------------------------------------------------------------------------------ models
    def galmod_mc(self, out, sr, ring_lo, ring_hi, seed, nv, blo, bhi):
        """``_galmod_mc`` on the device: out (by, bx, nz) float64 accumulated (``bbarolo/galmod.py:92-171``)."""
        sr = np.ascontiguousarray(sr, np.float64)
        nv = np.ascontiguousarray(nv, np.int64)
        assert out.dtype == np.float64 and out.flags.c_contiguous
        self.ctx.check(self.ctx.L.bbgpu_galmod_mc(self.ctx.h, _lib.ptr(out), _lib.ptr(sr), sr.shape[1],
                                                  int(ring_lo), int(ring_hi), int(seed) & 0xFFFFFFFFFFFFFFFF,
                                                  _lib.ptr(nv), int(blo[0]), int(blo[1]), int(bhi[0]), int(bhi[1])))
        return out

    def galmod_wind(self, out, sr, ring_lo, ring_hi, seed, sep, nv, blo, bhi):
        """``_galmod_wind`` on the device (GALWIND WTYPE 1, ``bbarolo/galmod.py:539-590``): sr (11, nsub) of the
        shells, out (by, bx, nz) float64 accumulated; the cloud density, CMODE and the lines are this model's."""
        sr = np.ascontiguousarray(sr, np.float64)
        nv = np.ascontiguousarray(nv, np.int64)
        assert out.dtype == np.float64 and out.flags.c_contiguous
        self.ctx.check(self.ctx.L.bbgpu_galmod_wind(self.ctx.h, _lib.ptr(out), _lib.ptr(sr), sr.shape[1],
                                                    int(ring_lo), int(ring_hi), int(seed) & 0xFFFFFFFFFFFFFFFF,
                                                    float(sep), _lib.ptr(nv), int(blo[0]), int(blo[1]), int(bhi[0]),
                                                    int(bhi[1])))
        return out

    def build(self, rings, blo=(0, 0), bhi=None, seed=None, galmodtype=None, layout="zyx"):
        """The non-convolved model of rings (used as nodes) in [blo, bhi) (``GalmodSetup.build``)."""
        st = self.setup
        if bhi is None:
            bhi = (st.dimx, st.dimy)
        gtype = (galmodtype or st.galmodtype).upper()
        sr, nv = st.subrings(rings)
        out = np.zeros((bhi[1] - blo[1], bhi[0] - blo[0], st.nsubs))
        if sr.shape[1]:
            if gtype == "ANALYTIC":
                nzq = 1 if not np.any(sr[6] > 0) else ZSAMPLES_MAX
                self.ctx.check(self.ctx.L.bbgpu_galmod_analytic(self.ctx.h, _lib.ptr(out), _lib.ptr(sr), sr.shape[1],
                                                                0, sr.shape[1], nzq, int(blo[0]), int(blo[1]),
                                                                int(bhi[0]), int(bhi[1])))
            else:
                s = seed32(st.iseed if seed is None else seed)
                self.galmod_mc(out, sr, 0, sr.shape[1], s, nv, blo, bhi)
        if layout == "zyx":
            return np.ascontiguousarray(out.transpose(2, 0, 1))
        return out

    def array(self, rings, blo=None, bhi=None, final=True, ringmode=None, seed=None, galmodtype=None,
              layout="zyx", support=None, threads=None):
        """The model of the rings, convolved with the beam if smoothing is on (``bbarolo/galmod.py:1242-1271``).
        The device builds one model per call, so ``threads`` has no effect (the reference's THREADS>1 final
        models use one stream per thread chunk; this path reproduces THREADS=1)."""
        if blo is None or bhi is None:
            blo, bhi = (0, 0), (self.cin.DimX(), self.cin.DimY())
        if final:
            rings = model_rings(rings, self.ringmode if ringmode is None else ringmode, self.setup.radsep)
        mod = self.build(rings, blo, bhi, seed=seed, galmodtype=galmodtype, layout="yxz")
        if self.cfield is not None:
            if final:
                return self.convolve(mod, layout)
            out = np.zeros_like(mod)
            k = np.ascontiguousarray(self.cfield, np.float64)
            self.ctx.check(self.ctx.L.bbgpu_conv_sparse(self.ctx.h, _lib.ptr(mod), _lib.ptr(out), *mod.shape,
                                                        _lib.ptr(k), k.shape[0], k.shape[1], float(self.scalefactor)))
            mod = out
        if layout == "zyx":
            return np.ascontiguousarray(mod.transpose(2, 0, 1))
        return mod

    def convolve(self, mod, layout="zyx", workers=1):
        """A dense model (ny, nx, nz) convolved with the beam, values below 1e-12 set to zero, times the scale
        factor (``bbarolo/galmod.py:1273-1283``), as (nz, ny, nx) or (ny, nx, nz) with layout='yxz'."""
        if self.cfield is None:
            return np.ascontiguousarray(mod.transpose(2, 0, 1) if layout == "zyx" else mod.copy())
        a = np.ascontiguousarray(np.asarray(mod, np.float64).transpose(2, 0, 1))
        out = np.empty_like(a)
        self.ctx.check(self.ctx.L.bbgpu_convolve(self.ctx.h, _lib.ptr(a), _lib.ptr(out), *a.shape,
                                                 float(self.scalefactor), 1))
        return out if layout == "zyx" else np.ascontiguousarray(out.transpose(1, 2, 0))

    def convolve_planes(self, planes, threshold=False, scale=1.0):
        """The "same" convolution of a stack (n, ny, nx) (``FFTConvolver.__call__``, bbarolo/smooth.py:145)."""
        a = np.ascontiguousarray(planes, np.float64)
        if a.ndim == 2:
            return self.convolve_planes(a[None], threshold, scale)[0]
        out = np.empty_like(a)
        self.ctx.check(self.ctx.L.bbgpu_convolve(self.ctx.h, _lib.ptr(a), _lib.ptr(out), *a.shape, float(scale),
                                                 1 if threshold else 0))
        return out

    # ------------------------------------------------------------------------------------------ ring maps
    def _ring_weights(self, rings, ringmode):
        """(widx, wval) (nsub, 2): the ring(s) whose density each sub-ring interpolates and the weights
        (``bbarolo/galmod.py:1285-1315``), computed with unit densities through ``subrings``; cached."""
        key = (tuple(np.asarray(rings.radii, float)), float(rings.radsep), ringmode, getattr(rings, "edge", None),
               float(getattr(rings, "edgewidth", 0.)), rings.thick(),
               tuple(np.asarray(rings.fthick, float)) if rings.thick() else ())
        cache = self.__dict__.setdefault("_wcache", {})
        if key in cache:
            return cache[key]
        st = self.setup
        cols = []
        for r in range(rings.nr):
            rr = rings.copy()
            rr.dens = np.zeros(rings.nr)
            rr.dens[r] = 1.
            cols.append(st.subrings(model_rings(rr, ringmode, st.radsep))[0][5])
        W = np.array(cols).T
        nsub = W.shape[0]
        widx = np.full((nsub, 2), -1, np.int64)
        wval = np.zeros((nsub, 2))
        for s in range(nsub):
            nz = np.flatnonzero(W[s] != 0)
            if len(nz) > 2:
                raise RuntimeError("ring_maps: a sub-ring depends on more than two rings.")
            widx[s, :len(nz)] = nz
            wval[s, :len(nz)] = W[s, nz]
        if len(cache) > 64:
            cache.clear()
        cache[key] = (widx, wval)
        return widx, wval

    @property
    def mapscale(self):
        """The factor of the ring maps: mean(cd2i) x sum(relint) (x the beam scale factor when smoothing)."""
        st = self.setup
        f = float(np.mean(st.cd2i)) * float(np.sum(st.relint))
        return f * self.scalefactor if self.cfield is not None else f

    def ring_maps(self, rings, blo=None, bhi=None, ringmode=None):
        """Total-intensity maps (nr, ny, nx) of each ring with unit density, convolved with the beam when
        smoothing is on (``bbarolo/galmod.py:1317-1345``): the ANALYTIC samples deposited on the device, the
        convolution on the device (float32, within 1e-6 of the peak of the float64 maps)."""
        if blo is None or bhi is None:
            blo, bhi = (0, 0), (self.cin.DimX(), self.cin.DimY())
        mode = self.ringmode if ringmode is None else ringmode_name(ringmode)
        st = self.setup
        mr = model_rings(rings, mode, st.radsep)
        mr = mr.copy() if mr is rings else mr
        mr.dens = np.ones(mr.nr)
        sr, _ = st.subrings(mr)
        widx, wval = self._ring_weights(rings, mode)
        out = np.zeros((rings.nr, bhi[1] - blo[1], bhi[0] - blo[0]))
        if sr.shape[1]:
            sr = np.ascontiguousarray(sr)
            nzq = 1 if not np.any(sr[6] > 0) else ZSAMPLES_MAX
            self.ctx.check(self.ctx.L.bbgpu_ring_maps_analytic(self.ctx.h, _lib.ptr(out), out.shape[0], _lib.ptr(sr),
                                                               sr.shape[1], _lib.ptr(widx), _lib.ptr(wval), nzq,
                                                               int(blo[0]), int(blo[1]), int(bhi[0]), int(bhi[1])))
        out *= float(np.mean(st.cd2i)) * float(np.sum(st.relint))
        if self.cfield is not None and out.size:
            out = self.convolve_planes(out) * self.scalefactor
        return out

    def model_rows(self, rows, proto, ringmode=None):
        """Ring-value rows (B, 17, nr) of ring sets like ``proto`` -> the rows of their model rings (with the
        ring convention) and the model-ring prototype."""
        mode = self.ringmode if ringmode is None else ringmode_name(ringmode)
        return model_rows(rows, proto, mode, self.setup.radsep)


class BatchLikelihood:
    """The Gaussian log-likelihood of ``LikelihoodMixin._log_likelihood`` for batches of ring sets.

    data (nz, ny, nx) float32, likemask (nz, ny, nx) bool (the voxels of the likelihood), maskmode 2 (only the
    voxels in the mask, the default of Bayesian3DFIT) or 1 (data * mask) or 0; region (ny, nx) bool or None;
    sigma (noise per voxel); likefactor (the noise-correlation factor); likebox ([blo], [bhi]) the likelihood
    region's box (default the cube). For each ring set: -likefactor * (0.5 (ss + ss_out) / sigma^2 +
    0.5 nvox log(2 pi sigma^2)), ss over the model box on the device, ss_out (the data outside the box) from a
    summed-area table (``likelihood.py:437-440``), fracerr eps optional (``likelihood.py:512-531``)."""

    def __init__(self, model, data, likemask=None, maskmode=2, region=None, sigma=1.0, likefactor=1.0,
                 likebox=None, fracerr=None, nvox=None):
        self.model = model
        d = np.ascontiguousarray(data, np.float32)
        nz, ny, nx = d.shape
        self.shape = d.shape
        self.maskmode = int(maskmode) if likemask is not None else 0
        self.mask = None if likemask is None else np.ascontiguousarray(likemask, dtype=bool)
        self.region = None if region is None else np.ascontiguousarray(region, dtype=bool)
        self.sigma = float(sigma)
        self.likefactor = float(likefactor)
        self.eps = None if fracerr is None else float(fracerr)
        self.likebox = likebox if likebox is not None else ([0, 0], [nx, ny])
        ctx = model.ctx
        mk = None if self.mask is None else self.mask.view(np.uint8)
        rg = None if self.region is None else self.region.view(np.uint8)
        ctx.check(ctx.L.bbgpu_set_cube(ctx.h, _lib.ptr(d), _lib.ptr(mk), _lib.ptr(rg)))
        # the data of the likelihood (the rule of _sumsq_residuals), its squares per pixel and their count
        valid = np.isfinite(d) & (d != 0)
        dd = np.where(valid, d, 0.).astype(np.float64)
        if self.maskmode == 2:
            valid &= self.mask
        elif self.maskmode == 1:
            dd = np.where(self.mask, dd, 0.)
        if self.region is not None:
            valid &= self.region[None]
        dm2 = np.where(valid, dd * dd, 0.).sum(axis=0)
        self._dm2_sat = np.zeros((ny + 1, nx + 1))
        self._dm2_sat[1:, 1:] = dm2.cumsum(0).cumsum(1)
        Lb, Hb = self.likebox
        self._dm2_box = self._boxsum(Lb, Hb)
        self.nvox = int(valid[:, Lb[1]:Hb[1], Lb[0]:Hb[0]].sum()) if nvox is None else int(nvox)
        self._prof = None
        self._data = d

    def set_profile(self, proto, data_map, rms_map, ok_map, smooth=0.3, corr=1., floor=None, beam_arcsec=None):
        """Recompute the density profile of the rings at every evaluation, as Bayesian3DFIT does when DENS is not
        fitted and the geometry is free (``bbarolo/bayesian/likelihood.py:595-596``,
        ``bbarolo/bayesian/density.py:39-88``): the ring maps of each member, their convolution, the weighted
        least squares against data_map (noise rms_map, pixels ok_map; all of the likelihood box) and the
        non-negative solve with the smoothness prior (``bbarolo/profile.py:91-138``), on the device, before its
        MC model. proto: the rings (radii and options) of the batches to come."""
        from . import profile as P
        dm = self.model
        Lb, Hb = self.likebox
        shape = (Hb[1] - Lb[1], Hb[0] - Lb[0])
        y = np.ascontiguousarray(data_map, np.float64)
        s = np.ascontiguousarray(rms_map, np.float64)
        ok = np.ascontiguousarray(ok_map, dtype=bool)
        if y.shape != shape or s.shape != shape or ok.shape != shape:
            raise ValueError(f"set_profile: the maps must have the shape of the likelihood box {shape}")
        ext, w = P.exterior_ring(dm, proto, beam_arcsec)
        Rc = np.ascontiguousarray(np.r_[np.asarray(proto.radii, float), float(ext.radii[0])])
        ctx = dm.ctx
        ctx.check(ctx.L.bbgpu_set_profile(ctx.h, proto.nr, int(Lb[0]), int(Lb[1]), int(Hb[0]), int(Hb[1]),
                                          _lib.ptr(y), _lib.ptr(s), _lib.ptr(ok.view(np.uint8)), _lib.ptr(Rc),
                                          float(smooth or 0.), float(corr),
                                          float(P.DENSPROF_FLOOR if floor is None else floor), dm.mapscale))
        wm = dm._ring_weights(proto, dm.ringmode)
        we = dm._ring_weights(ext, "CENTRED")
        widx = np.ascontiguousarray(np.concatenate([wm[0], np.where(we[0] >= 0, we[0] + proto.nr, -1)]), np.int64)
        wval = np.ascontiguousarray(np.concatenate([wm[1], we[1]]))
        self._prof = dict(nr=proto.nr, ext=ext, widx=widx, wval=wval, radii=np.asarray(proto.radii, float).copy(),
                          y=y, rms=s, ok=ok, Rc=Rc, smooth=float(smooth or 0.), corr=float(corr),
                          floor=P.DENSPROF_FLOOR if floor is None else float(floor))

    def data_maps(self):
        """(data_mom0, map_rms, ok) of the likelihood box, as Bayesian3DFIT builds them
        (``bbarolo/bayesian/likelihood.py:180-188, 206-221``, ``bbarolo/bayesian/density.py:80-83``): the sum of
        the data in the voxels of the likelihood, sigma x sqrt(their number) (channels independent), and the
        pixels of the region with such voxels."""
        d = self._data
        lm = self.mask if self.mask is not None else np.ones(d.shape, bool)
        v = lm & np.isfinite(d) & (d != 0)
        mom0 = np.where(v, d, 0.).astype(np.float64).sum(axis=0)
        nvox = v.sum(axis=0)
        rms = self.sigma * np.sqrt(nvox.astype(np.float64))
        ok = nvox > 0
        if self.region is not None:
            ok &= self.region
        Lb, Hb = self.likebox
        sl = (slice(Lb[1], Hb[1]), slice(Lb[0], Hb[0]))
        return mom0[sl], rms[sl], ok[sl]

    def profile_maps(self, rows, out=None):
        """The sub-ring tables of the exterior annulus of the ring maps of a batch (B, 16, nse: the values of
        each member's last ring, ``bbarolo/profile.py:66-69``); the ring maps' tables are the model's sub-rings,
        then these. out (B, 16, nse), e.g. a view of the last columns of the maps' table, receives them."""
        dm = self.model
        P = self._prof
        ext = P["ext"]
        rows = np.asarray(rows, float)
        er = np.zeros(rows.shape[:2] + (1,))
        keep = [RING_KEYS.index(k) for k in ("xpos", "ypos", "vsys", "vrot", "vdisp", "z0", "inc", "phi",
                                             "z0thick", "fthick", "vdispthick")]
        er[:, keep, 0] = rows[:, keep, -1]
        er[:, RING_KEYS.index("radii"), 0] = ext.radii[0]
        er[:, RING_KEYS.index("dens"), 0] = 1.
        # (the members of a batch mostly share member 0's last ring: its table, and those of the others)
        other = np.flatnonzero(np.any(er != er[:1], axis=(1, 2)))
        pick = np.concatenate([[0], other])
        emr_rows, emr = dm.model_rows(er[pick], ext, ringmode="CENTRED")
        sre, _ = subrings_batch(dm.setup, emr, emr_rows)
        if out is None:
            out = np.empty((er.shape[0],) + sre.shape[1:])
        out[:] = sre[:1]
        out[other] = sre[1:]
        return out

    def _boxsum(self, blo, bhi):
        S = self._dm2_sat
        return float(S[bhi[1], bhi[0]] - S[blo[1], bhi[0]] - S[bhi[1], blo[0]] + S[blo[1], blo[0]])

    def model_box(self, rings):
        blo, bhi = self.model.box(rings, final=True)
        Lb, Hb = self.likebox
        blo = [max(blo[0], Lb[0]), max(blo[1], Lb[1])]
        bhi = [max(min(bhi[0], Hb[0]), blo[0]), max(min(bhi[1], Hb[1]), blo[1])]
        return blo, bhi

    def _boxes(self, rows, proto):
        """The model boxes of a batch within the likelihood box (``model_box`` / ``DiskModel.box(final=True)``,
        ``bbarolo/galmod.py:1224-1240``, ``bbarolo/bayesian/likelihood.py:429-436``), vectorised: (blo, bhi)
        arrays (B, 2). The boxes depend on the last ring's centre and layer height only."""
        dm = self.model
        h = dm.cin.Head()
        rows = np.asarray(rows, float)
        K = {k: RING_KEYS.index(k) for k in ("xpos", "ypos", "z0", "z0thick", "fthick")}
        ext0 = proto.radii[-1] + proto.radsep / 2.
        ext0 = max(ext0, outer_edge(proto, dm.ringmode))
        z0 = rows[:, K["z0"], -1]
        if proto.thick():
            zt = rows[:, K["z0thick"], -1]
            zt = np.where(zt >= 0, zt, z0)
            z0 = np.where(rows[:, K["fthick"], -1] > 0, np.maximum(z0, zt), z0)
        ext = ext0 + 3 * z0
        xdis = np.ceil(ext / (abs(h.Cdelt(0)) * dm.arcconv)).astype(np.int64)
        ydis = np.ceil(ext / (abs(h.Cdelt(1)) * dm.arcconv)).astype(np.int64)
        xpos = np.ceil(rows[:, K["xpos"], -1]).astype(np.int64)
        ypos = np.ceil(rows[:, K["ypos"], -1]).astype(np.int64)
        blo = np.stack([np.maximum(xpos - xdis, 0), np.maximum(ypos - ydis, 0)], axis=1)
        bhi = np.stack([np.minimum(xpos + xdis + 1, dm.cin.DimX()), np.minimum(ypos + ydis + 1, dm.cin.DimY())], axis=1)
        Lb, Hb = self.likebox
        blo = np.maximum(blo, np.asarray(Lb, np.int64))
        bhi = np.maximum(np.minimum(bhi, np.asarray(Hb, np.int64)), blo)
        return blo, bhi

    def prepare(self, rows, proto, seed=None):
        """Host side of a batch: sub-ring tables, boxes and descriptors of the ring-value rows (B, 17, nr)."""
        dm = self.model
        mrows, mr = dm.model_rows(rows, proto)
        ms = None
        if self._prof is not None:
            if not np.array_equal(np.asarray(proto.radii, float), self._prof["radii"]):
                raise ValueError("the radii differ from those given to set_profile")
            # the ring maps' tables: the model's sub-rings (written by subrings_batch), then the exterior's
            nsub = dm.setup.grid(mr).nsub
            nse = self._prof.get("nse")
            if nse is None:
                nse = self._prof["nse"] = self.profile_maps(rows[:1]).shape[2]
            ms = np.empty((len(rows), 16, nsub + nse))
            self.profile_maps(rows, out=ms[:, :, nsub:])
        sr, nv = subrings_batch(dm.setup, mr, mrows, out_ms=ms)
        B = sr.shape[0]
        s = seed32(dm.setup.iseed if seed is None else seed)
        blo, bhi = self._boxes(rows, proto)
        descs = np.zeros(B, _lib.EVAL_DTYPE)
        descs["blo0"], descs["blo1"], descs["bhi0"], descs["bhi1"] = blo[:, 0], blo[:, 1], bhi[:, 0], bhi[:, 1]
        descs["seed"] = s
        descs["maskmode"] = self.maskmode
        descs["use_region"] = 1 if self.region is not None else 0
        descs["sigma2"] = self.sigma ** 2
        descs["eps2"] = (self.eps or 0.) ** 2
        boxes = list(zip(blo.tolist(), bhi.tolist()))
        if ms is not None:
            self._maps_sr = ms
        return sr, nv, descs, boxes

    def evaluate(self, rows, proto, seed=None, galmodtype=None):
        """log L of each ring set (rows (B, 17, nr) in RING_KEYS order, radii and options as proto)."""
        sr, nv, descs, boxes = self.prepare(rows, proto, seed)
        try:
            ss, lg = self.run(sr, nv, descs, galmodtype)
        except _lib.DeviceError as e:
            if self._prof is None or "changed the MC cloud layout" not in str(e):
                raise
            return self._evaluate_split(rows, proto, seed, galmodtype)
        return self.finish(ss, lg, boxes)

    def _evaluate_split(self, rows, proto, seed, galmodtype):
        """A batch whose recomputed density profile changed the MC cloud layout of a member (a ring at zero, or
        above the 10-clouds-per-pixel floor: the batch's layout, set up from the members' DENS, no longer holds).
        Its halves are evaluated apart, down to single members; a single member whose layout changes is evaluated
        with the profile's densities as its DENS and no profile, which is the reference's evaluation: its model is
        built from the rings whose DENS the profile has set (``bbarolo/bayesian/density.py:13-25``,
        ``bbarolo/bayesian/likelihood.py:595-596``), and so are its clouds."""
        rows = np.asarray(rows, float)
        if len(rows) > 1:
            h = len(rows) // 2
            return np.concatenate([self.evaluate(rows[:h], proto, seed, galmodtype),
                                   self.evaluate(rows[h:], proto, seed, galmodtype)])
        x, _ = self.last_profile()
        own = rows.copy()
        own[0, RING_KEYS.index("dens")] = x[0, :self._prof["nr"]]
        prof, self._prof = self._prof, None
        try:
            return self.evaluate(own, proto, seed, galmodtype)
        finally:
            self._prof = prof

    def run(self, sr, nv, descs, galmodtype=None):
        dm = self.model
        gt = (galmodtype or dm.setup.galmodtype).upper()
        B, _, nsub = sr.shape
        ss = np.zeros(B)
        lg = np.zeros(B)
        ctx = dm.ctx
        code = _lib.ANALYTIC if gt == "ANALYTIC" else _lib.MC
        if self._prof is None:
            ctx.check(ctx.L.bbgpu_eval_batch(ctx.h, code, B, nsub, _lib.ptr(sr), _lib.ptr(nv), _lib.ptr(descs),
                                             _lib.ptr(ss), _lib.ptr(lg)))
            return ss, lg
        ctx.check(ctx.L.bbgpu_eval_upload(ctx.h, code, B, nsub, _lib.ptr(sr), _lib.ptr(nv), _lib.ptr(descs)))
        P = self._prof
        ms = self._maps_sr
        ctx.check(ctx.L.bbgpu_eval_upload_profile(ctx.h, ms.shape[2], _lib.ptr(ms), _lib.ptr(P["widx"]),
                                                  _lib.ptr(P["wval"])))
        ctx.check(ctx.L.bbgpu_eval_run(ctx.h))
        ctx.check(ctx.L.bbgpu_eval_download(ctx.h, _lib.ptr(ss), _lib.ptr(lg)))
        return ss, lg

    def last_profile(self):
        """(x (B, nr + 1), status (B)) of the last evaluation: the ring densities (and the exterior annulus)."""
        ctx = self.model.ctx
        B = len(self._maps_sr)
        x = np.zeros((B, self._prof["nr"] + 1))
        st = np.zeros(B, np.int32)
        ctx.check(ctx.L.bbgpu_eval_profile(ctx.h, _lib.ptr(x), _lib.ptr(st)))
        return x, st

    def finish(self, ss, lg, boxes):
        """log L of the members from their sums (ss, lg) in their boxes and the data outside them."""
        s2 = self.sigma ** 2
        b = np.asarray(boxes, np.int64).reshape(len(ss), 2, 2)          # (member, lo/hi, x/y)
        S = self._dm2_sat
        inside = S[b[:, 1, 1], b[:, 1, 0]] - S[b[:, 0, 1], b[:, 1, 0]] - S[b[:, 1, 1], b[:, 0, 0]] + \
            S[b[:, 0, 1], b[:, 0, 0]]
        ss_out = np.maximum(self._dm2_box - inside, 0.)
        ss = np.asarray(ss, float)
        const = 0.5 * self.nvox * math.log(2. * math.pi * s2)
        if self.eps is not None and self.eps > 0:
            res = 0.5 * (ss + ss_out / s2) + const + 0.5 * np.asarray(lg, float)
        else:
            res = 0.5 * (ss + ss_out) / s2 + const
        return -self.likefactor * res
