"""GALWIND WTYPE 1: the Monte-Carlo model of a bi-conical wind made of spherical shells, on the GPU.

The reference's ``GalWind`` (``bbarolo/galwind.py``) builds it in two steps: ``_shells`` (``:257-299``) turns the
parameters into a table of thin shells (radius, rotation, radial wind, dispersion, density, inclination, position
angle, opening angle, centre and systemic velocity, linear between the given radii, every ``sep`` = 0.75 of the
smallest pixel), and ``_spherical`` (``:301-331``) deposits the clouds of the shells with ``_galmod_wind`` (chunks of
shells, one stream per chunk seeded ISEED + 7919 k). Here the shells are the same host computation and the clouds
are placed and deposited on the device (``DiskModel.galmod_wind``, ``csrc/galwind.cu``); the chunks' models are
summed in chunk order, as the reference.
"""

import copy
import math

import numpy as np

from .engine import DiskModel
from .galmod import BBaroloError, GalmodSetup


class GalWindPars:
    """The parameters of a GALWIND WTYPE 1 model: XPOS, YPOS (pixels), VSYS (km/s), INC, PHI (degrees), CONELEN
    (arcsec), NLAYERS or RADII (arcsec: the shells' radii), per radius (one value or a list) VROT, VWIND, VDISP
    (km/s), DENS and OPENANG (degrees, full opening angle); CDENS, NV, ISEED as GALMOD's."""

    def __init__(self, xpos, ypos, vsys=0., inc=60., phi=0., conelen=10., nlayers=10, radii=None, vrot=0.,
                 vwind=100., vdisp=10., dens=1., openang=60., cdens=10., nv=-1, iseed=-1):
        self.XPOS, self.YPOS, self.VSYS, self.INC, self.PHI = float(xpos), float(ypos), float(vsys), float(inc), \
            float(phi)
        self.CONELEN, self.NLAYERS, self.RADII = float(conelen), int(nlayers), radii
        self.VROT, self.VWIND, self.VDISP, self.DENS, self.OPENANG = vrot, vwind, vdisp, dens, openang
        self.CDENS, self.NV, self.ISEED = float(cdens), int(nv), int(iseed)


def _per_radius(name, v, n):
    a = np.atleast_1d(np.asarray(v, dtype=np.float64)).ravel()
    if a.size == 1:
        return np.repeat(a, n)
    if a.size < n:
        raise BBaroloError(f"GALWIND: {name} has {a.size} values, fewer than the {n} cylinders or shells.")
    return a[:n]


def wind_shells(par, setup):
    """The shells of the wind (``bbarolo/galwind.py:257-299``): (sr (11, nshell) in internal units, nv, sep)."""
    nr = int(par.NLAYERS)
    radsep = par.CONELEN / nr
    given = None if par.RADII is None else np.asarray(par.RADII, dtype=np.float64).ravel()
    if given is not None:
        radsep = float(np.mean(np.diff(given[1:]))) if given.size > 2 else radsep
        nr = given.size
    radii = given if given is not None else np.arange(nr) * radsep + radsep / 2.
    rows = np.vstack([_per_radius("VROT", par.VROT, nr) * 1000., _per_radius("VWIND", par.VWIND, nr) * 1000.,
                      _per_radius("VDISP", par.VDISP, nr) * 1000., _per_radius("DENS", par.DENS, nr),
                      np.full(nr, math.radians(par.INC)), np.full(nr, math.radians(par.PHI)),
                      np.radians(_per_radius("OPENANG", par.OPENANG, nr)), np.full(nr, par.XPOS),
                      np.full(nr, par.YPOS), np.full(nr, par.VSYS * 1000.)])
    if np.any(rows[2] < 0):
        raise BBaroloError("GALMOD error: Negative velocity dispersion not allowed.")
    if np.any(rows[3] < 0):
        raise BBaroloError("GALMOD error: Negative column-density not allowed.")
    urad = radii / 60.
    sep = 0.75 * min(setup.pixsize)
    if np.any(urad[:-1] + sep >= urad[1:]):
        raise BBaroloError("GALMOD error: Radii not in increasing order or separation too small.")
    # shells every sep (float32 radii, as the reference), the values linear between the given radii
    out_r, out_v = [], []
    r = np.float32(urad[0] + sep / 2.) if urad[0] != 0 else np.float32(sep / 2.)
    for i in range(1, nr):
        slope = (rows[:, i] - rows[:, i - 1]) / (urad[i] - urad[i - 1])
        while r < np.float32(urad[i]):
            out_r.append(float(r))
            out_v.append(rows[:, i - 1] + slope * (float(r) - urad[i - 1]))
            r = np.float32(float(r) + sep)
    sr = np.empty((11, len(out_r)))
    if out_r:
        sr[0] = out_r
        sr[1:] = np.array(out_v).T
    nvpar = par.NV if par.NV > 0 else 20
    nv = np.where(sr[3] == 0, 1, nvpar if nvpar >= 1 else setup.nsubs).astype(np.int64)
    return np.ascontiguousarray(sr), nv, sep


def wind_gmpar(cube, par):
    """The GALMOD parameters of the shells (``bbarolo/galwind.py:174-182, 304``): the cube's, with CDENS, NV and ISEED
    of the wind, CMODE 1 and DENSFLUX false (the clouds carry a column density)."""
    gm = copy.deepcopy(cube.pars().gm)
    gm.CDENS, gm.NV, gm.ISEED, gm.CMODE, gm.DENSFLUX = par.CDENS, par.NV, par.ISEED, 1, False
    return gm


def wind_setup(cube, par):
    """The GalmodSetup of the shells (host only)."""
    return GalmodSetup(cube, gmpar=wind_gmpar(cube, par), densflux=False)


class GalWindMC:
    """GALWIND WTYPE 1 on the grid of a cube (``bbarolo/galwind.py:301-331``): ``model()`` is the (nz, ny, nx)
    float64 cube of the clouds (before any smoothing), threads the chunks of shells (each its own stream)."""

    def __init__(self, cube, par, threads=1, device=0):
        self.cube, self.par, self.threads = cube, par, int(threads)
        self.dm = DiskModel(cube, par=wind_gmpar(cube, par), densflux=False, smooth=False, device=device)
        self.setup = self.dm.setup
        sr, nv, self.sep = wind_shells(par, self.setup)
        self.sr, self.nv = np.ascontiguousarray(sr, np.float64), np.ascontiguousarray(nv, np.int64)

    def chunks(self):
        ns = self.sr.shape[1]
        n = max(1, min(self.threads, ns))
        return [c for c in np.array_split(np.arange(ns), n) if len(c)]

    def model(self, host_threads=None):
        """The model cube (nz, ny, nx): the chunks' streams parsed on host_threads threads (default: as many as
        the chunks, at most the host's cores), every cloud deposited in one device pass."""
        import os
        from . import _lib
        c = self.cube
        out = np.zeros((c.DimY(), c.DimX(), c.DimZ()))
        seed = int(self.par.ISEED) & 0xFFFFFFFF
        ch = self.chunks()
        lo = np.array([int(x[0]) for x in ch], dtype=np.int32)
        hi = np.array([int(x[-1]) + 1 for x in ch], dtype=np.int32)
        seeds = np.array([(seed + 7919 * t) & 0xFFFFFFFF for t in range(len(ch))], dtype=np.uint64)
        nt = host_threads or min(len(ch), os.cpu_count() or 1)
        ctx = self.dm.ctx
        ctx.check(ctx.L.bbgpu_galwind_spherical(ctx.h, _lib.ptr(out), _lib.ptr(self.sr), self.sr.shape[1], len(ch),
                                                _lib.ptr(lo), _lib.ptr(hi), _lib.ptr(seeds), float(self.sep),
                                                _lib.ptr(self.nv), 0, 0, c.DimX(), c.DimY(), int(nt)))
        return np.ascontiguousarray(out.transpose(2, 0, 1))
