"""Host side of the GALMOD model: header-derived constants and the sub-ring tables the device kernels read.

This module mirrors the model-setup part of ``bbarolo/galmod.py``:

* ``GalmodSetup`` (``bbarolo/galmod.py:609-758``): cdelt in arcmin, pixel area, CROTA2, the spectral axis
  (velocity / frequency / wavelength, radio / optical / relativistic), the instrumental dispersion, the channel
  factor ``cd2i`` (float32-rounded as the reference) and the channel edges in velocity of each line;
* ``GalmodSetup.subrings`` (``bbarolo/galmod.py:761-851``): rings -> sub-rings 0.75 pixel apart, with the
  float32 accumulation of the sub-ring radii, linear interpolation of the ring values, the sharp/Gaussian
  outer edge, the thick layer and the edge weights of the two halves (rows 14-15);
* the ring conventions ``model_rings``/``edge_weights``/``outer_edge`` (``bbarolo/galmod.py:1043-1141``).

The sub-ring table ``sr`` has the reference's layout (16, nsub), internal units (arcmin, m/s, radians),
rows: radius, vrot, vrad, vvert, vdisp, dens, z0, dvdz, zcyl, inc, phi, xpos, ypos, vsys, wrec, wapp.
All arithmetic is elementwise IEEE float64 in the reference's operation order, so the table is bit-equal
to the reference's (checked against golden tables generated from the reference).
"""

import math
import sys

import numpy as np

C_MS = 2.99792458e08
VEL_UNITS = {"km/s": 1., "kms": 1., "m/s": 1E03, "ms": 1E03, "cm/s": 1E05}
WAVE_UNITS = {"m": 1., "cm": 1E02, "mm": 1E03, "um": 1E06, "mum": 1E06, "micron": 1E06, "nm": 1E09,
              "a": 1E10, "angstrom": 1E10}
_FREQ_UNITS = {"hz": 1., "khz": 1E03, "mhz": 1E06, "ghz": 1E09}

# vertical samples of the ANALYTIC model (bbarolo/galmod.py:262-273)
ZSAMPLES_MAX = 1024
ZSTEP_FINE = 0.25
ZSTEP_COARSE = 0.75
ZSTEP_BEAM = 3.0

# rows of the sub-ring table
SR_R, SR_VROT, SR_VRAD, SR_VVERT, SR_VDISP, SR_DENS, SR_Z0, SR_DVDZ, SR_ZCYL, SR_INC, SR_PHI, SR_XPOS, \
    SR_YPOS, SR_VSYS, SR_WREC, SR_WAPP = range(16)

RINGMODES = ("CENTRED", "NODES", "SHIFTED")


class BBaroloError(ValueError):
    """Invalid input of the model path (the reference's ``bbarolo.bbutils.BBaroloError``)."""


def seed32(iseed):
    """The seed of the MC stream: ISEED & 0xFFFFFFFF (ISEED -1 -> 0xFFFFFFFF), ``bbarolo/galmod.py:593-594``."""
    return int(iseed) & 0xFFFFFFFF


def arcsconv(cunit):
    c = cunit.lower()
    if "deg" in c:
        return 3600.
    if "arcm" in c:
        return 60.
    if "arcs" in c:
        return 1.
    raise ValueError(f"Conversion error (unknown CUNIT for RA-DEC): {cunit}. Cannot convert to ARCSEC.")


def delta_vel(h):
    """Channel width in km/s (``bbarolo/bbutils.py:159-180``): velocity axes directly; frequency and
    wavelength axes as the mean width of the channels in velocity."""
    dv = h.Cdelt(2)
    nz = h.DimAx(2)
    cu = h.Cunit(2).lower()
    if cu in VEL_UNITS:
        return dv / VEL_UNITS[cu]
    k = np.arange(nz - 1)
    lo = (k + 1 - h.Crpix(2)) * h.Cdelt(2) + h.Crval(2)
    hi = (k + 2 - h.Crpix(2)) * h.Cdelt(2) + h.Crval(2)
    vd = h.VelDef()
    if cu in _FREQ_UNITS:
        fc = _FREQ_UNITS[cu]
        frest = h.Freq0() / (1 + h.Redshift())
        if vd == "radio":
            return -C_MS / 1000. * dv * fc / frest
        return float(np.sum(_freq2vel(hi * fc, frest, vd) - _freq2vel(lo * fc, frest, vd)) / (nz - 1))
    if cu in WAVE_UNITS:
        raise BBaroloError("delta_vel: wavelength axes need the rest wavelength of the cube (not supported)")
    return dv


def _freq2vel(f, f0, vd):
    c = C_MS / 1000.
    if vd == "radio":
        return c * (1 - f / f0)
    if vd == "optical":
        return c * (f0 / f - 1)
    r = (f / f0) ** 2
    return c * (1 - r) / (1 + r)


def edge_weights(R, dr, edge, width=0.):
    """Weights of the density of sub-rings at radii R (arcsec, dr wide) for an outer edge at ``edge``
    (``bbarolo/galmod.py:1122-1131``): the fraction of each sub-ring within the edge (sharp), or a Gaussian
    edge 1/2 erfc((R - edge) / (sqrt(2) width))."""
    R = np.asarray(R, float)
    if width > 0:
        from scipy.special import erfc
        return 0.5 * erfc((R - edge) / (math.sqrt(2.) * width))
    if dr > 0:
        return np.clip((edge - (R - dr / 2.)) / dr, 0., 1.)
    return (R <= edge).astype(float)


def ringmode_name(mode):
    m = str(mode).strip().upper()
    m = "CENTRED" if m == "CENTERED" else m
    if m not in RINGMODES:
        raise ValueError(f"Unknown ring convention {mode!r}: RINGMODE can be CENTRED, NODES or SHIFTED.")
    return m


def _half_widths(rings):
    R = rings.radii
    if rings.nr == 1:
        w = rings.radsep / 2. if rings.radsep > 0 else R[0] / 2.
        return w, w
    return (R[1] - R[0]) / 2., (R[-1] - R[-2]) / 2.


def model_rings(rings, mode="CENTRED", subring=0.):
    """The rings whose model (radii as nodes) is the model of ``rings`` with a ring convention
    (``bbarolo/galmod.py:1066-1119``): CENTRED adds the inner and outer half rings with the values of the
    first and last ring (unless narrower than one sub-ring), SHIFTED moves the first/last radius by half of
    RADSEP, NODES returns the rings."""
    mode = ringmode_name(mode)
    if mode == "NODES" and rings.nr == 1:
        raise BBaroloError("RINGMODE NODES needs two radii at least: the disk covers the first to the last radius "
                           "(one ring gave an empty model).")
    if mode == "SHIFTED" and rings.nr == 1 and not rings.radsep > 0:
        raise BBaroloError("RINGMODE SHIFTED with one ring needs RADSEP > 0: the width of the ring.")
    if mode == "NODES" or rings.nr == 0:
        return rings
    r = rings.copy()
    if mode == "SHIFTED":
        if r.nr == 1:
            r.addRing(r.radii[0] + r.radsep / 2., r.xpos[0], r.ypos[0], r.vsys[0], r.vrot[0], r.vdisp[0],
                      r.vrad[0], r.vvert[0], r.dvdz[0], r.zcyl[0], r.dens[0], r.z0[0], r.inc[0], r.phi[0],
                      r.z0thick[0], r.fthick[0], r.vdispthick[0])
        else:
            r.radii[-1] += r.radsep / 2.
        r.radii[0] = max(r.radii[0] - r.radsep / 2., 0.)
        return r
    R = r.radii
    w0, wn = _half_widths(r)
    rin, rout = max(R[0] - w0, 0.), R[-1] + wn
    idx, rad = list(range(r.nr)), list(R)
    if rin / 60. + subring < R[0] / 60.:
        idx.insert(0, 0)
        rad.insert(0, rin)
    if R[-1] / 60. + subring < rout / 60.:
        idx.append(r.nr - 1)
        rad.append(rout)
    out = r.subset(np.array(idx))
    out.radii = np.array(rad, dtype=float)
    return out


def model_rows(rows, proto, mode, radsep):
    """Ring-value rows (B, 17, nr) of ring sets like ``proto`` -> (the rows of their model rings with the ring
    convention ``mode`` (``model_rings``), the model-ring prototype): CENTRED repeats the first/last ring at the
    added half rings, SHIFTED moves the end radii, NODES keeps the rings."""
    if ringmode_name(mode) != "NODES" and proto.nr and isinstance(proto.radii, np.ndarray) and \
            proto.radii.dtype == np.float64:
        mr = model_rings(proto, mode, radsep)        # (a new ring set: proto is copied, not changed)
    else:
        probe = proto.copy()
        probe.radii = np.asarray(proto.radii, float)
        mr = model_rings(probe, mode, radsep)
        if mr is probe:
            return np.asarray(rows, float), probe
    eq = np.asarray(mr.radii, float)[:, None] == np.asarray(proto.radii, float)[None, :]
    idx = np.where(eq.any(axis=1), eq.argmax(axis=1), -1).tolist()     # (the first equal radius, or -1)
    nr = proto.nr
    if idx and idx[0] == -1:
        idx[0] = 0
    if idx and idx[-1] == -1:
        idx[-1] = nr - 1
    if any(i < 0 for i in idx):
        raise ValueError("model_rows: ring convention not representable")
    out = np.asarray(rows, float)[:, :, idx].copy()
    out[:, 0, :] = mr.radii
    return out, mr


def outer_edge(rings, mode="CENTRED"):
    mode = ringmode_name(mode)
    if mode == "NODES":
        return float(rings.radii[-1])
    if mode == "SHIFTED":
        return float(rings.radii[-1] + rings.radsep / 2.)
    return float(rings.radii[-1] + _half_widths(rings)[1])


class SubringGrid:
    """The sub-ring radii of a set of radii (the part of ``subrings`` that depends only on the radii):
    float32-accumulated radii (arcmin), and for each sub-ring the interpolation segment and offset.
    Cached by the engines: during a fit the radii do not change."""

    def __init__(self, rad_arcmin, radsep, empty):
        f32 = np.float32
        rad = np.asarray(rad_arcmin, float)
        nr = rad.size
        radii, seg, dr, const = [], [], [], []
        inner = bool(rad[0] != 0 and empty)
        r = f32(rad[0] + radsep / 2.0) if inner else f32(radsep / 2.0)
        if not inner:
            first = f32(rad[0])
            while r < first:
                radii.append(float(r)); seg.append(0); dr.append(0.); const.append(True)
                r = f32(float(r) + radsep)
        for i in range(1, nr):
            ri = f32(rad[i])
            prev = float(f32(rad[i - 1]))
            while r < ri:
                radii.append(float(r)); seg.append(i); dr.append(float(r) - prev); const.append(False)
                r = f32(float(r) + radsep)
        self.radii = np.asarray(radii, float)
        self.seg = np.asarray(seg, np.int64)
        self.dr = np.asarray(dr, float)
        self.const = np.asarray(const, bool)
        self.nsub = self.radii.size
        i1 = np.maximum(self.seg, 1)
        self.i1 = i1
        if nr > 1:
            self.dur = rad[i1] - rad[i1 - 1]
            self._dseg = rad[1:] - rad[:-1]
        else:
            self.dur = np.ones(self.nsub)

    def interpolate(self, V):
        """V (..., nrow, nr) ring values -> (..., nrow, nsub) sub-ring values (reference operation order:
        v0 + ((v1 - v0) / dur) * dr, constant rows before the first radius)."""
        V = np.asarray(V, float)
        nr = V.shape[-1]
        if V.ndim == 3 and V.shape[0] > 8 and nr > 1 and self.nsub:
            out = self._interpolate_steps(V)
            if out is not None:
                return out
        return self._interpolate_all(V)

    def _interpolate_steps(self, V):
        """A batch whose members differ from member 0 in few rings (the steps of a finite-difference gradient):
        member 0's values, and the same operations on the sub-rings next to a ring that differs (the values
        are those of _interpolate_all, bit for bit); None when more than a quarter of the values differ."""
        i1 = self.i1
        D = np.any(V != V[:1], axis=1)                                   # (B, nr): rings that differ
        if np.count_nonzero(D) * 4 > D.size:
            return None
        A = D[:, i1 - 1] | D[:, i1] | (self.const[None, :] & D[:, :1])   # (B, nsub): sub-rings that differ
        bb, ss = np.nonzero(A)
        if bb.size * 4 > A.size:
            return None
        out = np.repeat(self._interpolate_all(V[:1]), V.shape[0], axis=0)
        if bb.size:
            j = i1[ss]
            v0 = V[bb, :, j - 1]                                         # (P, nrow)
            sl = (V[bb, :, j] - v0) / self._dseg[j - 1][:, None]
            sl *= self.dr[ss][:, None]
            v = v0 + sl
            c = self.const[ss]
            if c.any():
                v[c] = V[bb[c], :, 0]
            out[bb, :, ss] = v
        return out

    def _interpolate_all(self, V):
        nr = V.shape[-1]
        i1 = self.i1
        if nr > 1:
            # the slope of each segment once (dur depends on the segment only), then gathered per sub-ring
            seg = (V[..., 1:] - V[..., :-1]) / self._dseg
            vals = np.take(V, i1 - 1, axis=-1)
            slope = np.take(seg, i1 - 1, axis=-1)
            slope *= self.dr
            vals += slope
        else:
            vals = V[..., i1 - 1] + np.zeros(V.shape[:-1] + (self.nsub,)) * self.dr
        if self.const.any():
            vals[..., self.const] = V[..., 0:1]
        return vals


class GalmodSetup:
    """Header-derived constants of the models of a cube (``bbarolo/galmod.py:609-758``)."""

    def __init__(self, cube, gmpar=None, galmodtype=None, densflux=None):
        h = cube.Head()
        p = cube.pars()
        gm = p.gm if gmpar is None else gmpar
        self.nsubs = cube.DimZ()
        self.dimx, self.dimy = cube.DimX(), cube.DimY()
        cdelt = [0., 0.]
        arcmconv = 0.
        for i in range(2):
            cu = h.Cunit(i).lower()
            if "deg" in cu:
                arcmconv = 60.
            elif "arcs" in cu:
                arcmconv = 1 / 60.
            elif "arcm" in cu:
                arcmconv = 1.
            else:
                raise BBaroloError(f"GALMOD error (unknown CUNIT for RA-DEC): cannot convert to ARCMIN.\n{cu}")
            cdelt[i] = h.Cdelt(i) * arcmconv
        self.arcmconv = arcmconv
        self.cdelt = cdelt
        self.pixsize = [abs(cdelt[0]), abs(cdelt[1])]
        self.pixarea = self.pixsize[0] * self.pixsize[1]
        self.crota2 = h.Crota() * math.pi / 180.
        self.zstep = ZSTEP_FINE
        reds = p.getRedshift()
        cunit3 = h.Cunit(2).lower()
        self.cdelt3, self.crval3, self.crpix3 = h.Cdelt(2), h.Crval(2), h.Crpix(2)
        self.velsys = {"radio": 1, "optical": 2, "relativistic": 3}.get(h.VelDef(), 1)
        sptype = h.SpectralType()
        lfreq0 = None
        self.relint = np.array([1.])
        self.freq0 = 0.1420405751786E10
        if sptype == "wave":
            self.axtyp = 2
            if cunit3 not in WAVE_UNITS:
                raise BBaroloError(f"GALMOD ERROR: unknown CUNIT3={cunit3}. Cannot convert to meters.")
            mconv = 1. / WAVE_UNITS[cunit3]
            self.crval3 *= mconv
            self.cdelt3 *= mconv
            restw = p.getRestwave()
            self.freq0 = C_MS / (restw * (1 + reds) * mconv) if restw != -1 else C_MS / self.crval3
            if len(gm.RESTWAVE) > 1:
                lfreq0 = C_MS / (np.asarray(gm.RESTWAVE, float) * (1 + reds) * mconv)
                self.relint = _relint(gm.RELINT, len(gm.RESTWAVE), "RESTWAVE")
        elif sptype == "freq":
            self.axtyp = 3
            hz = _FREQ_UNITS.get(cunit3)
            if hz is None:
                raise BBaroloError(f"GALMOD ERROR: unknown CUNIT3={cunit3}. Cannot convert to Hz.")
            self.crval3 *= hz
            self.cdelt3 *= hz
            self.freq0 = h.Freq0() / (1 + reds)
            if self.freq0 == 0:
                self.freq0 = 0.1420405751786E10
            if len(gm.RESTFREQ) > 1:
                lfreq0 = np.asarray(gm.RESTFREQ, float) / (1 + reds)
                self.relint = _relint(gm.RELINT, len(gm.RESTFREQ), "RESTFREQ")
        elif "velo" in sptype:
            self.axtyp = 4
            if cunit3 not in VEL_UNITS:
                raise BBaroloError(f"GALMOD ERROR: unknown CUNIT3={cunit3}. Cannot convert to m/s.")
            msconv = 1.0E03 / VEL_UNITS[cunit3]
            self.freq0 = h.Freq0() / (1 + reds)
            if self.freq0 == 0:
                self.freq0 = 0.1420405751786E10
            self.crval3 *= msconv
            self.cdelt3 *= msconv
            if max(len(gm.RESTWAVE), len(gm.RESTFREQ)) > 1:
                sys.stderr.write(" GALMOD WARNING: several lines (RESTWAVE/RESTFREQ) on a velocity axis: only one "
                                 "line is modelled.\n")
        else:
            raise BBaroloError("GALMOD ERROR: unknown Spectral axis type. Check CTYPE3 and CUNIT3 keywords.")
        nch = p.specres if getattr(p, "specres", -1) != -1 else p.linear
        if nch == -1:
            nch = 1. / (2 * math.sqrt(2 * math.log(2)))
        self.chwidth = abs(delta_vel(h)) * 1000
        self.sig_instr = nch * self.chwidth
        self.ltype = gm.LTYPE
        self.cmode = gm.CMODE
        if self.cmode < 0 or self.cmode > 2:
            self.cmode = 1
        self.cdens = float(gm.CDENS)
        if self.cdens < 0:
            self.cdens = 1.
        self.iseed = gm.ISEED
        self.empty = gm.EMPTY
        self.radmaxa = float(getattr(gm, "RADMAXA", -1.))
        self.radmaxr = float(getattr(gm, "RADMAXR", -1.))
        self.densIsFlux = gm.DENSFLUX if densflux is None else densflux
        self.nvpar = gm.NV
        self.galmodtype = (galmodtype or getattr(p, "galmodtype", "MC")).upper()
        self.radsep = 0.75 * min(self.pixsize)
        if self.densIsFlux:
            self.cd2i = np.full(self.nsubs, np.float32(3600. / self.chwidth * 1000.), dtype=np.float64)
        else:
            self.cd2i = self._nhi_to_rad()
        self.lfreq0 = np.ascontiguousarray([self.freq0] if lfreq0 is None else lfreq0, dtype=np.float64)
        self.relint = np.ascontiguousarray(self.relint, dtype=np.float64)
        self._vedges = self._velocity_edges()
        self._vedges_lines = np.ascontiguousarray([self._velocity_edges(f) for f in self.lfreq0])
        self._chmin = float(np.min(np.abs(np.diff(self._vedges)))) if self.nsubs > 0 else self.chwidth
        self._grid_cache = {}

    def _nhi_to_rad(self):
        """Column density (1E20 atoms/cm2) -> flux per channel (``bbarolo/galmod.py:727-741``)."""
        jy, K = 1E-26, 1.3806488E-23
        k = np.arange(self.nsubs)
        w = self.crval3 + self.cdelt3 * (k + 1 - self.crpix3)
        if self.axtyp == 2:
            lab, fac = w, 2.588E04
        elif self.axtyp == 3:
            lab, fac = C_MS / w, 3.8475E-06
        else:
            f = self.freq0 * (1 - w / C_MS)
            if self.velsys == 2:
                f = self.freq0 * (C_MS / (C_MS + w))
            if self.velsys == 3:
                f = self.freq0 * np.sqrt((C_MS - w) / (C_MS + w))
            lab, fac = C_MS / f, 1.823E-05
        ddum = 2 * (K / jy) / (fac * lab * lab) / abs(self.cdelt3)
        return (ddum * (math.pi / (180.0 * 60.0)) ** 2).astype(np.float32).astype(np.float64)

    def _velocity_edges(self, freq0=None):
        """Velocity (m/s) of the channel edges, k - 0.5 for k = 0..nz (``bbarolo/galmod.py:743-758``)."""
        g = np.arange(self.nsubs + 1) - 0.5
        w = (g + 1 - self.crpix3) * self.cdelt3 + self.crval3
        if self.axtyp == 4:
            return w
        f = C_MS / w if self.axtyp == 2 else w
        r = f / (self.freq0 if freq0 is None else freq0)
        if self.velsys == 1:
            v = C_MS * (1 - r)
        elif self.velsys == 2:
            v = C_MS * (1 / r - 1)
        else:
            v = C_MS * (1 - r * r) / (1 + r * r)
        return np.ascontiguousarray(v, dtype=np.float64)

    def side_edges(self, rings):
        out = []
        for attr, default in (("edgeapp", self.radmaxa), ("edgerec", self.radmaxr)):
            e = getattr(rings, attr, None)
            e = default if e is None else float(e)
            out.append(e if e >= 0 else None)
        return tuple(out)

    def grid(self, rings):
        """The SubringGrid of the radii of ``rings`` (cached)."""
        empty = self.empty if getattr(rings, "empty", None) is None else rings.empty
        rad = np.asarray(rings.radii, float) / 60.
        key = (rad.tobytes(), bool(empty))
        g = self._grid_cache.get(key)
        if g is None:
            for i in range(1, rad.size):
                if rad[i - 1] + self.radsep >= rad[i]:
                    if rad[i - 1] > rad[i]:
                        raise BBaroloError("GALMOD ERROR: Radii not in increasing order.")
                    raise BBaroloError("GALMOD ERROR: Radius separation too small.")
            g = SubringGrid(rad, self.radsep, empty)
            if len(self._grid_cache) > 64:
                self._grid_cache.clear()
            self._grid_cache[key] = g
        return g

    def subrings(self, rings):
        """Sub-ring table (16, nsub) float64 and NV per sub-ring (int64), as ``bbarolo/galmod.py:761-851``."""
        if np.any(np.asarray(rings.vdisp) < 0):
            raise ValueError("GALMOD ERROR: Negative velocity dispersion not allowed.")
        if np.any(np.asarray(rings.dens) < 0):
            raise ValueError("GALMOD ERROR: Negative column-density or flux are not allowed.")
        if np.any(np.asarray(rings.z0) < 0):
            raise ValueError("GALMOD ERROR: Negative scale height not allowed.")
        thick = rings.thick() if hasattr(rings, "thick") else False
        if thick:
            ft = np.asarray(rings.fthick, float)
            if np.any((ft < 0) | (ft > 1)):
                raise ValueError("GALMOD ERROR: The fraction of gas in the thick layer (FTHICK) must be 0 to 1.")
        g = self.grid(rings)
        V = ring_value_rows(rings, thick)
        nsub = g.nsub
        sr = np.empty((V.shape[0] + 1, nsub))
        sr[0] = g.radii
        if nsub:
            sr[1:] = g.interpolate(V)
        edge = getattr(rings, "edge", None)
        if edge is not None and nsub:
            sr[5] *= edge_weights(sr[0] * 60., self.radsep * 60., float(edge),
                                  float(getattr(rings, "edgewidth", 0.)))
        if thick:
            f = sr[14]
            thin, thk = sr[:14].copy(), sr[:14].copy()
            thin[5] *= 1. - f
            thin[7] = 0.
            thk[5] *= f
            thk[6], thk[4] = sr[15], sr[16]
            sr = np.concatenate([thin, thk], axis=1)
        side = np.ones((2, sr.shape[1]))
        for k, e in enumerate(self.side_edges(rings)[::-1]):
            if e is not None and sr.shape[1]:
                side[k] = edge_weights(sr[0] * 60., self.radsep * 60., e)
        sr = np.concatenate([sr[:14], side])
        nvtmp = self.nvpar if self.nvpar >= 1 else self.nsubs
        nv = np.where(sr[4] == 0, 1, nvtmp).astype(np.int64)
        return np.ascontiguousarray(sr), nv

    def subcloud_flux(self, sr, nv):
        """Mean flux of one MC sub-cloud (``bbarolo/galmod.py:879-897``)."""
        R0, dens = sr[0], sr[5]
        area_pix = 2 * np.pi * R0 * self.radsep / self.pixarea
        with np.errstate(divide="ignore", invalid="ignore"):
            nc = np.floor(self.cdens * dens ** self.cmode * area_pix + 0.5)
            low = np.floor(nc / area_pix + 0.5) < 10.
            nc = np.where(low, np.floor(10 * area_pix + 0.5), nc)
            w = dens * area_pix
            ok = (w > 0) & (nc > 0)
            if not np.any(ok):
                return 0.
            fsc = w[ok] * self.pixarea / (nc[ok] * nv[ok])
            unit = w[ok].sum() / np.sum(w[ok] / fsc)
        ri = self.relint
        return float(unit * np.sum(ri * ri) / np.sum(ri))


def ring_value_rows(rings, thick):
    """The ring values in internal units, one row per quantity (13 rows, 16 with a thick layer)."""
    rows = [np.asarray(rings.vrot) * 1000., np.asarray(rings.vrad) * 1000.,
            np.asarray(rings.vvert) * 1000., np.asarray(rings.vdisp) * 1000.,
            np.asarray(rings.dens, float), np.asarray(rings.z0) / 60.,
            np.asarray(rings.dvdz) * 1000 * 60, np.asarray(rings.zcyl) / 60.,
            np.radians(np.asarray(rings.inc, float)), np.radians(np.asarray(rings.phi, float)),
            np.asarray(rings.xpos, float), np.asarray(rings.ypos, float),
            np.asarray(rings.vsys) * 1000.]
    if thick:
        vdt = np.asarray(rings.vdispthick, float)
        vdt = np.where(vdt >= 0, vdt, np.asarray(rings.vdisp, float))
        rows += [np.asarray(rings.fthick, float), rings.thick_z0() / 60., vdt * 1000.]
    return np.vstack(rows).astype(float)


def _relint(relint, nlines, name):
    if len(relint) != nlines:
        raise BBaroloError(f"GALMOD ERROR: {name} gives {nlines} lines, but RELINT has {len(relint)} values: give "
                           "one relative intensity per line.")
    return np.array(relint, float)


def ring_rows_batch(rings_list):
    """Ring values of a list of rings with the same radii, as one array (B, 17, nr) in RING_KEYS order."""
    from .rings import RING_KEYS
    return np.stack([np.vstack([np.asarray(getattr(r, k), float) for k in RING_KEYS]) for r in rings_list])


_NATIVE = None


def _native_subrings():
    """The library's ``bbgpu_subrings_rows`` (C++), or None where the library is not built."""
    global _NATIVE
    if _NATIVE is None:
        try:
            from . import _lib
            _NATIVE = _lib.load().bbgpu_subrings_rows
        except Exception:
            _NATIVE = False
    return _NATIVE or None


def subrings_batch(setup, proto, rows, out_ms=None, native=True):
    """Sub-ring tables of a batch of ring sets that share the radii and the options of ``proto`` (edges, thick
    layer, empty): rows (B, 17, nr) in RING_KEYS order -> (sr (B, 16, nsub), nv (B, nsub)).

    The same elementwise float64 operations as ``GalmodSetup.subrings`` (bit-equal tables), vectorised over
    the batch: the fits change ring values, not radii, between evaluations. A thin disk of two or more rings
    is tabulated in C++ (``bbgpu_subrings_rows``: the same operations, member 0 in full and the other members'
    sub-rings next to a ring that differs from member 0's), native=False or a thick layer with numpy.
    out_ms (B, 16, nsm) C-contiguous, nsm >= nsub: also receives the tables in its first nsub columns."""
    rows = np.asarray(rows, float)
    B = rows.shape[0]
    radii, xpos, ypos, vsys, vrot, vdisp, vrad, vvert, dvdz, zcyl, dens, z0, inc, phi, z0t, fth, vdt = \
        (rows[:, i] for i in range(17))
    if np.any(vdisp < 0):
        raise ValueError("GALMOD ERROR: Negative velocity dispersion not allowed.")
    if np.any(dens < 0):
        raise ValueError("GALMOD ERROR: Negative column-density or flux are not allowed.")
    if np.any(z0 < 0):
        raise ValueError("GALMOD ERROR: Negative scale height not allowed.")
    thick = proto.thick() if hasattr(proto, "thick") else False
    g = setup.grid(proto)
    nvtmp = setup.nvpar if setup.nvpar >= 1 else setup.nsubs
    fn = _native_subrings() if native and not thick and g.nsub and rows.shape[2] > 1 else None
    if fn is not None:
        from . import _lib
        edge = getattr(proto, "edge", None)
        edgew = None if edge is None else np.ascontiguousarray(
            edge_weights(g.radii * 60., setup.radsep * 60., float(edge), float(getattr(proto, "edgewidth", 0.))),
            dtype=float)
        side = np.ones((2, g.nsub))
        for k, e in enumerate(setup.side_edges(proto)[::-1]):
            if e is not None:
                side[k] = edge_weights(g.radii * 60., setup.radsep * 60., e)
        rows_c = np.ascontiguousarray(rows)
        sr = np.empty((B, 16, g.nsub))
        nv = np.empty((B, g.nsub), np.int64)
        if out_ms is not None and not (out_ms.flags.c_contiguous and out_ms.dtype == np.float64 and
                                       out_ms.shape[:2] == (B, 16) and out_ms.shape[2] >= g.nsub):
            raise ValueError("subrings_batch: out_ms must be a C-contiguous float64 (B, 16, >= nsub) array")
        rc = fn(_lib.ptr(rows_c), B, rows.shape[2], g.nsub, _lib.ptr(g.i1), _lib.ptr(g.dr), _lib.ptr(g._dseg),
                _lib.ptr(g.const.view(np.uint8)), _lib.ptr(g.radii), _lib.ptr(edgew), _lib.ptr(side), int(nvtmp),
                _lib.ptr(sr), _lib.ptr(nv), _lib.ptr(out_ms), 0 if out_ms is None else out_ms.shape[2])
        if rc != 0:
            raise ValueError(f"bbgpu_subrings_rows: status {rc}")
        return sr, nv
    V = [vrot * 1000., vrad * 1000., vvert * 1000., vdisp * 1000., dens, z0 / 60., dvdz * 1000 * 60, zcyl / 60.,
         np.radians(inc), np.radians(phi), xpos, ypos, vsys * 1000.]
    if thick:
        if np.any((fth < 0) | (fth > 1)):
            raise ValueError("GALMOD ERROR: The fraction of gas in the thick layer (FTHICK) must be 0 to 1.")
        V += [fth, np.where(z0t >= 0, z0t, z0) / 60., np.where(vdt >= 0, vdt, vdisp) * 1000.]
    V = np.stack(V, axis=1)                                    # (B, nrow, nr)
    nsub = g.nsub
    # (a thin layer's table is built in place: 16 rows, the side weights in rows 14-15)
    sr = np.empty((B, 16 if not thick else V.shape[1] + 1, nsub))
    sr[:, 0] = g.radii
    if nsub:
        sr[:, 1:V.shape[1] + 1] = g.interpolate(V)
    edge = getattr(proto, "edge", None)
    if edge is not None and nsub:
        sr[:, 5] *= edge_weights(sr[0, 0] * 60., setup.radsep * 60., float(edge),
                                 float(getattr(proto, "edgewidth", 0.)))
    if thick:
        f = sr[:, 14]
        thin, thk = sr[:, :14].copy(), sr[:, :14].copy()
        thin[:, 5] *= 1. - f
        thin[:, 7] = 0.
        thk[:, 5] *= f
        thk[:, 6], thk[:, 4] = sr[:, 15], sr[:, 16]
        sr = np.concatenate([thin, thk], axis=2)
    side = np.ones((2, sr.shape[2]))
    for k, e in enumerate(setup.side_edges(proto)[::-1]):
        if e is not None and sr.shape[2]:
            side[k] = edge_weights(sr[0, 0] * 60., setup.radsep * 60., e)
    if sr.shape[1] == 16:
        sr[:, 14:16] = side
    else:
        sr = np.concatenate([sr[:, :14], np.broadcast_to(side, (B, 2, sr.shape[2]))], axis=1)
    nv = np.where(sr[:, 4] == 0, 1, nvtmp).astype(np.int64)
    if out_ms is not None:
        out_ms[:, :, :sr.shape[2]] = sr
    return np.ascontiguousarray(sr), np.ascontiguousarray(nv)


def cloud_counts(setup, sr, nv):
    """(clouds, sub-clouds) of the MC model of a sub-ring table (``bbarolo/galmod.py:107-114``)."""
    R0, dens = sr[0], sr[5]
    rap = 2 * math.pi * R0 * setup.radsep / setup.pixarea
    act = dens != 0
    nc = np.floor(setup.cdens * np.where(act, dens, 0.) ** setup.cmode * rap + 0.5)
    with np.errstate(divide="ignore", invalid="ignore"):
        low = np.floor(nc / rap + 0.5) < 10.
    nc = np.where(low, np.floor(10 * rap + 0.5), nc)
    nc = np.where(act, nc, 0).astype(np.int64)
    return int(nc.sum()), int((nc * np.asarray(nv, np.int64)).sum())
