"""Host side of the GALMOD model: header-derived constants and the sub-ring tables the device kernels read.

What this module computes, and the reference code whose numbers it reproduces:

* ``GalmodSetup``: the constants of ``bbarolo/galmod.py:609-758`` (pixel sizes in arcmin, the pixel area, CROTA2
  in radians, the spectral axis in SI units with the reference frequency of each line, the instrumental
  dispersion, the channel factor ``cd2i`` rounded to float32 and the channel edges in velocity). Here the
  spectral axis is an object (``SpectralAxis``, one subclass per axis type) and the units are tables, but each
  number is formed by the reference's float64 operations in the reference's order: the device results are
  bit-exact only if these constants are;
* ``GalmodSetup.subrings`` (``bbarolo/galmod.py:761-851``): rings -> sub-rings 0.75 pixel apart (``SubringGrid``:
  float32 accumulation of the radii, linear interpolation of the ring values), the outer edge, the thick layer,
  the side weights (rows 14-15);
* the ring conventions (``RINGMODE``, ``bbarolo/galmod.py:1043-1141``) as ``RingConvention`` objects.

The sub-ring table ``sr`` has the reference's layout (16, nsub), internal units (arcmin, m/s, radians), rows:
radius, vrot, vrad, vvert, vdisp, dens, z0, dvdz, zcyl, inc, phi, xpos, ypos, vsys, wrec, wapp.
"""

import math
import sys

import numpy as np

C_MS = 2.99792458e08
# velocity, wavelength and frequency units: the number of units in km/s, m and Hz respectively
VEL_UNITS = {"km/s": 1., "kms": 1., "m/s": 1E03, "ms": 1E03, "cm/s": 1E05}
WAVE_UNITS = {"m": 1., "cm": 1E02, "mm": 1E03, "um": 1E06, "mum": 1E06, "micron": 1E06, "nm": 1E09,
              "a": 1E10, "angstrom": 1E10}
_HZ_PER_UNIT = {"hz": 1., "khz": 1E03, "mhz": 1E06, "ghz": 1E09}
# sky units (a substring of CUNIT) in arcmin and in arcsec
_ARCMIN_PER = (("deg", 60.), ("arcs", 1 / 60.), ("arcm", 1.))
_ARCSEC_PER = (("deg", 3600.), ("arcm", 60.), ("arcs", 1.))
HI_FREQ = 0.1420405751786E10

# vertical samples of the ANALYTIC model (bbarolo/galmod.py:262-273)
ZSAMPLES_MAX = 1024
ZSTEP_FINE = 0.25
ZSTEP_COARSE = 0.75
ZSTEP_BEAM = 3.0

# rows of the sub-ring table
SR_R, SR_VROT, SR_VRAD, SR_VVERT, SR_VDISP, SR_DENS, SR_Z0, SR_DVDZ, SR_ZCYL, SR_INC, SR_PHI, SR_XPOS, \
    SR_YPOS, SR_VSYS, SR_WREC, SR_WAPP = range(16)


class BBaroloError(ValueError):
    """Invalid input of the model path (the reference's ``bbarolo.bbutils.BBaroloError``)."""


def seed32(iseed):
    """The seed of the MC stream: ISEED & 0xFFFFFFFF (ISEED -1 -> 0xFFFFFFFF), ``bbarolo/galmod.py:593-594``."""
    return int(iseed) & 0xFFFFFFFF


def _lookup(cunit, table, what):
    c = cunit.lower()
    for key, f in table:
        if key in c:
            return f
    raise BBaroloError(f"{what}: sky axis unit {cunit!r} is not degrees, arcminutes or arcseconds")


def arcsconv(cunit):
    """Arcseconds per unit of a sky axis (``bbarolo/bbutils.py:227-232``)."""
    return _lookup(cunit, _ARCSEC_PER, "arcsconv")


def arcmconv(cunit):
    """Arcminutes per unit of a sky axis (the conversion of ``bbarolo/galmod.py:618-626``)."""
    return _lookup(cunit, _ARCMIN_PER, "GALMOD")


# Doppler conventions: velocity (m/s) of the ratio r = f / f0 of an observed to a reference frequency
_DOPPLER = {1: lambda r: C_MS * (1 - r),                        # radio
            2: lambda r: C_MS * (1 / r - 1),                    # optical
            3: lambda r: C_MS * (1 - r * r) / (1 + r * r)}      # relativistic
_VELDEF = {"radio": 1, "optical": 2, "relativistic": 3}


def delta_vel(h):
    """Channel width in km/s (``bbarolo/bbutils.py:159-180``): a velocity axis directly, a frequency axis as its
    radio width or the mean width of its channels in velocity."""
    unit = h.Cunit(2).lower()
    if unit in VEL_UNITS:
        return h.Cdelt(2) / VEL_UNITS[unit]
    if unit in _HZ_PER_UNIT:
        hz = _HZ_PER_UNIT[unit]
        frest = h.Freq0() / (1 + h.Redshift())
        vd = _VELDEF.get(h.VelDef(), 1)
        if vd == 1:
            return -(C_MS / 1000.) * h.Cdelt(2) * hz / frest
        nz = h.DimAx(2)
        k = np.arange(nz - 1)
        lo = (k + 1 - h.Crpix(2)) * h.Cdelt(2) + h.Crval(2)
        hi = (k + 2 - h.Crpix(2)) * h.Cdelt(2) + h.Crval(2)
        kms = {1: lambda f: (C_MS / 1000.) * (1 - f / frest),
               2: lambda f: (C_MS / 1000.) * (frest / f - 1),
               3: lambda f: (C_MS / 1000.) * (1 - (f / frest) ** 2) / (1 + (f / frest) ** 2)}[vd]
        return float(np.sum(kms(hi * hz) - kms(lo * hz)) / (nz - 1))
    if unit in WAVE_UNITS:
        raise BBaroloError("delta_vel: wavelength axes need the rest wavelength of the cube (not supported)")
    return h.Cdelt(2)


class SpectralAxis:
    """The spectral axis of a cube in SI units (``bbarolo/galmod.py:630-700``): ``code`` (2 wavelength, 3 frequency,
    4 velocity), ``crval``, ``cdelt``, ``crpix``, the reference frequency ``freq0`` of the first line, and the
    lines (``lfreq0``: their reference frequencies, ``relint``: their relative intensities)."""

    code = 0

    def __init__(self, h, p, gm):
        self.velsys = _VELDEF.get(h.VelDef(), 1)
        self.crpix = h.Crpix(2)
        self.redshift = p.getRedshift()
        self.freq0 = HI_FREQ
        self.lfreq0 = None
        self.relint = np.array([1.])

    @staticmethod
    def of(h, p, gm):
        kind = h.SpectralType()
        for cls in (WavelengthAxis, FrequencyAxis, VelocityAxis):
            if cls.matches(kind):
                return cls(h, p, gm)
        raise BBaroloError("GALMOD ERROR: unknown Spectral axis type. Check CTYPE3 and CUNIT3 keywords.")

    def _lines(self, given, name, gm, to_freq):
        """Several rest lines (RESTWAVE/RESTFREQ with more than one value): their frequencies and intensities."""
        if len(given) > 1:
            if len(gm.RELINT) != len(given):
                raise BBaroloError(f"GALMOD ERROR: {name} gives {len(given)} lines, but RELINT has {len(gm.RELINT)} "
                                   "values: give one relative intensity per line.")
            self.lfreq0 = to_freq(np.asarray(given, float))
            self.relint = np.array(gm.RELINT, float)

    def velocity(self, w, freq0):
        """Velocity (m/s) of axis values w (SI) for a line of reference frequency freq0."""
        return _DOPPLER[self.velsys]((C_MS / w if self.code == 2 else w) / freq0)

    def rest_wavelength(self, w):
        """The wavelength (m) of the line at axis values w, and the flux-conversion factor of this axis type
        (the column density of ``bbarolo/galmod.py:727-741``)."""
        raise NotImplementedError


class WavelengthAxis(SpectralAxis):
    code = 2

    @staticmethod
    def matches(kind):
        return kind == "wave"

    def __init__(self, h, p, gm):
        super().__init__(h, p, gm)
        unit = h.Cunit(2).lower()
        if unit not in WAVE_UNITS:
            raise BBaroloError(f"GALMOD ERROR: unknown CUNIT3={unit}. Cannot convert to meters.")
        to_m = 1. / WAVE_UNITS[unit]
        self.crval, self.cdelt = h.Crval(2) * to_m, h.Cdelt(2) * to_m
        restw = p.getRestwave()
        z1 = 1 + self.redshift
        self.freq0 = C_MS / (restw * z1 * to_m) if restw != -1 else C_MS / self.crval
        self._lines(gm.RESTWAVE, "RESTWAVE", gm, lambda w: C_MS / (w * z1 * to_m))

    def rest_wavelength(self, w):
        return w, 2.588E04


class FrequencyAxis(SpectralAxis):
    code = 3

    @staticmethod
    def matches(kind):
        return kind == "freq"

    def __init__(self, h, p, gm):
        super().__init__(h, p, gm)
        unit = h.Cunit(2).lower()
        hz = _HZ_PER_UNIT.get(unit)
        if hz is None:
            raise BBaroloError(f"GALMOD ERROR: unknown CUNIT3={unit}. Cannot convert to Hz.")
        self.crval, self.cdelt = h.Crval(2) * hz, h.Cdelt(2) * hz
        self.freq0 = h.Freq0() / (1 + self.redshift) or HI_FREQ
        self._lines(gm.RESTFREQ, "RESTFREQ", gm, lambda f: f / (1 + self.redshift))

    def rest_wavelength(self, w):
        return C_MS / w, 3.8475E-06


class VelocityAxis(SpectralAxis):
    code = 4

    @staticmethod
    def matches(kind):
        return "velo" in kind

    def __init__(self, h, p, gm):
        super().__init__(h, p, gm)
        unit = h.Cunit(2).lower()
        if unit not in VEL_UNITS:
            raise BBaroloError(f"GALMOD ERROR: unknown CUNIT3={unit}. Cannot convert to m/s.")
        to_ms = 1.0E03 / VEL_UNITS[unit]
        self.freq0 = h.Freq0() / (1 + self.redshift) or HI_FREQ
        self.crval, self.cdelt = h.Crval(2) * to_ms, h.Cdelt(2) * to_ms
        if max(len(gm.RESTWAVE), len(gm.RESTFREQ)) > 1:
            sys.stderr.write(" GALMOD WARNING: several lines (RESTWAVE/RESTFREQ) on a velocity axis: only one line "
                             "is modelled.\n")

    def velocity(self, w, freq0):
        return w

    def rest_wavelength(self, w):
        shift = {1: lambda: self.freq0 * (1 - w / C_MS),
                 2: lambda: self.freq0 * (C_MS / (C_MS + w)),
                 3: lambda: self.freq0 * np.sqrt((C_MS - w) / (C_MS + w))}[self.velsys]
        return C_MS / shift(), 1.823E-05


# ------------------------------------------------------------------------------------------ outer edges
def edge_weights(R, dr, edge, width=0.):
    """The weights of sub-rings of radii R (arcsec), each dr wide, for a disk ending at the radius ``edge``
    (``bbarolo/galmod.py:1122-1131``): the part of each sub-ring inside it for a sharp edge (width 0, and a step
    for dr 0), else the Gaussian edge 1/2 erfc((R - edge) / (sqrt(2) width))."""
    R = np.asarray(R, float)
    if width > 0:
        from scipy.special import erfc
        return 0.5 * erfc((R - edge) / (math.sqrt(2.) * width))
    if not dr > 0:
        return (R <= edge).astype(float)
    inside = (edge - (R - dr / 2.)) / dr
    return np.clip(inside, 0., 1.)


# ------------------------------------------------------------------------------------------ ring conventions
class RingConvention:
    """A ring convention (RINGMODE, ``bbarolo/galmod.py:1043-1141``): how the fitted rings map to the radii (used as
    nodes of the linear interpolation) of their model, and where the disk ends."""

    name = ""

    def model(self, rings, subring):
        raise NotImplementedError

    def outer(self, rings):
        raise NotImplementedError


class _Nodes(RingConvention):
    """The ring values sit at the radii; the disk covers the first to the last radius."""
    name = "NODES"

    def model(self, rings, subring):
        if rings.nr == 1:
            raise BBaroloError("RINGMODE NODES: a single ring makes an empty disk (the disk spans the first to the "
                               "last radius); give two radii at least.")
        return rings

    def outer(self, rings):
        return float(rings.radii[-1])


class _Shifted(RingConvention):
    """BBarolo 1.x: the first and last radius moved inwards and outwards by half of RADSEP."""
    name = "SHIFTED"

    def model(self, rings, subring):
        if rings.nr == 1 and not rings.radsep > 0:
            raise BBaroloError("RINGMODE SHIFTED: a single ring needs RADSEP > 0 (its width).")
        half = rings.radsep / 2.
        if rings.nr == 1:
            out = rings.subset(np.array([0, 0]))
            out.radii = np.array([rings.radii[0], rings.radii[0] + half], dtype=float)
        else:
            out = rings.copy()
            out.radii[-1] += half
        out.radii[0] = max(out.radii[0] - half, 0.)
        return out

    def outer(self, rings):
        return float(rings.radii[-1] + rings.radsep / 2.)


class _Centred(RingConvention):
    """Each ring an annulus reaching halfway to its neighbours (the rings 3DFIT fits): the disk extends half a ring
    beyond the first and last radius with their values, an extension narrower than one sub-ring left out."""
    name = "CENTRED"

    @staticmethod
    def halves(rings):
        R = rings.radii
        if rings.nr > 1:
            return (R[1] - R[0]) / 2., (R[-1] - R[-2]) / 2.
        w = rings.radsep / 2. if rings.radsep > 0 else R[0] / 2.
        return w, w

    def model(self, rings, subring):
        R = np.asarray(rings.radii, float)
        first, last = self.halves(rings)
        rin, rout = max(R[0] - first, 0.), R[-1] + last
        pre = int(rin / 60. + subring < R[0] / 60.)       # (compared in arcmin, the sub-ring's unit)
        post = int(R[-1] / 60. + subring < rout / 60.)
        idx = np.r_[[0] * pre, np.arange(rings.nr), [rings.nr - 1] * post].astype(int)
        out = rings.subset(idx)
        out.radii = np.r_[[rin] * pre, R, [rout] * post].astype(float)
        return out

    def outer(self, rings):
        return float(rings.radii[-1] + self.halves(rings)[1])


CONVENTIONS = {c.name: c for c in (_Centred(), _Nodes(), _Shifted())}
RINGMODES = tuple(CONVENTIONS)


def ringmode_name(mode):
    """The canonical name of a ring convention (CENTERED accepted)."""
    m = str(mode).strip().upper().replace("CENTERED", "CENTRED")
    if m not in CONVENTIONS:
        raise ValueError(f"RINGMODE {mode!r} unknown: the conventions are CENTRED, NODES and SHIFTED.")
    return m


def model_rings(rings, mode="CENTRED", subring=0.):
    """The rings whose model (radii as nodes) is the model of ``rings`` under a ring convention; subring: the
    sub-ring width in arcmin (GalmodSetup.radsep). A new ring set, or ``rings`` itself when nothing changes."""
    if rings.nr == 0:
        return rings
    return CONVENTIONS[ringmode_name(mode)].model(rings, subring)


def outer_edge(rings, mode="CENTRED"):
    """The outer radius (arcsec) of the disk of the rings under a ring convention."""
    return CONVENTIONS[ringmode_name(mode)].outer(rings)


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
    """The constants of the models of a cube, computed once per cube (``bbarolo/galmod.py:609-758``): the sky
    grid, the spectral axis (``SpectralAxis``), the line and cloud options of the GALMOD parameters, the channel
    factor ``cd2i`` and the channel edges in velocity of each line."""

    def __init__(self, cube, gmpar=None, galmodtype=None, densflux=None):
        h = cube.Head()
        p = cube.pars()
        gm = p.gm if gmpar is None else gmpar
        self.nsubs = cube.DimZ()
        self.dimx, self.dimy = cube.DimX(), cube.DimY()
        # the sky grid in arcmin
        conv = [arcmconv(h.Cunit(i)) for i in range(2)]
        self.arcmconv = conv[1]
        self.cdelt = [h.Cdelt(i) * conv[i] for i in range(2)]
        self.pixsize = [abs(c) for c in self.cdelt]
        self.pixarea = self.pixsize[0] * self.pixsize[1]
        self.crota2 = h.Crota() * math.pi / 180.
        self.radsep = 0.75 * min(self.pixsize)
        self.zstep = ZSTEP_FINE
        # the spectral axis (SI) and the lines
        ax = self.axis = SpectralAxis.of(h, p, gm)
        self.axtyp, self.velsys = ax.code, ax.velsys
        self.crval3, self.cdelt3, self.crpix3 = ax.crval, ax.cdelt, ax.crpix
        self.freq0 = ax.freq0
        self.lfreq0 = np.ascontiguousarray([ax.freq0] if ax.lfreq0 is None else ax.lfreq0, dtype=np.float64)
        self.relint = np.ascontiguousarray(ax.relint, dtype=np.float64)
        # the instrumental dispersion: SPECRES (or LINEAR) channels, by default the Gaussian of one channel's FWHM
        per_channel = p.specres if getattr(p, "specres", -1) != -1 else p.linear
        if per_channel == -1:
            per_channel = 1. / (2 * math.sqrt(2 * math.log(2)))
        self.chwidth = abs(delta_vel(h)) * 1000
        self.sig_instr = per_channel * self.chwidth
        # the clouds and the lines
        self.ltype = gm.LTYPE
        self.cmode = gm.CMODE if 0 <= gm.CMODE <= 2 else 1
        self.cdens = float(gm.CDENS) if gm.CDENS >= 0 else 1.
        self.iseed = gm.ISEED
        self.empty = gm.EMPTY
        self.radmaxa = float(getattr(gm, "RADMAXA", -1.))
        self.radmaxr = float(getattr(gm, "RADMAXR", -1.))
        self.densIsFlux = gm.DENSFLUX if densflux is None else densflux
        self.nvpar = gm.NV
        self.galmodtype = (galmodtype or getattr(p, "galmodtype", "MC")).upper()
        # flux per channel of a unit of DENS (arcsec^2 -> arcmin^2 and km/s -> m/s; float32 as the reference)
        self.cd2i = np.full(self.nsubs, np.float32(3600. / self.chwidth * 1000.), dtype=np.float64) \
            if self.densIsFlux else self._column_density_factor()
        self._vedges = self._velocity_edges()
        self._vedges_lines = np.ascontiguousarray([self._velocity_edges(f) for f in self.lfreq0])
        self._chmin = float(np.min(np.abs(np.diff(self._vedges)))) if self.nsubs > 0 else self.chwidth
        self._grid_cache = {}

    def _column_density_factor(self):
        """The flux per channel of a column density of 1E20 atoms/cm^2 (``bbarolo/galmod.py:727-741``): 2 k_B /
        (f lambda^2) per channel width, in the reference's order, rounded to float32."""
        w = self.crval3 + self.cdelt3 * (np.arange(self.nsubs) + 1 - self.crpix3)
        lam, fac = self.axis.rest_wavelength(w)
        per_jy = 1.3806488E-23 / 1E-26
        ddum = 2 * per_jy / (fac * lam * lam) / abs(self.cdelt3)
        return (ddum * (math.pi / (180.0 * 60.0)) ** 2).astype(np.float32).astype(np.float64)

    def _velocity_edges(self, freq0=None):
        """The velocity (m/s) of the channel edges k - 0.5, k = 0..nz (``bbarolo/galmod.py:743-758``), for the line of
        reference frequency freq0 (default: the first line)."""
        edges = np.arange(self.nsubs + 1) - 0.5
        w = (edges + 1 - self.crpix3) * self.cdelt3 + self.crval3
        return np.ascontiguousarray(self.axis.velocity(w, self.freq0 if freq0 is None else freq0),
                                    dtype=np.float64)

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
        """Sub-ring table (16, nsub) float64 and NV per sub-ring (int64) of a ring set (``bbarolo/galmod.py:761-851``):
        the batch tabulation of ``subrings_batch`` for one member (numpy)."""
        sr, nv = subrings_batch(self, rings, ring_rows_batch([rings]), native=False)
        return sr[0], nv[0]

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
