"""Header and cube objects with the accessors of BBarolo's ``Cube``/``Header`` that the model path reads.

The reference reads FITS files through astropy (``bbarolo/cube.py``, ``bbarolo/header.py``). The
model-evaluation path only needs the data array and a handful of header scalars, so these classes hold
exactly those, with the reference's accessor names (``Head().Cdelt(i)``, ``DimX()``, ``pars().gf``...):
a ``Cube`` built here can be passed wherever the reference's ``DiskModel(cube, ...)`` takes one.

Conventions follow ``bbarolo/header.py``: CDELT/CRVAL in the axis units (degrees for RA/DEC), BMAJ/BMIN
in degrees, BPA in degrees, the spectral type one of ``"velo-radio"``, ``"velo-opt"``, ``"freq"``,
``"wave"`` (``bbarolo/header.py:319-328``), the data array (nz, ny, nx) float32.
"""

import math
import re
from dataclasses import dataclass, field
from typing import List

import numpy as np


@dataclass
class GalfitPar:
    """The GALMOD/3DFIT parameters read by the model path, with the defaults of
    ``bbarolo/params.py:137-216`` (GalmodPar + GalfitPar)."""
    CDENS: float = 10
    CMODE: int = 1
    ISEED: int = -1
    LTYPE: int = 1
    NV: int = -1
    REDSHIFT: float = 0.0
    EMPTY: bool = True
    DENSFLUX: bool = True
    RESTWAVE: List[float] = field(default_factory=lambda: [-1.0])
    RESTFREQ: List[float] = field(default_factory=lambda: [-1.0])
    RELINT: List[float] = field(default_factory=lambda: [1.0])
    SM: bool = True
    RADMAXA: float = -1.0
    RADMAXR: float = -1.0
    FTYPE: int = 2
    WFUNC: int = 2
    NORM: str = "AZIM"
    BWEIGHT: float = 1.0
    SIDE: str = "B"


class Params:
    """The subset of ``bbarolo.params.Param`` used by the model path (``cube.pars()``)."""

    def __init__(self, **kw):
        self.gf = GalfitPar()
        self.gm = self.gf
        self.specres = -1
        self.linear = -1
        self.galmodtype = "MC"
        self.ringmode = "CENTRED"
        self.threads = 1
        self.verbose = False
        for k, v in kw.items():
            if hasattr(self.gf, k):
                setattr(self.gf, k, v)
            else:
                setattr(self, k, v)

    def getRedshift(self):
        z = self.gf.REDSHIFT
        return 0. if z <= -1 else z

    def getRestwave(self):
        return self.gf.RESTWAVE[0]

    def getRestfreq(self):
        return self.gf.RESTFREQ[0]


class Header:
    """Header scalars of a cube, with the accessors of ``bbarolo.header.Header``."""

    def __init__(self, nx, ny, nz, cdelt, crpix=None, crval=None, cunit=("deg", "deg", "km/s"),
                 sptype="velo-radio", bmaj=0., bmin=0., bpa=0., crota=0., veldef="radio",
                 freq0=0.1420405751786E10, redshift=0., bunit="JY/BEAM", name="SYNTH"):
        self.dims = [int(nx), int(ny), int(nz)]
        self.cdelt = [float(c) for c in cdelt]
        self.crpix = [float(c) for c in (crpix if crpix is not None else
                                         [(n - 1) / 2. + 1 for n in self.dims])]
        self.crval = [float(c) for c in (crval if crval is not None else [60., 0., 0.])]
        self.cunit = list(cunit)
        self.sptype = sptype
        self.bmaj, self.bmin, self.bpa = float(bmaj), float(bmin), float(bpa)
        self.crota = float(crota)
        self.veldef = veldef
        self.freq0 = float(freq0)
        self.redshift = float(redshift)
        self.bunit = bunit
        self.object = name
        self.fitsname = name

    def Cunit(self, i): return self.cunit[i]
    def Cdelt(self, i): return self.cdelt[i]
    def Crpix(self, i): return self.crpix[i]
    def Crval(self, i): return self.crval[i]
    def Crota(self): return self.crota
    def VelDef(self): return self.veldef
    def SpectralType(self): return self.sptype
    def Freq0(self): return self.freq0
    def Redshift(self): return self.redshift
    def Bmaj(self): return self.bmaj
    def Bmin(self): return self.bmin
    def Bpa(self): return self.bpa
    def Bunit(self): return self.bunit
    def Name(self): return self.object
    def DimAx(self, i): return self.dims[i]
    def NumAx(self): return 3
    def PixScale(self): return (abs(self.cdelt[0]) + abs(self.cdelt[1])) / 2.

    def setCrpix(self, i, v): self.crpix[i] = float(v)

    @classmethod
    def from_fits(cls, h):
        """The header of an image from its FITS cards (``fits.FitsHeader``), read as ``bbarolo.header.Header``
        reads them (``bbarolo/header.py:195-407``): pixel spacing from CDELTi (or CDi_i), CRPIX/CRVAL required,
        CTYPE and CUNIT defaults, spatial axes in arcsec or arcmin converted to degrees, the spectral axis (the
        last, or the 3rd/4th of a 4D cube with a Stokes axis) and its type, the rest frequency (FREQ0, RESTFREQ,
        RESTFRQ, else DRVAL3/DUNIT3, else the HI line), BUNIT, CROTA, OBJECT and the beam (BMAJ/BMIN/BPA, the GIPSY
        and CLEAN keywords, or HISTORY cards). The spectral axis of a cube with a Stokes third axis is moved to the
        third place, as ``bbarolo.cube.Cube`` does. ValueError for a header without spacing, CRPIX or CRVAL."""
        return _header_from_cards(cls, h)

    def copy(self):
        h = Header.__new__(Header)
        h.__dict__.update({k: (list(v) if isinstance(v, list) else v) for k, v in self.__dict__.items()})
        return h


class Cube:
    """A data cube (nz, ny, nx) float32 with its header and parameters (``bbarolo.cube.Cube`` accessors)."""

    def __init__(self, array, head, par=None):
        a = np.asarray(array, dtype=np.float32)
        if a.ndim != 3:
            raise ValueError("Cube: the data must be a 3D array (nz, ny, nx)")
        self.array = np.ascontiguousarray(a)
        self.head = head
        self.par = par if par is not None else Params()
        nz, ny, nx = self.array.shape
        if head.dims != [nx, ny, nz]:
            raise ValueError(f"Cube: header dimensions {head.dims} do not match the data {nx}x{ny}x{nz}")

    def Head(self): return self.head
    def pars(self): return self.par
    def DimX(self): return self.array.shape[2]
    def DimY(self): return self.array.shape[1]
    def DimZ(self): return self.array.shape[0]

    @classmethod
    def from_fits(cls, name, par=None):
        """A cube read from a FITS file (``bbarolo.cube.Cube(fname)``, ``bbarolo/cube.py:182-261``): the image of
        the file (``fits.read_fits``: the primary HDU or the first image extension; ``file.fits[n]`` names one),
        its header read as the reference reads it (``Header.from_fits``), the first Stokes plane of a 4D cube,
        blank (NaN) voxels set to 0, float32."""
        from . import fits
        fh, data = fits.read_fits(name)
        if data is None:
            raise ValueError(f"{name}: no image")
        head = Header.from_fits(fh)
        head.fitsname = str(name)
        nx, ny, nz = head.dims
        a = np.asarray(data)
        if a.ndim == 4:
            a = a[:, 0] if head._stokes3 else a[0]
        a = np.array(a.reshape(-1)[:nx * ny * nz].reshape(nz, ny, nx), dtype=np.float32)
        a[np.isnan(a)] = 0.0
        return cls(a, head, par)

    @classmethod
    def empty(cls, nx, ny, nz, cdelt, beam=None, par=None, **hkw):
        """An empty cube (as ``bbarolo.utils.emptyfits``): beam FWHM in degrees (one value: circular)."""
        if beam is not None:
            b = list(np.atleast_1d(beam).astype(float))
            hkw.setdefault("bmaj", b[0])
            hkw.setdefault("bmin", b[1] if len(b) > 1 else b[0])
            hkw.setdefault("bpa", b[2] if len(b) > 2 else 0.)
        h = Header(nx, ny, nz, cdelt, **hkw)
        return cls(np.zeros((nz, ny, nx), np.float32), h, par)


# ------------------------------------------------------------------------------------------ FITS header reading
_VEL_UNITS = ("km/s", "m/s", "cm/s")
_VEL_SPELLING = re.compile(r"((?:k|c)?m)(?:/s(?:ec)?|\.?s(?:\^|\*\*)?-1)")


def _velocity_unit(u):
    """km/s, m/s or cm/s for the spellings of a velocity unit (km s-1, km.s-1, m/sec, ...); others unchanged."""
    t = str(u).strip().lower().replace(" ", "")
    if t in _VEL_UNITS:
        return u
    m = _VEL_SPELLING.fullmatch(t)
    return m.group(1) + "/s" if m else u


def _deg_factor(unit):
    u = unit.lower()
    return 1.0 if "deg" in u else (1.0 / 60.0 if "arcm" in u else 1.0 / 3600.0)


def _object_name(obj):
    out = str(obj)
    for a in "/\\()":
        out = out.replace(a, "-")
    return "".join("_" if ch.isspace() else ch for ch in out)


def _header_from_cards(cls, h):
    n = int(h.get("NAXIS", 0))
    dims = [int(h.get(f"NAXIS{i + 1}", 1)) for i in range(n)]
    cd = [h.get(f"CD{i + 1}_{i + 1}") for i in range(n)]
    cdelt = [h.get(f"CDELT{i + 1}") for i in range(n)]
    if all(v is None for v in cdelt):
        if any(v is None for v in cd):
            raise ValueError("FITS header: no pixel spacing (CDELTi or CDi_i)")
        cdelt = cd
    cdelt = [float(c if c is not None else (cd[i] or 1.0)) for i, c in enumerate(cdelt)]
    crpix = [h.get(f"CRPIX{i + 1}") for i in range(n)]
    crval = [h.get(f"CRVAL{i + 1}") for i in range(n)]
    if n and all(v is None for v in crpix):
        raise ValueError("FITS header: no CRPIXi")
    if n and all(v is None for v in crval):
        raise ValueError("FITS header: no CRVALi")
    crpix = [float(v) if v is not None else 1.0 for v in crpix]
    crval = [float(v) if v is not None else 0.0 for v in crval]
    ctype = [h.get(f"CTYPE{i + 1}") for i in range(n)]
    if all(v is None for v in ctype):
        ctype = [("RA---NCP", "DEC--NCP", "VRAD")[i] if i < 3 else "" for i in range(n)]
    ctype = [str(v) if v is not None else "" for v in ctype]

    def spectral_default(i):
        # a velocity axis without unit: m/s when its channels are wider than 100 (km/s channels are never that wide)
        return "m/s" if abs(cdelt[i]) > 100 else "km/s"

    cunit = [h.get(f"CUNIT{i + 1}") for i in range(n)]
    if all(v is None for v in cunit):
        cunit = ["deg", "deg"] + (["hz" if "freq" in ctype[2].lower() else spectral_default(2)] if n > 2 else [])
        cunit = (cunit + [""] * n)[:n]
    else:
        cunit = [_velocity_unit(str(v)) if v is not None else "" for v in cunit]
        for i in range(n):
            if cunit[i] != "":
                continue
            ct = ctype[i].lower()
            if "stokes" in ct:
                cunit[i] = "stokes"
            elif i >= 2:
                cunit[i] = "hz" if "freq" in ct else spectral_default(i)
            else:
                cunit[i] = "deg"
    for i in range(min(n, 2)):
        cu = cunit[i].lower()
        if "arcs" in cu or "arcm" in cu:
            f = _deg_factor(cu)
            cdelt[i] *= f
            crval[i] *= f
            cunit[i] = "deg"
    if n > 0 and "RA" in ctype[0] and crval[0] < 0:
        crval[0] += 360.0
    bunit = str(h.get("BUNIT", "NONE"))
    if "beam-1" in bunit.lower() and "jy" in bunit.lower():
        m = re.match(r"\s*(m|u|\u00b5|\u03bc|mu)?\s*jy", bunit, re.I)
        pre = m.group(1) if m and m.group(1) else ""
        bunit = f"{pre}Jy/beam" if pre else "JY/BEAM"
    # the spectral axis
    sp = n - 1
    if n > 3:
        sp = 3 if "stokes" in ctype[2].lower() else 2
    cu2 = cunit[sp].lower() if n else ""
    ct2 = ctype[sp].lower() if n else ""
    if any(w in ct2 for w in ("wav",)) or any(w in cu2 for w in ("um", "nm", "ang", "micr")):
        sptype = "wave"
    elif "freq" in ct2 or "hz" in cu2:
        sptype = "freq"
    elif "vopt" in ct2 or "felo" in ct2:
        sptype = "velo-opt"
    elif "vel" in ct2 or "vrad" in ct2 or "m/s" in cu2:
        sptype = "velo-radio"
    else:
        sptype = "unknown"
    freq0 = None
    for k in ("FREQ0", "RESTFREQ", "RESTFRQ"):
        if k in h:
            v = h.get(k)
            try:
                freq0 = float(v) if v is not None and float(v) > 0 else None
            except (TypeError, ValueError):
                freq0 = None
            break
    if freq0 is None:
        dunit3, drval3 = str(h.get("DUNIT3", "NONE")), float(h.get("DRVAL3", 0.0))
        if dunit3 == "NONE" or drval3 == 0 or ("hz" in cu2 and "m/s" in cu2):
            freq0 = 0.1420405751786E10
        else:
            du = _velocity_unit(dunit3).lower()
            d = drval3 * (1000.0 / {"km/s": 1.0, "kms": 1.0, "m/s": 1E03, "ms": 1E03, "cm/s": 1E05}[du]) \
                if du in ("km/s", "kms", "m/s", "ms", "cm/s") else 0.0
            c3 = crval[sp] * {"hz": 1.0, "khz": 1E03, "mhz": 1E06, "ghz": 1E09}.get(cu2, 0.0)
            freq0 = c3 * math.sqrt((299792458. + d) / (299792458. - d))
    # the beam
    clmaj = clmin = 0.0
    bmaj = h.get("BMAJ", h.get("BMMAJ"))
    if bmaj is None:
        clmaj, bmaj = float(h.get("CLBMMAJ", 0.0)), 0.0
    bmin = h.get("BMIN", h.get("BMMIN"))
    if bmin is None:
        clmin, bmin = float(h.get("CLBMMIN", 0.0)), 0.0
    bpa = h.get("BPA", h.get("BMPA"))
    beam = {"bmaj": float(bmaj), "bmin": float(bmin), "bpa": float(0.0 if bpa is None else bpa)}
    if beam["bmaj"] == 0 and beam["bmin"] == 0 and beam["bpa"] == 0 and clmaj == 0 and clmin == 0:
        for c in h.cards:
            if c.keyword in ("", "END"):
                continue
            for kw, key in (("BMAJ=", "bmaj"), ("BMIN=", "bmin"), ("BPA=", "bpa")):
                f = c.image.find(kw)
                if f >= 0:
                    try:
                        beam[key] = float(c.image[f + len(kw):].split()[0])
                    except (ValueError, IndexError):
                        pass
    for kw, key in (("BMMAJ", "bmaj"), ("BMMIN", "bmin")):
        # GIPSY writes a beam in arcsec with a Fortran exponent (3.0000000D+01)
        if kw in h:
            c = h._first[kw]
            if c.image[8:10] == "= " and "D" in c.image[10:].split("/", 1)[0]:
                beam[key] /= 3600.0
    if clmaj != 0:
        beam["bmaj"] = clmaj / 3600.0
    if clmin != 0:
        beam["bmin"] = clmin / 3600.0
    # the first three axes, the spectral one third (a Stokes third axis of a 4D cube swapped out)
    stokes3 = n > 3 and ctype[2].lower() == "stokes"
    ax = [0, 1, 3 if stokes3 else 2]
    get = lambda arr, dflt: [arr[i] if i < n else dflt for i in ax]
    veldef = {"velo-radio": "radio", "velo-opt": "optical", "freq": "radio", "wave": "relativistic"}.get(sptype,
                                                                                                     "auto")
    head = cls(*get(dims, 1), cdelt=get(cdelt, 1.0), crpix=get(crpix, 1.0), crval=get(crval, 0.0),
               cunit=tuple(get(cunit, "")), sptype=sptype, crota=float(h.get("CROTA", 0.0)), veldef=veldef,
               freq0=freq0, bunit=bunit, name=_object_name(h.get("OBJECT", "NONE")), **beam)
    head.ctype = get(ctype, "")
    head._stokes3 = stokes3
    return head
