"""Header and cube objects with the accessors of BBarolo's ``Cube``/``Header`` that the model path reads.

The reference reads FITS files through astropy (``bbarolo/cube.py``, ``bbarolo/header.py``). The
model-evaluation path only needs the data array and a handful of header scalars, so these classes hold
exactly those, with the reference's accessor names (``Head().Cdelt(i)``, ``DimX()``, ``pars().gf``...):
a ``Cube`` built here can be passed wherever the reference's ``DiskModel(cube, ...)`` takes one.

Conventions follow ``bbarolo/header.py``: CDELT/CRVAL in the axis units (degrees for RA/DEC), BMAJ/BMIN
in degrees, BPA in degrees, the spectral type one of ``"velo-radio"``, ``"velo-opt"``, ``"freq"``,
``"wave"`` (``bbarolo/header.py:319-328``), the data array (nz, ny, nx) float32.
"""

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
    def empty(cls, nx, ny, nz, cdelt, beam=None, par=None, **hkw):
        """An empty cube (as ``bbarolo.utils.emptyfits``): beam FWHM in degrees (one value: circular)."""
        if beam is not None:
            b = list(np.atleast_1d(beam).astype(float))
            hkw.setdefault("bmaj", b[0])
            hkw.setdefault("bmin", b[1] if len(b) > 1 else b[0])
            hkw.setdefault("bpa", b[2] if len(b) > 2 else 0.)
        h = Header(nx, ny, nz, cdelt, **hkw)
        return cls(np.zeros((nz, ny, nx), np.float32), h, par)
