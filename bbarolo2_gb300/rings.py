"""Tilted rings: the parameter arrays of a set of rings, as ``bbarolo.rings.Rings`` (``bbarolo/rings.py:15-145``).

Same attribute names and meaning (arcsec, km/s, degrees, pixels for the centre), same defaults, so that a
reference ``Rings`` object and this one are interchangeable for the model path.
"""

import numpy as np

RING_KEYS = ("radii", "xpos", "ypos", "vsys", "vrot", "vdisp", "vrad", "vvert",
             "dvdz", "zcyl", "dens", "z0", "inc", "phi", "z0thick", "fthick", "vdispthick")


class Rings:
    def __init__(self, nr=0):
        self.radsep = 0.
        self.id = 0
        self.edge, self.edgewidth = None, 0.
        self.edgeapp, self.edgerec = None, None
        self.empty = None
        self.twolayer = None
        for k in RING_KEYS:
            setattr(self, k, np.zeros(nr))
        self.vdispthick = np.full(nr, -1.)

    @property
    def nr(self):
        return len(self.radii)

    def _copy_meta(self, r):
        r.radsep, r.id = self.radsep, self.id
        r.edge, r.edgewidth, r.empty = self.edge, self.edgewidth, getattr(self, "empty", None)
        r.edgeapp, r.edgerec = getattr(self, "edgeapp", None), getattr(self, "edgerec", None)
        r.twolayer = getattr(self, "twolayer", None)
        return r

    def copy(self):
        r = self._copy_meta(Rings())
        for k in RING_KEYS:
            setattr(r, k, np.array(getattr(self, k), dtype=float, copy=True))
        return r

    def subset(self, idx):
        r = self._copy_meta(Rings())
        for k in RING_KEYS:
            setattr(r, k, np.atleast_1d(np.asarray(getattr(self, k))[idx]).astype(float))
        return r

    def setRings(self, **kw):
        """All the ring arrays; scalars are broadcast to the length of radii (``bbarolo/rings.py:67-82``)."""
        radii = np.atleast_1d(np.asarray(kw["radii"], dtype=float))
        n = len(radii)
        dflt = dict(xpos=0, ypos=0, vsys=0, vrot=0, vdisp=0, vrad=0, vvert=0, dvdz=0, zcyl=0,
                    dens=1, z0=0, inc=0, phi=0, z0thick=0, fthick=0, vdispthick=-1)
        self.radii = radii.copy()
        for k in RING_KEYS[1:]:
            v = np.asarray(kw.get(k, dflt[k]), dtype=float)
            setattr(self, k, np.full(n, float(v)) if v.ndim == 0 else v.astype(float).copy())
        self.radsep = kw["radsep"] if "radsep" in kw else (radii[1] - radii[0] if n > 1 else 0)
        return self

    def addRing(self, radii, xpos, ypos, vsys, vrot, vdisp, vrad, vvert, dvdz, zcyl, dens, z0, inc, phi,
                z0thick=0., fthick=0., vdispthick=-1.):
        vals = (radii, xpos, ypos, vsys, vrot, vdisp, vrad, vvert, dvdz, zcyl, dens, z0, inc, phi, z0thick,
                fthick, vdispthick)
        for k, v in zip(RING_KEYS, vals):
            setattr(self, k, np.append(getattr(self, k), float(v)))

    def thick(self):
        tl = getattr(self, "twolayer", None)
        return bool(tl) if tl is not None else bool(np.any(np.asarray(self.fthick, float) > 0))

    def thick_z0(self):
        z = np.asarray(self.z0thick, float)
        return np.where(z >= 0, z, np.asarray(self.z0, float))

    def layer_height(self):
        z0 = np.asarray(self.z0, float)
        if not self.thick():
            return z0
        return np.where(np.asarray(self.fthick, float) > 0, np.maximum(z0, self.thick_z0()), z0)
