"""Loading of the golden fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py from the reference)."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


def cases(name):
    z = load(name)
    return z, json.loads(str(z["index"]))


def dense(idx, val, shape):
    a = np.zeros(int(np.prod(shape)))
    a[idx] = val
    return a.reshape(shape)


def call_args_mc(meta, arrs, nm):
    """The _galmod_mc arguments of a fixture case (after out, sr, ring_lo, ring_hi)."""
    m = meta
    return (m["seed32"], m["radsep"], arrs[nm + "/nv"], m["cdens"], m["cmode"], m["pixarea"], m["cdelt0"],
            m["cdelt1"], m["crota2"], m["blo"][0], m["blo"][1], m["bhi"][0], m["bhi"][1], m["ltype"],
            m["sig_instr"], m["axtyp"], m["velsys"], arrs[nm + "/lfreq0"], m["crval3"], m["cdelt3"], m["crpix3"],
            arrs[nm + "/relint"], arrs[nm + "/cd2i"])


def call_args_an(meta, arrs, nm, nzq):
    m = meta
    return (m["radsep"], m["cdens"], m["pixarea"], m["cdelt0"], m["cdelt1"], m["crota2"], m["blo"][0], m["blo"][1],
            m["bhi"][0], m["bhi"][1], m["ltype"], m["sig_instr"], arrs[nm + "/vedges"], arrs[nm + "/relint"],
            arrs[nm + "/cd2i"], nzq, m["axtyp"], m["velsys"], arrs[nm + "/lfreq0"], m["crval3"], m["cdelt3"],
            m["crpix3"], m["chmin"])


class DeviceCase:
    """A device context set up from the scalars of a fixture case."""

    def __init__(self, meta, arrs, nm):
        from bbarolo2_gb300 import _lib
        self.L = _lib
        self.c = _lib.Context(0)
        g = _lib.Grid()
        m = meta
        g.nx, g.ny, g.nz = m["dimx"], m["dimy"], m["nz"]
        nz = m["nz"]

        def arr(name, default):
            return np.ascontiguousarray(arrs[nm + name]) if (nm + name) in arrs else default

        cd2i = arr("/cd2i", np.full(nz, float(m.get("mean_cd2i", 1.0))))
        lf = arr("/lfreq0", np.zeros(1))
        ri = arr("/relint", np.ones(1))
        ve = arr("/vedges", None)
        g.nlines = lf.size
        g.axtyp, g.velsys, g.ltype, g.cmode = m["axtyp"], m["velsys"], m["ltype"], m["cmode"]
        g.radsep, g.cdens, g.pixarea = m["radsep"], m["cdens"], m["pixarea"]
        g.cdelt0, g.cdelt1, g.crota2 = m["cdelt0"], m["cdelt1"], m["crota2"]
        g.sig_instr, g.crval3, g.cdelt3, g.crpix3 = m["sig_instr"], m["crval3"], m["cdelt3"], m["crpix3"]
        g.chwidth, g.zstep, g.scalefactor = m["chmin"], m["zstep"], 1.0
        self.c.check(self.c.L.bbgpu_set_grid(self.c.h, g, _lib.ptr(cd2i), _lib.ptr(lf), _lib.ptr(ri), _lib.ptr(ve)))

    def analytic(self, out, sr, lo, hi, nzq, blo, bhi):
        sr = np.ascontiguousarray(sr)
        self.c.check(self.c.L.bbgpu_galmod_analytic(self.c.h, self.L.ptr(out), self.L.ptr(sr), sr.shape[1], lo, hi,
                                                    nzq, blo[0], blo[1], bhi[0], bhi[1]))
        return out

    def ring_maps(self, out, sr, widx, wval, nzq, blo, bhi):
        sr = np.ascontiguousarray(sr)
        widx = np.ascontiguousarray(widx, np.int64)
        wval = np.ascontiguousarray(wval, np.float64)
        self.c.check(self.c.L.bbgpu_ring_maps_analytic(self.c.h, self.L.ptr(out), out.shape[0], self.L.ptr(sr),
                                                       sr.shape[1], self.L.ptr(widx), self.L.ptr(wval), nzq, blo[0],
                                                       blo[1], bhi[0], bhi[1]))
        return out

    def mc(self, out, sr, lo, hi, seed, nv, blo, bhi):
        sr = np.ascontiguousarray(sr)
        nv = np.ascontiguousarray(nv, np.int64)
        self.c.check(self.c.L.bbgpu_galmod_mc(self.c.h, self.L.ptr(out), self.L.ptr(sr), sr.shape[1], lo, hi, seed,
                                              self.L.ptr(nv), blo[0], blo[1], bhi[0], bhi[1]))
        return out
