"""The reference's host-side set-up of the model path, restated in plain numpy: the constants of ``GalmodSetup``,
``subrings``, the CENTRED/NODES ring conventions, ``DiskModel.box``, the beam kernel and the inputs of the
deconvolved profile.

TEST INFRASTRUCTURE: used by the tests (as an independent check of ``bbarolo2_gb300.galmod``) and by the CPU
reference arm of ``bench.py`` (``oracle/cpu_baseline.py``), which must not load the product library. Each function
follows the reference's float64 operations in the reference's order (cited per function), with loops where the
reference is vectorised only where that does not change a rounding.
"""

import math

import numpy as np

C_MS = 2.99792458e08
_VEL_UNITS = {"km/s": 1., "kms": 1., "m/s": 1E03, "ms": 1E03, "cm/s": 1E05}
_FREQ_UNITS = {"hz": 1., "khz": 1E03, "mhz": 1E06, "ghz": 1E09}


class Setup:
    """``GalmodSetup.__init__`` (bbarolo/galmod.py:613-725) for velocity and frequency axes, DENSFLUX models."""

    def __init__(self, cube):
        h = cube.Head()
        p = cube.pars()
        gm = p.gm
        self.nsubs = cube.DimZ()
        self.dimx, self.dimy = cube.DimX(), cube.DimY()
        self.cdelt = [0., 0.]
        for i in range(2):                                              # galmod.py:618-626
            cu = h.Cunit(i).lower()
            if "deg" in cu:
                c = 60.
            elif "arcs" in cu:
                c = 1 / 60.
            elif "arcm" in cu:
                c = 1.
            else:
                raise ValueError(cu)
            self.cdelt[i] = h.Cdelt(i) * c
        self.pixsize = [abs(self.cdelt[0]), abs(self.cdelt[1])]
        self.pixarea = self.pixsize[0] * self.pixsize[1]
        self.crota2 = h.Crota() * math.pi / 180.
        reds = p.getRedshift()
        cunit3 = h.Cunit(2).lower()
        self.cdelt3, self.crval3, self.crpix3 = h.Cdelt(2), h.Crval(2), h.Crpix(2)
        self.velsys = {"radio": 1, "optical": 2, "relativistic": 3}.get(h.VelDef(), 1)
        sptype = h.SpectralType()
        if "velo" in sptype:                                            # galmod.py:673-690
            self.axtyp = 4
            msconv = 1.0E03 / _VEL_UNITS[cunit3]
            self.freq0 = h.Freq0() / (1 + reds)
            if self.freq0 == 0:
                self.freq0 = 0.1420405751786E10
            self.crval3 *= msconv
            self.cdelt3 *= msconv
            chw = h.Cdelt(2) / _VEL_UNITS[cunit3]                       # bbutils.DeltaVel, velocity axis
        elif sptype == "freq":                                          # galmod.py:657-672, radio velocities
            self.axtyp = 3
            hz = _FREQ_UNITS[cunit3]
            self.crval3 *= hz
            self.cdelt3 *= hz
            self.freq0 = h.Freq0() / (1 + reds)
            if self.freq0 == 0:
                self.freq0 = 0.1420405751786E10
            if self.velsys != 1:
                raise NotImplementedError("oracle Setup: optical/relativistic frequency axes")
            frest = h.Freq0() / (1 + h.Redshift())
            chw = -(C_MS / 1000.) * h.Cdelt(2) * hz / frest              # bbutils.py:172-173
        else:
            raise NotImplementedError("oracle Setup: wavelength axes")
        self.lfreq0 = np.array([self.freq0])
        self.relint = np.array([1.])
        nch = p.specres if getattr(p, "specres", -1) != -1 else p.linear
        if nch == -1:
            nch = 1. / (2 * math.sqrt(2 * math.log(2)))
        self.chwidth = abs(chw) * 1000
        self.sig_instr = nch * self.chwidth
        self.ltype = gm.LTYPE
        self.cmode = gm.CMODE if 0 <= gm.CMODE <= 2 else 1
        self.cdens = float(gm.CDENS) if gm.CDENS >= 0 else 1.
        self.iseed = gm.ISEED
        self.empty = gm.EMPTY
        self.nvpar = gm.NV
        self.radmaxa = float(getattr(gm, "RADMAXA", -1.))
        self.radmaxr = float(getattr(gm, "RADMAXR", -1.))
        if not gm.DENSFLUX:
            raise NotImplementedError("oracle Setup: column-density models")
        self.radsep = 0.75 * min(self.pixsize)
        self.cd2i = np.full(self.nsubs, np.float32(3600. / self.chwidth * 1000.), dtype=np.float64)
        g = np.arange(self.nsubs + 1) - 0.5                             # galmod.py:743-758
        w = (g + 1 - self.crpix3) * self.cdelt3 + self.crval3
        if self.axtyp == 4:
            self.vedges = w
        else:
            self.vedges = C_MS * (1 - w / self.freq0)
        self.chmin = float(np.min(np.abs(np.diff(self.vedges))))

    def side_edges(self, rings):
        """``GalmodSetup.side_edges``: (approaching, receding) outer edges (arcsec) or None."""
        out = []
        for attr, default in (("edgeapp", self.radmaxa), ("edgerec", self.radmaxr)):
            e = getattr(rings, attr, None)
            e = default if e is None else float(e)
            out.append(e if e >= 0 else None)
        return tuple(out)


def zstep(cube, st):
    """The vertical sample spacing of the ANALYTIC models (``DiskModel``, bbarolo/galmod.py:1193-1203): 0.75 pixel
    when the beam's minor axis spans at least 3 pixels, else 0.25."""
    h = cube.Head()
    pix = max(st.pixsize) / 60.
    bmin = min(abs(h.Bmaj()), abs(h.Bmin()))
    return 0.75 if pix > 0 and bmin / pix >= 3.0 else 0.25


def edge_weights(R, dr, edge, width=0.):
    """bbarolo/galmod.py:1122-1131."""
    R = np.asarray(R, float)
    if width > 0:
        from scipy.special import erfc
        return 0.5 * erfc((R - edge) / (math.sqrt(2.) * width))
    return np.clip((edge - (R - dr / 2.)) / dr, 0., 1.) if dr > 0 else (R <= edge).astype(float)


def subrings(st, rings):
    """``GalmodSetup.subrings`` (bbarolo/galmod.py:761-851) for a thin layer: (sr (16, nsub), nv (nsub))."""
    if rings.thick():
        raise NotImplementedError("oracle subrings: thick layers")
    nr = rings.nr
    radsep = st.radsep
    rad = np.asarray(rings.radii, float) / 60.
    V = np.vstack([np.asarray(rings.vrot) * 1000., np.asarray(rings.vrad) * 1000.,
                   np.asarray(rings.vvert) * 1000., np.asarray(rings.vdisp) * 1000.,
                   np.asarray(rings.dens, float), np.asarray(rings.z0) / 60.,
                   np.asarray(rings.dvdz) * 1000 * 60, np.asarray(rings.zcyl) / 60.,
                   np.radians(np.asarray(rings.inc, float)), np.radians(np.asarray(rings.phi, float)),
                   np.asarray(rings.xpos, float), np.asarray(rings.ypos, float),
                   np.asarray(rings.vsys) * 1000.]).astype(float)
    f32 = np.float32
    rads, segs = [], []
    empty = st.empty if getattr(rings, "empty", None) is None else rings.empty
    r = f32(rad[0] + radsep / 2.0) if (rad[0] != 0 and empty) else f32(radsep / 2.0)
    if not (rad[0] != 0 and empty):
        while r < f32(rad[0]):
            rads.append(r)
            segs.append((0, None))
            r = f32(float(r) + radsep)
    for i in range(1, nr):
        ri = f32(rad[i])
        while r < ri:
            rads.append(r)
            segs.append((i, float(r) - float(f32(rad[i - 1]))))
            r = f32(float(r) + radsep)
    nsub = len(rads)
    sr = np.empty((14, nsub))
    sr[0] = np.asarray(rads, float)
    if nsub:
        idx = np.array([s[0] for s in segs])
        dr = np.array([0. if s[1] is None else s[1] for s in segs])
        const = np.array([s[1] is None for s in segs])
        i1 = np.maximum(idx, 1)
        dur = rad[i1] - rad[i1 - 1] if nr > 1 else np.ones(nsub)
        slope = (V[:, i1] - V[:, i1 - 1]) / dur if nr > 1 else np.zeros((V.shape[0], nsub))
        vals = V[:, i1 - 1] + slope * dr
        vals[:, const] = V[:, [0]]
        sr[1:] = vals
    edge = getattr(rings, "edge", None)
    if edge is not None and nsub:
        sr[5] *= edge_weights(sr[0] * 60., radsep * 60., float(edge), float(getattr(rings, "edgewidth", 0.)))
    side = np.ones((2, nsub))
    for k, e in enumerate(st.side_edges(rings)[::-1]):
        if e is not None and nsub:
            side[k] = edge_weights(sr[0] * 60., radsep * 60., e)
    sr = np.concatenate([sr, side])
    nvtmp = st.nvpar if st.nvpar >= 1 else st.nsubs
    nv = np.where(sr[4] == 0, 1, nvtmp).astype(np.int64)
    return np.ascontiguousarray(sr), nv


def model_rings(rings, mode, subring):
    """``model_rings`` (bbarolo/galmod.py:1066-1119) for CENTRED and NODES."""
    if mode == "NODES" or rings.nr == 0:
        return rings
    if mode != "CENTRED":
        raise NotImplementedError("oracle model_rings: " + mode)
    R = rings.radii
    if rings.nr == 1:
        w0 = wn = rings.radsep / 2. if rings.radsep > 0 else R[0] / 2.
    else:
        w0, wn = (R[1] - R[0]) / 2., (R[-1] - R[-2]) / 2.
    rin, rout = max(R[0] - w0, 0.), R[-1] + wn
    idx, rad = list(range(rings.nr)), list(R)
    if rin / 60. + subring < R[0] / 60.:
        idx.insert(0, 0)
        rad.insert(0, rin)
    if R[-1] / 60. + subring < rout / 60.:
        idx.append(rings.nr - 1)
        rad.append(rout)
    out = rings.subset(np.array(idx))
    out.radii = np.array(rad, dtype=float)
    return out


def outer_edge_centred(rings):
    R = rings.radii
    wn = (R[-1] - R[-2]) / 2. if rings.nr > 1 else (rings.radsep / 2. if rings.radsep > 0 else R[0] / 2.)
    return float(R[-1] + wn)


def box(cube, rings, final=True):
    """``DiskModel.box`` (bbarolo/galmod.py:1224-1240), CENTRED rings, thin layer: ([blo], [bhi])."""
    h = cube.Head()
    conv = 3600. if "deg" in h.Cunit(0).lower() else (60. if "arcm" in h.Cunit(0).lower() else 1.)
    ext = rings.radii[-1] + rings.radsep / 2.
    if final:
        ext = max(ext, outer_edge_centred(rings))
    ext = ext + 3 * float(np.asarray(rings.z0, float)[-1])
    xdis = int(math.ceil(ext / (abs(h.Cdelt(0)) * conv)))
    ydis = int(math.ceil(ext / (abs(h.Cdelt(1)) * conv)))
    xpos = int(math.ceil(rings.xpos[-1]))
    ypos = int(math.ceil(rings.ypos[-1]))
    return ([max(xpos - xdis, 0), max(ypos - ydis, 0)],
            [min(xpos + xdis + 1, cube.DimX()), min(ypos + ydis + 1, cube.DimY())])


def beam_kernel(cube):
    """The convolution kernel of a cube's beam (``Smooth3D.defineBeam_Gaussian``, bbarolo/smooth.py:203-231, from
    a point source: ``convpars`` smooth.py:25-51 reduces to the new beam, then ``fillgauss2d`` smooth.py:62-88):
    the kernel (ky, kx), normalised, taps below 1e-4 of the peak zero."""
    h = cube.Head()
    conv = 3600. if "deg" in h.Cunit(0).lower() else (60. if "arcm" in h.Cunit(0).lower() else 1.)
    gs = (abs(h.Cdelt(0) * conv), abs(h.Cdelt(1) * conv))
    bmaj, bmin, bpa = h.Bmaj() * 3600., h.Bmin() * 3600., h.Bpa()
    if bmaj < bmin:
        bmaj, bmin, bpa = bmin, bmaj, bpa + 90.
    d2r = math.atan(1.) / 45.
    a0, b0 = bmaj / 2, bmin / 2
    D0 = a0 * a0 - b0 * b0
    th0 = bpa * d2r
    D1 = math.sqrt(max(D0 * D0, 0.))
    a1 = math.sqrt(0.5 * (a0 * a0 + b0 * b0 + D1))
    arg = 0.5 * (a0 * a0 + b0 * b0 - D1)
    b1 = math.sqrt(arg if arg > 0 else 0.)
    nom, den = D0 * math.sin(2 * th0), D0 * math.cos(2 * th0)
    th1 = 0. if (den == 0 and nom == 0) else math.atan2(nom, den) / 2
    cb = (2 * a1, 2 * b1, th1 / d2r - (h.Crota() - 90))
    phi = cb[2] * math.pi / 180.
    cs, sn = math.cos(phi), math.sin(phi)
    bm = (abs(cb[0]), abs(cb[1]))
    cutoff = 1e-4
    extend = math.sqrt(-1.0 * math.log(cutoff) / math.log(2.0))
    xr, yr = 0.5 * bm[0] * extend, 0.5 * bm[1] * extend
    x = max(abs(xr * cs), abs(-yr * sn))
    y = max(abs(xr * sn), abs(yr * cs))
    Xmax, Ymax = int(round(x / gs[0])), int(round(y / gs[1]))
    jj, ii = np.mgrid[-Ymax:Ymax + 1, -Xmax:Xmax + 1]
    xx, yy = ii * gs[0], jj * gs[1]
    xrr = xx * cs + yy * sn
    yrr = -xx * sn + yy * cs
    argX = xrr / bm[0] if bm[0] != 0 else 0 * xrr
    argY = yrr / bm[1] if bm[1] != 0 else 0 * yrr
    c = np.exp(-4.0 * math.log(2.0) * (argX * argX + argY * argY))
    c = np.where(c >= cutoff, c, 0.)
    return c / c.sum()


def ring_weights(st, rings, mode):
    """``DiskModel._ring_weights`` (bbarolo/galmod.py:1285-1315): (widx, wval) (nsub, 2)."""
    cols = []
    for r in range(rings.nr):
        rr = rings.copy()
        rr.dens = np.zeros(rings.nr)
        rr.dens[r] = 1.
        cols.append(subrings(st, model_rings(rr, mode, st.radsep))[0][5])
    W = np.array(cols).T
    widx = np.full((W.shape[0], 2), -1, np.int64)
    wval = np.zeros((W.shape[0], 2))
    for s in range(W.shape[0]):
        nz = np.flatnonzero(W[s] != 0)
        widx[s, :len(nz)] = nz
        wval[s, :len(nz)] = W[s, nz]
    return widx, wval


def exterior_ring(st, rings, beam_arcsec, ringmode="CENTRED"):
    """The exterior annulus of ``profile_system`` (bbarolo/profile.py:47-71): a one-ring set two beams wide
    beyond the outer edge, with the last ring's values and unit density."""
    from bbarolo2_gb300.rings import Rings
    r = rings
    R = np.asarray(r.radii, float)
    w = 2. * beam_arcsec if beam_arcsec else 2. * float(np.max(np.diff(R), initial=R[-1]))
    edge = outer_edge_centred(r) if ringmode == "CENTRED" else float(R[-1])
    if getattr(r, "edge", None) is not None:
        edge = min(edge, float(r.edge))
    ea, er = st.side_edges(r)
    if ea is not None and er is not None:
        edge = min(edge, max(ea, er))
    rext = edge + w / 2.
    ext = Rings().setRings(radii=[rext], xpos=r.xpos[-1], ypos=r.ypos[-1], vsys=r.vsys[-1], vrot=r.vrot[-1],
                           vdisp=r.vdisp[-1], z0=r.z0[-1], inc=r.inc[-1], phi=r.phi[-1], dens=1., radsep=w,
                           z0thick=r.z0thick[-1], fthick=r.fthick[-1], vdispthick=r.vdispthick[-1])
    ext.twolayer = r.thick()
    ext.edgeapp = ext.edgerec = -1.
    return ext


def rings_of_row(proto, row):
    """A ring set with proto's radii and options and the values of one row (17, nr) in the order of
    ``bbarolo.rings.Rings`` (radii, xpos, ypos, vsys, vrot, vdisp, vrad, vvert, dvdz, zcyl, dens, z0, inc, phi,
    z0thick, fthick, vdispthick)."""
    keys = ("radii", "xpos", "ypos", "vsys", "vrot", "vdisp", "vrad", "vvert", "dvdz", "zcyl", "dens", "z0", "inc",
            "phi", "z0thick", "fthick", "vdispthick")
    r = proto.copy()
    for i, k in enumerate(keys):
        setattr(r, k, np.array(row[i], dtype=float))
    return r
