"""Bi-conical wind models of WINDFIT: the columns of the linear wind model and their normal equations on the GPU.

The reference's ``bbarolo/windmodel.py`` (``WindPars``, ``WindCells``, ``WindModel``, ``Boxes``) with the same names,
arguments and results. The emission of a wind is a set of amplitudes on a fixed grid of cells of the two cones
(``WindCells``); the model cube is linear in them, M = A(geometry, kinematics) . amplitudes, and each column of A (one
cell) is a dense box of the cube. Per set of wind parameters (``WindPars``) the device computes the quadrature
points of the cells (sky position, line-of-sight velocity, weight), deposits them in the raw box of their cell
(the channel-integrated line, bilinear on the pixels), convolves each box with the beam and, for a likelihood, forms
the normal equations G = A'WA, b = A'Wd of the columns (``csrc/wind.cu``). The host keeps the cells and their
quadrature (fixed per fit), the beam kernel, and reads back the boxes' extents, G and b.

``WindModel.boxes`` returns a ``DeviceBoxes``: its columns stay on the device until ``buf`` is read; the device
holds the columns of the latest ``boxes`` call of a model, so a ``DeviceBoxes`` is used before the next call (as
``bbarolo/bayesian/wind.py`` uses them), or its values are read first (``buf``).
"""

import ctypes as C
import math
import sys

import numpy as np

from . import _lib
from .galmod import BBaroloError, GalmodSetup

PSF_CUTOFF = 1.0e-4                 # the beam is zero below this fraction of its peak (as CUTOFFRATIO of SMOOTH)
MAX_POINTS = 2_000_000              # the most quadrature points: beyond, the cones are sampled more coarsely


class WindPars:
    """The parameters of a wind (``bbarolo/windmodel.py:43-86``): centre (xpos, ypos: pixels), vsys (km/s), inc and
    pa (degrees), openang and openin (full outer and inner opening angles, degrees), conelen (outer radius, arcsec;
    default the last radius) and per shell (radii: arcsec, increasing) vwind, vdisp and vrot (km/s; one value or one
    per shell)."""

    NAMES = ("xpos", "ypos", "vsys", "inc", "pa", "openang", "openin", "conelen")
    SHELL = ("vwind", "vdisp", "vrot")

    def __init__(self, radii, vwind, vdisp, vrot=0., xpos=0., ypos=0., vsys=0., inc=60., pa=0., openang=60.,
                 openin=0., conelen=None):
        self.radii = np.atleast_1d(np.asarray(radii, dtype=np.float64))
        n = self.radii.size
        if n == 0 or np.any(np.diff(self.radii) <= 0):
            raise BBaroloError("WindModel: the radii of the shells must be increasing")
        for name, v in zip(self.SHELL, (vwind, vdisp, vrot)):
            a = np.asarray(v, dtype=np.float64).ravel()
            if a.size == 1:
                a = np.repeat(a, n)
            if a.size != n:
                raise BBaroloError(f"WindModel: {name} has {a.size} values, not one or {n} (one per shell)")
            setattr(self, name, a)
        self.xpos, self.ypos, self.vsys = float(xpos), float(ypos), float(vsys)
        self.inc, self.pa = float(inc), float(pa)
        self.openang, self.openin = float(openang), float(openin)
        self.conelen = float(self.radii[-1]) if conelen is None else float(conelen)

    def copy(self):
        out = WindPars.__new__(WindPars)
        out.__dict__ = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in self.__dict__.items()}
        return out

    def check(self):
        if not (0 <= self.openin < self.openang <= 180.):
            raise BBaroloError(f"WindModel: the opening angles must be 0 <= OPENIN < OPENANG <= 180 "
                               f"(OPENIN={self.openin:g}, OPENANG={self.openang:g})")
        if not self.conelen > 0:
            raise BBaroloError(f"WindModel: CONELEN must be positive (CONELEN={self.conelen:g})")

    def __repr__(self):
        geo = ", ".join(f"{k}={getattr(self, k):g}" for k in self.NAMES)
        return f"WindPars({geo}, {self.radii.size} shells)"


class WindCells:
    """The fixed grid of cells of the emission in the frame of the wind (``bbarolo/windmodel.py:89-209``).

    redges: edges of the radial bins (arcsec, increasing, non-negative); ntheta polar bins from the axis to thmax
    (degrees, the largest half opening angle); nphi azimuthal sectors; cones: 1 (along +z), -1 or both. Cell k is
    the row (cone, r0, r1, theta0, theta1, phi0, phi1) of ``cells``, ordered by cone, radius, polar angle, azimuth.
    """

    def __init__(self, redges, ntheta=1, nphi=1, thmax=90., cones=(1, -1)):
        self.redges = np.asarray(redges, dtype=np.float64).ravel()
        if self.redges.size < 2 or np.any(np.diff(self.redges) <= 0) or self.redges[0] < 0:
            raise BBaroloError("WindCells: the radial edges must be increasing and non-negative")
        self.ntheta, self.nphi = int(ntheta), int(nphi)
        if self.ntheta < 1 or self.nphi < 1:
            raise BBaroloError("WindCells: ntheta and nphi must be at least 1")
        if not 0 < thmax <= 90.:
            raise BBaroloError(f"WindCells: the largest half opening angle must be in (0, 90] degrees, not {thmax:g}")
        self.thmax = float(thmax)
        self.cones = tuple(int(c) for c in np.atleast_1d(cones))
        if not self.cones or any(c not in (1, -1) for c in self.cones) or len(set(self.cones)) != len(self.cones):
            raise BBaroloError("WindCells: cones must be 1, -1 or both")
        self.nr = self.redges.size - 1
        th = np.linspace(0., math.radians(self.thmax), self.ntheta + 1)
        ph = np.linspace(0., 2 * math.pi, self.nphi + 1)
        rows, ijk = [], []
        for ic, cone in enumerate(self.cones):
            for ir in range(self.nr):
                for it in range(self.ntheta):
                    for ip in range(self.nphi):
                        rows.append((cone, self.redges[ir], self.redges[ir + 1], th[it], th[it + 1], ph[ip],
                                     ph[ip + 1]))
                        ijk.append((ic, ir, it, ip))
        self._set(rows, ijk)

    def _set(self, rows, ijk):
        self.cells = np.ascontiguousarray(np.array(rows, dtype=np.float64).reshape(-1, 7))
        self.ijk = np.array(ijk, dtype=np.int64).reshape(-1, 4)
        self.qn = None
        self.qoff = None
        self.spacing = None

    @classmethod
    def resolved(cls, rmax, thmax, size, cones=(1, -1), rmin=0., minphi=1):
        """Cells about size (arcsec) across: radial bins of width ~size from rmin to rmax and, in each, as many polar
        bins and azimuthal sectors (at least minphi) as fit with that size at the bin's outer radius."""
        nr = max(1, int(round((rmax - rmin) / size)))
        redges = np.linspace(rmin, rmax, nr + 1)
        self = cls(redges, 1, 1, thmax=thmax, cones=cones)
        th = math.radians(thmax)
        rows, ijk = [], []
        for ic, cone in enumerate(self.cones):
            for ir in range(nr):
                ro = redges[ir + 1]
                nt = max(1, int(round(ro * th / size)))
                tedges = np.linspace(0., th, nt + 1)
                for it in range(nt):
                    npp = max(int(minphi), int(round(2 * math.pi * ro * math.sin(tedges[it + 1]) / size)))
                    pedges = np.linspace(0., 2 * math.pi, npp + 1)
                    for ip in range(npp):
                        rows.append((cone, redges[ir], redges[ir + 1], tedges[it], tedges[it + 1], pedges[ip],
                                     pedges[ip + 1]))
                        ijk.append((ic, ir, it, ip))
        self._set(rows, ijk)
        self.ntheta = self.nphi = None
        return self

    @property
    def ncell(self):
        return self.cells.shape[0]

    def index(self, cone, ir, it=0, ip=0):
        ic = self.cones.index(cone)
        hit = np.flatnonzero(np.all(self.ijk == np.array([ic, ir, it, ip]), axis=1))
        if hit.size == 0:
            raise BBaroloError(f"WindCells: no cell ({cone}, {ir}, {it}, {ip})")
        return int(hit[0])

    def set_quadrature(self, spacing, vmax, sigmin, cap=16, maxpoints=None):
        """Quadrature points per cell in r, theta, phi: at most spacing (arcsec) apart on the sky and with
        line-of-sight velocities at most sigmin/2 apart for winds up to vmax (at most cap per dimension for the
        velocities); with maxpoints the spacing grows until the total fits. Sets qn, qoff and spacing."""
        c = self.cells
        dr, dth, dph = c[:, 2] - c[:, 1], c[:, 4] - c[:, 3], c[:, 6] - c[:, 5]
        s1 = np.sin(c[:, 4])
        dv = max(0.5 * float(sigmin), 1e-3)
        vel_t = np.minimum(np.ceil(vmax * dth / dv), cap)
        vel_p = np.minimum(np.ceil(vmax * s1 * dph / dv), cap)
        sp = float(spacing)
        while True:
            q = np.stack([np.ceil(dr / sp), np.maximum(np.ceil(c[:, 2] * dth / sp), vel_t),
                          np.maximum(np.ceil(c[:, 2] * s1 * dph / sp), vel_p)], axis=1)
            qn = np.maximum(q, 1).astype(np.int64)
            tot = int(np.prod(qn, axis=1).sum())
            if maxpoints is None or tot <= maxpoints:
                break
            sp *= max(1.02, (tot / maxpoints) ** (1. / 3.))
        self.spacing = sp
        self.qn = np.ascontiguousarray(qn)
        self.qoff = np.concatenate([[0], np.cumsum(np.prod(qn, axis=1))]).astype(np.int64)
        return self

    @property
    def npoints(self):
        return int(self.qoff[-1]) if self.qoff is not None else 0

    def centres(self):
        """(cone, r, theta, phi) of the centres of the cells (arcsec, degrees)."""
        c = self.cells
        return (c[:, 0].astype(int), 0.5 * (c[:, 1] + c[:, 2]), np.degrees(0.5 * (c[:, 3] + c[:, 4])),
                np.degrees(0.5 * (c[:, 5] + c[:, 6])))


class Boxes:
    """Columns of a linear model, each a dense box of the cube (``bbarolo/windmodel.py:605-703``): column k holds
    ``buf[offs[k]:offs[k+1]]`` in the box ``boxes[k]`` = (x0, x1, y0, y1, k0, k1), [lo, hi), values in (channel, y,
    x) order. Host arrays; ``DeviceBoxes`` keeps them on the GPU."""

    def __init__(self, buf, offs, boxes):
        self._buf, self.offs, self.boxes = buf, offs, boxes

    @property
    def buf(self):
        return self._buf

    @property
    def n(self):
        return self.boxes.shape[0]

    @staticmethod
    def _offsets(boxes):
        size = (boxes[:, 1] - boxes[:, 0]) * (boxes[:, 3] - boxes[:, 2]) * (boxes[:, 5] - boxes[:, 4])
        return np.concatenate([[0], np.cumsum(np.maximum(size, 0))]).astype(np.int64)

    @staticmethod
    def from_boxes(boxes):
        boxes = np.ascontiguousarray(boxes, dtype=np.int64).reshape(-1, 6)
        offs = Boxes._offsets(boxes)
        return Boxes(np.zeros(int(offs[-1])), offs, boxes)

    @staticmethod
    def from_cubes(cubes, tiny=0.):
        """The columns of a list of (nz, ny, nx) arrays, each in the bounding box of its values above tiny."""
        ext = []
        for a in cubes:
            nzv = np.argwhere(np.abs(a) > tiny)
            if nzv.size == 0:
                ext.append((0, 0, 0, 0, 0, 0))
            else:
                lo, hi = nzv.min(axis=0), nzv.max(axis=0) + 1
                ext.append((lo[2], hi[2], lo[1], hi[1], lo[0], hi[0]))
        B = Boxes.from_boxes(np.array(ext, dtype=np.int64).reshape(-1, 6))
        for k, a in enumerate(cubes):
            x0, x1, y0, y1, k0, k1 = B.boxes[k]
            if x1 > x0:
                B.buf[B.offs[k]:B.offs[k + 1]] = a[k0:k1, y0:y1, x0:x1].ravel()
        return B

    def _view(self, k):
        x0, x1, y0, y1, k0, k1 = self.boxes[k]
        if x1 <= x0 or y1 <= y0 or k1 <= k0:
            return None
        return self.buf[self.offs[k]:self.offs[k + 1]].reshape(k1 - k0, y1 - y0, x1 - x0)

    def column(self, k, shape):
        out = np.zeros(shape)
        v = self._view(k)
        if v is not None:
            x0, x1, y0, y1, k0, k1 = self.boxes[k]
            out[k0:k1, y0:y1, x0:x1] = v
        return out

    def dense(self, shape, mask=None):
        """The matrix A (voxels, n) over all the voxels of shape or those of the boolean mask."""
        cols = [self.column(k, shape).ravel() for k in range(self.n)]
        A = np.array(cols).T if cols else np.zeros((int(np.prod(shape)), 0))
        return A[np.ravel(mask)] if mask is not None else A

    def model(self, amp, shape):
        out = np.zeros(shape)
        for k in range(self.n):
            v = self._view(k)
            if v is not None and amp[k] != 0.:
                x0, x1, y0, y1, k0, k1 = self.boxes[k]
                out[k0:k1, y0:y1, x0:x1] += amp[k] * v
        return out

    def lim(self):
        b = self.boxes
        ok = (b[:, 1] > b[:, 0]) & (b[:, 3] > b[:, 2]) & (b[:, 5] > b[:, 4])
        if not np.any(ok):
            return np.zeros(6, dtype=np.int64)
        b = b[ok]
        return np.array([b[:, 0].min(), b[:, 1].max(), b[:, 2].min(), b[:, 3].max(), b[:, 4].min(), b[:, 5].max()],
                        dtype=np.int64)

    def voxel_lists(self, wm, lim=None, rel=0.):
        """The selection of the column values of the normal equations: those != 0, with wm != 0 and at least rel times
        the peak of their column (the reference's voxel lists; here the lim and rel they are made with)."""
        lim = self.lim() if lim is None else np.asarray(lim, dtype=np.int64)
        return (lim, float(rel))

    def normal(self, wd, wm, lists=None):
        """(G, b) = (A'WA, A'Wd) over the selected values (lists: voxel_lists(wm, ...))."""
        rel = 0. if lists is None else float(lists[1])
        return _host_normal(self, wd, wm, rel)

    def cross(self, other, wm, lists=None, other_lists=None):
        """Gab = A'WB with the columns B of other (over the values selected in both)."""
        ra = 0. if lists is None else float(lists[1])
        rb = 0. if other_lists is None else float(other_lists[1])
        return _host_cross(self, other, wm, ra, rb)


def _selected(B, k, wm, rel):
    """Column k's values in its box with the values outside the selection set to 0."""
    v = B._view(k)
    if v is None:
        return None
    x0, x1, y0, y1, k0, k1 = B.boxes[k]
    keep = (v != 0.) & (wm[k0:k1, y0:y1, x0:x1] != 0.)
    if rel > 0.:
        keep &= np.abs(v) >= rel * np.abs(v).max()
    return np.where(keep, v, 0.)


def _host_cross(A, B, wm, ra, rb):
    G = np.zeros((A.n, B.n))
    sa = [_selected(A, k, wm, ra) for k in range(A.n)]
    sb = sa if B is A and ra == rb else [_selected(B, k, wm, rb) for k in range(B.n)]
    for k in range(A.n):
        if sa[k] is None:
            continue
        a = A.boxes[k]
        for l in range(B.n):
            if sb[l] is None:
                continue
            b = B.boxes[l]
            x0, x1 = max(a[0], b[0]), min(a[1], b[1])
            y0, y1 = max(a[2], b[2]), min(a[3], b[3])
            z0, z1 = max(a[4], b[4]), min(a[5], b[5])
            if x1 <= x0 or y1 <= y0 or z1 <= z0:
                continue
            va = sa[k][z0 - a[4]:z1 - a[4], y0 - a[2]:y1 - a[2], x0 - a[0]:x1 - a[0]]
            vb = sb[l][z0 - b[4]:z1 - b[4], y0 - b[2]:y1 - b[2], x0 - b[0]:x1 - b[0]]
            G[k, l] = np.sum(wm[z0:z1, y0:y1, x0:x1] * va * vb)
    return G


def _host_normal(B, wd, wm, rel):
    G = _host_cross(B, B, wm, rel, rel)
    b = np.zeros(B.n)
    for k in range(B.n):
        s = _selected(B, k, wm, rel)
        if s is not None:
            x0, x1, y0, y1, k0, k1 = B.boxes[k]
            b[k] = np.sum(s * wd[k0:k1, y0:y1, x0:x1])
    return G, b


class DeviceBoxes(Boxes):
    """The columns of one ``WindModel.boxes`` call, on the device: boxes (host), offsets and values read on demand;
    ``normal`` and ``model`` run on the device while these are the model's latest columns."""

    def __init__(self, wm, boxes, total, gen):
        self._wm, self._gen, self.total = wm, gen, int(total)
        self.boxes = boxes
        self._offs = None
        self._buf = None

    def _live(self, what):
        if self._gen != self._wm._gen_boxes:
            raise BBaroloError(f"WindModel: {what} of columns replaced by a later boxes() call (read .buf first)")

    def _read(self):
        self._live("reading the values")
        offs = np.zeros(self.n + 1, dtype=np.int64)
        buf = np.empty(self.total)
        self._wm._call("bbgpu_wind_columns", _lib.ptr(buf), _lib.ptr(offs))
        self._offs, self._buf = offs, buf

    @property
    def offs(self):
        if self._offs is None:
            self._read()
        return self._offs

    @property
    def buf(self):
        if self._buf is None:
            self._read()
        return self._buf

    def normal(self, wd, wm, lists=None):
        if self._gen != self._wm._gen_boxes and self._buf is not None:
            return super().normal(wd, wm, lists)
        self._live("normal equations")
        lim, rel = (self.lim(), 0.) if lists is None else lists
        return self._wm._normal(wd, wm, lim, float(rel))

    def model(self, amp, shape):
        if tuple(shape) != self._wm.shape:
            raise BBaroloError(f"WindModel: the model shape must be the cube's {self._wm.shape}")
        if self._gen != self._wm._gen_boxes and self._buf is not None:
            return super().model(amp, shape)
        self._live("the model")
        a = np.ascontiguousarray(amp, dtype=np.float64)
        if a.size != self.n:
            raise BBaroloError(f"WindModel: {a.size} amplitudes for {self.n} columns")
        out = np.empty(self._wm.shape)
        self._wm._call("bbgpu_wind_model", _lib.ptr(a), _lib.ptr(out))
        return out


class WindModel:
    """Models of bi-conical winds on the grid of a cube (``bbarolo/windmodel.py:706-889``).

    WindModel(cube, cells, smooth=True): the cube's header and parameters (spectral axis, lines, beam), the cells of
    the emission (their quadrature set by ``quadrature``) and smooth: spread the points with the beam of the cube,
    else bilinearly on the pixels. Then for parameters p (``WindPars``): ``points(p)``, ``boxes(p, lim, pts,
    weight)`` (the columns, on the device) and ``cube(p, amp)``.
    """

    def __init__(self, cube, cells, smooth=True, device=0):
        self.cin = cube
        self.cells = cells
        self.device = device
        self.setup = GalmodSetup(cube, densflux=True)
        su = self.setup
        self.shape = (cube.DimZ(), cube.DimY(), cube.DimX())
        self.cdelt = (su.cdelt[0] * 60., su.cdelt[1] * 60.)
        self.pixsize = min(abs(self.cdelt[0]), abs(self.cdelt[1]))
        self.psfq = np.zeros(5)
        self.hx = self.hy = 0
        self.kern = np.ones((1, 1))
        self.kx = self.ky = np.ones(1)
        self.separable = True
        self.beam = None
        self.sigbeam = None
        h = cube.Head()
        if smooth and h.Bmaj() > 0 and h.Bmin() > 0:
            self.beam = (h.Bmaj() * 3600., h.Bmin() * 3600., h.Bpa())
            self._set_psf()
        self._h = None
        self._cells_on_device = None
        self._gen_points = 0
        self._gen_boxes = 0
        self._wkey = None

    def _set_psf(self):
        """The beam as a quadratic form of the pixel offsets, exp(-(a dx^2 + 2 b dx dy + c dy^2)/2) (the major axis
        at BPA + 90 - CROTA from x, as SMOOTH), and the kernel convolved with the bilinear deposit: the Gaussian of
        the beam's covariance less the 1/6 pixel^2 of the bilinear weights per axis (the whole beam when that leaves
        less than 0.05 pixel^2), sampled on the pixels, zero below PSF_CUTOFF of the peak, normalised to 1
        (``bbarolo/windmodel.py:743-783``)."""
        bmaj, bmin, bpa = self.beam
        ang = math.radians(bpa + 90. - self.cin.Head().Crota())
        co, si = math.cos(ang), math.sin(ang)
        px, py = abs(self.cdelt[0]), abs(self.cdelt[1])
        f = 8. * math.log(2.)
        a = f * px * px * (co * co / bmaj ** 2 + si * si / bmin ** 2)
        b = f * px * py * co * si * (1. / bmaj ** 2 - 1. / bmin ** 2)
        c = f * py * py * (si * si / bmaj ** 2 + co * co / bmin ** 2)
        if abs(b) < 1e-12 * math.sqrt(a * c):
            b = 0.
        qcut = -2. * math.log(PSF_CUTOFF)
        self.psfq = np.array([a, b, c, math.sqrt(a * c - b * b) / (2. * math.pi), qcut])
        self.sigbeam = min(bmaj, bmin) / (2. * math.sqrt(2. * math.log(2.)))
        Q = np.array([[a, b], [b, c]])
        cov = np.linalg.inv(Q) - np.eye(2) / 6.
        if np.min(np.linalg.eigvalsh(cov)) <= 0.05:
            cov = np.linalg.inv(Q)
        P = np.linalg.inv(cov)
        ka, kb, kc = P[0, 0], P[0, 1], P[1, 1]
        kdet = ka * kc - kb * kb
        self.hx = int(math.ceil(math.sqrt(qcut * kc / kdet)))
        self.hy = int(math.ceil(math.sqrt(qcut * ka / kdet)))
        yy, xx = np.mgrid[-self.hy:self.hy + 1, -self.hx:self.hx + 1].astype(float)
        q = ka * xx * xx + 2 * kb * xx * yy + kc * yy * yy
        kern = np.where(q <= qcut, np.exp(-0.5 * q), 0.)
        self.kern = np.ascontiguousarray(kern / kern.sum())
        self.separable = b == 0.
        if self.separable:
            gx = np.exp(-0.5 * ka * np.arange(-self.hx, self.hx + 1.) ** 2)
            gy = np.exp(-0.5 * kc * np.arange(-self.hy, self.hy + 1.) ** 2)
            self.kx, self.ky = gx / gx.sum(), gy / gy.sum()

    def quadrature(self, vmax, sigmin, spacing=None, cap=16):
        """The quadrature of the cells for winds up to vmax (km/s) and lines at least sigmin (km/s) wide (the
        instrumental dispersion added): points at most spacing (arcsec; default the beam's dispersion, one pixel
        without a beam) and one line dispersion apart."""
        if spacing is None:
            spacing = self.pixsize if self.beam is None else self.sigbeam
        sig = math.hypot(sigmin, self.setup.sig_instr / 1000.)
        self.cells.set_quadrature(spacing, vmax, 2. * sig, cap=cap, maxpoints=MAX_POINTS)
        if self.cells.spacing > 2. * spacing:
            sys.stderr.write(f" WindModel WARNING: the cones are sampled every {self.cells.spacing:.3g} arcsec, more "
                             f"than twice the {spacing:.3g} arcsec needed (at most {MAX_POINTS} quadrature points): "
                             "the model is lumpier than the beam.\n")
        self._cells_on_device = None
        return self

    # ------------------------------------------------------------------ device
    def _handle(self):
        if self._h is None:
            L = _lib.load()
            su = self.setup
            nz, ny, nx = self.shape
            g = _lib.WindGrid(nx=nx, ny=ny, nz=nz, nlines=len(su.lfreq0), axtyp=int(su.axtyp),
                              velsys=int(su.velsys), cdelt0=self.cdelt[0], cdelt1=self.cdelt[1],
                              sig_instr=su.sig_instr, chmin=su._chmin, crval3=su.crval3, cdelt3=su.cdelt3,
                              crpix3=su.crpix3)
            self._keep = [np.ascontiguousarray(a, dtype=np.float64) for a in
                          (su.lfreq0, su.relint, su._vedges_lines, self.kern, self.kx, self.ky)]
            lf, ri, ve, ke, kx, ky = self._keep
            h = C.c_void_p()
            rc = L.bbgpu_wind_create(C.byref(h), self.device, C.byref(g), _lib.ptr(lf), _lib.ptr(ri), _lib.ptr(ve),
                                     _lib.ptr(ke), self.hy, self.hx, _lib.ptr(kx), _lib.ptr(ky), int(self.separable))
            if rc != 0:
                raise _lib.DeviceError(rc, "bbgpu_wind_create failed")
            self._L, self._h = L, h
        if self._cells_on_device is not self.cells.qoff:
            c = self.cells
            if c.qoff is None:
                raise BBaroloError("WindModel: the quadrature of the cells is not set (call quadrature first)")
            self._call("bbgpu_wind_set_cells", int(c.ncell), _lib.ptr(c.cells), _lib.ptr(c.qn), _lib.ptr(c.qoff))
            self._cells_on_device = c.qoff
        return self._h

    def _call(self, name, *args):
        h = self._handle() if name != "bbgpu_wind_set_cells" else self._h
        rc = getattr(self._L, name)(h, *args)
        if rc != 0:
            msg = self._L.bbgpu_wind_last_error(h)
            raise _lib.DeviceError(rc, f"{name}: {msg.decode() if msg else ''}")

    def close(self):
        if self._h is not None:
            self._L.bbgpu_wind_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def launches(self):
        """Kernels launched by this model's device handle so far."""
        return int(self._L.bbgpu_wind_launch_count(self._h)) if self._h is not None else 0

    def _geometry(self, p):
        p.check()
        inc = math.radians(p.inc)
        ang = math.radians(p.pa) + self.setup.crota2
        return _lib.WindGeometry(x0=p.xpos, y0=p.ypos, vsys=p.vsys * 1000., sinc=math.sin(inc), cinc=math.cos(inc),
                                 spa=math.sin(ang), cpa=math.cos(ang), th_in=math.radians(0.5 * p.openin),
                                 th_out=math.radians(0.5 * p.openang), rmax=p.conelen)

    def _points(self, p, out=None):
        g = self._geometry(p)
        sh = [np.ascontiguousarray(a, dtype=np.float64) for a in (p.radii, p.vwind, p.vdisp, p.vrot)]
        o = out or {}
        names = ("gx", "gy", "vel", "sig", "w", "r", "vol", "rbar")
        self._call("bbgpu_wind_points", C.byref(g), int(sh[0].size), *[_lib.ptr(a) for a in sh],
                   *[_lib.ptr(o.get(k)) for k in names])
        self._gen_points += 1
        return o

    def points(self, p):
        """The quadrature points of the wind p: a dict of gx, gy (pixels), vel, sig (m/s), w (arcsec^3), r (arcsec)
        per point and vol (clipped volume), rbar (mean radius) per cell."""
        c = self.cells
        if c.qoff is None:
            raise BBaroloError("WindModel: the quadrature of the cells is not set (call quadrature first)")
        n, m = c.npoints, c.ncell
        out = {k: np.empty(n) for k in ("gx", "gy", "vel", "sig", "w", "r")}
        out.update(vol=np.empty(m), rbar=np.empty(m))
        self._points(p, out)
        out["_wind_points"] = (id(self), self._gen_points)
        return out

    def boxes(self, p, lim=None, pts=None, weight=None):
        """The columns (``DeviceBoxes``) of the wind p within lim = (x0, x1, y0, y1, k0, k1) (default the cube); pts:
        the points (default computed on the device); weight: an extra weight per point."""
        nz, ny, nx = self.shape
        lim = np.ascontiguousarray([0, nx, 0, ny, 0, nz] if lim is None else lim, dtype=np.int64)
        if pts is None:
            self._points(p)
        elif pts.get("_wind_points") != (id(self), self._gen_points):
            arr = [np.ascontiguousarray(pts[k], dtype=np.float64) for k in ("gx", "gy", "vel", "sig", "w")]
            if any(a.size != self.cells.npoints for a in arr):
                raise BBaroloError("WindModel: the points do not match the quadrature of the cells")
            self._call("bbgpu_wind_set_points", *[_lib.ptr(a) for a in arr])
        wt = None
        if weight is not None:
            wt = np.ascontiguousarray(np.broadcast_to(np.asarray(weight, dtype=np.float64), (self.cells.npoints,)))
        boxes = np.empty((self.cells.ncell, 6), dtype=np.int64)
        total = C.c_int64()
        self._call("bbgpu_wind_boxes", _lib.ptr(lim), _lib.ptr(wt), _lib.ptr(boxes), C.byref(total))
        self._gen_boxes += 1
        return DeviceBoxes(self, boxes, total.value, self._gen_boxes)

    def _normal(self, wd, wm, lim, rel):
        key = (id(wm), id(wd))
        if self._wkey != key:
            W = np.ascontiguousarray(wm, dtype=np.float64)
            Wd = np.ascontiguousarray(wd, dtype=np.float64)
            if W.shape != self.shape or Wd.shape != self.shape:
                raise BBaroloError(f"WindModel: the weights must have the cube's shape {self.shape}")
            self._call("bbgpu_wind_set_weights", _lib.ptr(W), _lib.ptr(Wd))
            self._wkey, self._wref = key, (wm, wd)
        n = self.cells.ncell
        G, b = np.empty((n, n)), np.empty(n)
        lim = np.ascontiguousarray(lim, dtype=np.int64)
        self._call("bbgpu_wind_normal", _lib.ptr(lim), float(rel), _lib.ptr(G), _lib.ptr(b))
        return G, b

    def cube(self, p, amp=None, weight=None, lim=None):
        """The model cube (nz, ny, nx) of the wind p with the amplitudes amp of the cells (default 1)."""
        B = self.boxes(p, lim=lim, weight=weight)
        return B.model(np.ones(B.n) if amp is None else amp, self.shape)
