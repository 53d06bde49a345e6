"""The beam kernel of the model convolution (host side, float64).

Restates ``bbarolo/smooth.py``:

* ``convpars`` (``smooth.py:25-51``): the Gaussian that convolves an old beam into a new one (Wild 1970);
* ``fillgauss2d`` (``smooth.py:62-88``): a rotated 2D Gaussian sampled on the pixel grid, taps below 1e-4 of
  the peak set to zero, normalised to unit sum;
* ``gaussian_scalefactor`` (``smooth.py:91-101``) and the kernel set-up of ``Smooth3D.defineBeam_Gaussian``
  (``smooth.py:203-231``) as used by ``DiskModel._set_kernel`` (``galmod.py:1205-1214``): from a point
  source (old beam 0) to the beam of the cube, position angle measured from +X after CROTA.

The kernel is computed once per cube on the host and uploaded to the device as float32 taps (and the float64
original for the CLASSIC sparse path).
"""

import math

import numpy as np

CUTOFFRATIO = 1.0 / 10000.0
MAXCONV = 512 * 512


def convpars(oldbeam, newbeam):
    d2r = math.atan(1.) / 45.
    a2, b2 = oldbeam[0] / 2, oldbeam[1] / 2
    a0, b0 = newbeam[0] / 2, newbeam[1] / 2
    D0 = a0 * a0 - b0 * b0
    D2 = a2 * a2 - b2 * b2
    th2, th0 = oldbeam[2] * d2r, newbeam[2] * d2r
    D1 = math.sqrt(max(D0 * D0 + D2 * D2 - 2 * D0 * D2 * math.cos(2 * (th0 - th2)), 0.))
    s = a0 * a0 + b0 * b0 - a2 * a2 - b2 * b2
    arg = 0.5 * (s + D1)
    if arg < 0:
        return None
    a1 = math.sqrt(arg)
    arg = 0.5 * (s - D1)
    if arg < 0:
        if arg > -1e-9 * max(a0 * a0, 1e-30):
            arg = 0.
        else:
            return None
    b1 = math.sqrt(arg)
    nom = D0 * math.sin(2 * th0) - D2 * math.sin(2 * th2)
    den = D0 * math.cos(2 * th0) - D2 * math.cos(2 * th2)
    th1 = 0. if (den == 0 and nom == 0) else math.atan2(nom, den) / 2
    return (2 * a1, 2 * b1, th1 / d2r)


def fillgauss2d(beam, gridspace, ampl=1.0, norm=True, cutoff=CUTOFFRATIO):
    """Rotated Gaussian (bmaj, bmin, pa [deg from +X]) on a grid of spacing gridspace: array (ny, nx)."""
    amplitude = 1.0 if norm else ampl
    phi = beam[2] * math.pi / 180.
    cs, sn = math.cos(phi), math.sin(phi)
    bmaj, bmin = abs(beam[0]), abs(beam[1])
    extend = math.sqrt(-1.0 * math.log(cutoff) / math.log(2.0))
    xr, yr = 0.5 * bmaj * extend, 0.5 * bmin * extend
    xext = max(abs(xr * cs), abs(-yr * sn))
    yext = max(abs(xr * sn), abs(yr * cs))
    gx, gy = abs(gridspace[0]), abs(gridspace[1])
    Xmax, Ymax = int(round(xext / gx)), int(round(yext / gy))
    if (2 * Xmax + 1) * (2 * Ymax + 1) > MAXCONV:
        return None
    jj, ii = np.mgrid[-Ymax:Ymax + 1, -Xmax:Xmax + 1]
    xx, yy = ii * gx, jj * gy
    xrot = xx * cs + yy * sn
    yrot = -xx * sn + yy * cs
    ax = xrot / bmaj if bmaj != 0 else 0 * xrot
    ay = yrot / bmin if bmin != 0 else 0 * yrot
    c = np.exp(-4.0 * math.log(2.0) * (ax * ax + ay * ay))
    c = np.where(c >= cutoff, c * amplitude, 0.)
    if norm:
        c = c / c.sum()
    return c


def gaussian_scalefactor(oldbeam_rot, kernel, gridspace):
    """1 / (G_old * K)(0): the flux scaling of the convolution of column densities."""
    g = fillgauss2d(oldbeam_rot, gridspace, 1.0, norm=False)
    ky, kx = kernel.shape
    gy, gx = g.shape
    hy, hx = min(ky, gy) // 2, min(kx, gx) // 2
    cg = g[gy // 2 - hy:gy // 2 + hy + 1, gx // 2 - hx:gx // 2 + hx + 1]
    ck = kernel[ky // 2 - hy:ky // 2 + hy + 1, kx // 2 - hx:kx // 2 + hx + 1]
    val = float(np.sum(cg * ck[::-1, ::-1]))
    return 1.0 / val if val != 0 else 1.0


class BeamKernel:
    """The convolution kernel of the models of a cube and its flux scale factor.

    ``BeamKernel.from_cube(cube)`` follows ``DiskModel._set_kernel``: old beam (0, 0, 0), new beam the cube's
    (BMAJ, BMIN in arcsec, BPA), a beam given with BMAJ < BMIN has its axes swapped and PA + 90, the kernel's
    PA is BPA - (CROTA - 90) on the grid (CDELT1, CDELT2 in arcsec). ``kernel`` is None when the beam cannot be
    set (no smoothing)."""

    def __init__(self, kernel, scalefac, conbeam=None):
        self.kernel = None if kernel is None else np.ascontiguousarray(kernel, dtype=np.float64)
        self.scalefac = float(scalefac)
        self.conbeam = conbeam

    @classmethod
    def from_cube(cls, cube):
        h = cube.Head()
        from .galmod import arcsconv, BBaroloError
        conv = arcsconv(h.Cunit(0))
        gridspace = (h.Cdelt(0) * conv, h.Cdelt(1) * conv)
        crota = h.Crota()
        ob = [0., 0., 0.]
        nb = [h.Bmaj() * 3600., h.Bmin() * 3600., h.Bpa()]
        for b in (ob, nb):
            if b[0] < b[1]:
                b[0], b[1], b[2] = b[1], b[0], b[2] + 90.
        if not (nb[0] >= ob[0] and nb[1] >= ob[1]):
            raise BBaroloError("SMOOTH: the new beam is smaller than the old beam.")
        cb = convpars(ob, nb)
        if cb is None:
            raise BBaroloError(f"SMOOTH: cannot calculate the convolution from the beam {ob} to the beam {nb}.")
        cb = [cb[0], cb[1], cb[2] - (crota - 90)]
        k = fillgauss2d(cb, gridspace, 1.0, norm=True)
        if k is None:
            return cls(None, 1.0)
        obr = (ob[0], ob[1], ob[2] + 90 - crota)
        sf = gaussian_scalefactor(obr, k, gridspace)
        cb[2] += crota
        return cls(k, sf, tuple(cb))
