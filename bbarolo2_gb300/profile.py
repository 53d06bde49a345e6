"""The deconvolved density profile (``bbarolo/profile.py:33-185``) with the maps and the solve on the device.

The total-intensity map of a disk model is linear in the densities of its rings, sum_r dens_r K_r, K_r the map
of ring r with unit density convolved with the beam (``DiskModel.ring_maps``). ``profile_system`` builds the
weighted least-squares system of the reference (the maps of the rings and of an exterior annulus two beams wide,
divided by the noise, in the pixels used) and ``solve_profile`` its non-negative solution with the smoothness
prior of the reference (two solves), on the GPU: the normal equations in float64 and a Lawson-Hanson active-set
solve in one CTA (``libbbgpu.so``: ``bbgpu_solve_profile``). The batched likelihood runs the same solve for every
member inside its evaluation (``BatchLikelihood.set_profile``).
"""

import numpy as np

from . import _lib
from .galmod import outer_edge
from .rings import Rings

DENSPROF_SMOOTH = 0.3
DENSPROF_FLOOR = 0.05


def exterior_ring(model, rings, beam_arcsec=None):
    """(ext, w): the exterior annulus of ``profile_system`` (``bbarolo/profile.py:49-71``), from the outer edge of
    the disk to two beams (w) beyond, with the values of the last ring and unit density."""
    r = rings
    R = np.asarray(r.radii, float)
    if beam_arcsec:
        w = 2. * beam_arcsec
    else:
        w = 2. * float(np.max(np.diff(R), initial=R[-1]))
    edge = outer_edge(r, model.ringmode)
    if getattr(r, "edge", None) is not None:
        edge = min(edge, float(r.edge))
    ea, er = model.setup.side_edges(r)
    if ea is not None and er is not None:
        edge = min(edge, max(ea, er))
    rext = edge + w / 2.
    ext = Rings().setRings(radii=[rext], xpos=r.xpos[-1], ypos=r.ypos[-1], vsys=r.vsys[-1], vrot=r.vrot[-1],
                           vdisp=r.vdisp[-1], z0=r.z0[-1], inc=r.inc[-1], phi=r.phi[-1], dens=1., radsep=w,
                           z0thick=r.z0thick[-1], fthick=r.fthick[-1], vdispthick=r.vdispthick[-1])
    ext.twolayer = r.thick()
    ext.edgeapp = ext.edgerec = -1.
    return ext, w


def profile_system(model, rings, box, data_map, rms_map, ok_map, beam_arcsec=None):
    """(A, b, ok, Rc) of ``bbarolo/profile.py:33-79``: A (npix, nr + 1) the beam-convolved maps of the rings and
    of the exterior annulus with unit density, b the data map, both divided by the noise, in the pixels ok; Rc
    the radii of the rings and of the annulus. None with fewer than 2 nr pixels."""
    Lb, Hb = box
    K = model.ring_maps(rings, Lb, Hb)
    ext, _ = exterior_ring(model, rings, beam_arcsec)
    K = np.concatenate([K, model.ring_maps(ext, Lb, Hb, ringmode="CENTRED")])
    y, s = np.asarray(data_map, float), np.asarray(rms_map, float)
    ok = np.asarray(ok_map, bool) & (s > 0) & np.isfinite(y)
    if ok.sum() < 2 * rings.nr:
        return None
    return K[:, ok].T / s[ok, None], y[ok] / s[ok], ok, np.r_[np.asarray(rings.radii, float), float(ext.radii[0])]


def solve_profile(A, b, radii, smooth=DENSPROF_SMOOTH, corr=1., floor=None, ctx=None):
    """The non-negative densities of ``A dens = b`` with the smoothness prior (``bbarolo/profile.py:91-138``),
    solved on the device. ``ctx``: a ``_lib.Context`` (default: the module's context on device 0)."""
    from .galfit import context
    c = ctx or context()
    A = np.ascontiguousarray(A, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    R = np.ascontiguousarray(radii, np.float64)
    m, n = A.shape
    x = np.zeros(n)
    st = np.zeros(1, np.int32)
    c.check(c.L.bbgpu_solve_profile(c.h, _lib.ptr(A), _lib.ptr(b), m, n, _lib.ptr(R), float(smooth or 0.),
                                    float(corr), float(DENSPROF_FLOOR if floor is None else floor), _lib.ptr(x),
                                    _lib.ptr(st)))
    if st[0] & 1:
        raise _lib.DeviceError(_lib.ERR_KERNEL, "solve_profile: the system is rank deficient")
    return x


def deconvolved_profile(model, rings, box, data_map, rms_map, ok_map, smooth=DENSPROF_SMOOTH, beam_arcsec=None,
                        corr=1.):
    """The ring densities whose beam-convolved model reproduces data_map (``bbarolo/profile.py:175-185``), or
    None with too few pixels."""
    sysm = profile_system(model, rings, box, data_map, rms_map, ok_map, beam_arcsec=beam_arcsec)
    if sysm is None:
        return None
    A, b, _, Rc = sysm
    return solve_profile(A, b, Rc, smooth, corr, ctx=model.ctx)[:rings.nr]
