"""CLASSIC 3DFIT (``bbarolo/galfit.py:455-1238``) with every model and residual on the device.

The reference fits one ring at a time: a downhill simplex over the free parameters of the ring, each trial point
moved into the parameter bounds (redrawn at random inside them for VROT and VDISP), then the model of the ring
alone built (MC GALMOD), convolved (``_conv_sparse``) and normalised against the data (``_norm``). The rings of a
stage are independent; the reference spreads them over threads.

Here the rings of a stage advance together, in rounds: each ring's simplex is a coroutine (``simplex``) that yields
its next trial point and receives the value, and a round evaluates the pending point of every ring still running on
the device. The arithmetic of a fit is the reference's: the same steps of the simplex (the Nelder-Mead method in the
form of Numerical Recipes' ``amoeba``, with the reference's initial steps, tolerance and budget of 200 evaluations per
free parameter), the same bounds, the same seeded generator per ring for the redraws, so each ring visits the
reference's points and ends at its minimum (tested against fits recorded from the reference). Not here: the
second stage (regularisation), REVERSE passes and error estimates of the reference, which call the same evaluation.
"""

import math
from dataclasses import dataclass

import numpy as np

from .galfit import _norm, context
from .galmod import arcsconv

TINY = 1.0e-10
NORMCODE = {"LOCAL": 0, "AZIM": 1, "AZIMUTHAL": 1, "NONE": 2}
SIDECODE = {"R": 1, "A": 2}

# the free parameters in the reference's order, with the FREE keyword that selects each and its Rings attribute
PARAMS = ("vrot", "vdisp", "dens", "z0", "inc", "phi", "xpos", "ypos", "vsys", "vrad")
_KEYWORD = {"vrot": "vrot", "vdisp": "disp", "dens": "dens", "z0": "z0", "inc": "inc", "phi": "pa",
            "xpos": "xpos", "ypos": "ypos", "vsys": "vsys", "vrad": "vrad"}


def free_parameters(free):
    """The free parameters named in FREE (``bbarolo/galfit.py`` setFree): in PARAMS order; 'ALL' frees every one."""
    f = str(free).lower()
    if "all" in f:
        return list(PARAMS)
    out = [p for p in PARAMS if _KEYWORD[p] in f or (p == "phi" and "phi" in f)]
    if not out:
        raise ValueError(" 3DFIT ERROR: NO free parameters!")
    return out


def default_par(**kw):
    """The 3DFIT parameters a CLASSIC fit reads, with the reference's defaults (``bbarolo/params.py``): FREE "VROT
    VDISP", one stage, NORM AZIM, FTYPE 2, WFUNC 2, SIDE B, TOL 1e-3, and the GALMOD ones of the cube; keywords
    override them."""
    import types
    par = types.SimpleNamespace(FREE="VROT VDISP", DELTAVROT=1000.0, MINVDISP=0.1, MAXVDISP=1000.0, DELTAINC=5.0,
                                DELTAPHI=15.0, TOL=1e-3, FTYPE=2, WFUNC=2, SIDE="B", BWEIGHT=1.0, NORM="AZIM",
                                NORMALCUBE=True, TWOSTAGE=False, flagERRORS=False, STARTRAD=0, DENSFLUX=True,
                                CDENS=10, CMODE=1, ISEED=1, LTYPE=1, NV=-1, REDSHIFT=0.0, EMPTY=True,
                                RESTWAVE=[-1.0], RESTFREQ=[-1.0], RELINT=[1.0], SM=True, RADMAXA=-1.0,
                                RADMAXR=-1.0)
    for k, v in kw.items():
        setattr(par, k, v)
    return par


@dataclass
class Limits:
    """The bounds of one free parameter for a stage: [lo, hi] from the initial rings, and how a trial value outside
    them comes back in: 'redraw' (uniform within `span` of the bound), 'clip' (to the bound, within `delta` of the
    ring's initial value) or 'reset' (to the ring's initial value)."""
    lo: float
    hi: float
    rule: str
    delta: float = 0.0


def stage_limits(par, inr, cube, axis_kms):
    """The bounds of every parameter (``bbarolo/galfit.py:600-633``): VROT within DELTAVROT of the initial values and
    not negative, VDISP within [MINVDISP, MAXVDISP], Z0 in [0, 1000], INC within DELTAINC of the initial values and
    [0, 90], PA within DELTAPHI and [-360, 360], the centre within 10 pixels and the cube, VSYS within the band, VRAD
    in [-500, 500]. axis_kms: the velocities (km/s) of the first and last channel."""
    lim = {
        "vrot": Limits(max(inr.vrot.min() - par.DELTAVROT, 0), inr.vrot.max() + par.DELTAVROT, "redraw",
                       par.DELTAVROT),
        "vdisp": Limits(par.MINVDISP, par.MAXVDISP, "redraw"),
        "dens": Limits(0., math.inf, "reset"),
        "z0": Limits(0., 1000., "reset"),
        "inc": Limits(max(inr.inc.min() - par.DELTAINC, 0), min(inr.inc.max() + par.DELTAINC, 90), "clip",
                      par.DELTAINC),
        "phi": Limits(max(inr.phi.min() - par.DELTAPHI, -360), min(inr.phi.max() + par.DELTAPHI, 360), "clip",
                      par.DELTAPHI),
        "xpos": Limits(max(inr.xpos.min() - 10, 0), min(inr.xpos.max() + 10, cube.DimX()), "reset"),
        "ypos": Limits(max(inr.ypos.min() - 10, 0), min(inr.ypos.max() + 10, cube.DimY()), "reset"),
        "vsys": Limits(min(axis_kms), max(axis_kms), "reset"),
        "vrad": Limits(-500., 500., "reset"),
    }
    return lim


def into_bounds(name, z, lim, init, draw):
    """The value of parameter `name` actually evaluated for the trial value z (``bbarolo/galfit.py:832-886``): z
    inside the bounds, else the rule of `lim`; init: the ring's initial value; draw(): a uniform deviate, taken only
    for a redraw."""
    if lim.rule == "redraw":
        if name == "vrot":
            lo, hi, span = max(init - lim.delta, lim.lo), min(init + lim.delta, lim.hi), lim.delta
        else:
            lo, hi, span = lim.lo, lim.hi, min(init, lim.hi - lim.lo)
        if z > hi:
            return hi - draw() * span
        if z < lo:
            return lo + draw() * span
        return z
    if lim.rule == "clip":
        lo, hi = max(init - lim.delta, lim.lo), min(init + lim.delta, lim.hi)
        return hi if z > hi else (lo if z < lo else z)
    if name == "dens":
        return init if z < 0 else z
    return init if (z < lim.lo or z > lim.hi) else z


def initial_step(name, v, lim):
    """The simplex's initial step of a parameter at value v (``bbarolo/galfit.py:900-914``)."""
    if name == "vrot":
        return 30. if v > 40 else 5
    if name == "vdisp":
        return 20. if v > 80 else (10. if 20. < v <= 80. else (0.2 if v <= 2 else 5))
    if name in ("dens", "z0"):
        return 0.2 * v
    if name == "inc":
        return 5.
    if name == "phi":
        return 10.
    if name == "vrad":
        return 25
    return (lim.hi - lim.lo) / 4.


# ------------------------------------------------------------------------------------------------ the simplex
def _rank(y):
    """(best, worst, second worst) vertices of the simplex, ties resolved as Numerical Recipes' amoeba resolves
    them (the last of equal best values; the worst found first)."""
    best = 0
    worst, second = (0, 1) if y[0] > y[1] else (1, 0)
    for i, v in enumerate(y):
        if v <= y[best]:
            best = i
        if v > y[worst]:
            second, worst = worst, i
        elif v > y[second] and i != worst:
            second = i
    return best, worst, second


def _move(P, y, psum, worst, fac):
    """A trial point on the line through the worst vertex and the centroid of the others (fac -1 reflects, 2
    expands, 0.5 contracts); the vertex is replaced by the point (as evaluated, inside the bounds) if it is better.
    A sub-coroutine of ``simplex``: yields the point, receives (value, point evaluated)."""
    n = P.shape[1]
    f1 = (1.0 - fac) / n
    f2 = f1 - fac
    value, got = yield psum * f1 - P[worst] * f2
    if value < y[worst]:
        y[worst] = value
        psum += got - P[worst]
        P[worst] = got
    return value


def simplex(x0, steps, tol, nmax):
    """The downhill simplex of Nelder and Mead as a coroutine: yields trial points and receives (value, point as
    evaluated) for each; returns (converged, minimum, parameters at the minimum). The vertices start at x0 and x0
    plus each step; the fit converges when the spread of the values 2 |f_worst - f_best| / (|f_worst| + |f_best| +
    1e-10) falls below tol, and fails after nmax evaluations (not counting the first n + 1)."""
    x0 = np.asarray(x0, float)
    n = x0.size
    P = np.tile(x0, (n + 1, 1))
    for i in range(1, n + 1):
        P[i, i - 1] += steps[i - 1]
    y = np.empty(n + 1)
    for i in range(n + 1):
        y[i], _ = yield P[i].copy()
    used = 0
    psum = P.sum(axis=0)
    while True:
        best, worst, second = _rank(y)
        spread = 2.0 * abs(y[worst] - y[best]) / (abs(y[worst]) + abs(y[best]) + TINY)
        if spread < tol:
            return True, float(y[best]), P[best].copy()
        if used >= nmax:
            return False, float(y[best]), P[best].copy()
        used += 2
        value = yield from _move(P, y, psum, worst, -1.0)
        if value <= y[best]:
            yield from _move(P, y, psum, worst, 2.0)
        elif value >= y[second]:
            before = y[worst]
            value = yield from _move(P, y, psum, worst, 0.5)
            if value >= before:
                # shrink towards the best vertex: the new vertices are kept as computed (their evaluated copies,
                # moved into the bounds, are not)
                for i in range(n + 1):
                    if i != best:
                        P[i] = 0.5 * (P[i] + P[best])
                        y[i], _ = yield P[i].copy()
                used += n
                psum = P.sum(axis=0)
        else:
            used -= 1


# ------------------------------------------------------------------------------------------------ the fit
def ring_pixels(mask2d, blo, bhi, x0, y0, phi, inc, r1, r2):
    """(pixels of the ring's annulus in the box [blo, bhi] (inclusive), those with mask voxels): the count that
    decides whether a ring is fitted (``bbarolo/galfit.py:199-216``)."""
    F = math.pi / 180.
    sphi, cphi, cinc = math.sin(F * phi), math.cos(F * phi), math.cos(F * inc)
    y, x = np.mgrid[blo[1]:bhi[1] + 1, blo[0]:bhi[0] + 1]
    dx = (x - blo[0]).astype(np.float64) - x0
    dy = (y - blo[1]).astype(np.float64) - y0
    along = -dx * sphi + dy * cphi
    across = (-dx * cphi - dy * sphi) / cinc
    r = np.sqrt(along * along + across * across)
    ring = (r >= r1) & (r <= r2)
    ny, nx = mask2d.shape
    inside = (y < ny) & (x < nx)
    masked = np.zeros(ring.shape, bool)
    masked[inside] = mask2d[y[inside], x[inside]] > 0
    return int(ring.sum()), int((ring & masked).sum())


def ring_annulus(inr, ir, values=None):
    """The ring ir as 3DFIT fits it (``bbarolo/galfit.py:978-1000``): an annulus from halfway to the previous radius to
    halfway to the next (the radius spacing at the ends, RADSEP for a single ring), its edges rounded to float32 as the
    reference, with the values of ring ir of `values` (default the initial rings)."""
    from .rings import Rings
    R = inr.radii
    v = inr if values is None else values
    nr = inr.nr
    if nr == 1:
        inner = outer = inr.radsep / 2. if inr.radsep > 0 else R[0] / 2.
    else:
        inner = (R[ir] - R[ir - 1]) / 2. if ir > 0 else (R[1] - R[0]) / 2.
        outer = (R[ir + 1] - R[ir]) / 2. if ir < nr - 1 else inner
    inner, outer = np.float32(inner), np.float32(outer)
    edges = [max(float(np.float32(R[ir] - inner)), 0.), max(float(np.float32(R[ir] + outer)), 0.)]
    d = Rings()
    d.setRings(radii=edges, **{k: getattr(v, k)[ir] for k in ("xpos", "ypos", "vsys", "vrot", "vdisp", "vrad",
                                                               "vvert", "dvdz", "zcyl", "dens", "z0", "inc", "phi",
                                                               "z0thick", "fthick", "vdispthick")})
    d.twolayer = v.thick()
    d.radsep = edges[1] - edges[0]
    d.id = ir
    return d


class ClassicFit:
    """The CLASSIC fit of the rings of a cube, one stage (``bbarolo/galfit.py:1162-1238`` without REVERSE passes,
    second stage or errors), the rings advanced together in rounds (see the module docstring).

    cube: a ``Cube`` (data (nz, ny, nx) and header); rings: the initial ``Rings``; par: the 3DFIT parameters (FREE,
    DELTAVROT, DELTAINC, DELTAPHI, MINVDISP, MAXVDISP, TOL, FTYPE, WFUNC, SIDE, BWEIGHT, NORM, NORMALCUBE, STARTRAD and
    the GALMOD ones); data_noise: the noise of the data; mask (nz, ny, nx) bool; chan_noise (nz), default ones.
    After ``run``: ``status[ir]`` (text, minimum) and ``log[ir]``, the evaluations of ring ir as (parameters as
    evaluated, value)."""

    def __init__(self, cube, rings, par, data_noise, mask, chan_noise=None, device=0):
        from .engine import DiskModel
        self.cube, self.par, self.inr = cube, par, rings.copy()
        h = cube.Head()
        self.free = free_parameters(par.FREE)
        self.model = DiskModel(cube, par=par, densflux=True, device=device)
        self.ctx = self.model.ctx
        st = self.model.setup
        band = np.asarray(st._vedges_lines[0], float) / 1000.
        centres = 0.5 * (band[:-1] + band[1:])
        self.limits = stage_limits(par, self.inr, cube, (centres[0], centres[-1]))
        self.band = (band[0], band[-1])
        conv = arcsconv(h.Cunit(0))
        self.pixscale = ((abs(h.Cdelt(0)) * conv) + (abs(h.Cdelt(1)) * conv)) / 2.
        self.mask_yxz = np.ascontiguousarray(np.asarray(mask, bool).transpose(1, 2, 0))
        self.mask2d = np.asarray(mask, bool).sum(axis=0).astype(np.int32)
        self.data_noise = float(data_noise)
        self.chan_noise = np.ones(cube.DimZ()) if chan_noise is None else np.asarray(chan_noise, np.float64)
        norms = [("AZIM" if n == "AZIMUTHAL" else n) for n in str(par.NORM).split()] or ["LOCAL"]
        self.norms = [n if n in NORMCODE else "LOCAL" for n in (norms + norms[-1:] * 2)[:3]]
        self.status, self.log = {}, {}

    def _residual(self, dring, data_yxz, noise, normtype):
        """The CLASSIC residual of the model of one ring (``Galfit.getFuncValue``, ``bbarolo/galfit.py:736-749``):
        its MC model and sparse convolution on the device, then ``_norm`` on the device."""
        blo, bhi = self.model.box(dring)
        mod = np.ascontiguousarray(self.model.array(dring, blo, bhi, final=False, layout="yxz"), np.float64)
        p = self.par
        return _norm(mod, data_yxz, self.mask_yxz, blo[0], blo[1], dring.xpos[-1] - blo[0], dring.ypos[-1] - blo[1],
                     dring.phi[-1], dring.inc[-1], dring.radii[0] / self.pixscale, dring.radii[-1] / self.pixscale,
                     float(p.WFUNC), SIDECODE.get(p.SIDE, 0), p.FTYPE, self.chan_noise, noise, float(p.BWEIGHT),
                     normtype, None, None, None, None, None, 0, 0., ctx=self.ctx)

    def _start(self, ir, stage):
        """The coroutine of ring ir and its state, or None (ring skipped: too few pixels of the mask)."""
        dring = ring_annulus(self.inr, ir)
        blo, bhi = self.model.box(dring)
        total, masked = ring_pixels(self.mask2d, blo, bhi, dring.xpos[-1] - blo[0], dring.ypos[-1] - blo[1],
                                    dring.phi[-1], dring.inc[-1], dring.radii[0] / self.pixscale,
                                    dring.radii[-1] / self.pixscale)
        if masked < 20 and (masked == 0 or masked < 0.7 * total):
            self.status[ir] = ("skipped: few pixels in the mask", None)
            return None
        x0 = [float(getattr(dring, k)[0]) for k in self.free]
        steps = [initial_step(k, x, self.limits[k]) for k, x in zip(self.free, x0)]
        co = simplex(x0, steps, self.par.TOL, 200 * len(self.free))
        return dict(ir=ir, ring=dring, co=co, rng=np.random.default_rng([12345, stage, ir]), point=next(co))

    def _evaluate(self, job, data_yxz, noise, normtype):
        """Moves the job's pending point into the bounds (in PARAMS order, redraws from the ring's generator), sets
        it in the ring and returns (value, point as evaluated)."""
        ir, dring, x = job["ir"], job["ring"], np.array(job["point"], float)
        draw = job["rng"].random
        for i, k in enumerate(self.free):
            x[i] = into_bounds(k, x[i], self.limits[k], float(getattr(self.inr, k)[ir]), draw)
            getattr(dring, k)[:] = x[i]
        value = self._residual(dring, data_yxz, noise, normtype)
        self.log[ir].append((x.copy(), value))
        return value, x

    def run(self, rings=None, stage=1):
        """One fitting stage over the rings (default: from STARTRAD), the data normalised to a peak of 10 during the
        fit (NORMALCUBE). Returns (fitted Rings, converged per ring)."""
        data = np.asarray(self.cube.array)
        noise = self.data_noise
        if getattr(self.par, "NORMALCUBE", True):
            scaling = 10. / float(np.nanmax(data))
            data = (data * scaling).astype(data.dtype)
            noise = noise * scaling
        data_yxz = np.ascontiguousarray(np.asarray(data, np.float32).transpose(1, 2, 0))
        normtype = NORMCODE[self.norms[stage - 1]]
        nr = self.inr.nr
        start = self.par.STARTRAD if self.par.STARTRAD < nr else 0
        order = list(range(start, nr)) if rings is None else list(rings)
        out, ok = self.inr.copy(), [False] * nr
        jobs = []
        for ir in order:
            self.log[ir] = []
            job = self._start(ir, stage)
            if job is not None:
                jobs.append(job)
        while jobs:                                          # one round: every running ring's pending point
            running = []
            for job in jobs:
                try:
                    job["point"] = job["co"].send(self._evaluate(job, data_yxz, noise, normtype))
                    running.append(job)
                except StopIteration as done:
                    self._finish(job, done.value, out, ok)
            jobs = running
        return out, ok

    def _finish(self, job, result, out, ok):
        converged, minimum, xmin = result
        ir = job["ir"]
        if not converged:
            self.status[ir] = ("not converged", minimum)
            return
        for k, v in zip(self.free, xmin):
            getattr(out, k)[ir] = v
        sini = math.sin(out.inc[ir] * math.pi / 180.)
        reach = max(abs(self.band[1] - out.vsys[ir]), abs(self.band[0] - out.vsys[ir]))
        vmax = reach / sini if sini != 0 else math.inf
        if out.vrot[ir] > vmax:                              # (bbarolo/galfit.py:1066-1094: beyond the band)
            self.status[ir] = ("rejected: VROT beyond the band", minimum)
            return
        ok[ir] = True
        self.status[ir] = ("ok", minimum)
