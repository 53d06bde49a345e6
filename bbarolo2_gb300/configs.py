"""Synthetic workloads of the model-evaluation path, with the shapes of the benchmark problems.

There is no public dataset for these problems: each is a mock cube on a header of the stated size, with
rings of the stated shape. Choices not fixed by the problem statements are made here once and documented:

* ``classic64``  - 64x64 px x 64 channels, 10" pixels, 5 km/s channels centred on 1000 km/s (channel 32),
  8 rings at 10-150" (step 20"), centre (32, 32), vrot 150 (1 - exp(-r/40")), vdisp 10, inc 55, pa 45, z0 0,
  dens exp(-r/60"), CDENS 10, 30" circular beam.
* ``global160``  - 160x160 px x 128 channels, 8" pixels, 4 km/s channels centred on 1000 km/s (channel 64),
  40 rings at 8 + 16k" (k = 0..39), centre (79.5, 79.5), vrot 200 (2/pi) atan(r/60"), vdisp 12 -> 6 km/s
  linearly, inc 65, pa 120, z0 10" with a sech2 layer (LTYPE 2), dens 0.8 exp(-r/160"), 30"x20" beam at
  BPA 30.  The density peak below 0.95 keeps CDENS * DENS under 10 clouds per pixel, where the cloud count of
  every sub-ring is the floor of 10 per pixel of ring area (``bbarolo/galmod.py:112-114``).
* ``bayes256``   - 256x256 px x 192 channels, 4" pixels, 6 km/s channels, 20 rings at 8 + 16k", beam 4 px FWHM
  (16"), truth drawn from the priors (vrot U(0,350), vdisp U(1,40), inc U(30,80), pa U(0,360)) with seed 7.
* ``wind_circinus`` - a WINDFIT problem with the shapes of the reference's Circinus example (MUSE [OIII]): 173x238
  px of 0.2" x 41 channels of 75 km/s (on a velocity axis) from -1725 to +1275 km/s, 0.9" beam, SPECRES 0.85
  channels; cells of 3.6" on the approaching cone (OPENANG 110, CONELEN 52": 3192 cells), quadrature for winds up to
  1600 km/s (the prior's bound) and no intrinsic dispersion; the wind at VWIND 338 km/s, INC 71.6, PA 25, apex at
  pixel (20, 40) (about half of the cone's quadrature points fall in the cube).
"""

import math

import numpy as np

from .cube import Cube, Params
from .rings import Rings


def classic64(galmodtype="MC", iseed=1):
    par = Params(CDENS=10, ISEED=iseed, LTYPE=1, galmodtype=galmodtype)
    cube = Cube.empty(64, 64, 64, [-10. / 3600., 10. / 3600., 5.], beam=30. / 3600., par=par,
                      crpix=[33., 33., 33.], crval=[60., 0., 1000.], cunit=("deg", "deg", "km/s"))
    r = np.arange(10., 151., 20.)
    rings = Rings().setRings(radii=r, xpos=32., ypos=32., vsys=1000., vrot=150. * (1 - np.exp(-r / 40.)),
                             vdisp=10., inc=55., phi=45., z0=0., dens=np.exp(-r / 60.))
    return cube, rings


def global160(galmodtype="MC", iseed=1):
    par = Params(CDENS=10, ISEED=iseed, LTYPE=2, galmodtype=galmodtype)
    cube = Cube.empty(160, 160, 128, [-8. / 3600., 8. / 3600., 4.], beam=[30. / 3600., 20. / 3600., 30.],
                      par=par, crpix=[80.5, 80.5, 65.], crval=[60., 0., 1000.], cunit=("deg", "deg", "km/s"))
    r = 8. + 16. * np.arange(40)
    rings = Rings().setRings(radii=r, xpos=79.5, ypos=79.5, vsys=1000.,
                             vrot=200. * (2 / math.pi) * np.arctan(r / 60.),
                             vdisp=np.linspace(12., 6., r.size), inc=65., phi=120., z0=10.,
                             dens=0.8 * np.exp(-r / 160.))
    return cube, rings


def bayes256(galmodtype="ANALYTIC", iseed=1, seed=7):
    par = Params(CDENS=10, ISEED=iseed, LTYPE=1, galmodtype=galmodtype)
    cube = Cube.empty(256, 256, 192, [-4. / 3600., 4. / 3600., 6.], beam=16. / 3600., par=par,
                      crpix=[128.5, 128.5, 97.], crval=[60., 0., 1000.], cunit=("deg", "deg", "km/s"))
    r = 8. + 16. * np.arange(20)
    g = np.random.default_rng(seed)
    rings = Rings().setRings(radii=r, xpos=127.5, ypos=127.5, vsys=1000.,
                             vrot=g.uniform(0., 350., r.size), vdisp=g.uniform(1., 40., r.size),
                             inc=g.uniform(30., 80.), phi=g.uniform(0., 360.), z0=0.,
                             dens=np.exp(-r / 100.))
    return cube, rings


def galaxy_population(n, seed=11, nmax=320, zmax=256):
    """n mock galaxies with the spread of the heterogeneous batch: cubes of nx = ny uniform in [32, nmax] pixels of
    10" and nz uniform in [32, zmax] channels, 5-50 rings (at most one per two pixels) out to 0.4 of the cube, inclination 20-80 degrees, position
    angle 0-360, flat rotation 50-300 km/s reached as (2/pi) arctan(r / (0.2 rmax)), dispersion 5-30 km/s, scale
    height 0-0.2 rmax, circular beam of 2-6 pixels FWHM, noise 0.5-2% of the peak (ANALYTIC model); the channel
    width makes the line span about 80% of the band. Returns a list of (cube, rings, noise fraction)."""
    g = np.random.default_rng(seed)
    out = []
    for _ in range(int(n)):
        nx = int(g.integers(32, nmax + 1))
        nz = int(g.integers(32, zmax + 1))
        nr = int(g.integers(5, 51))
        nr = min(nr, int(0.4 * nx / 2))          # (rings at least two pixels apart: GALMOD's sub-ring spacing)
        inc, pa = float(g.uniform(20., 80.)), float(g.uniform(0., 360.))
        vflat, vdisp = float(g.uniform(50., 300.)), float(g.uniform(5., 30.))
        pix = 10.
        rmax = 0.4 * nx * pix
        z0 = float(g.uniform(0., 0.2)) * rmax
        fwhm = float(g.uniform(2., 6.)) * pix
        noise = float(g.uniform(0.005, 0.02))
        dv = 2. * (vflat * math.sin(math.radians(inc)) + 4. * vdisp) / (0.8 * nz)
        par = Params(CDENS=10, ISEED=1, LTYPE=1, galmodtype="ANALYTIC")
        cube = Cube.empty(nx, nx, nz, [-pix / 3600., pix / 3600., dv], beam=fwhm / 3600., par=par,
                          crpix=[nx / 2. + 0.5, nx / 2. + 0.5, nz / 2. + 0.5], crval=[60., 0., 1000.],
                          cunit=("deg", "deg", "km/s"))
        r = (np.arange(nr) + 0.5) * (rmax / nr)
        c = (nx - 1) / 2.
        rings = Rings().setRings(radii=r, xpos=c, ypos=c, vsys=1000.,
                                 vrot=vflat * (2 / math.pi) * np.arctan(r / (0.2 * rmax)), vdisp=vdisp, inc=inc,
                                 phi=pa, z0=z0, dens=np.exp(-r / (0.5 * rmax)))
        out.append((cube, rings, noise))
    return out


def bayes256_subproblem(free_rings=(2, 7, 12, 17), noise=0.02, seed=7):
    """The BAYESIAN problem of the screen's benchmark: the ``bayes256`` cube and rings (ANALYTIC), the mock its model
    plus white noise of `noise` of the peak, the mask the model above twice the noise; VROT and VDISP of `free_rings`
    free (uniform priors: VROT within 40 km/s of the free rings' truths, VDISP 1-40 km/s), the other rings and the
    geometry at the truth. Returns (BatchLikelihood, bayesian.Problem)."""
    from . import bayesian, engine
    cube, truth = bayes256(galmodtype="ANALYTIC")
    dm = engine.DiskModel(cube, galmodtype="ANALYTIC")
    model = dm.array(truth, seed=1)
    sigma = noise * float(model.max())
    g = np.random.default_rng(seed)
    data = (model + g.normal(0., sigma, model.shape)).astype(np.float32)
    like = engine.BatchLikelihood(dm, data, model > 2 * sigma, maskmode=2, sigma=sigma)
    vr = np.asarray(truth.vrot, float)[list(free_rings)]
    prob = bayesian.Problem(truth, per_ring=("vrot", "vdisp"), global_=(), free_rings=free_rings,
                            priors={"vrot": (float(vr.min()) - 40., float(vr.max()) + 40.), "vdisp": (1., 40.)})
    return like, prob


WORKLOADS = {"classic64": classic64, "global160": global160, "bayes256": bayes256}


def wind_circinus():
    """The Circinus-shaped WINDFIT problem (module docstring): (WindModel with its quadrature, WindPars of the
    wind)."""
    from .wind import WindCells, WindModel, WindPars
    par = Params(specres=0.85)
    cube = Cube.empty(173, 238, 41, [-0.2 / 3600., 0.2 / 3600., 75.], beam=0.9 / 3600., par=par,
                      crpix=[87., 120., 24.], crval=[213.29, -65.34, 0.], cunit=("deg", "deg", "km/s"))
    wm = WindModel(cube, WindCells.resolved(52., 55., 3.6, cones=(-1,))).quadrature(vmax=1600., sigmin=0.)
    p = WindPars([26.], 338., 0., xpos=20., ypos=40., inc=71.6, pa=25., openang=110., conelen=52.)
    return wm, p


def wind_data(wm, p, noise=0.05, seed=1):
    """Mock data of the wind p: the model with the emissivity (r / 26")^-3.4 of the cells plus Gaussian noise of
    noise times its peak; W = 1 / sigma^2 on the voxels where the model is above 1e-3 of its peak, 0 elsewhere (the
    mask of the fit). Returns (W, W d)."""
    c = wm.cells.cells
    r = 0.5 * (c[:, 1] + c[:, 2])
    model = wm.cube(p, amp=(r / 26.) ** -3.4)
    peak = float(model.max())
    sig = noise * peak
    d = model + np.random.default_rng(seed).normal(0., sig, model.shape)
    W = np.where(model > 1e-3 * peak, 1. / sig ** 2, 0.)
    return W, W * d
