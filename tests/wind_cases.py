"""The wind-model cases of the golden fixtures and the tests (``tests/golden/wind.npz``): each a cube, a grid of
cells with its quadrature, the parameters of one wind, the box of the columns, a weight per point, the pruning of
the voxel lists and the weights of the normal equations, all built with the package's own classes so that the tests
rebuild what the reference was run on."""
import math

import numpy as np

from bbarolo2_gb300.cube import Cube, Params

F0 = 1.42040575e9


def cube(nx, nz, pix=10., beam=(30.,), freq=False, crota=0.):
    """An empty cube nx x nx x nz: pixels of pix arcsec; 15 km/s channels centred on 0, or a frequency axis of
    50 kHz channels around the HI line with a second line 60 km/s away (RELINT 1, 0.5); beam (arcsec, arcsec,
    degrees) or None."""
    par = Params()
    b = None if beam is None else [beam[0] / 3600., (beam[1] if len(beam) > 1 else beam[0]) / 3600.] + list(beam[2:])
    if freq:
        par.gf.RESTFREQ = [F0, F0 * (1 + 60e3 / 2.99792458e8)]
        par.gf.RELINT = [1.0, 0.5]
        return Cube.empty(nx, nx, nz, [-pix / 3600., pix / 3600., -50e3], beam=b, par=par,
                          crpix=[nx / 2., nx / 2., nz / 2. + 0.5], crval=[60., 0., F0], cunit=("deg", "deg", "hz"),
                          sptype="freq", freq0=F0, crota=crota)
    return Cube.empty(nx, nx, nz, [-pix / 3600., pix / 3600., 15.], beam=b, par=par,
                      crpix=[nx / 2., nx / 2., nz / 2. + 0.5], crval=[60., 0., 0.], cunit=("deg", "deg", "km/s"),
                      crota=crota)


# name: cube kwargs, cells (("resolved", args, kwargs) or ("grid", args, kwargs)), quadrature (vmax, sigmin),
# smooth, wind parameters, lim (None: the cube), weight (None or "exp": exp(-r/30)), rel, zeros in the weights
CASES = {
    "sep": dict(cube=dict(nx=24, nz=20), cells=("resolved", (110., 40., 35.), {}), quad=(150., 10.), smooth=True,
                pars=dict(radii=[50.], vwind=150., vdisp=10., xpos=11.5, ypos=11.5, inc=60., pa=45., openang=60.,
                          conelen=100.),
                lim=None, weight=None, rel=0., holes=False),
    "ell": dict(cube=dict(nx=24, nz=20, beam=(40., 20., 30.)), cells=("grid", ([0., 40., 80., 120.], 2, 3),
                                                                      dict(thmax=35.)),
                quad=(220., 8.), smooth=True,
                pars=dict(radii=[20., 90.], vwind=[100., 200.], vdisp=[15., 8.], vrot=[30., 10.], xpos=12.3,
                          ypos=10.8, vsys=20., inc=50., pa=120., openang=64., openin=20., conelen=105.),
                lim=[3, 21, 2, 22, 2, 18], weight="exp", rel=1e-3, holes=True),
    "freq_nobeam": dict(cube=dict(nx=20, nz=16, pix=8., beam=None, freq=True, crota=15.),
                        cells=("resolved", (80., 30., 20.), dict(cones=(-1,))), quad=(150., 12.), smooth=False,
                        pars=dict(radii=[40.], vwind=120., vdisp=12., vrot=20., xpos=9.7, ypos=10.2, inc=70.,
                                  pa=-30., openang=50., conelen=70.),
                        lim=None, weight=None, rel=0., holes=False),
}


def make_cells(mod, spec):
    """The cells of a case with the WindCells class of module mod (the package's or the reference's)."""
    kind, args, kw = spec
    return mod.WindCells.resolved(*args, **kw) if kind == "resolved" else mod.WindCells(*args, **kw)


def weights(name, shape):
    """Seeded weights W, data d and the weighted data W d of the normal equations of a case."""
    g = np.random.default_rng(sum(map(ord, name)))
    W = g.uniform(0.5, 2., shape)
    if CASES[name]["holes"]:
        W[g.random(shape) < 0.1] = 0.
    d = g.normal(0., 1e-3, shape)
    return W, d, W * d


def point_weight(name, r):
    return None if CASES[name]["weight"] is None else np.exp(-np.asarray(r) / 30.)


def geometry(p, crota2):
    """The scalars of WindModel.points (bbarolo/windmodel.py:808-827) for parameters p."""
    inc = math.radians(p["inc"])
    ang = math.radians(p["pa"]) + crota2
    return dict(vsys=p.get("vsys", 0.) * 1000., sinc=math.sin(inc), cinc=math.cos(inc), spa=math.sin(ang),
                cpa=math.cos(ang), th_in=math.radians(0.5 * p.get("openin", 0.)),
                th_out=math.radians(0.5 * p["openang"]), rmax=p["conelen"])


# GALWIND WTYPE 1 (the Monte-Carlo shells): cube kwargs, the GalWindPars, threads (chunks of shells, one stream each)
# and the box of the kernel call (None: the cube)
GW_CASES = {
    "gw_velo": dict(cube=dict(nx=24, nz=20),
                    par=dict(xpos=11.5, ypos=11.5, vsys=0., inc=60., phi=45., conelen=140., nlayers=10, vwind=150.,
                             vdisp=10., dens=10., openang=60., cdens=50., nv=10, iseed=3),
                    threads=3, box=None),
    "gw_radii_freq": dict(cube=dict(nx=20, nz=16, pix=8., beam=None, freq=True, crota=15.),
                          par=dict(xpos=9.7, ypos=10.2, vsys=20., inc=70., phi=-30., conelen=120.,
                                   radii=[10., 40., 80., 120.], vrot=20., vwind=[100., 150., 200., 180.],
                                   vdisp=[0., 0., 8., 12.], dens=[5., 3., 2., 1.], openang=[40., 50., 60., 70.],
                                   cdens=20., nv=-1, iseed=7),
                          threads=2, box=((3, 2), (17, 19))),
}


def gw_reference_par(p):
    """The parameters of a GW case as the reference's parameter file gives them (strings for the per-radius
    values, RADII "-1" when not given)."""
    def text(v):
        return " ".join(str(float(x)) for x in np.atleast_1d(v))
    return dict(PHI=p["phi"], INC=p["inc"], VSYS=p["vsys"], CONELEN=p["conelen"], NLAYERS=p.get("nlayers", 25),
                RADII="-1" if p.get("radii") is None else text(p["radii"]), VROT=text(p.get("vrot", 0.)),
                VWIND=text(p["vwind"]), VDISP=text(p["vdisp"]), DENS=text(p["dens"]), OPENANG=text(p["openang"]),
                NV=p["nv"], CDENS=p["cdens"], ISEED=p["iseed"])
