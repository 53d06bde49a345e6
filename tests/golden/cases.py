"""The inputs of the golden fixture cases (shared by make_golden.py and the tests): cubes and rings built with
the package's own Cube/Rings, so that the tests rebuild exactly what the reference was run on."""
import numpy as np

from bbarolo2_gb300 import configs
from bbarolo2_gb300.cube import Cube, Params
from bbarolo2_gb300.rings import Rings


def cube64(ltype=1, nv=-1, cdens=10, cmode=1, sptype="velo-radio", nlines=1, crota=0.):
    par = Params(CDENS=cdens, CMODE=cmode, ISEED=1, LTYPE=ltype, NV=nv)
    if sptype == "freq":
        # 64 channels of 24.4 kHz around the redshifted HI line; two lines (RESTFREQ) when nlines == 2
        f0 = 1.42040575e9
        cube = Cube.empty(64, 64, 64, [-10. / 3600., 10. / 3600., -24.4e3], beam=30. / 3600., par=par,
                          crpix=[33., 33., 33.], crval=[60., 0., f0 * (1 - 1000e3 / 2.99792458e8)],
                          cunit=("deg", "deg", "hz"), sptype="freq", freq0=f0, crota=crota)
        if nlines == 2:
            par.gf.RESTFREQ = [f0, f0 * (1 + 80e3 / 2.99792458e8)]
            par.gf.RELINT = [1.0, 0.4]
        return cube
    return Cube.empty(64, 64, 64, [-10. / 3600., 10. / 3600., 5.], beam=30. / 3600., par=par,
                      crpix=[33., 33., 33.], crval=[60., 0., 1000.], cunit=("deg", "deg", "km/s"), crota=crota)


def rings64(**kw):
    r = np.arange(10., 151., 20.)
    d = dict(radii=r, xpos=32., ypos=32., vsys=1000., vrot=150. * (1 - np.exp(-r / 40.)), vdisp=10., inc=55.,
             phi=45., z0=0., dens=np.exp(-r / 60.))
    d.update(kw)
    return Rings().setRings(**d)


def mc_cases():
    """(name, cube, rings, ringmode, box, seed) of the model fixtures."""
    c = []
    cube, rings = configs.classic64()
    c.append(("classic64", cube, rings, "CENTRED", None, 1))
    c.append(("classic64_box", cube, rings, "CENTRED", ((10, 5), (50, 60)), 1))
    c.append(("classic64_seedm1", cube, rings, "CENTRED", None, -1))
    c.append(("sech2_lag", cube64(ltype=2), rings64(z0=12., dvdz=8., zcyl=5., vrad=10., vvert=-5.), "CENTRED",
              None, 3))
    c.append(("exp_layer_nv20", cube64(ltype=3, nv=20), rings64(z0=8.), "NODES", None, 4))
    c.append(("lorentz_box", cube64(ltype=4), rings64(z0=6.), "CENTRED", ((8, 8), (56, 50)), 5))
    c.append(("box_layer_vdisp0", cube64(ltype=5), rings64(z0=15., vdisp=np.r_[0., 0., 8, 8, 8, 8, 8, 8]),
              "SHIFTED", None, 6))
    r = rings64(z0=5., fthick=0.3, z0thick=20., vdispthick=25., dvdz=10., zcyl=0.)
    r.edgeapp, r.edgerec = 100., -1.
    c.append(("thick_sideedge", cube64(ltype=1), r, "CENTRED", None, 7))
    r = rings64(inc=np.linspace(40, 70, 8), phi=np.linspace(30, 60, 8))
    r.edge, r.edgewidth = 120., 10.
    c.append(("warp_gaussedge_crota", cube64(crota=20.), r, "CENTRED", None, 8))
    c.append(("freq_axis", cube64(sptype="freq"), rings64(), "CENTRED", None, 9))
    c.append(("freq_2lines", cube64(sptype="freq", nlines=2), rings64(), "CENTRED", None, 10))
    c.append(("cmode2_dense", cube64(cdens=40, cmode=2), rings64(dens=2.0 * np.exp(-np.arange(10., 151., 20.) / 60.)),
              "CENTRED", None, 11))
    return c


def subring_cases():
    out = []
    for wl in ("classic64", "global160", "bayes256"):
        cube, rings = configs.WORKLOADS[wl]()
        out.append((wl, cube, rings, "CENTRED"))
    for case in mc_cases()[3:]:
        out.append((case[0], case[1], case[2], case[3]))
    r = rings64()
    r.empty = False
    out.append(("not_empty", cube64(), r, "NODES"))
    return out


def case(name):
    """(cube, rings, ringmode) of a named case."""
    for nm, cube, rings, mode in subring_cases():
        if nm == name:
            return cube, rings, mode
    for nm, cube, rings, mode, box, seed in mc_cases():
        if nm == name:
            return cube, rings, mode
    raise KeyError(name)


def galfit_par():
    """The 3DFIT parameters of the CLASSIC fit fixture: the defaults of bbarolo/params.py, FREE "VROT VDISP",
    one stage, no errors."""
    import types
    return types.SimpleNamespace(FREE="VROT VDISP", DELTAVROT=1000.0, MINVDISP=0.1, MAXVDISP=1000.0, DELTAINC=5.0,
                                 DELTAPHI=15.0, TOL=1e-3, FTYPE=2, WFUNC=2, SIDE="B", BWEIGHT=1.0, NORM="AZIM",
                                 NORMALCUBE=True, TWOSTAGE=False, flagERRORS=False, STARTRAD=0, DENSFLUX=True,
                                 CDENS=10, CMODE=1, ISEED=1, LTYPE=1, NV=-1, REDSHIFT=0.0, EMPTY=True,
                                 RESTWAVE=[-1.0], RESTFREQ=[-1.0], RELINT=[1.0], SM=True, RADMAXA=-1.0,
                                 RADMAXR=-1.0)
