"""Generates the golden fixtures of the wind models (``wind.npz``) by running the REFERENCE's own kernels.

Run in a container that has the reference source tree, named by the ``BBAROLO_REF`` environment variable:

    python tests/golden/make_wind.py

``bbarolo/windmodel.py`` is imported with a stub numba (``_refimport.py``), so its kernels run as plain Python:
``WindCells`` (cells and quadrature), ``WindModel._set_psf`` (the beam kernel), ``_wind_points``, ``_raw_boxes``,
``_deposit_raw``, ``_convolve_boxes``, ``_voxel_lists``, ``_normal_lists`` and ``_scatter``; for GALWIND WTYPE 1
``bbarolo/galwind.py``'s ``GalWind._shells`` and ``bbarolo/galmod.py``'s ``_galmod_wind``. The glue of
``WindModel.boxes`` (``bbarolo/windmodel.py:829-859``) is repeated here around them. The cubes, the spectral
constants (``GalmodSetup``) and the cases come from the package and ``tests/wind_cases.py``.
"""

import importlib
import json
import math
import os
import sys
import types
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
warnings.simplefilter("ignore")

import _refimport  # noqa: E402
import wind_cases as WC  # noqa: E402

ns = _refimport.load()
WM = importlib.import_module("bbarolo.windmodel")
from bbarolo2_gb300.galmod import GalmodSetup  # noqa: E402


def run_case(name):
    c = WC.CASES[name]
    cube = WC.cube(**c["cube"])
    su = GalmodSetup(cube, densflux=True)
    cdelt = (su.cdelt[0] * 60., su.cdelt[1] * 60.)
    pixsize = min(abs(cdelt[0]), abs(cdelt[1]))
    # the beam (WindModel.__init__ and _set_psf, run on a stand-in of the model object)
    fake = types.SimpleNamespace(cin=cube, cdelt=cdelt, beam=None, hx=0, hy=0, kern=np.ones((1, 1)),
                                 kx=np.ones(1), ky=np.ones(1), separable=True, sigbeam=None, psfq=np.zeros(5))
    h = cube.Head()
    if c["smooth"] and h.Bmaj() > 0 and h.Bmin() > 0:
        fake.beam = (h.Bmaj() * 3600., h.Bmin() * 3600., h.Bpa())
        WM.WindModel._set_psf(fake)
    # the cells and their quadrature (WindModel.quadrature)
    cells = WC.make_cells(WM, c["cells"])
    vmax, sigmin = c["quad"]
    spacing = pixsize if fake.beam is None else fake.sigbeam
    sig = math.hypot(sigmin, su.sig_instr / 1000.)
    cells.set_quadrature(spacing, vmax, 2. * sig, cap=16, maxpoints=WM.MAX_POINTS)
    # the points (WindModel.points)
    P = WM.WindPars(**c["pars"])
    g = WC.geometry(c["pars"], su.crota2)
    n, m = cells.npoints, cells.ncell
    pts = {k: np.empty(n) for k in ("gx", "gy", "vel", "sig", "w", "r")}
    vol, rbar = np.empty(m), np.empty(m)
    WM._wind_points(cells.cells, cells.qn, cells.qoff, P.radii, P.vwind, P.vdisp, P.vrot, P.xpos, P.ypos, g["vsys"],
                    g["sinc"], g["cinc"], g["spa"], g["cpa"], cdelt[0], cdelt[1], g["th_in"], g["th_out"], g["rmax"],
                    su.sig_instr, pts["gx"], pts["gy"], pts["vel"], pts["sig"], pts["w"], pts["r"], vol, rbar)
    # the columns (WindModel.boxes)
    wt = WC.point_weight(name, pts["r"])
    w = pts["w"] if wt is None else pts["w"] * wt
    nz, ny, nx = cube.DimZ(), cube.DimY(), cube.DimX()
    lim = np.array([0, nx, 0, ny, 0, nz] if c["lim"] is None else c["lim"], dtype=np.int64)
    hx, hy = fake.hx, fake.hy
    rlim = lim + np.array([-hx, hx, -hy, hy, 0, 0])
    spec = (su.axtyp, su.velsys, su.lfreq0, su.crval3, su.cdelt3, su.crpix3)
    rboxes = np.empty((m, 6), dtype=np.int64)
    WM._raw_boxes(cells.qoff, pts["gx"], pts["gy"], pts["vel"], pts["sig"], w, rlim, su._chmin, *spec, rboxes)
    R = WM.Boxes.from_boxes(rboxes)
    WM._deposit_raw(R.buf, R.offs, R.boxes, cells.qoff, pts["gx"], pts["gy"], pts["vel"], pts["sig"], w,
                    su._vedges_lines, su.relint, np.ones(nz), ns.galmod._PHI_TAB, su._chmin, *spec, nz)
    if hx == 0 and hy == 0:
        B = WM.Boxes(R.buf, R.offs, np.ascontiguousarray(np.clip(rboxes, np.repeat(lim[::2], 2),
                                                                 np.repeat(lim[1::2], 2))))
    else:
        boxes = rboxes + np.array([-hx, hx, -hy, hy, 0, 0])
        boxes[:, 0:2] = np.clip(boxes[:, 0:2], lim[0], lim[1])
        boxes[:, 2:4] = np.clip(boxes[:, 2:4], lim[2], lim[3])
        empty = (rboxes[:, 1] <= rboxes[:, 0]) | (boxes[:, 1] <= boxes[:, 0]) | (boxes[:, 3] <= boxes[:, 2])
        boxes[empty] = (lim[0], lim[0], lim[2], lim[2], lim[4], lim[4])
        B = WM.Boxes.from_boxes(boxes)
        WM._convolve_boxes(R.buf, R.offs, R.boxes, fake.kern, fake.kx, fake.ky, fake.separable, B.buf, B.offs,
                           B.boxes)
    # the normal equations and a model
    W, d, Wd = WC.weights(name, (nz, ny, nx))
    lists = B.voxel_lists(W, lim, rel=c["rel"])
    G, b = B.normal(Wd, W, lists)
    amp = np.random.default_rng(5).exponential(1., m)
    model = B.model(amp, (nz, ny, nx))
    out = dict(cells=cells.cells, qn=cells.qn, qoff=cells.qoff, spacing=cells.spacing, kern=fake.kern, kx=fake.kx,
               ky=fake.ky, psfq=fake.psfq, hxhy=np.array([hx, hy]), separable=np.array(fake.separable),
               vedges=su._vedges_lines, relint=su.relint, lfreq0=su.lfreq0, lim=lim, vol=vol, rbar=rbar,
               rboxes=rboxes, roffs=R.offs, rbuf=R.buf, boxes=B.boxes, offs=B.offs, buf=B.buf, G=G, b=b, amp=amp,
               model=model, **{"pts_" + k: v for k, v in pts.items()})
    meta = dict(chmin=su._chmin, sig_instr=su.sig_instr, axtyp=int(su.axtyp), velsys=int(su.velsys),
                crval3=su.crval3, cdelt3=su.cdelt3, crpix3=su.crpix3, cdelt0=cdelt[0], cdelt1=cdelt[1],
                crota2=su.crota2, sigbeam=fake.sigbeam, shape=[nz, ny, nx], rel=c["rel"])
    print(f"  {name}: {m} cells, {n} points, {int(B.offs[-1])} column values, hx={hx} hy={hy} "
          f"separable={fake.separable}")
    return out, meta


def run_galwind(name):
    """GALWIND WTYPE 1: the reference's GalWind._shells (on a stand-in of the GalWind object) and _galmod_wind over
    the chunks of shells (the loop of GalWind._spherical, bbarolo/galwind.py:301-331)."""
    for mod, attrs in (("bbarolo.moments", ("MomentMap",)), ("bbarolo.pvslice", ("PositionVelocity",)),
                       ("bbarolo.plotscripts", ("run_scripts", "F"))):
        if mod not in sys.modules:                       # (plotting modules: not needed by the model)
            m = types.ModuleType(mod)
            for a in attrs:
                setattr(m, a, None)
            sys.modules[mod] = m
    GW = importlib.import_module("bbarolo.galwind")
    from bbarolo2_gb300.galwind import GalWindPars, wind_setup
    c = WC.GW_CASES[name]
    cube = WC.cube(**c["cube"])
    p = c["par"]
    su = wind_setup(cube, GalWindPars(**p))
    fake = types.SimpleNamespace(par=types.SimpleNamespace(**WC.gw_reference_par(p)),
                                 _center=lambda: (p["xpos"], p["ypos"]))
    sr, nv, sep = GW.GalWind._shells(fake, su)
    nz, ny, nx = cube.DimZ(), cube.DimY(), cube.DimX()
    (b0, b1), (e0, e1) = c["box"] if c["box"] is not None else ((0, 0), (nx, ny))
    out = np.zeros((e1 - b1, e0 - b0, nz))
    nsh = sr.shape[1]
    chunks = [ch for ch in np.array_split(np.arange(nsh), max(1, min(c["threads"], nsh))) if len(ch)]
    seed = int(p["iseed"]) & 0xFFFFFFFF
    for t, ch in enumerate(chunks):
        buf = np.zeros_like(out)
        ns.galmod._galmod_wind(buf, sr, int(ch[0]), int(ch[-1]) + 1, (seed + 7919 * t) & 0xFFFFFFFF, sep, nv,
                               su.cdens, 1, su.pixarea, su.cdelt[0], su.cdelt[1], su.crota2, b0, b1, e0, e1,
                               su.sig_instr, su.axtyp, su.velsys, su.lfreq0, su.crval3, su.cdelt3, su.crpix3,
                               su.relint, su.cd2i)
        out += buf
    idx = np.flatnonzero(out)
    arrays = dict(sr=sr, nv=nv, idx=idx, val=out.ravel()[idx], cd2i=su.cd2i, lfreq0=su.lfreq0, relint=su.relint,
                  chunks=np.array([[int(ch[0]), int(ch[-1]) + 1] for ch in chunks]))
    meta = dict(sep=sep, cdens=su.cdens, pixarea=su.pixarea, cdelt0=su.cdelt[0], cdelt1=su.cdelt[1],
                crota2=su.crota2, sig_instr=su.sig_instr, axtyp=int(su.axtyp), velsys=int(su.velsys),
                crval3=su.crval3, cdelt3=su.cdelt3, crpix3=su.crpix3, seed=seed, box=[[b0, b1], [e0, e1]],
                shape=list(out.shape))
    print(f"  {name}: {nsh} shells, {len(chunks)} chunks, {idx.size} voxels with clouds")
    return arrays, meta


def main():
    arrays, index = {}, {}
    for name in WC.CASES:
        out, meta = run_case(name)
        for k, v in out.items():
            arrays[f"{name}/{k}"] = np.asarray(v)
        index[name] = meta
    for name in WC.GW_CASES:
        out, meta = run_galwind(name)
        for k, v in out.items():
            arrays[f"{name}/{k}"] = np.asarray(v)
        index[name] = meta
    arrays["index"] = np.array(json.dumps(index))
    path = os.path.join(HERE, "wind.npz")
    np.savez_compressed(path, **arrays)
    print(f"  wind.npz: {os.path.getsize(path) / 1024:.0f} KB")


if __name__ == "__main__":
    main()
