"""Generates the golden fixtures of the model path by running the REFERENCE's own kernels.

Run in a container that has the reference source tree, named by the ``BBAROLO_REF`` environment variable:

    python tests/golden/make_golden.py

The reference's modules are imported with a stub numba (``_refimport.py``), so its kernels run as plain
Python: ``bbarolo/_rng.py`` (stream), ``bbarolo/galmod.py`` (sub-rings, MC and ANALYTIC models, ring maps,
sparse convolution), ``bbarolo/smooth.py`` (beam kernel, FFT convolution), ``bbarolo/galfit.py`` (CLASSIC
``_norm``) and ``bbarolo/bayesian/likelihood.py`` (residual kernels). The inputs are the synthetic workloads of
``bbarolo2_gb300.configs`` and small variants of them that exercise the code paths (layers, lags, edges, lines,
boxes). Models are stored sparsely (flat index, value) in float64. The fixtures pin the CPU oracle and the GPU
path; nothing reads the reference tree at test time.
"""

import json
import os
import sys
import time
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
warnings.simplefilter("ignore")

import _refimport  # noqa: E402

ns = _refimport.load()
from bbarolo2_gb300 import configs  # noqa: E402
from bbarolo2_gb300.cube import Cube  # noqa: E402

G = ns.galmod


def sparse(a):
    a = np.asarray(a, np.float64)
    idx = np.flatnonzero(a)
    return idx.astype(np.int64), a.ravel()[idx]


def setup_dict(st):
    """The setup scalars a kernel call used (so that the tests replay it without the reference)."""
    return dict(radsep=st.radsep, cdens=st.cdens, cmode=st.cmode, pixarea=st.pixarea, cdelt0=st.cdelt[0],
                cdelt1=st.cdelt[1], crota2=st.crota2, ltype=st.ltype, sig_instr=st.sig_instr, axtyp=st.axtyp,
                velsys=st.velsys, crval3=st.crval3, cdelt3=st.cdelt3, crpix3=st.crpix3, chmin=st._chmin,
                zstep=st.zstep, nz=st.nsubs, dimx=st.dimx, dimy=st.dimy)


def save(name, **arrays):
    path = os.path.join(HERE, name)
    np.savez_compressed(path, **arrays)
    print(f"  {name}: {os.path.getsize(path) / 1024:.0f} KB")


# ---------------------------------------------------------------------------------------------- RNG
def gen_rng():
    R = ns.rng
    out = {}
    seeds = [0, 1, 12345, 0xFFFFFFFF, 7 + 7919 * 3]
    states, words = [], []
    for sd in seeds:
        s = R.rng_init(sd)
        states.append(s.copy())
        words.append([int(R.rng_next(s)) for _ in range(32)])
    out["seeds"] = np.array(seeds, np.uint64)
    out["init_states"] = np.array(states, np.uint64)
    out["words"] = np.array(words, np.uint64)
    s = R.rng_init(12345)
    nrm, uni = np.empty(4000), np.empty(4000)
    for i in range(4000):
        nrm[i] = R.rng_normal(s)
        uni[i] = R.rng_uniform(s)
    out["normals"], out["uniforms"], out["final_state"] = nrm, uni, s.copy()
    out["KN"], out["WN"], out["FN"] = R.KN, R.WN, R.FN
    out["PHI_TAB"] = G._PHI_TAB
    save("rng.npz", **out)


# ---------------------------------------------------------------------------------------------- cases
from cases import cube64, galfit_par, rings64, mc_cases, subring_cases  # noqa: E402


def run_model(galmodtype, case):
    name, cube, rings, mode, box, seed = case
    st = G.GalmodSetup(cube, densflux=True)
    dm = G.DiskModel(cube, ringmode=mode, galmodtype=galmodtype)
    st = dm.setup
    mr = G.model_rings(rings, mode, st.radsep)
    sr, nv = st.subrings(mr)
    blo, bhi = box if box is not None else ((0, 0), (cube.DimX(), cube.DimY()))
    t = time.time()
    mod = st.build(mr, blo, bhi, seed=seed, galmodtype=galmodtype, layout="yxz")
    dt = time.time() - t
    meta = setup_dict(st)
    meta.update(name=name, seed=int(seed), seed32=int(seed) & 0xFFFFFFFF, blo=list(blo), bhi=list(bhi),
                ringmode=mode, shape=list(mod.shape))
    return dict(sr=sr, nv=nv, lfreq0=st.lfreq0, relint=st.relint, cd2i=st.cd2i, vedges=st._vedges_lines,
                model=mod, meta=meta, dt=dt, dm=dm, rings=rings, mr=mr)


def gen_models():
    for gtype, cases in (("MC", mc_cases()), ("ANALYTIC", [c for c in mc_cases()
                                                            if c[0] not in ("classic64_seedm1",)])):
        arrays = {}
        index = []
        for case in cases:
            r = run_model(gtype, case)
            nm = case[0]
            idx, val = sparse(r["model"])
            arrays[nm + "/sr"] = r["sr"]
            arrays[nm + "/nv"] = r["nv"]
            arrays[nm + "/lfreq0"] = r["lfreq0"]
            arrays[nm + "/relint"] = r["relint"]
            arrays[nm + "/cd2i"] = r["cd2i"]
            arrays[nm + "/vedges"] = r["vedges"]
            arrays[nm + "/idx"] = idx
            arrays[nm + "/val"] = val
            index.append(r["meta"])
            print(f"  {gtype} {nm}: nsub={r['sr'].shape[1]} nonzero={idx.size} ({r['dt']:.1f} s)")
        arrays["index"] = np.array(json.dumps(index))
        save("mc.npz" if gtype == "MC" else "analytic.npz", **arrays)


# ---------------------------------------------------------------------------------------------- subrings
def gen_subrings():
    arrays, index = {}, []
    for nm, cube, rings, mode in subring_cases():
        st = G.GalmodSetup(cube, densflux=True)
        mr = G.model_rings(rings, mode, st.radsep)
        sr, nv = st.subrings(mr)
        arrays[nm + "/sr"], arrays[nm + "/nv"] = sr, nv
        arrays[nm + "/model_radii"] = np.asarray(mr.radii, float)
        index.append(dict(name=nm, ringmode=mode))
    arrays["index"] = np.array(json.dumps(index))
    save("subrings.npz", **arrays)


# ---------------------------------------------------------------------------------------------- beam + conv
def gen_beam_conv():
    arrays = {}
    for wl in ("classic64", "global160", "bayes256"):
        cube, _ = configs.WORKLOADS[wl]()
        dm = G.DiskModel(cube)
        arrays[wl + "/kernel"] = dm.cfield
        arrays[wl + "/scalefactor"] = np.array(dm.scalefactor)
        sm = ns.smooth.Smooth3D()
        h = cube.Head()
        sm.setfromCube(cube, (0, 0, 0), (h.Bmaj() * 3600., h.Bmin() * 3600., h.Bpa()))
        arrays[wl + "/scalefac_coldens"] = np.array(sm.Scalefac())
    # a beam with BMAJ < BMIN and CROTA: the axes swap
    cube = Cube.empty(64, 64, 64, [-10. / 3600., 10. / 3600., 5.], beam=[20. / 3600., 40. / 3600., 10.],
                      crota=15., cunit=("deg", "deg", "km/s"))
    dm = G.DiskModel(cube)
    arrays["swapped/kernel"] = dm.cfield
    # the FFT convolution of the classic64 MC model (DiskModel.array with smoothing: threshold, scale 1)
    cube, rings = configs.classic64()
    dm = G.DiskModel(cube)
    sm = dm.array(rings, seed=1)
    unsm = G.DiskModel(cube, smooth=False).array(rings, seed=1)
    arrays["classic64/unsmoothed_idx"], arrays["classic64/unsmoothed_val"] = sparse(unsm)
    arrays["classic64/smoothed_idx"], arrays["classic64/smoothed_val"] = sparse(sm)
    # column densities: scale factor
    dmc = G.DiskModel(cube, densflux=False)
    smc = dmc.convolve(unsm.transpose(1, 2, 0).copy())
    arrays["classic64/coldens_smoothed_idx"], arrays["classic64/coldens_smoothed_val"] = sparse(smc)
    arrays["classic64/coldens_scalefactor"] = np.array(dmc.scalefactor)
    save("beam_conv.npz", **arrays)


# ---------------------------------------------------------------------------------------------- residuals
def gen_residuals():
    g = np.random.default_rng(3)
    nz, ny, nx = 12, 10, 9
    model = np.abs(g.normal(0, 1, (nz, ny, nx)))
    model[g.random(model.shape) < 0.3] = 0.
    data = (model + g.normal(0, 0.3, model.shape)).astype(np.float32)
    data[g.random(data.shape) < 0.05] = np.nan
    data[g.random(data.shape) < 0.05] = 0.
    mask = g.random(data.shape) < 0.6
    region = g.random((ny, nx)) < 0.8
    arrays = dict(model=model, data=data, mask=mask, region=region)
    L = ns.likelihood
    out = []
    for mm in (0, 1, 2):
        for reg in (np.zeros((0, 0), bool), region):
            ss = L._sumsq_residuals(model, data, mask, mm, reg)
            fr = L._residuals_fracerr(model, data, mask, mm, reg, 0.09, 0.04)
            out.append([mm, reg.size > 0, ss, fr[0], fr[1]])
    arrays["results"] = np.array(out, float)
    save("residuals.npz", **arrays)


# ---------------------------------------------------------------------------------------------- CLASSIC
def gen_classic():
    """_conv_sparse and _norm on single-ring models (as Galfit.getFuncValue)."""
    gf = ns.galfit
    cube, rings = configs.classic64()
    dm = G.DiskModel(cube)
    st = dm.setup
    arrays, index = {}, []
    one = rings.subset(np.array([2, 3]))
    one.radsep = 20.
    blo, bhi = dm.box(one)
    mod = st.build(one, blo, bhi, seed=1, galmodtype="MC", layout="yxz")
    cs = G._conv_sparse(mod, dm.cfield, 1.0)
    arrays["conv_sparse/model"] = mod
    arrays["conv_sparse/out"] = cs
    arrays["conv_sparse/kernel"] = dm.cfield
    cs2 = G._conv_sparse(mod, dm.cfield, 2.5)
    arrays["conv_sparse/out_scaled"] = cs2
    # _norm: data = classic64 smoothed model with noise, mask above a threshold
    full = dm.array(rings, seed=1)
    g = np.random.default_rng(1)
    data = (full + g.normal(0, 0.01 * full.max(), full.shape)).astype(np.float32)
    # (the residual reads the data in the box only: the fixture keeps that crop, passed with blo = 0)
    data_T = np.ascontiguousarray(data.transpose(1, 2, 0)[blo[1]:bhi[1], blo[0]:bhi[0]])
    mask_T = np.ascontiguousarray((full > 0.05 * full.max()).transpose(1, 2, 0)[blo[1]:bhi[1], blo[0]:bhi[0]])
    arrays["norm/data_T"], arrays["norm/mask_T"] = data_T, mask_T
    arrays["norm/model"] = cs
    chan_noise = np.full(64, 0.01 * full.max())
    arrays["norm/chan_noise"] = chan_noise
    ky, kx = dm.cfield.shape
    ilo = np.full(ky, -(kx // 2), np.int64)
    ihi = np.full(ky, kx // 2, np.int64)
    arrays["norm/ilo"], arrays["norm/ihi"] = ilo, ihi
    x0, y0 = 32. - blo[0], 32. - blo[1]
    r1, r2 = 3.5, 8.0                  # (pixels: the annulus of the rings in the 17 x 17 box)
    # The kernel runs here as Python: a float32 scalar added to a Python float accumulator stays float32 under
    # NumPy 2's promotion rules, where numba accumulates in float64. The data are therefore passed as float64
    # (exact conversions): the numba kernel's arithmetic on the float32 data.
    data64 = data_T.astype(np.float64)
    res = []
    for normtype in (0, 1, 2):
        for ftype in (1, 2, 3, 4):
            for wpow, side, foot in ((2., 0, 0), (1., 1, 0), (-1., 2, 0), (0., 0, 1)):
                m = cs.copy()
                v = gf._norm(m, data64, mask_T, 0, 0, x0, y0, 45., 55., r1, r2, wpow, side, ftype,
                             chan_noise, 0.001, 1.0, normtype, np.zeros((0, 0, 0)), np.zeros(0, np.int64),
                             np.zeros(0, np.int64), np.zeros(0), np.zeros((0, 0, 0)), foot, 4.0)
                res.append([normtype, ftype, wpow, side, foot, 0, v, float(np.sum(m))])
    # with the MC support emulation (pre, thr)
    thr = np.full(64, 0.3 * float(np.max(mod)))
    for normtype in (0, 1):
        m = cs.copy()
        P = np.zeros((ky, mod.shape[1] + 1, 64))
        v = gf._norm(m, data64, mask_T, 0, 0, x0, y0, 45., 55., r1, r2, 2., 0, 2, chan_noise, 0.001,
                     1.0, normtype, mod, ilo, ihi, thr, P, 0, 4.0)
        res.append([normtype, 2, 2., 0, 0, 1, v, float(np.sum(m))])
    arrays["norm/thr"] = thr
    arrays["norm/results"] = np.array(res, float)
    arrays["norm/meta"] = np.array(json.dumps(dict(blo=list(blo), bhi=list(bhi), x0=x0, y0=y0, r1=r1, r2=r2)))
    save("classic.npz", **arrays)


# ---------------------------------------------------------------------------------------------- ring maps
def gen_ringmaps():
    arrays, index = {}, []
    cube = cube64(ltype=2)
    for mode, z0 in (("CENTRED", 10.), ("NODES", 0.), ("SHIFTED", 20.)):
        dm = G.DiskModel(cube, ringmode=mode, galmodtype="ANALYTIC")
        r = rings64(z0=z0, dens=np.linspace(3., 0.5, 8), inc=np.linspace(50., 70., 8))
        blo, bhi = (5, 8), (60, 58)
        K = dm.ring_maps(r, blo, bhi)
        st = dm.setup
        mr = G.model_rings(r, mode, st.radsep)
        mr = mr.copy() if mr is r else mr
        mr.dens = np.ones(mr.nr)
        sr, _ = st.subrings(mr)
        widx, wval = dm._ring_weights(r, mode)
        raw = np.zeros((r.nr, bhi[1] - blo[1], bhi[0] - blo[0]))
        G._ring_maps_analytic(raw, sr, widx, wval, st.radsep, st.pixarea, st.cdelt[0], st.cdelt[1], st.crota2,
                              blo[0], blo[1], bhi[0], bhi[1], st.ltype, 1 if not np.any(sr[6] > 0) else 1024,
                              st.sig_instr, st._chmin, st.zstep)
        arrays[mode + "/sr"], arrays[mode + "/widx"], arrays[mode + "/wval"] = sr, widx, wval
        arrays[mode + "/raw"], arrays[mode + "/maps"] = raw, K
        meta = setup_dict(st)
        meta.update(mode=mode, blo=list(blo), bhi=list(bhi), mean_cd2i=float(np.mean(st.cd2i)),
                    sum_relint=float(np.sum(st.relint)), nzq=1 if not np.any(sr[6] > 0) else 1024)
        index.append(meta)
        # the deconvolved profile of the maps: A, b from the map of a model with noise
        if mode == "CENTRED" and ns.profile is not None:
            mom0 = dm.array(r, blo, bhi).sum(axis=0)
            g = np.random.default_rng(2)
            rms = np.full(mom0.shape, 0.01 * mom0.max())
            y = mom0 + g.normal(0, 1, mom0.shape) * rms
            ok = mom0 > 0.001 * mom0.max()
            A = K[:, ok].T / rms[ok, None]
            b = y[ok] / rms[ok]
            Rc = np.asarray(r.radii, float)
            arrays["profile/A"], arrays["profile/b"], arrays["profile/radii"] = A, b, Rc
            arrays["profile/x_smooth"] = ns.profile.solve_profile(A, b, Rc, 0.3, 4.0)
            arrays["profile/x_nosmooth"] = ns.profile.solve_profile(A, b, Rc, 0.0)
    arrays["index"] = np.array(json.dumps(index))
    save("ringmaps.npz", **arrays)


# ---------------------------------------------------------------------------------------------- PROFILE
def gen_profile():
    """profile_system + solve_profile (bbarolo/profile.py:33-138) on two geometries: the maps of the rings and of
    the exterior annulus, the system (A, b, ok, Rc) and the densities with and without the smoothness prior."""
    P = ns.profile
    arrays, index = {}, []
    cases = [("flat", cube64(ltype=2), rings64(z0=10., dens=np.linspace(3., 0.5, 8), inc=np.linspace(50., 70., 8)),
              "CENTRED", ((5, 8), (60, 58))),
             ("warp", cube64(ltype=1, crota=15.), rings64(z0=0., inc=np.linspace(40., 65., 8),
                                                           phi=np.linspace(30., 55., 8)), "NODES", ((0, 0), (64, 64)))]
    for name, cube, r, mode, (blo, bhi) in cases:
        dm = G.DiskModel(cube, ringmode=mode, galmodtype="ANALYTIC")
        mom0 = dm.array(r, blo, bhi).sum(axis=0)
        g = np.random.default_rng(3)
        rms = np.full(mom0.shape, 0.01 * mom0.max())
        y = mom0 + g.normal(0, 1, mom0.shape) * rms
        ok = mom0 > 0.002 * mom0.max()
        h = cube.Head()
        beam = abs(h.Bmaj()) * 3600.
        A, b, okk, Rc = P.profile_system(dm, r, (blo, bhi), y, rms, ok, beam_arcsec=beam)
        # the maps of the rings and of the exterior annulus (as profile_system builds them)
        K = dm.ring_maps(r, blo, bhi)
        edge = G.outer_edge(r, dm.ringmode)
        rext = edge + beam
        ext = ns.rings.Rings().setRings(radii=[rext], xpos=r.xpos[-1], ypos=r.ypos[-1], vsys=r.vsys[-1],
                                        vrot=r.vrot[-1], vdisp=r.vdisp[-1], z0=r.z0[-1], inc=r.inc[-1],
                                        phi=r.phi[-1], dens=1., radsep=2. * beam, z0thick=r.z0thick[-1],
                                        fthick=r.fthick[-1], vdispthick=r.vdispthick[-1])
        ext.twolayer = r.thick()
        ext.edgeapp = ext.edgerec = -1.
        K = np.concatenate([K, dm.ring_maps(ext, blo, bhi, ringmode="CENTRED")])
        # (A and b are exactly maps[:, okk].T / rms[okk] and y[okk] / rms[okk]: not stored)
        assert np.array_equal(K[:, okk].T / rms[okk, None], A) and np.array_equal(y[okk] / rms[okk], b)
        assert Rc[-1] == rext
        arrays[name + "/y"], arrays[name + "/rms"], arrays[name + "/ok"] = y, rms, ok
        arrays[name + "/okk"], arrays[name + "/Rc"], arrays[name + "/maps"] = okk, Rc, K
        for smooth, corr in ((0.3, 1.0), (0.3, 4.0), (0.0, 1.0), (1.0, 2.0)):
            arrays[name + f"/x_{smooth}_{corr}"] = P.solve_profile(A, b, Rc, smooth, corr)
        index.append(dict(name=name, mode=mode, blo=list(blo), bhi=list(bhi), beam_arcsec=beam,
                          rings={k: np.asarray(getattr(r, k), float).tolist()
                                 for k in ("radii", "xpos", "ypos", "vsys", "vrot", "vdisp", "dens", "z0", "inc",
                                           "phi")}))
    arrays["index"] = np.array(json.dumps(index))
    save("profile.npz", **arrays)


# ---------------------------------------------------------------------------------------------- CLASSIC fit
GALFIT_RINGS = (1, 2, 3)
GALFIT_CROP = (12, 52)          # (the fits of these rings read the data in [12, 52)^2 only)


def gen_galfit():
    """The CLASSIC fit of single rings (bbarolo/galfit.py:736-1160: _fit_ring, minimize, _mtry, func3D,
    getFuncValue, _norm_value; first stage, one thread, no REVERSE passes) on the 64^3 mock: the reference's
    Galfit set up as Galfit.setup does, with the cube statistics given (the noise of the mock) and the VROT
    band check left out (the cube of the fixture has no spectral-axis conversion). Recorded: each ring's fit
    (converged, minimum, VROT, VDISP) and the sequence of its function values."""
    import threading
    gf = ns.galfit
    cube, rings = configs.classic64()
    dm = G.DiskModel(cube)
    full = dm.array(rings, seed=1)
    g = np.random.default_rng(1)
    sigma = 0.01 * float(full.max())
    data = (full + g.normal(0, sigma, full.shape)).astype(np.float32)
    mask = full > 0.02 * full.max()
    par = galfit_par()
    inr = rings.copy()
    inr.vrot = np.full(inr.nr, 120.)
    inr.vdisp = np.full(inr.nr, 8.)
    F = gf.Galfit()
    F.cin, F.par, F.inr, F.verb = cube, par, inr.copy(), 0
    F.arcconv = G.arcsconv(cube.Head().Cunit(0))
    F.chan_noise = np.ones(cube.DimZ())
    F.data_noise = sigma
    F.wpow = par.WFUNC
    F.setFree()
    F.mask = mask
    F.mask_T = np.ascontiguousarray(mask.transpose(1, 2, 0))
    F.mask2D = mask.sum(axis=0).astype(np.int32)
    F.norms = ["AZIM", "AZIM", "AZIM"]
    P = gf
    F.maxs, F.mins = np.zeros(P.MAXPAR), np.zeros(P.MAXPAR)
    F.maxs[P.VROT] = inr.vrot.max() + par.DELTAVROT
    F.mins[P.VROT] = max(inr.vrot.min() - par.DELTAVROT, 0)
    F.maxs[P.VDISP], F.mins[P.VDISP] = par.MAXVDISP, par.MINVDISP
    F.model = G.DiskModel(cube, par=par, densflux=True)
    h = cube.Head()
    F.pixScale = ((abs(h.Cdelt(0)) * F.arcconv) + (abs(h.Cdelt(1)) * F.arcconv)) / 2.
    F._rngs, F._tls, F._ringstat = {}, threading.local(), {}
    F._check_vrot = lambda ir: True
    # galfit(): stage 1 with the data normalised (NORMALCUBE)
    F.n_galfit = 1
    F.outr = F.inr.copy()
    scaling = 10. / float(data.max())
    # (float64 copies of the float32 data: the arithmetic of the numba kernels, see gen_classic)
    F.data_T = np.ascontiguousarray((data * scaling).astype(np.float32).transpose(1, 2, 0)).astype(np.float64)
    F.data_noise = sigma * scaling
    nr = inr.nr
    errors = np.zeros((nr, 2, F.nfree))
    fitok = [False] * nr
    F._cstat = np.full(nr, F.CS_NONE)
    F._pass = 0
    calls = []
    f3 = F.func3D

    def counted(dring, zpar, ctx=None):
        v = f3(dring, zpar, ctx)
        calls[-1].append((float(zpar[0]), float(zpar[1]), float(v)))
        return v
    F.func3D = counted
    res = []
    for ir in GALFIT_RINGS:
        calls.append([])
        t0 = time.time()
        F._fit_ring(ir, errors, fitok, 1)
        st = F._ringstat.get(ir, ("", None))
        res.append([ir, 1.0 if fitok[ir] else 0.0, st[1] if st[1] is not None else np.nan, F.outr.vrot[ir],
                    F.outr.vdisp[ir], len(calls[-1])])
        print(f"  ring {ir}: {res[-1]} ({time.time() - t0:.0f} s)")
    a, b = GALFIT_CROP
    arrays = dict(data=np.ascontiguousarray(data[:, a:b, a:b]), mask=np.ascontiguousarray(mask[:, a:b, a:b]),
                  results=np.array(res, float), scaling=np.array(scaling), sigma=np.array(sigma))
    for k, c in zip(GALFIT_RINGS, calls):
        arrays[f"calls_{k}"] = np.array(c, float)
    arrays["index"] = np.array(json.dumps(dict(crop=list(GALFIT_CROP), rings=list(GALFIT_RINGS),
                                               par=vars(par), vrot0=120., vdisp0=8.)))
    save("galfit.npz", **arrays)


if __name__ == "__main__":
    which = sys.argv[1:] or ["rng", "subrings", "beam_conv", "residuals", "classic", "ringmaps", "models", "profile", "galfit"]
    for w in which:
        print(w)
        {"rng": gen_rng, "subrings": gen_subrings, "beam_conv": gen_beam_conv, "residuals": gen_residuals,
         "classic": gen_classic, "ringmaps": gen_ringmaps, "models": gen_models, "profile": gen_profile, "galfit": gen_galfit}[w]()
