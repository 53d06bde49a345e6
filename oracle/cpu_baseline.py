"""The reference's CPU likelihood evaluation, timed on the host cores (the CPU baseline of the benchmark), and the
float64 pipeline the GPU evaluations are checked against.

TEST INFRASTRUCTURE: used only by the CPU-baseline leg of ``bench.py`` (and its ``--impl reference`` arm).

numba is not available where the benchmark runs, so the reference's numba kernels are timed through their C
restatement (``oracle/bbref.c``, bit-exact with the reference): the MC model (``_galmod_mc``) and the residual
(``_sumsq_residuals``). The beam convolution is the reference's own algorithm with the same library:
``FFTConvolver.__call__`` (``bbarolo/smooth.py:145-165``) restated here with scipy.fft (real FFTs padded to
``next_fast_len(n + k // 2)``, empty planes skipped), followed by the threshold of ``DiskModel.convolve``.
With a profile in the payload, each evaluation first recomputes the deconvolved density profile as
``Bayesian3DFIT._log_likelihood`` does when DENS is not fitted and the geometry is free
(``bbarolo/bayesian/likelihood.py:595-596``): the ring maps (``_ring_maps_analytic`` through its C restatement,
times mean(cd2i) sum(relint), FFT convolution, times the scale factor), the weighted least squares and
``solve_profile`` (``oracle/profile.py``), the model's sub-rings with the new densities (the reference's
``subrings`` restated in ``oracle/host.py``), then the MC model (or, with ``galmodtype`` ANALYTIC in the payload,
the ANALYTIC model ``_galmod_analytic`` through its C restatement). ``reference_payload`` builds a whole batch with
the oracle alone (the reference arm of ``bench.py``, which loads no product library).
One evaluation per process, as the reference's fork pool (``bbarolo/bayesian/sampling.py:184-193``), with the
FFT on one worker thread; throughput = evaluations / wall time over all processes.
"""

import multiprocessing as mp
import os
import time

import numpy as np

_W = {}


def fft_convolve(data, kernel):
    """"Same" convolution of the planes (nz, ny, nx) by the FFT, as FFTConvolver (empty planes skipped)."""
    import scipy.fft as sfft
    nz = data.shape[0]
    full = data.reshape(nz, -1).any(axis=1)
    out = np.zeros(data.shape, np.float64)
    if not full.any():
        return out
    d = data[full]
    ny, nx = d.shape[-2:]
    ky, kx = kernel.shape
    Ny = sfft.next_fast_len(ny + ky // 2, real=True)
    Nx = sfft.next_fast_len(nx + kx // 2, real=True)
    kf = _W.get(("kf", Ny, Nx))
    if kf is None:
        kf = sfft.rfft2(kernel, s=(Ny, Nx))
        _W[("kf", Ny, Nx)] = kf
    f = sfft.rfft2(d, s=(Ny, Nx), workers=1)
    f *= kf
    r = sfft.irfft2(f, s=(Ny, Nx), workers=1)
    out[full] = r[..., ky // 2:ky // 2 + ny, kx // 2:kx // 2 + nx]
    return out


def _init(payload):
    _W.update(payload)
    from oracle import oracle
    oracle.lib()


def profile_dens(k, P=None):
    """The ring densities (and the exterior annulus) of member k from its ring maps (see the module docstring)."""
    from oracle import oracle as O
    from oracle import profile as OP
    P = P or _W
    pr = P["prof"]
    st = P["setup"]
    (Lb, Hb) = pr["box"]
    ms = pr["maps_sr"][k]
    raw = np.zeros((pr["nr"] + 1, Hb[1] - Lb[1], Hb[0] - Lb[0]))
    O.ring_maps_analytic(raw, ms, pr["widx"], pr["wval"], st["radsep"], st["pixarea"], st["cdelt0"], st["cdelt1"],
                         st["crota2"], Lb[0], Lb[1], Hb[0], Hb[1], st["ltype"], pr["nzq"], st["sig_instr"],
                         st["chwidth"], st["zstep"])
    raw *= pr["mcd_relint"]
    K = fft_convolve(raw, P["kernel"]) * pr["scalefactor"] if P["kernel"] is not None else raw
    ok, s, y = pr["ok"], pr["rms"], pr["y"]
    A = K[:, ok].T / s[ok, None]
    b = y[ok] / s[ok]
    return OP.solve_profile(A, b, pr["Rc"], pr["smooth"], pr["corr"], pr["floor"])


def model_table(k, x, P=None):
    """The MC sub-ring table of member k with the ring densities x (nr): the reference's ``subrings`` of its
    CENTRED model rings (``oracle/host.py``)."""
    from oracle import host
    P = P or _W
    pr = P["prof"]
    row = pr["rows"][k].copy()
    row[pr["dens_row"]] = x[:pr["nr"]]
    st = pr["hsetup"]
    return host.subrings(st, host.model_rings(host.rings_of_row(pr["proto"], row), pr["mode"], st.radsep))


def evaluate(k):
    """log-likelihood sum of squares of member k of the batch in the worker's payload."""
    from oracle import oracle as O
    P = _W
    st = P["setup"]
    blo, bhi = P["boxes"][k]
    sr, nv = P["sr"][k], P["nv"][k]
    if P.get("prof") is not None:
        sr, nv = model_table(k, profile_dens(k))
    m = np.zeros((bhi[1] - blo[1], bhi[0] - blo[0], st["nz"]))
    if P.get("galmodtype", "MC") == "ANALYTIC":
        nzq = 1 if not np.any(sr[6] > 0) else 1024      # (bbarolo/galmod.py:912)
        O.galmod_analytic(m, sr, 0, sr.shape[1], st["radsep"], st["cdens"], st["pixarea"], st["cdelt0"],
                          st["cdelt1"], st["crota2"], blo[0], blo[1], bhi[0], bhi[1], st["ltype"], st["sig_instr"],
                          P["vedges"], P["relint"], P["cd2i"], nzq, st["axtyp"], st["velsys"], P["lfreq0"],
                          st["crval3"], st["cdelt3"], st["crpix3"], st["chwidth"], None, st["zstep"])
    else:
        O.galmod_mc(m, sr, 0, sr.shape[1], P["seed"], st["radsep"], nv, st["cdens"], st["cmode"],
                    st["pixarea"], st["cdelt0"], st["cdelt1"], st["crota2"], blo[0], blo[1], bhi[0], bhi[1],
                    st["ltype"], st["sig_instr"], st["axtyp"], st["velsys"], P["lfreq0"], st["crval3"], st["cdelt3"],
                    st["crpix3"], P["relint"], P["cd2i"])
    sm = fft_convolve(np.ascontiguousarray(m.transpose(2, 0, 1)), P["kernel"])
    sm[sm < 1e-12] = 0.
    sl = (slice(None), slice(blo[1], bhi[1]), slice(blo[0], bhi[0]))
    return O.sumsq_residuals(sm, P["data"][sl], P["mask"][sl], P["maskmode"], None)


def setup_payload(dm, sr, nv, boxes, seed, data, mask, maskmode, like=None, rows=None, proto=None,
                  galmodtype="MC"):
    """The worker payload of a batch; like: a BatchLikelihood with a profile (set_profile) to recompute it."""
    st = dm.setup
    P = dict(setup=dict(nz=st.nsubs, radsep=st.radsep, cdens=st.cdens, cmode=st.cmode, pixarea=st.pixarea,
                        cdelt0=st.cdelt[0], cdelt1=st.cdelt[1], crota2=st.crota2, ltype=st.ltype,
                        sig_instr=st.sig_instr, axtyp=st.axtyp, velsys=st.velsys, crval3=st.crval3,
                        cdelt3=st.cdelt3, crpix3=st.crpix3, chwidth=st._chmin, zstep=st.zstep),
             sr=sr, nv=nv, boxes=boxes, seed=seed, lfreq0=st.lfreq0, relint=st.relint, cd2i=st.cd2i,
             kernel=dm.cfield, data=data, mask=mask, maskmode=maskmode, prof=None, galmodtype=galmodtype.upper(),
             vedges=st._vedges_lines)
    if like is not None and like._prof is not None:
        from bbarolo2_gb300.rings import RING_KEYS
        pr = like._prof
        ms = like._maps_sr
        P["prof"] = dict(maps_sr=ms, widx=pr["widx"], wval=pr["wval"], box=like.likebox, y=pr["y"], rms=pr["rms"],
                         ok=pr["ok"], Rc=pr["Rc"], smooth=pr["smooth"], corr=pr["corr"], floor=pr["floor"],
                         nr=pr["nr"], nzq=1 if not np.any(ms[:, 6] > 0) else 1024,
                         mcd_relint=float(np.mean(st.cd2i)) * float(np.sum(st.relint)),
                         scalefactor=dm.scalefactor, rows=np.asarray(rows, float), proto=proto, mode=dm.ringmode,
                         dens_row=RING_KEYS.index("dens"), hsetup=_host_setup(dm.cin))
    return P


def _host_setup(cube):
    from oracle import host
    return host.Setup(cube)


# ---------------------------------------------------------------------------------------- the reference arm
RING_KEYS = ("radii", "xpos", "ypos", "vsys", "vrot", "vdisp", "vrad", "vvert", "dvdz", "zcyl", "dens", "z0", "inc",
             "phi", "z0thick", "fthick", "vdispthick")


def ring_rows(rings):
    return np.vstack([np.asarray(getattr(rings, k), float) for k in RING_KEYS])


def reference_payload(cube, rings, rows, seed=1, noise=0.005, galmodtype="MC"):
    """The worker payload of a batch of the 160x160x128 workload built by the oracle alone (the reference's host
    set-up restated in ``oracle/host.py``, the mock from the oracle's MC model and the FFT convolution): what the
    CPU reference arm evaluates, without the device library. rows (B, 17, nr) in RING_KEYS order."""
    import math
    from scipy import ndimage
    from oracle import host
    from oracle import oracle as O
    O.lib()
    st = host.Setup(cube)
    kern = host.beam_kernel(cube)
    h = cube.Head()
    nx, ny, nz = cube.DimX(), cube.DimY(), cube.DimZ()
    mr = host.model_rings(rings, "CENTRED", st.radsep)
    sr0, nv0 = host.subrings(st, mr)
    m = np.zeros((ny, nx, nz))
    O.galmod_mc(m, sr0, 0, sr0.shape[1], seed, st.radsep, nv0, st.cdens, st.cmode, st.pixarea, st.cdelt[0],
                st.cdelt[1], st.crota2, 0, 0, nx, ny, st.ltype, st.sig_instr, st.axtyp, st.velsys, st.lfreq0,
                st.crval3, st.cdelt3, st.crpix3, st.relint, st.cd2i)
    truth = fft_convolve(np.ascontiguousarray(m.transpose(2, 0, 1)), kern)
    truth[truth < 1e-12] = 0.
    rms = noise * float(truth.max())
    g = np.random.default_rng(1)
    nse = fft_convolve(g.normal(0., rms, truth.shape), kern)
    nse *= rms / np.std(nse)
    data = (truth + nse).astype(np.float32)
    rad = abs(h.Bmaj() / h.Cdelt(1))
    yy, xx = np.mgrid[-int(rad) - 1:int(rad) + 2, -int(rad) - 1:int(rad) + 2]
    disk = (xx * xx + yy * yy) <= rad * rad
    mask = ndimage.binary_dilation(truth > 3 * rms, structure=disk[None])
    mask = ndimage.binary_dilation(mask, structure=np.ones((7, 1, 1), bool))
    # the likelihood's total-intensity maps (bbarolo/bayesian/likelihood.py:180-221, density.py:80-83)
    v = mask & np.isfinite(data) & (data != 0)
    y = np.where(v, data, 0.).astype(np.float64).sum(axis=0)
    cnt = v.sum(axis=0)
    srms = rms * np.sqrt(cnt.astype(np.float64))
    ok = cnt > 0
    bmaj, bmin = abs(h.Bmaj()), abs(h.Bmin())
    corr = math.pi * bmaj * bmin / (4. * math.log(2.)) / abs(h.Cdelt(0) * h.Cdelt(1))
    members = []
    for row in np.asarray(rows, float):
        rk = host.rings_of_row(rings, row)
        mk = host.model_rings(rk, "CENTRED", st.radsep)
        srk, nvk = host.subrings(st, mk)
        ext = host.exterior_ring(st, rk, bmaj * 3600.)
        sre, _ = host.subrings(st, host.model_rings(ext, "CENTRED", st.radsep))
        members.append((srk, nvk, host.box(cube, rk, final=True), np.concatenate([srk, sre], axis=1)))
    wm = host.ring_weights(st, rings, "CENTRED")
    we = host.ring_weights(st, host.exterior_ring(st, rings, bmaj * 3600.), "CENTRED")
    widx = np.ascontiguousarray(np.concatenate([wm[0], np.where(we[0] >= 0, we[0] + rings.nr, -1)]), np.int64)
    wval = np.ascontiguousarray(np.concatenate([wm[1], we[1]]))
    ext0 = host.exterior_ring(st, rings, bmaj * 3600.)
    ms = np.stack([mm[3] for mm in members])
    P = dict(setup=dict(nz=nz, radsep=st.radsep, cdens=st.cdens, cmode=st.cmode, pixarea=st.pixarea,
                        cdelt0=st.cdelt[0], cdelt1=st.cdelt[1], crota2=st.crota2, ltype=st.ltype,
                        sig_instr=st.sig_instr, axtyp=st.axtyp, velsys=st.velsys, crval3=st.crval3,
                        cdelt3=st.cdelt3, crpix3=st.crpix3, chwidth=st.chmin, zstep=host.zstep(cube, st)),
             sr=[mm[0] for mm in members], nv=[mm[1] for mm in members], boxes=[mm[2] for mm in members],
             seed=seed, lfreq0=st.lfreq0, relint=st.relint, cd2i=st.cd2i, kernel=kern, data=data, mask=mask,
             maskmode=2, galmodtype=galmodtype.upper(), vedges=np.ascontiguousarray(st.vedges[None]),
             prof=dict(maps_sr=ms, widx=widx, wval=wval, box=([0, 0], [nx, ny]), y=y, rms=srms, ok=ok,
                       Rc=np.r_[np.asarray(rings.radii, float), float(ext0.radii[0])], smooth=0.3, corr=corr,
                       floor=0.05, nr=rings.nr, nzq=1 if not np.any(ms[:, 6] > 0) else 1024,
                       mcd_relint=float(np.mean(st.cd2i)) * float(np.sum(st.relint)), scalefactor=1.0,
                       rows=np.asarray(rows, float), proto=rings, mode="CENTRED",
                       dens_row=RING_KEYS.index("dens"), hsetup=st))
    return P


class Pool:
    """A spawn pool of `cores` processes holding the payload (started before any GPU work of the caller)."""

    def __init__(self, payload, cores=None):
        self.cores = int(cores or os.cpu_count() or 1)
        ctx = mp.get_context("spawn")
        # one BLAS / OpenMP thread per process, as the reference's pool (the workers inherit the environment
        # before they import numpy)
        keys = ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS", "BLIS_NUM_THREADS")
        old = {k: os.environ.get(k) for k in keys}
        for k in keys:
            os.environ[k] = "1"
        try:
            self.pool = ctx.Pool(self.cores, initializer=_init, initargs=(payload,))
            self.pool.map(_noop, range(self.cores))
        finally:
            for k, v in old.items():
                if v is None:
                    os.environ.pop(k, None)
                else:
                    os.environ[k] = v

    def run(self, members):
        """Evaluates the members (indices); returns (sums of squares, wall seconds)."""
        t0 = time.perf_counter()
        out = self.pool.map(evaluate, list(members), chunksize=1)
        return np.array(out), time.perf_counter() - t0

    def close(self):
        self.pool.terminate()
        self.pool.join()


def _noop(_):
    return 0
