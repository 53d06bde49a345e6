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
``solve_profile`` (``oracle/profile.py``), the model's sub-rings with the new densities (the package's host
``subrings_batch``, bit-equal to the reference's ``subrings``), then the MC model (or, with ``galmodtype``
ANALYTIC in the payload, the ANALYTIC model ``_galmod_analytic`` through its C restatement).
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
    """The MC sub-ring table of member k with the ring densities x (nr)."""
    from bbarolo2_gb300.galmod import model_rows, subrings_batch
    P = P or _W
    pr = P["prof"]
    rows = pr["rows"][k:k + 1].copy()
    rows[0, pr["dens_row"]] = x[:pr["nr"]]
    mrows, mr = model_rows(rows, pr["proto"], pr["mode"], pr["gsetup"].radsep)
    sr, nv = subrings_batch(pr["gsetup"], mr, mrows)
    return sr[0], nv[0]


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
                         dens_row=RING_KEYS.index("dens"), gsetup=st)
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
