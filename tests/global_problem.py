"""The reduced GLOBAL problem of the fit-level parity tests, built from the oracle alone.

A 64x64x64 cube (10" pixels, 5 km/s channels, 30" beam), four rings at 20-110", the ANALYTIC model of a thin disk
(z0 = 0), uniform priors. Two cases: "kin", VROT and VDISP per ring (8 free parameters, the geometry at the truth),
and "geo", VROT and VDISP per ring with INC and PA global (10 free parameters). The mock is the oracle's
ANALYTIC model of the truth, convolved in float64, plus white noise of 2% of its peak (seed 7); the likelihood mask is
the convolved truth above twice the noise, mask mode 2 (Bayesian3DFIT's default).

``oracle_loglikes(P)`` is the reference's log L of a list of parameter vectors computed by the oracle
(``bbarolo/bayesian/likelihood.py:567-619``: the model in its box, the "same" convolution, the residual of the box and
the data outside it), the likelihood the reference's own GLOBAL fit is run on to make ``tests/golden/global.npz``.

The likelihood is smooth in VROT and VDISP, but in INC and PA it is a staircase: the ANALYTIC model puts each
azimuth sample in one pixel, so that a change of the geometry moves flux between pixels in steps (of up to several
units of log L at this noise, over fractions of the Laplace sigma of PA). A fit of "geo" therefore ends wherever its
path meets the staircase; ``STARTS`` gives the starts of the reference's fits that measure how far apart its own
fits from nearby starts land.
"""

import math

import numpy as np

FREE = {"kin": (("vrot", 4, (20., 200.)), ("vdisp", 4, (2., 30.))),
        "geo": (("vrot", 4, (20., 200.)), ("vdisp", 4, (2., 30.)), ("inc", 1, (40., 70.)), ("phi", 1, (30., 60.)))}
X0 = {"kin": np.array([70., 100., 120., 140., 14., 8., 12., 9.]),             # the start of the fits
      "geo": np.array([70., 100., 120., 140., 14., 8., 12., 9., 50., 40.])}
# the reference's fits of "geo" from nearby starts (its own scatter on the staircase)
STARTS = [X0["geo"] + d for d in (np.r_[[2., -2., 2., -2.], [1., -1., 1., -1.], 0.5, 0.5],
                                 np.r_[[-2., 2., -2., 2.], [-1., 1., -1., 1.], -0.5, 0.5],
                                 np.r_[[1., 1., 1., 1.], [0.5, 0.5, 0.5, 0.5], 0.5, -0.5])]


def cube_and_truth():
    from bbarolo2_gb300 import configs
    from bbarolo2_gb300.rings import Rings
    cube, _ = configs.classic64(galmodtype="ANALYTIC")
    r = np.array([20., 50., 80., 110.])
    truth = Rings().setRings(radii=r, xpos=32., ypos=32., vsys=1000., vrot=150. * (1 - np.exp(-r / 40.)),
                             vdisp=10., inc=55., phi=45., z0=0., dens=np.exp(-r / 60.))
    return cube, truth


def bounds(case):
    lo, hi, names = [], [], []
    for name, n, (a, b) in FREE[case]:
        lo += [a] * n
        hi += [b] * n
        names += [name] * n
    return np.array(lo), np.array(hi), names


class Problem:
    """The cube, truth, mock and the oracle's set-up of the reduced GLOBAL problem (case "kin" or "geo")."""

    def __init__(self, case):
        from oracle import host
        from oracle import oracle as O
        O.lib()
        self.cube, self.truth = cube_and_truth()
        self.st = host.Setup(self.cube)
        self.kernel = host.beam_kernel(self.cube)
        self.zstep = host.zstep(self.cube, self.st)
        self.nx, self.ny, self.nz = self.cube.DimX(), self.cube.DimY(), self.cube.DimZ()
        model = self.model(self.row(None))
        self.sigma = 0.02 * float(model.max())
        g = np.random.default_rng(7)
        self.data = (model + g.normal(0., self.sigma, model.shape)).astype(np.float32)
        self.mask = model > 2 * self.sigma
        valid = np.isfinite(self.data) & (self.data != 0) & self.mask
        self.valid = valid
        self.d2 = np.where(valid, self.data.astype(np.float64) ** 2, 0.)
        self.nvox = int(valid.sum())
        self.case = case
        self.lo, self.hi, self.names = bounds(case)

    def row(self, theta):
        """The ring-value row (17, nr) of a parameter vector (None: the truth)."""
        from oracle.cpu_baseline import RING_KEYS, ring_rows
        row = ring_rows(self.truth)
        if theta is None:
            return row
        th = np.asarray(theta, float)
        k = 0
        for name, n, _ in FREE[self.case]:
            row[RING_KEYS.index(name)] = th[k:k + n] if n > 1 else th[k]
            k += n
        return row

    def model(self, row, box=False):
        """The convolved ANALYTIC model of a ring-value row in its box (box=True: also the box)."""
        from oracle import host
        from oracle import oracle as O
        st = self.st
        rk = host.rings_of_row(self.truth, row)
        sr, _ = host.subrings(st, host.model_rings(rk, "CENTRED", st.radsep))
        blo, bhi = host.box(self.cube, rk, final=True)
        m = np.zeros((bhi[1] - blo[1], bhi[0] - blo[0], self.nz))
        nzq = 1 if not np.any(sr[6] > 0) else 1024
        O.galmod_analytic(m, sr, 0, sr.shape[1], st.radsep, st.cdens, st.pixarea, st.cdelt[0], st.cdelt[1],
                          st.crota2, blo[0], blo[1], bhi[0], bhi[1], st.ltype, st.sig_instr,
                          np.ascontiguousarray(st.vedges[None]), st.relint, st.cd2i, nzq, st.axtyp, st.velsys,
                          st.lfreq0, st.crval3, st.cdelt3, st.crpix3, st.chmin, None, self.zstep)
        sm = O.conv_same(m.transpose(2, 0, 1), self.kernel)
        if box:
            return sm, (blo, bhi)
        full = np.zeros((self.nz, self.ny, self.nx))
        full[:, blo[1]:bhi[1], blo[0]:bhi[0]] = sm
        return full

    def loglike(self, theta):
        """log L of one parameter vector: -(0.5 (ss_box + ss_out) / sigma^2 + 0.5 nvox log(2 pi sigma^2))."""
        from oracle import oracle as O
        sm, (blo, bhi) = self.model(self.row(theta), box=True)
        sl = (slice(None), slice(blo[1], bhi[1]), slice(blo[0], bhi[0]))
        ss = O.sumsq_residuals(sm, self.data[sl], self.mask[sl], 2, None)
        out = self.d2.sum() - self.d2[sl].sum()
        s2 = self.sigma ** 2
        return -(0.5 * (ss + out) / s2 + 0.5 * self.nvox * math.log(2. * math.pi * s2))

    def loglikes(self, thetas):
        return np.array([self.loglike(t) for t in thetas], float)
