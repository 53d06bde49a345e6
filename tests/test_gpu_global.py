"""Fit-level parity of METHOD GLOBAL on the device: the reduced problem of ``global_problem.py`` (10 free parameters,
the ANALYTIC model) fitted through ``bayesian.global_fit`` (every gradient and Hessian stencil one device batch)
lands within 0.05 sigma of the reference's own GLOBAL fit (``tests/golden/global.npz``: the reference's ``optimize``
on the oracle's log L), sigma the reference's Laplace errors; the device's errors agree with the reference's within
2%."""
import numpy as np
import pytest

import global_problem as G
from golden_io import load

pytestmark = pytest.mark.gpu

SIGMA_FRAC = 0.05


def test_global_fit_matches_reference(gpu_lib, oracle_lib):
    from bbarolo2_gb300 import bayesian, engine
    P = G.Problem()
    ref = load("global.npz")
    dm = engine.DiskModel(P.cube, galmodtype="ANALYTIC")
    like = engine.BatchLikelihood(dm, P.data, P.mask, maskmode=2, sigma=P.sigma)
    prob = bayesian.Problem(P.truth, per_ring=("vrot", "vdisp"), global_=("inc", "phi"),
                            priors={name: b for name, _, b in G.FREE})
    # the device log L of the start and of the reference's best fit against the oracle's
    for th in (G.X0, ref["x"]):
        dev = bayesian.DeviceLogLike(like, prob, galmodtype="ANALYTIC").of_theta([th])[0]
        cpu = P.loglike(th)
        assert abs(dev - cpu) <= 1e-5 * abs(cpu) + 0.05, (dev, cpu)
    res = bayesian.global_fit(like, prob, G.X0, galmodtype="ANALYTIC", seed=1, nsamples=200)
    err = ref["errors"]
    dx = np.abs(res.x - ref["x"]) / err
    print("GLOBAL fit: |x - x_ref| / sigma_ref max", dx.max(), "likelihoods", res.nfev, "vs", int(ref["nfev"]),
          "time", round(res.time, 2), "s")
    assert np.all(dx <= SIGMA_FRAC), (res.x, ref["x"], dx)
    np.testing.assert_allclose(res.errors, err, rtol=0.02)
    assert res.calls == res.nfev
