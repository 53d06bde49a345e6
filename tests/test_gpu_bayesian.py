"""BAYESIAN fit on the device: nested sampling of a reduced problem (a 64^3 cube, four rings, VROT and VDISP per
ring, INC and PA global: 10 dimensions), with and without the learned screen of the proposals. Same seed, so the
screened run can differ from the plain one only where the screen turned away a point the exact likelihood would have
accepted: log Z within 0.1 of the plain run's and every posterior median within 0.1 of its sigma, with no more exact
likelihood evaluations."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _problem(galmodtype="ANALYTIC"):
    from bbarolo2_gb300 import bayesian, configs, engine
    from bbarolo2_gb300.rings import Rings
    cube, _ = configs.classic64(galmodtype=galmodtype)
    r = np.array([20., 50., 80., 110.])
    truth = Rings().setRings(radii=r, xpos=32., ypos=32., vsys=1000., vrot=150. * (1 - np.exp(-r / 40.)),
                             vdisp=10., inc=55., phi=45., z0=0., dens=np.exp(-r / 60.))
    dm = engine.DiskModel(cube, galmodtype=galmodtype)
    model = dm.array(truth, seed=1)
    sigma = 0.02 * float(model.max())
    g = np.random.default_rng(7)
    data = (model + dm.convolve_planes(g.normal(0., sigma, model.shape)) * 2.).astype(np.float32)
    mask = model > 2 * sigma
    like = engine.BatchLikelihood(dm, data, mask, maskmode=2, sigma=sigma)
    prob = bayesian.Problem(truth, per_ring=("vrot", "vdisp"), global_=("inc", "phi"),
                            priors={"vrot": (20., 200.), "vdisp": (2., 30.), "inc": (40., 70.), "phi": (30., 60.)})
    return like, prob, truth


def test_screened_fit_matches_plain_fit(gpu_lib):
    from bbarolo2_gb300 import bayesian
    like, prob, truth = _problem()
    kw = dict(n_live=100, n_batch=1024, dlogz=0.1, seed=11, galmodtype="ANALYTIC")
    plain = bayesian.fit(like, prob, **kw)
    screened = bayesian.fit(like, prob, surrogate=True, **kw)
    print({k: plain[k] for k in ("logz", "logzerr", "n_like", "wall", "iterations")},
          {k: screened[k] for k in ("logz", "n_like", "n_screened", "wall", "screen_batches", "surrogate_rmse")})
    assert abs(screened["logz"] - plain["logz"]) <= 0.1, (screened["logz"], plain["logz"])
    sd = plain["theta_std"]
    assert np.all(np.abs(screened["theta_median"] - plain["theta_median"]) <= 0.1 * sd), \
        (screened["theta_median"] - plain["theta_median"]) / sd
    # the screen only ever removes exact evaluations (it engages while its held-out error near the threshold stays
    # below 0.5 in log L; otherwise the exact likelihood judges every proposal)
    assert screened["n_like"] <= 1.02 * plain["n_like"], (screened["n_like"], plain["n_like"])
    # the truth within the posterior (4 sigma)
    t = np.r_[truth.vrot, truth.vdisp, truth.inc[0], truth.phi[0]]
    assert np.all(np.abs(plain["theta_median"] - t) <= 4 * sd + 1e-9), (plain["theta_median"] - t) / sd


def test_screen_gain_on_full_size_cube(gpu_lib):
    """The 256x256x192 BAYESIAN cube (20 rings, ANALYTIC), VROT and VDISP of four rings free (8 dimensions, a smooth
    likelihood): the screened run reaches the same log Z and medians with fewer exact evaluations. The gain is bounded
    by the share of the run in which the surrogate's held-out error near the threshold is below 0.5 (the last fifth
    or so, once the live points span a few tens of log L); the wall times are printed."""
    from bbarolo2_gb300 import bayesian, configs
    like, prob = configs.bayes256_subproblem()
    kw = dict(n_live=100, n_batch=1024, dlogz=0.1, seed=11, galmodtype="ANALYTIC")
    plain = bayesian.fit(like, prob, **kw)
    screened = bayesian.fit(like, prob, surrogate=True, **kw)
    print("plain", {k: plain[k] for k in ("logz", "n_like", "wall")},
          "screened", {k: screened[k] for k in ("logz", "n_like", "n_screened", "wall", "screen_batches",
                                                "surrogate_rmse")})
    assert abs(screened["logz"] - plain["logz"]) <= 0.1
    sd = plain["theta_std"]
    assert np.all(np.abs(screened["theta_median"] - plain["theta_median"]) <= 0.1 * sd)
    assert screened["n_like"] <= 0.9 * plain["n_like"], (screened["n_like"], plain["n_like"])
