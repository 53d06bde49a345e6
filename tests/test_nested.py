"""The batched nested sampler (host code) on likelihoods with a known evidence, on the CPU."""
import math

import numpy as np


def _gauss(mu, sd):
    d = len(mu)

    def loglike(u):
        z = (np.asarray(u) - mu) / sd
        return -0.5 * (z * z).sum(axis=1) - d * math.log(sd * math.sqrt(2 * math.pi))
    return loglike


def test_evidence_of_a_gaussian_in_the_unit_cube():
    """A normalised Gaussian well inside the cube: log Z = 0 within the sampler's stated error (4 sigma), and the
    posterior median and spread of each coordinate those of the Gaussian."""
    from bbarolo2_gb300 import nested
    mu, sd = np.array([0.4, 0.5, 0.55, 0.6, 0.45]), 0.05
    res = nested.sample(_gauss(mu, sd), 5, n_live=300, n_batch=512, dlogz=0.05, seed=3)
    assert abs(res["logz"]) < 4 * res["logzerr"], (res["logz"], res["logzerr"])
    med = nested.posterior_median(res)
    std = nested.posterior_std(res)
    assert np.all(np.abs(med - mu) < 0.2 * sd), med
    assert np.all(np.abs(std / sd - 1) < 0.15), std
    assert res["n_like"] >= res["iterations"]


def test_same_seed_same_run():
    from bbarolo2_gb300 import nested
    f = _gauss(np.full(3, 0.5), 0.1)
    a = nested.sample(f, 3, n_live=100, n_batch=256, seed=5)
    b = nested.sample(f, 3, n_live=100, n_batch=256, seed=5)
    assert a["logz"] == b["logz"] and a["n_like"] == b["n_like"]
