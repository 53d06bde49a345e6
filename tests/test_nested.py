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


def test_screen_plays_the_rising_threshold():
    """The screen keeps every proposal the exact pass would accept when the surrogate's error is within the margin,
    and turns away those below the threshold the earlier proposals of the batch raise."""
    from bbarolo2_gb300.nested import _screen
    g = np.random.default_rng(3)
    for trial in range(50):
        live = g.normal(0., 3., 40)
        exact = g.normal(0., 4., 300)
        delta = 0.5
        pred = exact + g.uniform(-0.49, 0.49, exact.size)
        use = _screen(pred, live, delta)
        # the exact pass
        cur = live.copy()
        for c, v in enumerate(exact):
            w = int(np.argmin(cur))
            if v > cur[w]:
                assert use[c], (trial, c)
                cur[w] = v
        # a proposal far below the initial threshold is turned away
        assert not _screen(np.array([live.min() - 10.]), live, delta)[0]
    # the rising threshold: the same value offered twice after the live minimum rose past it is turned away once
    live = np.array([0., 5., 5., 5.])
    assert list(_screen(np.array([4., 1.]), live, 0.5)) == [True, False]
