"""A batched nested sampler for the device likelihood, with an optional learned screen of its proposals.

Nested sampling (Skilling 2004) on the unit cube of the priors: n_live live points; at each step the worst is
replaced by a point drawn from the prior restricted to a higher likelihood, the prior volume shrinking by a factor
exp(-1/n_live) a step, and the evidence is the sum of the dead points' likelihoods times their volume shells plus the
live points' share at the end. The constrained draws are rejection samples from a bound of the live points (their
ellipsoid, enlarged, within the cube), proposed ``n_batch`` at a time so that the likelihood runs as one device batch:
a proposal that beats the current worst point replaces it (a uniform draw within the old bound, kept when above the
new threshold, is a uniform draw within the new region).

Screen (``surrogate``): the proposals pass through the learned surrogate first, and only those it predicts above the
threshold they would meet, minus a margin, reach the exact likelihood; the others count as rejected. The threshold a
proposal meets is the one after the replacements by the proposals before it in the batch: the pass is played on the
predictions less the margin (``_screen``), which keeps that threshold at or below the exact pass's whenever the
surrogate's error is within the margin, so that no proposal the exact pass would accept is turned away. The surrogate
is retrained on the exact evaluations every n_live / 4 replacements once the live points' log L span less than
``fit_range`` (40; before, the threshold moves by more than the surrogate's window between fits, and no fit passes the
check below), and the screen is used only while its error on the latest evaluations it was not trained on, near the
threshold, stays below ``max_rmse`` (0.5 in log L): else every proposal is evaluated exactly.
The proposals are the same random draws with and without the screen, so a run with a screen that never turns away a
point the exact likelihood would accept is the run without it, point for point.

The reference samples its posterior with a vendored nautilus (``bbarolo/bayesian/sampling.py:252-320``,
``bbarolo/bayesian/nautilus/sampler.py``), an importance nested sampler with neural bounds; this sampler is the
simpler ellipsoidal form, written for batched device likelihoods.
"""

import math
import time

import numpy as np


def _logaddexp(a, b):
    return np.logaddexp(a, b)


class _Ellipsoid:
    """The bound of the live points: their ellipsoid (mean, covariance) scaled to contain them all, enlarged."""

    def __init__(self, u, enlarge):
        self.mu = u.mean(axis=0)
        c = np.cov(u, rowvar=False) + 1e-12 * np.eye(u.shape[1])
        self.L = np.linalg.cholesky(c)
        z = np.linalg.solve(self.L, (u - self.mu).T)
        self.r = math.sqrt(float((z * z).sum(axis=0).max())) * enlarge

    def sample(self, n, rng):
        d = self.mu.size
        out = np.empty((0, d))
        while len(out) < n:
            m = 2 * (n - len(out)) + 16
            g = rng.standard_normal((m, d))
            g /= np.linalg.norm(g, axis=1)[:, None]
            g *= (rng.random(m) ** (1.0 / d))[:, None] * self.r
            x = self.mu + g @ self.L.T
            x = x[np.all((x >= 0) & (x <= 1), axis=1)]
            out = np.vstack([out, x])
        return out[:n]


def sample(loglike, ndim, n_live=400, n_batch=1024, dlogz=0.1, seed=0, enlarge=1.25, surrogate=None,
           retrain_every=None, max_rmse=0.5, margin=None, fit_range=40.0, max_batches=100000, verbose=False):
    """Nested sampling of loglike (a function of an (n, ndim) array of unit-cube points -> n log-likelihoods) until
    the live points can add at most dlogz to log Z. Returns a dict: logz, logzerr, samples (unit cube), logl, logwt
    (log weights), n_like (exact evaluations), n_proposed, n_screened (proposals the screen turned away), iterations,
    wall (s), screen_batches (batches that used the screen)."""
    rng = np.random.default_rng(seed)
    t0 = time.perf_counter()
    u = rng.random((n_live, ndim))
    logl = np.asarray(loglike(u), float)
    n_like = n_live
    hist_u, hist_l = [u.copy()], [logl.copy()]
    dead_u, dead_l, dead_w = [], [], []
    logz, h = -np.inf, 0.0
    logx = 0.0
    it = 0
    n_prop = n_screen = screen_batches = 0
    untrained_from = 0                       # (first history entry the surrogate was not fitted on)
    screen_ok = False
    # the surrogate is refitted every `retrain_every` replacements of a live point (default a quarter of the live
    # points: the prior volume has shrunk by a quarter of an e-fold since the last fit)
    retrain_every = retrain_every or max(n_live // 4, 1)
    next_fit = retrain_every
    for batch in range(max_batches):
        # stop when the live points can add little: log Z against log(Z + L_max X)
        lmax = float(logl.max())
        if np.isfinite(logz) and _logaddexp(logz, lmax + logx) - logz < dlogz:
            break
        thr = float(logl.min())
        cand = _Ellipsoid(u, enlarge).sample(n_batch, rng)
        n_prop += len(cand)
        vals = np.full(len(cand), -np.inf)
        use = np.ones(len(cand), bool)
        if surrogate is not None and screen_ok:
            delta = margin if margin is not None else max(4.0 * surrogate.last_rmse, 0.5)
            use = _screen(surrogate.predict(cand), logl, delta)
            n_screen += int((~use).sum())
            screen_batches += 1
        if use.any():
            vals[use] = np.asarray(loglike(cand[use]), float)
            n_like += int(use.sum())
            hist_u.append(cand[use])
            hist_l.append(vals[use])
        for c in np.flatnonzero(vals > thr):             # (the threshold only rises: the others cannot enter)
            worst = int(np.argmin(logl))
            if not vals[c] > logl[worst]:
                continue
            # the worst point dies: its shell of prior volume exp(logx) (1 - exp(-1/n_live))
            logw = logx + math.log1p(-math.exp(-1.0 / n_live)) + float(logl[worst])
            znew = _logaddexp(logz, logw)
            h = (math.exp(logw - znew) * float(logl[worst]) +
                 (math.exp(logz - znew) * (h + logz) if np.isfinite(logz) else 0.0) - znew)
            logz = znew
            dead_u.append(u[worst].copy())
            dead_l.append(float(logl[worst]))
            dead_w.append(logw)
            logx -= 1.0 / n_live
            u[worst] = cand[c]
            logl[worst] = vals[c]
            it += 1
        if surrogate is not None and it >= next_fit and float(logl.max() - logl.min()) < fit_range:
            screen_ok = _refit(surrogate, hist_u, hist_l, untrained_from, u, logl, max_rmse)
            untrained_from = len(hist_u)
            next_fit = it + retrain_every
        if verbose and batch % 20 == 0:
            print(f"batch {batch}: it {it} logz {logz:.3f} thr {thr:.3f} calls {n_like} screened {n_screen}")
    # the live points' share
    for k in np.argsort(logl):
        logw = logx - math.log(n_live) + float(logl[k])
        znew = _logaddexp(logz, logw)
        h = (math.exp(logw - znew) * float(logl[k]) +
             (math.exp(logz - znew) * (h + logz) if np.isfinite(logz) else 0.0) - znew)
        logz = znew
        dead_u.append(u[k].copy())
        dead_l.append(float(logl[k]))
        dead_w.append(logw)
    logwt = np.asarray(dead_w) - logz
    return dict(logz=float(logz), logzerr=math.sqrt(max(h, 0.0) / n_live), samples=np.asarray(dead_u),
                logl=np.asarray(dead_l), logwt=logwt, n_like=n_like, n_proposed=n_prop, n_screened=n_screen,
                iterations=it, wall=time.perf_counter() - t0, screen_batches=screen_batches, information=h)


def _screen(pred, live_l, delta):
    """The proposals worth an exact evaluation: those predicted above the threshold of their turn in the pass, less
    delta. The pass is played with the predictions less delta as the values of the replacing points, a lower bound of
    their exact values when the surrogate's error is below delta, so the played threshold stays at or below the exact
    one at every turn (the sorted live values of the play never exceed the exact ones)."""
    play = np.array(live_l, float)
    use = np.zeros(len(pred), bool)
    for c, p in enumerate(np.asarray(pred, float)):
        w = int(np.argmin(play))
        if p > play[w] - delta:
            use[c] = True
            if p - delta > play[w]:
                play[w] = p - delta
    return use


def _refit(sur, hist_u, hist_l, untrained_from, live_u, live_l, max_rmse):
    """Checks the surrogate on the evaluations it has not seen (near the threshold), then refits it on the recent
    ones; True when the check passed (the screen may be used until the next refit)."""
    thr = float(live_l.min())
    ok = False
    if sur.trained and untrained_from < len(hist_u):
        hu = np.vstack(hist_u[untrained_from:])
        hl = np.concatenate(hist_l[untrained_from:])
        near = np.abs(hl - thr) < 5.0                   # (the points whose screening decision is close)
        if near.sum() >= 32:
            sur.last_rmse = sur.rmse(hu[near], hl[near])
            ok = sur.last_rmse < max_rmse
    u = np.vstack(hist_u)[-32768:]
    y = np.concatenate(hist_l)[-32768:]
    sur.fit(u, y, center=thr, region=live_u)
    return ok


def posterior_median(res):
    """The weighted median of each coordinate of the samples of a run."""
    w = np.exp(res["logwt"] - res["logwt"].max())
    w /= w.sum()
    out = []
    for j in range(res["samples"].shape[1]):
        o = np.argsort(res["samples"][:, j])
        c = np.cumsum(w[o])
        out.append(float(res["samples"][o[np.searchsorted(c, 0.5)], j]))
    return np.asarray(out)


def posterior_std(res):
    w = np.exp(res["logwt"] - res["logwt"].max())
    w /= w.sum()
    m = (w[:, None] * res["samples"]).sum(axis=0)
    return np.sqrt((w[:, None] * (res["samples"] - m) ** 2).sum(axis=0))
