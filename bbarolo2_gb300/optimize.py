"""METHOD GLOBAL on the device: the maximum of log L within the priors by L-BFGS-B in the unit cube of the priors, every
gradient (its 2n + 1 likelihoods) one device batch, then the Laplace errors from a finite-difference Hessian whose
stencils are device batches too.

The function ``optimize`` takes a batch log-likelihood (a function of a list of parameter vectors returning their
log L: ``bayesian.DeviceLogLike`` over ``BatchLikelihood``, or any other) and uniform priors (lo, hi), and returns the
fields of the reference's result (``bbarolo/bayesian/optimize.py:388-468``): x, u, logl, fun, nfev, nit, message,
errors, cov, hessian, steps, samples, regularised, at_bound. The steps that decide the result are those of the
reference, so that the fit lands where the reference's does on the same likelihood:

* the search space: u in [0, 1]^n, theta = lo + u (hi - lo); non-finite -log L is 1e30;
* the gradient: central differences of step ``step`` in u, one-sided (or none) where a bound cuts the stencil
  (``optimize.py:205-229``); scipy's L-BFGS-B (the reference's default minimiser);
* the answer: the minimiser's point, or the best point any batch evaluated if that is better by 1e-9;
* the Hessian in theta (``optimize.py:298-352``): diagonal steps 1e-3 of the prior's scale, resized up to three times
  to a change of 8 in -log L (sqrt(16 / d2), within [1e-8, 0.25] of the scale), the stencil moved inside the
  bounds, then the off-diagonal terms from the points +-(h_i e_i + h_j e_j);
* the errors (``optimize.py:355-385``): the covariance of the Hessian in u floored at the prior's (eigenvalues >= 12),
  mapped back to theta.
"""

import math
import time

import numpy as np

BIG = 1e30          # the objective where log L is not finite
HESS_CHANGE = 8.    # the change of -log L the Hessian's steps aim at (about four conditional sigma)
PRIOR_CURV = 12.    # the curvature of a uniform prior in u (1 / its variance): the floor of the Hessian's eigenvalues


class Result(dict):
    """The result of ``optimize``: a dict whose keys are also attributes."""

    __getattr__ = dict.__getitem__


class _Batches:
    """-log L of lists of points, each list one call of the batch log-likelihood; tracks the best point in u and
    counts the likelihoods."""

    def __init__(self, loglikes, lo, hi):
        self.loglikes = loglikes
        self.lo, self.hi = np.asarray(lo, float), np.asarray(hi, float)
        self.scale = self.hi - self.lo
        self.nfev = 0
        self.fbest, self.ubest = np.inf, None

    def theta(self, u):
        return self.lo + np.clip(u, 0., 1.) * self.scale

    def of_theta(self, thetas):
        th = np.clip(np.atleast_2d(np.asarray(thetas, float)), self.lo, self.hi)
        f = -np.asarray(self.loglikes(list(th)), float)
        self.nfev += len(th)
        return np.where(np.isfinite(f), f, BIG)

    def of_u(self, us):
        us = np.clip(np.atleast_2d(np.asarray(us, float)), 0., 1.)
        f = self.of_theta(self.theta(us))
        k = int(np.argmin(f))
        if f[k] < self.fbest:
            self.fbest, self.ubest = float(f[k]), us[k].copy()
        return f

    def value_and_gradient(self, u, h):
        """-log L at u and its gradient in u: the 2n + 1 points in one batch."""
        u = np.clip(np.asarray(u, float), 0., 1.)
        n = u.size
        up = np.minimum(h, 1. - u)
        dn = np.minimum(h, u)
        stencil = np.vstack([u, u + np.diag(up), u - np.diag(dn)])
        f = self.of_u(stencil)
        f0, fp, fm = f[0], f[1:n + 1], f[n + 1:]
        okp = (up > 0) & (fp < BIG)
        okm = (dn > 0) & (fm < BIG)
        g = np.zeros(n)
        both = okp & okm
        g[both] = (fp[both] - fm[both]) / (up[both] + dn[both])
        only = okp & ~okm
        g[only] = (fp[only] - f0) / up[only]
        only = okm & ~okp
        g[only] = (f0 - fm[only]) / dn[only]
        return float(f0), g


def _hessian(B, x):
    """The Hessian of -log L in theta at x and its steps (see the module docstring)."""
    lo, hi, S = B.lo, B.hi, B.scale
    n = x.size
    eye = np.eye(n)

    def stencil(h):
        c = np.clip(x, lo + h, hi - h)
        f = B.of_theta(np.vstack([c, c + eye * h, c - eye * h]))
        return c, f[0], f[1:n + 1], f[n + 1:]

    h = 1e-3 * S
    for _ in range(3):
        h = np.minimum(h, 0.25 * S)
        _, f0, fp, fm = stencil(h)
        d2 = (fp + fm - 2. * f0) / h ** 2
        good = (d2 > 0) & (fp < BIG) & (fm < BIG)
        new = np.where(good, np.sqrt(2. * HESS_CHANGE / np.maximum(d2, 1e-300)), 10. * h)
        new = np.clip(new, 1e-8 * S, 0.25 * S)
        settled = bool(np.all(np.abs(np.log(new / h)) < math.log(1.5)))
        h = new
        if settled:
            break
    c, f0, fp, fm = stencil(h)
    H = np.diag((fp + fm - 2. * f0) / h ** 2)
    iu, ju = np.triu_indices(n, 1)
    if iu.size:
        step = eye[iu] * h[iu, None] + eye[ju] * h[ju, None]
        f = B.of_theta(np.vstack([c + step, c - step]))
        npair = iu.size
        v = (f[:npair] + f[npair:] - fp[iu] - fm[iu] - fp[ju] - fm[ju] + 2. * f0) / (2. * h[iu] * h[ju])
        H[iu, ju] = v
        H[ju, iu] = v
    if np.any(np.r_[fp, fm, f0] >= BIG) or not np.all(np.isfinite(H)):
        H = np.where(np.isfinite(H) & (np.abs(H) < BIG), H, 0.)
    return H, h


def _laplace(S, x, H, lo, hi, nsamples, seed):
    """Covariance in theta and in u of the Hessian H (theta) floored at the prior's curvature, and nsamples draws of
    the Gaussian within the priors."""
    Hu = S[:, None] * (0.5 * (H + H.T)) * S[None, :]
    w, V = np.linalg.eigh(Hu)
    regularised = bool(np.any(w < PRIOR_CURV))
    w = np.maximum(w, PRIOR_CURV)
    A = S[:, None] * (V / np.sqrt(w))
    cov = A @ A.T
    cov_u = (V / w) @ V.T
    rng = np.random.default_rng(seed)
    kept, tries = [], 0
    while sum(len(k) for k in kept) < nsamples and tries < 50:
        z = x + rng.standard_normal((nsamples, x.size)) @ A.T
        kept.append(z[np.all((z >= lo) & (z <= hi), axis=1)])
        tries += 1
    s = np.concatenate(kept) if kept else np.empty((0, x.size))
    if len(s) < nsamples:
        z = np.clip(x + rng.standard_normal((nsamples - len(s), x.size)) @ A.T, lo, hi)
        s = np.concatenate([s, z])
    return cov, cov_u, s[:nsamples], regularised


def optimize(loglikes, lo, hi, theta0, step=1e-3, errors=True, options=None, nsamples=4000, seed=None, names=None):
    """Maximum of log L within the uniform priors [lo, hi] from theta0 (see the module docstring); loglikes: a
    function of a list of parameter vectors returning their log L (one device batch per call)."""
    from scipy import optimize as sopt
    t0 = time.time()
    lo, hi = np.asarray(lo, float), np.asarray(hi, float)
    n = lo.size
    th0 = np.asarray(theta0, float)
    if th0.shape != (n,):
        raise ValueError(f"optimize: theta0 has {th0.size} values, the free parameters are {n}")
    B = _Batches(loglikes, lo, hi)
    u0 = np.clip((th0 - lo) / B.scale, 0., 1.)
    if not B.of_u(u0)[0] < BIG:
        raise ValueError("optimize: the likelihood is not finite at theta0")
    h = np.full(n, float(step))
    res = sopt.minimize(lambda u: B.value_and_gradient(u, h), u0, jac=True, method="L-BFGS-B",
                        bounds=sopt.Bounds(np.zeros(n), np.ones(n)), options=dict(options or {}))
    msg = str(res.message)
    if msg.strip().rstrip(":").startswith("ABNORMAL"):
        msg = "ABNORMAL: the line search found no better point, even along the gradient"
    u = np.clip(np.asarray(res.x, float), 0., 1.)
    if B.ubest is not None and B.fbest < B.of_u(u)[0] - 1e-9:
        u = B.ubest
    x = B.theta(u)
    logl = -float(B.of_theta(x)[0])
    out = Result(x=x, u=u, logl=logl, fun=-logl, method="L-BFGS-B", success=bool(res.success), message=msg,
                 nit=int(res.nit))
    tol = np.full(n, 1e-3)
    if errors:
        H, hs = _hessian(B, x)
        cov, cov_u, samples, reg = _laplace(B.scale, x, H, lo, hi, int(nsamples), seed)
        out.update(hessian=H, steps=hs, cov=cov, samples=samples, regularised=reg, errors=np.sqrt(np.diag(cov)))
        tol = np.maximum(tol, np.sqrt(np.diag(cov_u)))
    else:
        out.update(hessian=None, steps=None, cov=None, errors=None, samples=x[None].copy(), regularised=False)
    names = list(names) if names is not None else [f"p{i}" for i in range(n)]
    out["at_bound"] = [nm for nm, ui, t in zip(names, u, tol) if ui < t or 1. - ui < t]
    out["nfev"] = B.nfev
    out["time"] = time.time() - t0
    return out
