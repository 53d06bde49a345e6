"""BAYESIAN 3DFIT on the device: the posterior of ring parameters under the Gaussian likelihood of
``LikelihoodMixin._log_likelihood`` (``bbarolo/bayesian/likelihood.py:567-619``), sampled by the batched nested
sampler of ``bbarolo2_gb300.nested`` with every likelihood of a batch evaluated in one device pass
(``BatchLikelihood``), and optionally screened by the learned surrogate (``bbarolo2_gb300.surrogate``).

The free parameters follow ``Bayesian3DFIT`` (``bbarolo/bayesian/fitter.py:597-616``, ``:679-685``, ``:1109-1136``):
per-ring parameters (one value per ring, e.g. VROT and VDISP) and global ones (one value for every ring, e.g. INC and
PA), each with a uniform prior; a point of the unit cube maps to the ring values linearly within the priors.
"""

import numpy as np

from .rings import RING_KEYS


class Problem:
    """The parameter space of a fit: per_ring (names of per-ring parameters), global_ (names of parameters shared by
    the rings), priors {name: (lo, hi)}; proto: the rings (radii and the values of the fixed parameters); free_rings:
    the rings whose per-ring parameters are free (default all; the others keep proto's values)."""

    def __init__(self, proto, per_ring=("vrot", "vdisp"), global_=("inc", "phi"), priors=None, free_rings=None):
        self.proto = proto
        self.per_ring, self.global_ = tuple(per_ring), tuple(global_)
        self.priors = dict(priors or {})
        nr = proto.nr
        rings = range(nr) if free_rings is None else [int(r) for r in free_rings]
        self.cols = []                                       # (row of RING_KEYS, rings it sets, lo, hi)
        for name in self.per_ring:
            lo, hi = self.priors[name]
            for r in rings:
                self.cols.append((RING_KEYS.index(name), [r], float(lo), float(hi)))
        for name in self.global_:
            lo, hi = self.priors[name]
            self.cols.append((RING_KEYS.index(name), list(range(nr)), float(lo), float(hi)))
        self.ndim = len(self.cols)
        self.base = np.vstack([np.asarray(getattr(proto, k), float) for k in RING_KEYS])

    def theta(self, u):
        """Parameter values (n, ndim) of unit-cube points (the prior transform)."""
        u = np.atleast_2d(np.asarray(u, float))
        lo = np.array([c[2] for c in self.cols])
        hi = np.array([c[3] for c in self.cols])
        return lo + u * (hi - lo)

    def unit(self, theta):
        lo = np.array([c[2] for c in self.cols])
        hi = np.array([c[3] for c in self.cols])
        return (np.atleast_2d(theta) - lo) / (hi - lo)

    def rows(self, u):
        """The ring-value rows (n, 17, nr) of unit-cube points."""
        return self.rows_theta(self.theta(u))

    def rows_theta(self, theta):
        """The ring-value rows (n, 17, nr) of parameter vectors."""
        th = np.atleast_2d(np.asarray(theta, float))
        rows = np.repeat(self.base[None], len(th), axis=0)
        for j, (row, rings, _, _) in enumerate(self.cols):
            rows[:, row, rings] = th[:, j:j + 1]
        return rows


class DeviceLogLike:
    """log L of unit-cube points for a nested sampler: the points in device batches of at most ``chunk`` members
    (``BatchLikelihood.evaluate``); counts the evaluations."""

    def __init__(self, like, problem, galmodtype=None, seed=None, chunk=1024):
        self.like, self.problem = like, problem
        self.galmodtype, self.seed, self.chunk = galmodtype, seed, int(chunk)
        self.calls = 0

    def __call__(self, u):
        u = np.atleast_2d(np.asarray(u, float))
        out = np.empty(len(u))
        for a in range(0, len(u), self.chunk):
            rows = self.problem.rows(u[a:a + self.chunk])
            out[a:a + len(rows)] = self.like.evaluate(rows, self.problem.proto, seed=self.seed,
                                                      galmodtype=self.galmodtype)
        self.calls += len(u)
        return out

    def of_theta(self, thetas):
        """log L of parameter vectors (the batch log-likelihood of the GLOBAL fit)."""
        th = np.atleast_2d(np.asarray(thetas, float))
        out = np.empty(len(th))
        for a in range(0, len(th), self.chunk):
            rows = self.problem.rows_theta(th[a:a + self.chunk])
            out[a:a + len(rows)] = self.like.evaluate(rows, self.problem.proto, seed=self.seed,
                                                      galmodtype=self.galmodtype)
        self.calls += len(th)
        return out


def global_fit(like, problem, theta0, galmodtype=None, step=1e-3, errors=True, options=None, nsamples=4000,
               seed=None):
    """METHOD GLOBAL: the maximum of log L within the priors from theta0 (``bbarolo2_gb300.optimize``), every
    gradient and Hessian stencil one device batch. Returns the result of ``optimize.optimize`` with ``calls``."""
    from .optimize import optimize
    ll = DeviceLogLike(like, problem, galmodtype=galmodtype)
    lo = np.array([c[2] for c in problem.cols])
    hi = np.array([c[3] for c in problem.cols])
    names = [RING_KEYS[c[0]] for c in problem.cols]
    res = optimize(ll.of_theta, lo, hi, theta0, step=step, errors=errors, options=options, nsamples=nsamples,
                   seed=seed, names=names)
    res["calls"] = ll.calls
    return res


def fit(like, problem, n_live=400, n_batch=1024, dlogz=0.1, seed=0, surrogate=False, galmodtype=None,
        enlarge=1.25, hidden=256, device=0, **kw):
    """Samples the posterior of the problem; returns the sampler's result with ``theta_median`` and ``theta_std``
    (the weighted median and spread of each parameter) and, with surrogate=True, the surrogate's statistics."""
    from . import nested
    ll = DeviceLogLike(like, problem, galmodtype=galmodtype)
    sur = None
    if surrogate:
        from .surrogate import Surrogate
        sur = Surrogate(problem.ndim, hidden=hidden, seed=seed, device=device)
    res = nested.sample(ll, problem.ndim, n_live=n_live, n_batch=n_batch, dlogz=dlogz, seed=seed, enlarge=enlarge,
                        surrogate=sur, **kw)
    lo = np.array([c[2] for c in problem.cols])
    hi = np.array([c[3] for c in problem.cols])
    res["theta_median"] = lo + nested.posterior_median(res) * (hi - lo)
    res["theta_std"] = nested.posterior_std(res) * (hi - lo)
    if sur is not None:
        res["surrogate_rmse"] = float(sur.last_rmse)
    return res
