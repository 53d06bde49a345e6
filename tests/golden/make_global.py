"""Generates ``global.npz``: the reference's own GLOBAL fit (``optimize`` of ``bbarolo/bayesian/optimize.py:388-468``,
L-BFGS-B in the unit cube of the priors with central differences, the Laplace errors) of the reduced problem of
``tests/global_problem.py``, run on the oracle's log L (the reference's likelihood restated bit-exact in C).

The reference is imported from its source tree (``_refimport``; BBAROLO_REF must name it); its ``optimize`` takes a
fitter, which here is a minimal object with the fitter attributes ``optimize`` reads (ndim, free parameters and their
uniform priors, the prior transform and ``_log_like_func``).

Run: BBAROLO_REF=<reference tree> python tests/golden/make_global.py
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))                       # tests/
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))      # the repository

import _refimport  # noqa: E402
import global_problem as G  # noqa: E402


class _Fitter:
    def __init__(self, P):
        from scipy import stats
        self.P = P
        self.ndim = len(P.lo)
        self.freepar_names = list(P.names)
        self.freepar_idx, self.prior_distr = {}, {}
        k = 0
        for name, n, (a, b) in G.FREE:
            self.freepar_idx[name] = np.arange(k, k + n) if n > 1 else k
            self.prior_distr[name] = stats.uniform(loc=a, scale=b - a)
            k += n

    def _prior_transform(self, u):
        return self.P.lo + np.asarray(u, float) * (self.P.hi - self.P.lo)

    def _log_like_func(self, theta):
        return self.P.loglike(theta)


def main():
    _refimport.load()
    import importlib
    opt = importlib.import_module("bbarolo.bayesian.optimize")
    P = G.Problem()
    res = opt.optimize(_Fitter(P), {}, G.X0, minimiser="L-BFGS-B", threads=1, errors=True, seed=1, nsamples=200,
                       verbose=False, showbar=False)
    out = os.path.join(HERE, "global.npz")
    np.savez_compressed(out, x=res.x, u=res.u, errors=res.errors, cov=res.cov, hessian=res.hessian,
                        steps=res.steps, logl=res.logl, nfev=res.nfev, nit=res.nit, x0=G.X0,
                        data_sum=float(P.data.astype(np.float64).sum()), nvox=P.nvox,
                        message=np.array(res.message))
    print(out, "x", np.round(res.x, 4), "errors", np.round(res.errors, 4), "nfev", res.nfev, "nit", res.nit,
          "logl", res.logl, res.message)


if __name__ == "__main__":
    main()
