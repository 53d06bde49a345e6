"""Generates ``global.npz``: the reference's own GLOBAL fits (``optimize`` of ``bbarolo/bayesian/optimize.py:388-468``,
L-BFGS-B in the unit cube of the priors with central differences, the Laplace errors) of the reduced problems of
``tests/global_problem.py`` ("kin" and "geo" from their starts, and "geo" from the nearby starts ``STARTS``), run on
the oracle's log L (the reference's likelihood restated bit-exact in C). Keys: <case>/x, /errors, ... and
geo/starts_x (the fits from ``STARTS``).

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
        for name, n, (a, b) in G.FREE[P.case]:
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
    arrays = {}
    for case in ("kin", "geo"):
        P = G.Problem(case)
        res = opt.optimize(_Fitter(P), {}, G.X0[case], minimiser="L-BFGS-B", threads=1, errors=True, seed=1,
                           nsamples=200, verbose=False, showbar=False)
        for k in ("x", "u", "errors", "cov", "hessian", "steps", "logl", "nfev", "nit"):
            arrays[f"{case}/{k}"] = np.asarray(res[k])
        arrays[f"{case}/message"] = np.array(res.message)
        arrays[f"{case}/x0"] = G.X0[case]
        print(case, "x", np.round(res.x, 4), "errors", np.round(res.errors, 4), "nfev", res.nfev, "nit", res.nit,
              "logl", res.logl, res.message)
    arrays["data_sum"] = float(P.data.astype(np.float64).sum())
    arrays["nvox"] = P.nvox
    xs = []
    for x0 in G.STARTS:
        r = opt.optimize(_Fitter(P), {}, x0, minimiser="L-BFGS-B", threads=1, errors=False, verbose=False,
                         showbar=False)
        xs.append(r.x)
        print("geo from", np.round(x0, 2), "->", np.round((r.x - arrays["geo/x"]) / arrays["geo/errors"], 2))
    arrays["geo/starts_x"] = np.array(xs)
    out = os.path.join(HERE, "global.npz")
    np.savez_compressed(out, **arrays)
    print(out)


if __name__ == "__main__":
    main()
