"""The GLOBAL driver (``bbarolo2_gb300.optimize``) against the reference's own GLOBAL fit.

``tests/golden/global.npz`` holds the reference's ``optimize`` (``bbarolo/bayesian/optimize.py``) run on the oracle's
log L of the reduced problem of ``global_problem.py``. On the same likelihood the driver must take the same steps: the
same best fit, Hessian, errors and likelihood count."""
import numpy as np
import pytest

import global_problem as G
from golden_io import load


@pytest.fixture(scope="module")
def problem(oracle_lib):
    return G.Problem()


def test_mock_matches_fixture(problem):
    ref = load("global.npz")
    assert problem.nvox == int(ref["nvox"])
    assert abs(problem.data.astype(np.float64).sum() - float(ref["data_sum"])) <= 1e-9 * abs(float(ref["data_sum"]))


def test_driver_reproduces_reference_fit(problem):
    from bbarolo2_gb300.optimize import optimize
    ref = load("global.npz")
    res = optimize(problem.loglikes, problem.lo, problem.hi, G.X0, seed=1, nsamples=200, names=problem.names)
    err = ref["errors"]
    assert np.all(np.abs(res.x - ref["x"]) <= 1e-6 * err), (res.x, ref["x"])
    np.testing.assert_allclose(res.errors, err, rtol=1e-6)
    np.testing.assert_allclose(res.hessian, ref["hessian"], rtol=1e-6, atol=1e-9 * np.abs(ref["hessian"]).max())
    assert res.nfev == int(ref["nfev"]) and res.nit == int(ref["nit"])
    assert abs(res.logl - float(ref["logl"])) <= 1e-9 * abs(float(ref["logl"]))
    assert res.message == str(ref["message"])


def test_driver_bounds_and_errors():
    """A quadratic log L with its maximum outside the priors: the fit stops at the bound, the parameter is reported
    there, and the errors of a Gaussian are its sigmas."""
    from bbarolo2_gb300.optimize import optimize
    mu = np.array([0.3, 1.4])
    sig = np.array([0.05, 0.1])

    def ll(th):
        th = np.atleast_2d(th)
        return -0.5 * (((th - mu) / sig) ** 2).sum(axis=1)

    res = optimize(ll, [0., 0.], [1., 1.], [0.5, 0.5], names=["a", "b"], nsamples=100, seed=0)
    assert abs(res.x[0] - 0.3) < 1e-3 and res.x[1] == 1.0
    assert res.at_bound == ["b"]
    np.testing.assert_allclose(res.errors, sig, rtol=1e-3)
    with pytest.raises(ValueError, match="theta0"):
        optimize(ll, [0., 0.], [1., 1.], [0.5])
    with pytest.raises(ValueError, match="not finite"):
        optimize(lambda th: np.full(len(th), -np.inf), [0.], [1.], [0.5])
