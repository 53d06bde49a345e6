"""The GLOBAL driver (``bbarolo2_gb300.optimize``) against the reference's own GLOBAL fit.

``tests/golden/global.npz`` holds the reference's ``optimize`` (``bbarolo/bayesian/optimize.py``) run on the oracle's
log L of the reduced problem of ``global_problem.py``. On the same likelihood the driver must take the same steps: the
same best fit, Hessian, errors and likelihood count."""
import numpy as np
import pytest

import global_problem as G
from golden_io import load


def test_mock_matches_fixture(oracle_lib):
    P = G.Problem("kin")
    ref = load("global.npz")
    assert P.nvox == int(ref["nvox"])
    assert abs(P.data.astype(np.float64).sum() - float(ref["data_sum"])) <= 1e-9 * abs(float(ref["data_sum"]))


@pytest.mark.parametrize("case", ["kin", "geo"])
def test_driver_reproduces_reference_fit(oracle_lib, case):
    from bbarolo2_gb300.optimize import optimize
    P = G.Problem(case)
    ref = load("global.npz")
    res = optimize(P.loglikes, P.lo, P.hi, G.X0[case], seed=1, nsamples=200, names=P.names)
    x, err, H = ref[f"{case}/x"], ref[f"{case}/errors"], ref[f"{case}/hessian"]
    assert np.all(np.abs(res.x - x) <= 1e-6 * err), (res.x, x)
    np.testing.assert_allclose(res.errors, err, rtol=1e-6)
    np.testing.assert_allclose(res.hessian, H, rtol=1e-6, atol=1e-9 * np.abs(H).max())
    assert res.nfev == int(ref[f"{case}/nfev"]) and res.nit == int(ref[f"{case}/nit"])
    assert abs(res.logl - float(ref[f"{case}/logl"])) <= 1e-9 * abs(float(ref[f"{case}/logl"]))
    assert res.message == str(ref[f"{case}/message"])


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
