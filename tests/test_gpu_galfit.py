"""GPU parity of the CLASSIC fit of single rings (``bbarolo/galfit.py``: the downhill simplex with its bounds and
seeded redraws, the model of the ring built and convolved on the device, ``_norm`` on the device) against the
reference's fits of three rings of the 64^3 mock (``tests/golden/galfit.npz``).

The model of a ring is the reference's to rounding (bit-exact cloud indices, fixed-point sums, bit-exact sparse
convolution) and the residual differs from the reference's running sum by rounding only, so the simplex visits the
same points: the function values along the fit agree within FUNC_RTOL, and the fitted VROT and VDISP within PAR_TOL
(km/s)."""
import json

import numpy as np
import pytest

import golden_io as G

pytestmark = pytest.mark.gpu

FUNC_RTOL = 1e-9
PAR_TOL = 1e-6


def _setup():
    from bbarolo2_gb300 import configs
    from bbarolo2_gb300.classic import ClassicFit
    from golden.cases import galfit_par
    z = G.load("galfit.npz")
    meta = json.loads(str(z["index"]))
    cube, rings = configs.classic64()
    a, b = meta["crop"]
    data = np.zeros(cube.array.shape, np.float32)
    mask = np.zeros(cube.array.shape, bool)
    data[:, a:b, a:b] = z["data"]
    mask[:, a:b, a:b] = z["mask"]
    cube.array = data
    assert 10. / float(data.max()) == float(z["scaling"])
    inr = rings.copy()
    inr.vrot = np.full(inr.nr, meta["vrot0"])
    inr.vdisp = np.full(inr.nr, meta["vdisp0"])
    fit = ClassicFit(cube, inr, galfit_par(), float(z["sigma"]), mask)
    return z, meta, fit


def test_classic_ring_fits_match_reference(gpu_lib):
    """The rings of the stage fitted together (one round evaluates every running ring's point): each ring's sequence
    of evaluations, its convergence, minimum and fitted values are the reference's."""
    z, meta, fit = _setup()
    outr, fitok = fit.run(rings=meta["rings"])
    for ir, ok, minimum, vrot, vdisp, ncalls in z["results"]:
        ir = int(ir)
        ref_calls = z[f"calls_{ir}"]
        got = np.array([[x[0], x[1], f] for x, f in fit.log[ir]])
        n = min(len(got), len(ref_calls))
        np.testing.assert_allclose(got[:n, 2], ref_calls[:n, 2], rtol=FUNC_RTOL, err_msg=f"ring {ir}")
        np.testing.assert_allclose(got[:n, :2], ref_calls[:n, :2], rtol=0, atol=PAR_TOL, err_msg=f"ring {ir}")
        assert len(got) == int(ncalls), (ir, len(got), ncalls)
        assert bool(fitok[ir]) == bool(ok)
        assert abs(outr.vrot[ir] - vrot) <= PAR_TOL and abs(outr.vdisp[ir] - vdisp) <= PAR_TOL, ir
        assert abs(fit.status[ir][1] - minimum) <= FUNC_RTOL * abs(minimum)


def test_classic_rings_alone_equal_rings_together(gpu_lib):
    """A ring fitted alone gives the evaluations it gives among the others (the rounds only interleave rings)."""
    z, meta, fit = _setup()
    fit.run(rings=meta["rings"])
    together = {ir: [f for _, f in fit.log[ir]] for ir in meta["rings"]}
    _, _, fit1 = _setup()
    fit1.run(rings=[meta["rings"][1]])
    assert [f for _, f in fit1.log[meta["rings"][1]]] == together[meta["rings"][1]]
