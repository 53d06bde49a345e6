"""GPU parity of GALWIND WTYPE 1 (``bbarolo2_gb300.galwind``, ``csrc/galwind.cu``: the Monte-Carlo clouds of the
shells of a bi-cone, the reference's ``_galmod_wind``) against the reference's own runs (``tests/golden/wind.npz``)
and the CPU oracle.

Every cloud's pixel and every velocity sample's channel must equal the reference's: the device sums the deposits in
64-bit fixed point, so equal indices give the reference's float64 sums within 1e-12 relative; one misplaced sample
changes a voxel by a whole deposit."""
import numpy as np
import pytest

import wind_cases as WC
from golden_io import cases
from test_wind_oracle import gw_oracle

pytestmark = pytest.mark.gpu

GW_NAMES = list(WC.GW_CASES)


def _case(name):
    z, idx = cases("wind.npz")
    return {k.split("/", 1)[1]: z[k] for k in z.files if k.startswith(name + "/")}, idx[name]


def _model(name):
    from bbarolo2_gb300.galwind import GalWindMC, GalWindPars
    c = WC.GW_CASES[name]
    return GalWindMC(WC.cube(**c["cube"]), GalWindPars(**c["par"]), threads=c["threads"])


@pytest.mark.parametrize("name", GW_NAMES)
def test_galmod_wind_matches_reference(gpu_lib, oracle_lib, name):
    a, m = _case(name)
    gw = _model(name)
    np.testing.assert_array_equal(gw.sr, a["sr"])
    (b0, b1), (e0, e1) = m["box"]
    dev = np.zeros(m["shape"])
    ora = np.zeros(m["shape"])
    for t, (lo, hi) in enumerate(a["chunks"]):
        seed = (m["seed"] + 7919 * t) & 0xFFFFFFFF
        buf = gw.dm.galmod_wind(np.zeros(m["shape"]), gw.sr, int(lo), int(hi), seed, gw.sep, gw.nv, (b0, b1), (e0, e1))
        dev += buf
        ora += gw_oracle(oracle_lib, a, m, int(lo), int(hi), seed, np.zeros(m["shape"]))
    ref = np.zeros(int(np.prod(m["shape"])))
    ref[a["idx"]] = a["val"]
    ref = ref.reshape(m["shape"])
    assert np.array_equal(dev != 0, ora != 0), "different voxels than the oracle"
    np.testing.assert_allclose(dev, ora, rtol=1e-12, atol=0)
    assert np.array_equal(dev != 0, ref != 0), "different voxels than the reference"
    np.testing.assert_allclose(dev, ref, rtol=1e-12, atol=0)


def test_galwind_model_of_the_cube(gpu_lib, oracle_lib):
    """GalWindMC.model(): the chunks of shells with their streams, the whole cube, (nz, ny, nx); deterministic."""
    a, m = _case("gw_velo")
    gw = _model("gw_velo")
    mod = gw.model()
    ref = np.zeros(int(np.prod(m["shape"])))
    ref[a["idx"]] = a["val"]
    ref = ref.reshape(m["shape"]).transpose(2, 0, 1)
    assert np.array_equal(mod != 0, ref != 0)
    np.testing.assert_allclose(mod, ref, rtol=1e-12, atol=0)
    np.testing.assert_array_equal(gw.model(), mod)
