"""The wind models on the CPU: the oracle's restatement of ``bbarolo/windmodel.py`` against the reference's own
kernels (``tests/golden/wind.npz``, made by ``tests/golden/make_wind.py``), and the package's host side of
``bbarolo2_gb300.wind`` (cells, quadrature, beam kernel, host Boxes) against the same fixtures."""
import numpy as np
import pytest

import wind_cases as WC
from golden_io import cases

NAMES = list(WC.CASES)


def _case(name):
    z, idx = cases("wind.npz")
    return {k.split("/", 1)[1]: z[k] for k in z.files if k.startswith(name + "/")}, idx[name]


def _oracle_points(O, a, m, name):
    c = WC.CASES[name]
    g = WC.geometry(c["pars"], m["crota2"])
    from bbarolo2_gb300.wind import WindPars
    P = WindPars(**c["pars"])
    return O.wind_points(a["cells"], a["qn"], a["qoff"], P.radii, P.vwind, P.vdisp, P.vrot, P.xpos, P.ypos, g["vsys"],
                         g["sinc"], g["cinc"], g["spa"], g["cpa"], m["cdelt0"], m["cdelt1"], g["th_in"], g["th_out"],
                         g["rmax"], m["sig_instr"])


@pytest.mark.parametrize("name", NAMES)
def test_oracle_wind_points_match_reference(oracle_lib, name):
    a, m = _case(name)
    pts = _oracle_points(oracle_lib, a, m, name)
    for k in ("gx", "gy", "vel", "sig", "w", "r"):
        np.testing.assert_array_equal(pts[k], a["pts_" + k], err_msg=k)
    np.testing.assert_array_equal(pts["vol"], a["vol"])
    np.testing.assert_array_equal(pts["rbar"], a["rbar"])


@pytest.mark.parametrize("name", NAMES)
def test_oracle_wind_columns_match_reference(oracle_lib, name):
    """Raw boxes, deposit, grown boxes and convolution of the reference's points: bit-equal to the reference."""
    O = oracle_lib
    a, m = _case(name)
    pts = {k: a["pts_" + k] for k in ("gx", "gy", "vel", "sig", "w", "r")}
    wt = WC.point_weight(name, pts["r"])
    w = pts["w"] if wt is None else pts["w"] * wt
    spec = dict(chmin=m["chmin"], axtyp=m["axtyp"], velsys=m["velsys"], lfreq0=a["lfreq0"], crval3=m["crval3"],
                cdelt3=m["cdelt3"], crpix3=m["crpix3"])
    buf, offs, boxes = O.wind_boxes(pts, w, a["lim"], tuple(m["shape"]), a["kern"], a["kx"], a["ky"],
                                    bool(a["separable"]), spec, a["vedges"], a["relint"], a["qoff"])
    np.testing.assert_array_equal(boxes, a["boxes"])
    np.testing.assert_array_equal(offs, a["offs"])
    np.testing.assert_array_equal(buf, a["buf"])


@pytest.mark.parametrize("name", NAMES)
def test_oracle_wind_normal_and_model_match_reference(oracle_lib, name):
    O = oracle_lib
    a, m = _case(name)
    shape = tuple(m["shape"])
    W, d, Wd = WC.weights(name, shape)
    G, b = O.wind_normal(a["buf"], a["offs"], a["boxes"], Wd, W, a["lim"], m["rel"])
    np.testing.assert_array_equal(G, a["G"])
    np.testing.assert_array_equal(b, a["b"])
    np.testing.assert_array_equal(O.wind_scatter(shape, a["buf"], a["offs"], a["boxes"], a["amp"]), a["model"])


@pytest.mark.parametrize("name", NAMES)
def test_host_cells_quadrature_and_beam_match_reference(name):
    """The package's WindCells, quadrature and beam kernel (no device needed) equal the reference's."""
    from bbarolo2_gb300 import wind
    a, m = _case(name)
    c = WC.CASES[name]
    wm = wind.WindModel(WC.cube(**c["cube"]), WC.make_cells(wind, c["cells"]), smooth=c["smooth"])
    wm.quadrature(*c["quad"])
    np.testing.assert_array_equal(wm.cells.cells, a["cells"])
    np.testing.assert_array_equal(wm.cells.qn, a["qn"])
    np.testing.assert_array_equal(wm.cells.qoff, a["qoff"])
    assert wm.cells.spacing == float(a["spacing"])
    assert (wm.hx, wm.hy) == tuple(a["hxhy"]) and wm.separable == bool(a["separable"])
    np.testing.assert_allclose(wm.kern, a["kern"], rtol=1e-13, atol=1e-17)
    np.testing.assert_allclose(wm.kx, a["kx"], rtol=1e-13)
    np.testing.assert_allclose(wm.ky, a["ky"], rtol=1e-13)
    np.testing.assert_allclose(wm.psfq, a["psfq"], rtol=1e-13)
    np.testing.assert_array_equal(wm.setup._vedges_lines, a["vedges"])
    assert wm.cdelt == (m["cdelt0"], m["cdelt1"])


@pytest.mark.parametrize("name", ["sep", "ell"])
def test_host_boxes_normal_equals_dense(name):
    """Host Boxes (the reference's values): G = A'WA and b = A'Wd of the dense columns when nothing is pruned, and
    the pruned selection equal to the reference's lists."""
    from bbarolo2_gb300 import wind
    a, m = _case(name)
    shape = tuple(m["shape"])
    W, d, Wd = WC.weights(name, shape)
    B = wind.Boxes(a["buf"].copy(), a["offs"], a["boxes"])
    G, b = B.normal(Wd, W, B.voxel_lists(W, a["lim"], rel=m["rel"]))
    np.testing.assert_allclose(G, a["G"], rtol=1e-12, atol=1e-12 * np.abs(a["G"]).max())
    np.testing.assert_allclose(b, a["b"], rtol=1e-12, atol=1e-12 * np.abs(a["b"]).max())
    if m["rel"] == 0:
        A = B.dense(shape)
        np.testing.assert_allclose(G, A.T @ (W.ravel()[:, None] * A), rtol=1e-12, atol=1e-12 * np.abs(G).max())
    np.testing.assert_allclose(B.model(a["amp"], shape), a["model"], rtol=1e-12, atol=1e-15)


# ---------------------------------------------------------------------------------------------- GALWIND WTYPE 1
GW_NAMES = list(WC.GW_CASES)


@pytest.mark.parametrize("name", GW_NAMES)
def test_host_wind_shells_match_reference(name):
    """The package's shells of a GALWIND WTYPE 1 model equal the reference's GalWind._shells."""
    from bbarolo2_gb300.galwind import GalWindPars, wind_setup, wind_shells
    a, m = _case(name)
    c = WC.GW_CASES[name]
    par = GalWindPars(**c["par"])
    sr, nv, sep = wind_shells(par, wind_setup(WC.cube(**c["cube"]), par))
    np.testing.assert_array_equal(sr, a["sr"])
    np.testing.assert_array_equal(nv, a["nv"])
    assert sep == m["sep"]


def gw_oracle(O, a, m, ring_lo, ring_hi, seed, out):
    (b0, b1), (e0, e1) = m["box"]
    return O.galmod_wind(out, a["sr"], ring_lo, ring_hi, seed, m["sep"], a["nv"], m["cdens"], 1, m["pixarea"],
                         m["cdelt0"], m["cdelt1"], m["crota2"], b0, b1, e0, e1, m["sig_instr"], m["axtyp"], m["velsys"],
                         a["lfreq0"], m["crval3"], m["cdelt3"], m["crpix3"], a["relint"], a["cd2i"])


@pytest.mark.parametrize("name", GW_NAMES)
def test_oracle_galmod_wind_matches_reference(oracle_lib, name):
    """The oracle's _galmod_wind over the chunks of shells, summed in chunk order: bit-equal to the reference's."""
    a, m = _case(name)
    out = np.zeros(m["shape"])
    for t, (lo, hi) in enumerate(a["chunks"]):
        buf = gw_oracle(oracle_lib, a, m, int(lo), int(hi), (m["seed"] + 7919 * t) & 0xFFFFFFFF, np.zeros(m["shape"]))
        out += buf
    idx = np.flatnonzero(out)
    np.testing.assert_array_equal(idx, a["idx"])
    np.testing.assert_array_equal(out.ravel()[idx], a["val"])


def test_host_wind_parameter_checks():
    """The reference's refusals: opening angles out of order, a non-positive CONELEN, shells too close, bad cells."""
    from bbarolo2_gb300.galmod import BBaroloError
    from bbarolo2_gb300.galwind import GalWindPars, wind_setup, wind_shells
    from bbarolo2_gb300.wind import WindCells, WindPars
    with pytest.raises(BBaroloError):
        WindPars([50.], 100., 10., openang=30., openin=40.).check()
    with pytest.raises(BBaroloError):
        WindPars([50.], 100., 10., conelen=-1.).check()
    with pytest.raises(BBaroloError):
        WindPars([50., 40.], 100., 10.)
    with pytest.raises(BBaroloError):
        WindPars([10., 50.], [100., 200., 300.], 10.)
    for bad in (dict(redges=[0.]), dict(redges=[10., 5.]), dict(redges=[0., 10.], ntheta=0),
                dict(redges=[0., 10.], thmax=95.), dict(redges=[0., 10.], cones=(2,))):
        with pytest.raises(BBaroloError):
            WindCells(**bad)
    c = WC.GW_CASES["gw_velo"]
    par = GalWindPars(**dict(c["par"], radii=[10., 10.5, 40.]))
    with pytest.raises(BBaroloError):
        wind_shells(par, wind_setup(WC.cube(**c["cube"]), par))
    par = GalWindPars(**dict(c["par"], vdisp=-1.))
    with pytest.raises(BBaroloError):
        wind_shells(par, wind_setup(WC.cube(**c["cube"]), par))


def test_circinus_workload_shapes():
    """The bench's WINDFIT problem has the shapes of the reference's Circinus example (docs/examples/circinus.md:
    3192 cells of 3.6 arcsec on the approaching cone of OPENANG 110 and CONELEN 52 arcsec, 173 x 238 x 41 voxels,
    0.9 arcsec beam), with the quadrature capped at MAX_POINTS."""
    from bbarolo2_gb300 import configs, wind
    wm, p = configs.wind_circinus()
    assert wm.cells.ncell == 3192
    assert wm.shape == (41, 238, 173)
    assert 0 < wm.cells.npoints <= wind.MAX_POINTS
    assert set(wm.cells.cells[:, 0]) == {-1.0}
    assert wm.separable and wm.hx == wm.hy
