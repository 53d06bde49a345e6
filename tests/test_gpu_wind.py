"""GPU parity of the wind-model column engine (``bbarolo2_gb300.wind``, ``csrc/wind.cu``) against the reference's
own kernels (``tests/golden/wind.npz``) and the CPU oracle.

Tolerances: the device computes in float64 with the reference's operations; the deposits are float64 atomics (their
order is not fixed) and the sums are trees, so the columns, G and b agree with the reference's sequential sums to
rounding (1e-12 of the largest value). The points use the device's sin and cos (within 2 ulp of the C library's):
positions and velocities agree to 1e-12 relative, which leaves the boxes (integers) equal."""
import numpy as np
import pytest

import wind_cases as WC
from golden_io import cases

pytestmark = pytest.mark.gpu

NAMES = list(WC.CASES)


def _case(name):
    z, idx = cases("wind.npz")
    return {k.split("/", 1)[1]: z[k] for k in z.files if k.startswith(name + "/")}, idx[name]


def _model(name):
    from bbarolo2_gb300 import wind
    c = WC.CASES[name]
    wm = wind.WindModel(WC.cube(**c["cube"]), WC.make_cells(wind, c["cells"]), smooth=c["smooth"])
    return wm.quadrature(*c["quad"]), wind.WindPars(**c["pars"])


def _close(x, ref, rel=1e-12, what=""):
    scale = max(float(np.abs(ref).max()), 1e-300)
    err = float(np.abs(np.asarray(x) - ref).max()) / scale if np.size(ref) else 0.
    assert err <= rel, f"{what}: max error {err:.3g} of the peak (bound {rel:g})"


@pytest.mark.parametrize("name", NAMES)
def test_wind_points_match_reference(gpu_lib, name):
    a, m = _case(name)
    wm, P = _model(name)
    pts = wm.points(P)
    for k in ("gx", "gy", "vel", "sig"):
        np.testing.assert_allclose(pts[k], a["pts_" + k], rtol=1e-12, atol=1e-9, err_msg=k)
    np.testing.assert_allclose(pts["w"], a["pts_w"], rtol=1e-12, atol=0, err_msg="w")
    np.testing.assert_array_equal(pts["r"], a["pts_r"])
    np.testing.assert_allclose(pts["vol"], a["vol"], rtol=1e-12, atol=0)
    np.testing.assert_allclose(pts["rbar"], a["rbar"], rtol=1e-12, atol=0)


@pytest.mark.parametrize("name", NAMES)
def test_wind_columns_of_reference_points(gpu_lib, name):
    """The reference's points in: boxes equal, column values within 1e-12 of the peak."""
    a, m = _case(name)
    wm, P = _model(name)
    pts = {k: a["pts_" + k] for k in ("gx", "gy", "vel", "sig", "w", "r")}
    B = wm.boxes(P, lim=a["lim"], pts=pts, weight=WC.point_weight(name, pts["r"]))
    np.testing.assert_array_equal(B.boxes, a["boxes"])
    np.testing.assert_array_equal(B.offs, a["offs"])
    _close(B.buf, a["buf"], what="columns")


@pytest.mark.parametrize("name", NAMES)
def test_wind_normal_equations_match_reference(gpu_lib, name):
    """The whole path on the device (points, columns, normal equations, model) against the reference."""
    a, m = _case(name)
    wm, P = _model(name)
    shape = tuple(m["shape"])
    W, d, Wd = WC.weights(name, shape)
    pts = wm.points(P)
    B = wm.boxes(P, lim=a["lim"], pts=pts, weight=WC.point_weight(name, pts["r"]))
    np.testing.assert_array_equal(B.boxes, a["boxes"])
    G, b = B.normal(Wd, W, B.voxel_lists(W, a["lim"], rel=m["rel"]))
    _close(G, a["G"], 1e-11, "G")
    _close(b, a["b"], 1e-11, "b")
    np.testing.assert_array_equal(G, G.T)
    _close(B.model(a["amp"], shape), a["model"], 1e-12, "model")
    assert wm.launches() > 0


def test_wind_normal_equals_dense_columns(gpu_lib):
    """G = A'WA and b = A'Wd of the dense columns read back, the model = A x (bbarolo's
    test_wind_boxes_normal_equations)."""
    wm, P = _model("sep")
    shape = wm.shape
    g = np.random.default_rng(0)
    B = wm.boxes(P)
    A = B.dense(shape)
    x = g.exponential(1., B.n)
    d = A @ x + g.normal(0, 0.1, A.shape[0])
    W = g.uniform(0.5, 2., shape)
    G, b = B.normal(W * d.reshape(shape), W)
    np.testing.assert_allclose(G, A.T @ (W.ravel()[:, None] * A), rtol=1e-12, atol=1e-12 * np.abs(G).max())
    np.testing.assert_allclose(b, A.T @ (W.ravel() * d), rtol=1e-12, atol=1e-12 * np.abs(b).max())
    np.testing.assert_allclose(B.model(x, shape).ravel(), A @ x, rtol=1e-12, atol=1e-12 * np.abs(A @ x).max())
    pts = wm.points(P)
    inside = np.abs(A.sum(axis=0) / np.where(pts["vol"] > 0, pts["vol"], 1.) - 1)[pts["vol"] > 0]
    assert np.median(inside) < 1e-3


def test_wind_stale_boxes_refused(gpu_lib):
    from bbarolo2_gb300.galmod import BBaroloError
    wm, P = _model("sep")
    B1 = wm.boxes(P)
    B2 = wm.boxes(P)
    with pytest.raises(BBaroloError):
        B1.model(np.ones(B1.n), wm.shape)
    B2.model(np.ones(B2.n), wm.shape)


@pytest.mark.parametrize("size", [(48, 40, 160., 12.), (96, 64, 300., 15.)])
def test_wind_large_vs_oracle(gpu_lib, oracle_lib, size):
    """Larger grids of cells (hundreds to a thousand cells, up to 10^6 points) against the oracle run on the device's
    own points (the columns) and on the columns read back (the normal equations)."""
    from bbarolo2_gb300 import wind
    nx, nz, rmax, csize = size
    cube = WC.cube(nx, nz, beam=(30.,))
    wm = wind.WindModel(cube, wind.WindCells.resolved(rmax, 40., csize)).quadrature(200., 10.)
    P = wind.WindPars([rmax * 0.3, rmax * 0.9], [120., 220.], [12., 9.], vrot=[40., 10.], xpos=nx / 2 - 0.3,
                      ypos=nx / 2 + 0.4, inc=55., pa=30., openang=70., openin=10., conelen=rmax * 0.95)
    pts = wm.points(P)
    B = wm.boxes(P, pts=pts)
    su = wm.setup
    spec = dict(chmin=su._chmin, axtyp=su.axtyp, velsys=su.velsys, lfreq0=su.lfreq0, crval3=su.crval3,
                cdelt3=su.cdelt3, crpix3=su.crpix3)
    lim = np.array([0, nx, 0, nx, 0, nz])
    buf, offs, boxes = oracle_lib.wind_boxes(pts, pts["w"], lim, wm.shape, wm.kern, wm.kx, wm.ky, wm.separable, spec,
                                             su._vedges_lines, su.relint, wm.cells.qoff)
    np.testing.assert_array_equal(B.boxes, boxes)
    _close(B.buf, buf, what="columns")
    W, d, Wd = WC.weights("sep", wm.shape)
    G, b = B.normal(Wd, W, B.voxel_lists(W, lim, rel=1e-3))
    Go, bo = oracle_lib.wind_normal(B.buf, B.offs, B.boxes, Wd, W, lim, 1e-3)
    print(f"{wm.cells.ncell} cells, {wm.cells.npoints} points, {B.total} column values")
    _close(G, Go, 1e-11, "G")
    _close(b, bo, 1e-11, "b")


def test_wind_cells_with_large_raw_boxes(gpu_lib, oracle_lib):
    """Cells whose raw boxes exceed the shared-memory deposit (more than 26,624 values: float64 atomics in global
    memory) beside small ones, on one cube: the columns and normal equations against the oracle."""
    import math
    from bbarolo2_gb300 import wind
    cube = WC.cube(96, 60, beam=(30.,))
    wm = wind.WindModel(cube, wind.WindCells([0., 30., 60., 450.], 1, 1, thmax=50.)).quadrature(250., 10.)
    P = wind.WindPars([100.], 220., 10., vrot=30., xpos=47.5, ypos=48.2, inc=55., pa=20., openang=90., conelen=430.)
    pts = wm.points(P)
    B = wm.boxes(P, pts=pts)
    su = wm.setup
    hx, hy = wm.hx, wm.hy
    lim = np.array([0, 96, 0, 96, 0, 60])
    rb = oracle_lib.wind_raw_boxes(wm.cells.qoff, pts["gx"], pts["gy"], pts["vel"], pts["sig"], pts["w"],
                                   lim + np.array([-hx, hx, -hy, hy, 0, 0]), su._chmin, su.axtyp, su.velsys,
                                   su.lfreq0, su.crval3, su.cdelt3, su.crpix3)
    size = (rb[:, 1] - rb[:, 0]) * (rb[:, 3] - rb[:, 2]) * (rb[:, 5] - rb[:, 4])
    assert size.max() > 26624 and np.any((size > 0) & (size < 26624)), size
    spec = dict(chmin=su._chmin, axtyp=su.axtyp, velsys=su.velsys, lfreq0=su.lfreq0, crval3=su.crval3,
                cdelt3=su.cdelt3, crpix3=su.crpix3)
    buf, offs, boxes = oracle_lib.wind_boxes(pts, pts["w"], lim, wm.shape, wm.kern, wm.kx, wm.ky, wm.separable, spec,
                                             su._vedges_lines, su.relint, wm.cells.qoff)
    np.testing.assert_array_equal(B.boxes, boxes)
    _close(B.buf, buf, what="columns")
    W, d, Wd = WC.weights("sep", wm.shape)
    G, b = B.normal(Wd, W)
    Go, bo = oracle_lib.wind_normal(B.buf, B.offs, B.boxes, Wd, W, B.lim(), 0.)
    _close(G, Go, 1e-11, "G")
    _close(b, bo, 1e-11, "b")
    assert math.isfinite(float(G.sum()))


def test_wind_columns_survive_a_points_call(gpu_lib):
    """The columns of a boxes() call stay usable after the points of another wind are computed."""
    wm, P = _model("sep")
    B = wm.boxes(P)
    m1 = B.model(np.ones(B.n), wm.shape)
    wm.points(WindParsShift(P))
    # (the model's sums of overlapping columns are float64 atomics: equal to rounding)
    np.testing.assert_allclose(B.model(np.ones(B.n), wm.shape), m1, rtol=1e-13, atol=1e-15 * np.abs(m1).max())


def WindParsShift(P):
    q = P.copy()
    q.inc += 5.
    return q
