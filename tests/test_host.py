"""Host-side mirror of the reference interface: sub-ring tables, model rings, beam kernels (no GPU)."""
import json

import numpy as np
import pytest

import golden_io as G
from bbarolo2_gb300 import configs, galmod
from bbarolo2_gb300.beam import BeamKernel


def _cases():
    z = G.load("subrings.npz")
    return [(z, m) for m in json.loads(str(z["index"]))]


def _rebuild(name):
    """The (cube, rings, ringmode) of a named fixture case (same constructions as make_golden.py)."""
    import importlib.util
    import os
    import sys
    spec = importlib.util.spec_from_file_location("mg_cases", os.path.join(G.GOLDEN, "cases.py"))
    mod = importlib.util.module_from_spec(spec)
    sys.modules["mg_cases"] = mod
    spec.loader.exec_module(mod)
    return mod.case(name)


@pytest.mark.parametrize("case", _cases(), ids=lambda c: c[1]["name"])
def test_subrings_bit_equal(case):
    z, m = case
    cube, rings, mode = _rebuild(m["name"])
    st = galmod.GalmodSetup(cube, densflux=True)
    mr = galmod.model_rings(rings, mode, st.radsep)
    assert np.array_equal(np.asarray(mr.radii, float), z[m["name"] + "/model_radii"])
    sr, nv = st.subrings(mr)
    assert np.array_equal(sr, z[m["name"] + "/sr"])
    assert np.array_equal(nv, z[m["name"] + "/nv"])


@pytest.mark.parametrize("case", _cases(), ids=lambda c: c[1]["name"])
def test_subrings_batch_equal_single(case):
    """The vectorised batch tables equal the per-set tables."""
    z, m = case
    cube, rings, mode = _rebuild(m["name"])
    st = galmod.GalmodSetup(cube, densflux=True)
    mr = galmod.model_rings(rings, mode, st.radsep)
    rows = galmod.ring_rows_batch([mr, mr])
    rows[1, 4] *= 1.1          # vrot
    sr, nv = galmod.subrings_batch(st, mr, rows)
    assert np.array_equal(sr[0], z[m["name"] + "/sr"])
    r2 = mr.copy()
    r2.vrot = rows[1, 4].copy()
    s2, n2 = st.subrings(r2)
    assert np.array_equal(sr[1], s2) and np.array_equal(nv[1], n2)


@pytest.mark.parametrize("case", _cases(), ids=lambda c: c[1]["name"])
def test_subrings_batch_gradient_steps(case):
    """A finite-difference batch (member 0, then one ring's value stepped per member, fewer than a quarter of
    the values changed): the tables built from member 0's plus the sub-rings next to the stepped rings equal,
    bit for bit, the per-set tables."""
    z, m = case
    cube, rings, mode = _rebuild(m["name"])
    st = galmod.GalmodSetup(cube, densflux=True)
    mr = galmod.model_rings(rings, mode, st.radsep)
    base = galmod.ring_rows_batch([mr])[0]
    rows = [base]
    for j in range(mr.nr):
        for row, step in ((4, 3.0), (12, 1.0)):
            r = base.copy()
            r[row, j] += step
            rows.append(r)
    rows = np.stack(rows)
    sr, nv = galmod.subrings_batch(st, mr, rows)
    for k in (0, 1, 2, len(rows) // 2, len(rows) - 1):
        r2 = mr.copy()
        r2.vrot, r2.inc = rows[k, 4].copy(), rows[k, 12].copy()
        s2, n2 = st.subrings(r2)
        assert np.array_equal(sr[k], s2) and np.array_equal(nv[k], n2), k


@pytest.mark.parametrize("edges", [False, True])
@pytest.mark.parametrize("case", _cases(), ids=lambda c: c[1]["name"])
def test_subrings_batch_native(case, edges):
    """The C++ tables (bbgpu_subrings_rows) against the numpy ones, bit for bit: random batches (every member
    differs from member 0 in random rings), gradient batches, an outer edge and side edges, the copy into the
    first columns of a wider table."""
    if galmod._native_subrings() is None:
        pytest.skip("library not built")
    z, m = case
    cube, rings, mode = _rebuild(m["name"])
    st = galmod.GalmodSetup(cube, densflux=True)
    mr = galmod.model_rings(rings, mode, st.radsep)
    if edges:
        mr.edge, mr.edgewidth = float(mr.radii[-1] * 60. * 0.8), 0.
        mr.edgeapp, mr.edgerec = float(mr.radii[-1] * 60. * 0.7), float(mr.radii[-1] * 60. * 0.9)
    if mr.thick() or mr.nr < 2:
        pytest.skip("thick layer or one ring: numpy tables")
    base = galmod.ring_rows_batch([mr])[0]
    rng = np.random.default_rng(5)
    rand = base[None].repeat(12, axis=0)
    for k in range(1, 12):
        sel = rng.random(mr.nr) < 0.3
        for row in (1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13):
            rand[k, row, sel] += rng.normal(0., 0.5, sel.sum()) * (1. + abs(base[row, sel]))
        rand[k, 5] = np.abs(rand[k, 5])
        rand[k, 10] = np.abs(rand[k, 10])
        rand[k, 11] = np.abs(rand[k, 11])
    rand[3, 5, :] = 0.                               # (no dispersion: one velocity sample)
    grad = [base]
    for j in range(mr.nr):
        for row, step in ((4, 3.0), (12, 1.0), (10, 0.5)):
            r = base.copy()
            r[row, j] += step
            grad.append(r)
    for rows in (rand, np.stack(grad)):
        sr0, nv0 = galmod.subrings_batch(st, mr, rows, native=False)
        ms = np.full(sr0.shape[:2] + (sr0.shape[2] + 3,), 7.)
        sr1, nv1 = galmod.subrings_batch(st, mr, rows, out_ms=ms)
        assert np.array_equal(sr0.view(np.uint64), sr1.view(np.uint64))
        assert np.array_equal(nv0, nv1)
        assert np.array_equal(ms[:, :, :sr0.shape[2]], sr0) and np.all(ms[:, :, sr0.shape[2]:] == 7.)


@pytest.mark.parametrize("wl", ["classic64", "global160", "bayes256"])
def test_beam_kernel(wl):
    z = G.load("beam_conv.npz")
    cube, _ = configs.WORKLOADS[wl]()
    bk = BeamKernel.from_cube(cube)
    assert np.array_equal(bk.kernel, z[wl + "/kernel"])
    assert bk.scalefac == float(z[wl + "/scalefac_coldens"])


def test_beam_kernel_swapped_axes():
    from bbarolo2_gb300.cube import Cube
    z = G.load("beam_conv.npz")
    cube = Cube.empty(64, 64, 64, [-10. / 3600., 10. / 3600., 5.], beam=[20. / 3600., 40. / 3600., 10.], crota=15.,
                      cunit=("deg", "deg", "km/s"))
    assert np.array_equal(BeamKernel.from_cube(cube).kernel, z["swapped/kernel"])


def test_subring_errors():
    cube, rings = configs.classic64()
    st = galmod.GalmodSetup(cube)
    r = rings.copy()
    r.vdisp[2] = -1
    with pytest.raises(ValueError):
        st.subrings(r)
    r = rings.copy()
    r.radii[3] = r.radii[2]
    with pytest.raises(galmod.BBaroloError):
        st.subrings(r)
    with pytest.raises(galmod.BBaroloError):
        galmod.model_rings(rings.subset(np.array([0])), "NODES")


def test_batch_boxes_match_model_box():
    """The vectorised model boxes of a batch equal DiskModel.box(final=True) clipped to the likelihood box, ring
    set by ring (bbarolo/bayesian/likelihood.py:429-436)."""
    import types
    from bbarolo2_gb300 import configs, engine
    from bbarolo2_gb300.galmod import arcsconv, ring_rows_batch
    from bbarolo2_gb300.rings import RING_KEYS
    cube, rings = configs.global160()
    g = np.random.default_rng(3)
    for mode, thick in (("CENTRED", False), ("NODES", True), ("SHIFTED", False)):
        r = rings.copy()
        if thick:
            r.fthick = np.full(r.nr, 0.3)
            r.z0thick = np.full(r.nr, 25.)
        fake = types.SimpleNamespace(cin=cube, ringmode=mode, arcconv=arcsconv(cube.Head().Cunit(0)))
        rows = np.repeat(ring_rows_batch([r])[0][None], 12, axis=0)
        rows[:, RING_KEYS.index("xpos")] += g.uniform(-20, 20, (12, 1))
        rows[:, RING_KEYS.index("ypos")] += g.uniform(-20, 20, (12, 1))
        rows[:, RING_KEYS.index("z0")] *= g.uniform(0.5, 3., (12, 1))
        like = types.SimpleNamespace(model=fake, likebox=([7, 3], [150, 155]))
        blo, bhi = engine.BatchLikelihood._boxes(like, rows, r)
        for k in range(12):
            rk = r.copy()
            for j, key in enumerate(RING_KEYS):
                setattr(rk, key, rows[k, j].copy())
            lo, hi = engine.DiskModel.box(fake, rk, final=True)
            lo = [max(lo[0], 7), max(lo[1], 3)]
            hi = [max(min(hi[0], 150), lo[0]), max(min(hi[1], 155), lo[1])]
            assert list(blo[k]) == lo and list(bhi[k]) == hi, (mode, k)


def test_count_ring_pixels_matches_reference_rule():
    """The annulus pixel count of a ring (``_count_ring_pixels`` of bbarolo/galfit.py:199-216) on a box crossing
    the cube edge."""
    from bbarolo2_gb300.classic import ring_pixels
    m = np.zeros((30, 40), np.int32)
    m[5:20, 10:35] = 3
    nt, ni = ring_pixels(m, (2, 3), (39, 32), 20.5, 12.0, 30., 50., 4., 9.)
    # the same count written out pixel by pixel
    import math
    F = math.pi / 180.
    sphi, cphi, cinc = math.sin(F * 30.), math.cos(F * 30.), math.cos(F * 50.)
    t = i = 0
    for y in range(3, 33):
        for x in range(2, 40):
            xx, yy = x - 2, y - 3
            xr = -(xx - 20.5) * sphi + (yy - 12.0) * cphi
            yr = (-(xx - 20.5) * cphi - (yy - 12.0) * sphi) / cinc
            r = math.sqrt(xr * xr + yr * yr)
            if 4. <= r <= 9.:
                t += 1
                if y < 30 and x < 40 and m[y, x] > 0:
                    i += 1
    assert (nt, ni) == (t, i)


def test_prepare_maps_table(monkeypatch):
    """BatchLikelihood.prepare (no device: a stub context): the ring maps' table is the model's sub-ring tables
    followed by the exterior annulus' (written in place), bit for bit the tables of the numpy path, for a
    finite-difference batch and a batch of independent points."""
    from bbarolo2_gb300 import _lib, engine

    class _Calls:
        def __getattr__(self, name):
            return lambda *a, **k: 0

    class _StubContext:
        def __init__(self, device=0):
            self.L, self.h = _Calls(), None

        def check(self, rc):
            return rc

    monkeypatch.setattr(_lib, "Context", _StubContext)
    cube, rings = configs.global160(galmodtype="MC")
    dm = engine.DiskModel(cube)
    data = np.ones(cube.array.shape, np.float32)
    L = engine.BatchLikelihood(dm, data, np.ones(cube.array.shape, bool), maskmode=2, sigma=1.0)
    L.set_profile(rings, *L.data_maps(), smooth=0.3, corr=2.0, beam_arcsec=30.)
    base = galmod.ring_rows_batch([rings])[0]
    grad = [base]
    for j in (0, rings.nr // 2, rings.nr - 1):
        for row, step in ((4, 5.0), (12, 2.0), (13, 3.0)):
            r = base.copy()
            r[row, j] += step
            grad.append(r)
    rng = np.random.default_rng(7)
    rand = np.repeat(base[None], 9, axis=0)
    rand[1:, 4] += rng.normal(0., 5., rand[1:, 4].shape)
    rand[1:, 12] += rng.normal(0., 2., rand[1:, 12].shape)
    for rows in (np.stack(grad), rand):
        sr, nv, _, _ = L.prepare(rows, rings, seed=1)
        ms = L._maps_sr.copy()
        assert np.array_equal(ms, np.concatenate([sr, L.profile_maps(rows)], axis=2))
        monkeypatch.setattr(galmod, "_NATIVE", False)
        sr0, nv0, _, _ = L.prepare(rows, rings, seed=1)
        monkeypatch.setattr(galmod, "_NATIVE", None)
        assert np.array_equal(sr.view(np.uint64), sr0.view(np.uint64)) and np.array_equal(nv, nv0)
        assert np.array_equal(ms.view(np.uint64), L._maps_sr.view(np.uint64))


@pytest.mark.parametrize("wl", ["classic64", "global160"])
def test_oracle_host_setup_equals_package(wl):
    """The package's host set-up (constants, sub-ring tables, boxes, beam kernel, ring weights) equals the plain
    restatement of the reference under oracle/ on the benchmark workloads (the CPU reference arm uses the latter)."""
    from bbarolo2_gb300 import configs, galmod
    from bbarolo2_gb300.beam import BeamKernel
    from oracle import host
    cube, rings = configs.WORKLOADS[wl]()
    st = galmod.GalmodSetup(cube)
    ho = host.Setup(cube)
    for a in ("pixarea", "crota2", "crval3", "cdelt3", "crpix3", "chwidth", "sig_instr", "radsep", "freq0"):
        assert getattr(st, a) == getattr(ho, a), a
    assert st.cdelt == ho.cdelt
    np.testing.assert_array_equal(st.cd2i, ho.cd2i)
    np.testing.assert_array_equal(st._vedges, ho.vedges)
    assert st._chmin == ho.chmin
    mr = galmod.model_rings(rings, "CENTRED", st.radsep)
    mo = host.model_rings(rings, "CENTRED", ho.radsep)
    np.testing.assert_array_equal(mr.radii, mo.radii)
    sr, nv = st.subrings(mr)
    so, no = host.subrings(ho, mo)
    np.testing.assert_array_equal(sr, so)
    np.testing.assert_array_equal(nv, no)
    np.testing.assert_array_equal(BeamKernel.from_cube(cube).kernel, host.beam_kernel(cube))
    assert galmod.outer_edge(rings, "CENTRED") == host.outer_edge_centred(rings)


def test_classic_simplex_on_a_quadratic():
    """The simplex coroutine of the CLASSIC fit minimises a quadratic bowl (no bounds: each point evaluated as
    given), converging within its tolerance and budget."""
    from bbarolo2_gb300.classic import simplex
    co = simplex([3.0, -2.0], [1.0, 1.0], 1e-10, 2000)
    pt = next(co)
    n = 0
    try:
        while True:
            f = (pt[0] - 1.0) ** 2 + 2.0 * (pt[1] + 0.5) ** 2 + 3.0
            n += 1
            pt = co.send((f, np.array(pt)))
    except StopIteration as e:
        ok, fmin, xmin = e.value
    assert ok and abs(fmin - 3.0) < 1e-8 and np.allclose(xmin, [1.0, -0.5], atol=1e-4), (ok, fmin, xmin, n)


def test_classic_bounds_rules():
    """Trial values outside the bounds: VROT and VDISP redrawn inside (one deviate each), INC and PA clipped within
    their deltas of the initial value, the others reset to it."""
    from bbarolo2_gb300.classic import Limits, into_bounds
    draws = iter([0.25, 0.5])
    vrot = Limits(0., 1000., "redraw", 50.)
    assert into_bounds("vrot", 300., vrot, 120., lambda: next(draws)) == 170. - 0.25 * 50.
    vd = Limits(1., 40., "redraw")
    assert into_bounds("vdisp", 0.5, vd, 8., lambda: next(draws)) == 1. + 0.5 * 8.
    assert into_bounds("inc", 80., Limits(40., 70., "clip", 5.), 60., None) == 65.
    assert into_bounds("z0", -1., Limits(0., 1000., "reset"), 3., None) == 3.
    assert into_bounds("dens", -1., Limits(0., np.inf, "reset"), 0.7, None) == 0.7
    assert into_bounds("vrot", 130., vrot, 120., None) == 130.
