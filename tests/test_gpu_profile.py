"""GPU parity of the flux normalisation: the ring maps, the profile solve (``bbarolo/profile.py``) and the batched
likelihood that recomputes the deconvolved profile of every member (Bayesian3DFIT with DENS not fitted and the
geometry free), against the reference's fixtures and the float64 oracle pipeline.

Tolerances: the device convolves the ring maps in float32 (MAP_TOL of the peak); the densities of a well
conditioned system move by ~1e-8 with float32 map errors (DENS_RTOL), the device solve of the reference's system
(float64 normal equations, SOLVE_RTOL); log L as the other likelihood tests (SS_RTOL)."""
import json

import numpy as np
import pytest

import golden_io as G

pytestmark = pytest.mark.gpu

MAP_TOL = 1e-6
SOLVE_RTOL = 1e-8
DENS_RTOL = 1e-6
SS_RTOL = 1e-5


def _profile_cases():
    z = G.load("profile.npz")
    return z, json.loads(str(z["index"]))


def _model(meta):
    from bbarolo2_gb300 import engine
    from golden.cases import cube64
    cube = cube64(ltype=2) if meta["name"] == "flat" else cube64(ltype=1, crota=15.)
    return engine.DiskModel(cube, ringmode=meta["mode"], galmodtype="ANALYTIC")


def _rings(meta):
    from golden.cases import rings64
    return rings64(**{k: np.asarray(v) for k, v in meta["rings"].items()})


def test_solve_profile_matches_reference(gpu_lib):
    from bbarolo2_gb300 import profile as P
    z, idx = _profile_cases()
    for m in idx:
        nm = m["name"]
        okk, rms, y = z[nm + "/okk"], z[nm + "/rms"], z[nm + "/y"]
        A = z[nm + "/maps"][:, okk].T / rms[okk, None]
        b = y[okk] / rms[okk]
        for smooth, corr in ((0.3, 1.0), (0.3, 4.0), (0.0, 1.0), (1.0, 2.0)):
            x = P.solve_profile(A, b, z[nm + "/Rc"], smooth, corr)
            ref = z[nm + f"/x_{smooth}_{corr}"]
            np.testing.assert_allclose(x, ref, rtol=SOLVE_RTOL, atol=SOLVE_RTOL * np.abs(ref).max())


def test_ring_maps_and_system_match_reference(gpu_lib):
    from bbarolo2_gb300 import profile as P
    z, idx = _profile_cases()
    for m in idx:
        nm = m["name"]
        dm, r = _model(m), _rings(m)
        (Lb, Hb) = m["blo"], m["bhi"]
        A, b, ok, Rc = P.profile_system(dm, r, (Lb, Hb), z[nm + "/y"], z[nm + "/rms"], z[nm + "/ok"],
                                        beam_arcsec=m["beam_arcsec"])
        okk, rms = z[nm + "/okk"], z[nm + "/rms"]
        ref = z[nm + "/maps"][:, okk].T / rms[okk, None]
        assert np.array_equal(ok, okk) and np.array_equal(Rc, z[nm + "/Rc"])
        assert np.abs(A - ref).max() <= MAP_TOL * np.abs(ref).max(), nm
        x = P.solve_profile(A, b, Rc, 0.3, 1.0)
        xr = z[nm + "/x_0.3_1.0"]
        np.testing.assert_allclose(x, xr, rtol=DENS_RTOL, atol=DENS_RTOL * np.abs(xr).max())


def test_ring_maps_fixture(gpu_lib):
    """DiskModel.ring_maps against the reference's maps of ringmaps.npz (three ring conventions)."""
    from bbarolo2_gb300 import engine
    from golden.cases import cube64, rings64
    z, idx = G.cases("ringmaps.npz")
    for m in idx:
        mode = m["mode"]
        z0 = {"CENTRED": 10., "NODES": 0., "SHIFTED": 20.}[mode]
        dm = engine.DiskModel(cube64(ltype=2), ringmode=mode, galmodtype="ANALYTIC")
        r = rings64(z0=z0, dens=np.linspace(3., 0.5, 8), inc=np.linspace(50., 70., 8))
        K = dm.ring_maps(r, m["blo"], m["bhi"])
        ref = z[mode + "/maps"]
        assert np.abs(K - ref).max() <= MAP_TOL * np.abs(ref).max(), mode


def _batch_workload(B=5, bright=1.0):
    """A 64x64x64 MC fit with a sech2 layer: the mock (its flux times `bright`), its likelihood and B ring sets
    (base + steps of INC, PA, VROT: the geometry is free, so the profile changes with each member)."""
    from bbarolo2_gb300 import engine
    from bbarolo2_gb300.galmod import ring_rows_batch
    from golden.cases import cube64, rings64
    cube = cube64(ltype=2)
    r = np.arange(10., 151., 20.)
    rings = rings64(z0=10., dens=0.8 * np.exp(-r / 60.), inc=np.linspace(50., 65., 8))
    dm = engine.DiskModel(cube, galmodtype="MC")
    truth = dm.array(rings, seed=1)
    rms = 0.01 * float(truth.max())
    g = np.random.default_rng(4)
    data = (bright * truth + dm.convolve_planes(g.normal(0., rms, truth.shape)) * 3.).astype(np.float32)
    mask = truth > 0.02 * truth.max()
    L = engine.BatchLikelihood(dm, data, mask, maskmode=2, sigma=rms)
    mom0, mrms, ok = L.data_maps()
    L.set_profile(rings, mom0, mrms, ok, smooth=0.3, corr=2.0, beam_arcsec=30.)
    base = ring_rows_batch([rings])[0]
    rows = np.repeat(base[None], B, axis=0)
    steps = [(12, 3.0), (13, 4.0), (4, 10.0), (12, -2.0)]
    for k in range(1, B):
        row, st = steps[(k - 1) % len(steps)]
        rows[k, row, (2 * k) % rings.nr:] += st
    return dm, L, rings, rows, data


@pytest.mark.parametrize("galmodtype", ["MC", "ANALYTIC"])
def test_batch_profile_vs_oracle(gpu_lib, oracle_lib, galmodtype):
    from oracle import cpu_baseline as CB
    dm, L, rings, rows, data = _batch_workload()
    ll = L.evaluate(rows, rings, seed=1, galmodtype=galmodtype)
    x, st = L.last_profile()
    assert np.all(st == 0), st
    sr, nv, descs, boxes = L.prepare(rows, rings, seed=1)
    P = CB.setup_payload(dm, sr, nv, boxes, 1, data, L.mask, L.maskmode, like=L, rows=rows, proto=rings,
                         galmodtype=galmodtype)
    CB._W.clear()
    CB._W.update(P)
    for k in range(len(rows)):
        xr = CB.profile_dens(k)
        np.testing.assert_allclose(x[k], xr, rtol=DENS_RTOL, atol=DENS_RTOL * np.abs(xr).max())
        ss = CB.evaluate(k)
        ll_ref = L.finish(np.array([ss]), np.zeros(1), [boxes[k]])[0]
        assert abs(ll[k] - ll_ref) <= SS_RTOL * abs(ll_ref), (k, ll[k], ll_ref)
    # the profile is recomputed at each run: a second evaluation gives the same values
    ll2 = L.evaluate(rows, rings, seed=1, galmodtype=galmodtype)
    np.testing.assert_array_equal(ll, ll2)


@pytest.mark.parametrize("galmodtype", ["MC", "ANALYTIC"])
def test_batch_profile_shared_members(gpu_lib, oracle_lib, galmodtype):
    """A finite-difference batch (steps of one ring's VROT, VDISP, INC or PA): the members whose ring maps are
    the base member's (velocity steps) share its profile, those that differ in a few sub-rings (geometry steps)
    get member 0's maps plus the difference; both give, bit for bit, what every member computed from all its
    samples gives, and the densities agree with the oracle's. The same with the stage timers on (the MC clouds'
    lists then built on the context's stream after the flux normalisation, not beside it on the second stream)."""
    from bbarolo2_gb300 import _lib
    from bbarolo2_gb300.galmod import ring_rows_batch
    from oracle import cpu_baseline as CB
    dm, L, rings, _, data = _batch_workload()
    base = ring_rows_batch([rings])[0]
    steps = [(4, 5.0), (5, 1.0), (12, 2.0), (13, 3.0)]
    rows = [base]
    for j in (1, 4, 7):
        for row, st in steps:
            r = base.copy()
            r[row, j] += st
            rows.append(r)
    rows = np.stack(rows)
    ctx = dm.ctx
    res = {}
    try:
        for share, timing in ((0, 0), (1, 0), (1, 1)):
            ctx.set_option(_lib.OPT_SHARE, share)
            ctx.set_option(_lib.OPT_TIMING, timing)
            ll = L.evaluate(rows, rings, seed=1, galmodtype=galmodtype)
            x, st = L.last_profile()
            res[share, timing] = (ll, x, st)
            if share:
                nprof, full, delta, replay = ctx.shared_members()
                assert nprof < len(rows)
                if galmodtype == "MC":    # (velocity steps as a difference, geometry steps replaying member 0's)
                    assert delta > 0 and replay > 0, (full, delta, replay)
            if timing:
                assert ctx.run_times()["prof_solve"] > 0
    finally:
        ctx.set_option(_lib.OPT_SHARE, 1)
        ctx.set_option(_lib.OPT_TIMING, 0)
    for key in ((0, 0), (1, 1)):
        for i in range(3):
            np.testing.assert_array_equal(res[key][i], res[1, 0][i])
    ll, x, st = res[1, 0]
    assert np.all(st == 0), st
    sr, nv, descs, boxes = L.prepare(rows, rings, seed=1)
    P = CB.setup_payload(dm, sr, nv, boxes, 1, data, L.mask, L.maskmode, like=L, rows=rows, proto=rings,
                         galmodtype=galmodtype)
    CB._W.clear()
    CB._W.update(P)
    for k in (0, 1, 3, 4, 11, 12):
        xr = CB.profile_dens(k)
        np.testing.assert_allclose(x[k], xr, rtol=DENS_RTOL, atol=DENS_RTOL * np.abs(xr).max())
    # a batch of other members after it (the rows of the maps are rebuilt at every upload)
    ll2 = L.evaluate(rows[::-1].copy(), rings, seed=1, galmodtype=galmodtype)
    x2, _ = L.last_profile()
    np.testing.assert_array_equal(x2, x[::-1])


def test_batch_profile_changes_mc_layout(gpu_lib, oracle_lib):
    """Data three times brighter than the rings' DENS (8 clouds per pixel of ring area, under the floor of 10): the
    deconvolved profile lifts the densities above the floor, so the members' cloud counts are not those of the
    batch's layout. The batch falls back to evaluating each such member with the profile's densities as its DENS,
    the reference's model: log L against the oracle pipeline, which builds each member's sub-rings from its profile."""
    from oracle import cpu_baseline as CB
    dm, L, rings, rows, data = _batch_workload(B=4, bright=3.0)
    ll = L.evaluate(rows, rings, seed=1)
    sr, nv, descs, boxes = L.prepare(rows, rings, seed=1)
    P = CB.setup_payload(dm, sr, nv, boxes, 1, data, L.mask, L.maskmode, like=L, rows=rows, proto=rings)
    CB._W.clear()
    CB._W.update(P)
    for k in range(len(rows)):
        x = CB.profile_dens(k)
        assert x[:rings.nr].max() * 10 > 10, x            # (above the floor: another layout)
        ll_ref = L.finish(np.array([CB.evaluate(k)]), np.zeros(1), [boxes[k]])[0]
        assert abs(ll[k] - ll_ref) <= SS_RTOL * abs(ll_ref), (k, ll[k], ll_ref)
