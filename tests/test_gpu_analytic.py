"""GPU parity of the ANALYTIC model and ring maps (the reference's _galmod_analytic / _ring_maps_analytic) against
the golden fixtures and the CPU oracle.

Pixels, channels and the float64 value of every deposit are the reference's; the device sums the deposits in
64-bit fixed point (units of 2^-62 of the model's total-flux bound), so the model differs from the reference's
running float64 sums by rounding only: within AN_TOL of the model's peak. A misplaced sample would change a
voxel by a whole deposit (above 1e-4 of the peak)."""
import numpy as np
import pytest

import golden_io as G

pytestmark = pytest.mark.gpu

AN_TOL = 1e-12


def _cases(name):
    z, idx = G.cases(name)
    return [(z, m) for m in idx]


def _nzq(sr):
    return 1 if not np.any(sr[6] > 0) else 1024


def _close(out, ref, what):
    peak = np.abs(ref).max()
    err = np.abs(out - ref).max()
    assert err <= AN_TOL * peak, (what, err / peak)
    # every voxel the reference fills above the rounding level is filled, and no other
    big = np.abs(ref) > 1e-9 * peak
    assert np.all(out[big] != 0), what
    assert np.all(np.abs(out[~big]) <= 2e-9 * peak), what


@pytest.mark.parametrize("case", _cases("analytic.npz"), ids=lambda c: c[1]["name"])
def test_analytic_matches_reference(gpu_lib, case):
    z, m = case
    nm = m["name"]
    ctx = G.DeviceCase(m, z, nm)
    sr = z[nm + "/sr"]
    out = np.zeros(m["shape"])
    ctx.analytic(out, sr, 0, sr.shape[1], _nzq(sr), m["blo"], m["bhi"])
    ref = G.dense(z[nm + "/idx"], z[nm + "/val"], m["shape"])
    _close(out, ref, nm)
    # deterministic, and accumulated as the reference kernel: a second call adds exactly the same model
    first = out.copy()
    ctx.analytic(out, sr, 0, sr.shape[1], _nzq(sr), m["blo"], m["bhi"])
    np.testing.assert_array_equal(out, 2 * first)


def test_analytic_ring_range_vs_oracle(gpu_lib, oracle_lib):
    """ring_lo/ring_hi select sub-rings; a thick lagging layer with a vertical gradient (profiles per height)."""
    z, idx = G.cases("analytic.npz")
    m = [c for c in idx if c["name"] == "thick_sideedge"][0]
    nm = m["name"]
    ctx = G.DeviceCase(m, z, nm)
    sr = z[nm + "/sr"]
    lo, hi = 3, sr.shape[1] - 2
    for blo, bhi in (((0, 0), (64, 64)), ((13, 7), (41, 59))):
        shape = (bhi[1] - blo[1], bhi[0] - blo[0], m["nz"])
        out = ctx.analytic(np.zeros(shape), sr, lo, hi, 1024, blo, bhi)
        mm = dict(m, blo=list(blo), bhi=list(bhi))
        ref = oracle_lib.galmod_analytic(np.zeros(shape), sr, lo, hi, *G.call_args_an(mm, z, nm, 1024), None,
                                         m["zstep"])
        _close(out, ref, (blo, bhi))


def test_analytic_nzq_limits(gpu_lib, oracle_lib):
    """Few vertical samples allowed (nzq = 2, 7): the grid coarsens as the reference's."""
    z, idx = G.cases("analytic.npz")
    m = [c for c in idx if c["name"] == "exp_layer_nv20"][0]
    nm = m["name"]
    ctx = G.DeviceCase(m, z, nm)
    sr = z[nm + "/sr"]
    for nzq in (2, 7):
        out = ctx.analytic(np.zeros(m["shape"]), sr, 0, sr.shape[1], nzq, m["blo"], m["bhi"])
        ref = oracle_lib.galmod_analytic(np.zeros(m["shape"]), sr, 0, sr.shape[1], *G.call_args_an(m, z, nm, nzq),
                                         None, m["zstep"])
        _close(out, ref, nzq)


def test_analytic_empty_and_zero_density(gpu_lib):
    z, idx = G.cases("analytic.npz")
    m = idx[0]
    nm = m["name"]
    ctx = G.DeviceCase(m, z, nm)
    sr = z[nm + "/sr"].copy()
    out = np.zeros(m["shape"])
    ctx.analytic(out, sr, 2, 2, 1, m["blo"], m["bhi"])
    assert not out.any()
    sr[5] = 0.
    ctx.analytic(out, sr, 0, sr.shape[1], 1, m["blo"], m["bhi"])
    assert not out.any()


@pytest.mark.parametrize("case", _cases("ringmaps.npz"), ids=lambda c: c[1]["mode"])
def test_ring_maps_match_reference(gpu_lib, case):
    z, m = case
    mode = m["mode"]
    ctx = G.DeviceCase(m, z, mode)
    ref = z[mode + "/raw"]
    out = np.zeros_like(ref)
    ctx.ring_maps(out, z[mode + "/sr"], z[mode + "/widx"], z[mode + "/wval"], m["nzq"], m["blo"], m["bhi"])
    peak = np.abs(ref).max()
    assert np.abs(out - ref).max() <= AN_TOL * peak, mode
    assert np.array_equal(out != 0, ref != 0), mode


@pytest.mark.parametrize("variant", ["thin", "thick_lag"])
def test_batch_path_analytic_models(gpu_lib, oracle_lib, variant):
    """The float32 models of the batch path's ANALYTIC GALMOD against the oracle (the reference's float64
    kernel): the float32 path of the line profiles and deposits agrees within 1e-5 of the peak; with a vertical
    lag above zcyl, the sub-rings whose velocity depends on the height take the exact kernel in the same batch."""
    from bbarolo2_gb300 import _lib, configs, engine
    from bbarolo2_gb300.galmod import ring_rows_batch
    cube, rings = configs.classic64(galmodtype="ANALYTIC")
    if variant == "thick_lag":
        rings.z0[:] = 12.
        rings.dvdz[4:] = 6.
        rings.zcyl[:] = 8.
    dm = engine.DiskModel(cube)
    st = dm.setup
    L = engine.BatchLikelihood(dm, np.ones(cube.array.shape, np.float32), None, maskmode=0, sigma=1.0)
    rows = ring_rows_batch([rings] * 3)
    rows[1, 4] *= 1.07
    rows[2, 12] += 3.0
    sr, nv, descs, boxes = L.prepare(rows, rings, seed=1)
    L.run(sr, nv, descs, galmodtype="ANALYTIC")
    for k in range(3):
        (blo, bhi) = boxes[k]
        by, bx = bhi[1] - blo[1], bhi[0] - blo[0]
        got = np.zeros((by, bx, st.nsubs), np.float32)
        dm.ctx.check(dm.ctx.L.bbgpu_eval_model(dm.ctx.h, k, 0, _lib.ptr(got), by, bx, st.nsubs))
        ref = np.zeros((by, bx, st.nsubs))
        nzq = 1 if not np.any(sr[k, 6] > 0) else 1024
        oracle_lib.galmod_analytic(ref, sr[k], 0, sr.shape[2], st.radsep, st.cdens, st.pixarea, st.cdelt[0],
                                   st.cdelt[1], st.crota2, blo[0], blo[1], bhi[0], bhi[1], st.ltype, st.sig_instr,
                                   st._vedges_lines, st.relint, st.cd2i, nzq, st.axtyp, st.velsys, st.lfreq0,
                                   st.crval3, st.cdelt3, st.crpix3, st._chmin, None, st.zstep)
        np.testing.assert_allclose(got, ref, rtol=0, atol=1e-5 * ref.max())
        assert abs(got.sum() - ref.sum()) <= 1e-5 * ref.sum()


@pytest.mark.parametrize("variant", ["thin", "thick_lag"])
def test_batch_path_analytic_gradient_shared(gpu_lib, oracle_lib, variant):
    """A finite-difference batch of the ANALYTIC model (one ring's VROT, VDISP, INC or PA stepped per member): the
    members computed as member 0's model plus the difference of a few sub-rings' samples give, bit for bit, the
    models computed from all their samples (option 3 off), and agree with the oracle's."""
    from bbarolo2_gb300 import _lib, configs, engine
    from bbarolo2_gb300.galmod import ring_rows_batch
    cube, rings = configs.classic64(galmodtype="ANALYTIC")
    if variant == "thick_lag":
        rings.z0[:] = 12.
        rings.dvdz[4:] = 6.
        rings.zcyl[:] = 8.
    dm = engine.DiskModel(cube)
    st = dm.setup
    L = engine.BatchLikelihood(dm, np.ones(cube.array.shape, np.float32), None, maskmode=0, sigma=1.0)
    base = ring_rows_batch([rings])[0]
    rows = [base]
    for j in (1, 5):
        for row, step in ((4, 5.0), (5, 1.0), (12, 2.0), (13, 3.0)):
            r = base.copy()
            r[row, j] += step
            rows.append(r)
    rows = np.stack(rows)
    sr, nv, descs, boxes = L.prepare(rows, rings, seed=1)
    models = {}
    for share in (0, 1):
        dm.ctx.set_option(_lib.OPT_SHARE, share)
        ss, _ = L.run(sr, nv, descs, galmodtype="ANALYTIC")
        ms = []
        for k in range(len(rows)):
            (blo, bhi) = boxes[k]
            got = np.zeros((bhi[1] - blo[1], bhi[0] - blo[0], st.nsubs), np.float32)
            dm.ctx.check(dm.ctx.L.bbgpu_eval_model(dm.ctx.h, k, 0, _lib.ptr(got), got.shape[0], got.shape[1],
                                                   st.nsubs))
            ms.append(got)
        models[share] = (ss, ms)
        if share:
            _, full, delta, _ = dm.ctx.shared_members()
            assert delta > 0, (full, delta)
    dm.ctx.set_option(_lib.OPT_SHARE, 1)
    np.testing.assert_array_equal(models[0][0], models[1][0])
    for k in range(len(rows)):
        np.testing.assert_array_equal(models[0][1][k], models[1][1][k], err_msg=str(k))
    for k in (1, 2, 5):
        (blo, bhi) = boxes[k]
        got = models[1][1][k]
        ref = np.zeros(got.shape)
        nzq = 1 if not np.any(sr[k, 6] > 0) else 1024
        oracle_lib.galmod_analytic(ref, sr[k], 0, sr.shape[2], st.radsep, st.cdens, st.pixarea, st.cdelt[0],
                                   st.cdelt[1], st.crota2, blo[0], blo[1], bhi[0], bhi[1], st.ltype, st.sig_instr,
                                   st._vedges_lines, st.relint, st.cd2i, nzq, st.axtyp, st.velsys, st.lfreq0,
                                   st.crval3, st.cdelt3, st.crpix3, st._chmin, None, st.zstep)
        np.testing.assert_allclose(got, ref, rtol=0, atol=1e-5 * ref.max())
