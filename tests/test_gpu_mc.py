"""GPU parity of the MC model (the reference's _galmod_mc) against the golden fixtures and the CPU oracle.

Every sub-cloud's pixel and channel index must equal the reference's: the device sums the deposits in 64-bit
fixed point, so equal indices give values equal to the reference's float64 sums within 1e-12 relative, and a
single misplaced sub-cloud changes a voxel by a whole deposit (~1e-3 of a voxel or more)."""
import numpy as np
import pytest

import golden_io as G

pytestmark = pytest.mark.gpu


_Ctx = G.DeviceCase


def _cases():
    z, idx = G.cases("mc.npz")
    return [(z, m) for m in idx]


@pytest.mark.parametrize("case", _cases(), ids=lambda c: c[1]["name"])
def test_mc_matches_reference(gpu_lib, case):
    z, m = case
    nm = m["name"]
    ctx = _Ctx(m, z, nm)
    sr = z[nm + "/sr"]
    out = np.zeros(m["shape"])
    ctx.mc(out, sr, 0, sr.shape[1], m["seed32"], z[nm + "/nv"], m["blo"], m["bhi"])
    ref = G.dense(z[nm + "/idx"], z[nm + "/val"], m["shape"])
    assert np.array_equal(out != 0, ref != 0), "different voxels"
    np.testing.assert_allclose(out, ref, rtol=1e-12, atol=0)
    # deterministic, and accumulated as the reference kernel: a second call adds exactly the same model
    first = out.copy()
    ctx.mc(out, sr, 0, sr.shape[1], m["seed32"], z[nm + "/nv"], m["blo"], m["bhi"])
    np.testing.assert_array_equal(out, 2 * first)


def test_mc_box_is_crop(gpu_lib):
    """The model in a box is the crop of the full model (the reference's test_mc_model_in_box_is_crop)."""
    z, idx = G.cases("mc.npz")
    m = [c for c in idx if c["name"] == "classic64"][0]
    ctx = _Ctx(m, z, "classic64")
    sr, nv = z["classic64/sr"], z["classic64/nv"]
    full = ctx.mc(np.zeros((64, 64, 64)), sr, 0, sr.shape[1], 1, nv, (0, 0), (64, 64))
    box = ctx.mc(np.zeros((37, 29, 64)), sr, 0, sr.shape[1], 1, nv, (20, 11), (49, 48))
    np.testing.assert_array_equal(box, full[11:48, 20:49])


def test_mc_ring_range_is_chunk(gpu_lib, oracle_lib):
    """ring_lo/ring_hi: a chunk of sub-rings with its own stream (the threaded builds, seed + 7919 k)."""
    z, idx = G.cases("mc.npz")
    m = [c for c in idx if c["name"] == "sech2_lag"][0]
    ctx = _Ctx(m, z, "sech2_lag")
    sr, nv = z["sech2_lag/sr"], z["sech2_lag/nv"]
    seed = (m["seed32"] + 7919 * 2) & 0xFFFFFFFF
    out = ctx.mc(np.zeros(m["shape"]), sr, 5, 14, seed, nv, m["blo"], m["bhi"])
    ref = np.zeros(m["shape"])
    args = list(G.call_args_mc(m, z, "sech2_lag"))
    args[0] = seed
    oracle_lib.galmod_mc(ref, sr, 5, 14, *args)
    np.testing.assert_allclose(out, ref, rtol=1e-12, atol=0)


@pytest.mark.parametrize("wl", ["global160", "bayes256"])
def test_mc_full_workloads_vs_oracle(gpu_lib, oracle_lib, wl):
    """The benchmark workloads at full size: device vs the CPU oracle (bit-exact indices)."""
    from bbarolo2_gb300 import configs, engine
    from bbarolo2_gb300.galmod import model_rings
    cube, rings = configs.WORKLOADS[wl](galmodtype="MC")
    dm = engine.DiskModel(cube)
    st = dm.setup
    mr = model_rings(rings, dm.ringmode, st.radsep)
    sr, nv = st.subrings(mr)
    nx, ny, nz = cube.DimX(), cube.DimY(), cube.DimZ()
    out = dm.galmod_mc(np.zeros((ny, nx, nz)), sr, 0, sr.shape[1], 1, nv, (0, 0), (nx, ny))
    ref = np.zeros((ny, nx, nz))
    oracle_lib.galmod_mc(ref, sr, 0, sr.shape[1], 1, st.radsep, nv, st.cdens, st.cmode, st.pixarea, st.cdelt[0],
                         st.cdelt[1], st.crota2, 0, 0, nx, ny, st.ltype, st.sig_instr, st.axtyp, st.velsys, st.lfreq0,
                         st.crval3, st.cdelt3, st.crpix3, st.relint, st.cd2i)
    assert np.array_equal(out != 0, ref != 0)
    np.testing.assert_allclose(out, ref, rtol=1e-12, atol=0)


@pytest.mark.parametrize("wl", ["classic64", "global160"])
def test_batch_path_models_bit_exact(gpu_lib, oracle_lib, wl):
    """The unsmoothed float32 models of the batch path (the kernels the likelihood uses) against the oracle:
    the same voxels, values within float32 rounding (a misplaced sub-cloud moves a whole deposit)."""
    from bbarolo2_gb300 import _lib, configs, engine
    from bbarolo2_gb300.galmod import ring_rows_batch
    cube, rings = configs.WORKLOADS[wl](galmodtype="MC")
    dm = engine.DiskModel(cube)
    st = dm.setup
    data = np.zeros(cube.array.shape, np.float32)
    L = engine.BatchLikelihood(dm, data + 1.0, None, maskmode=0, sigma=1.0)
    rows = ring_rows_batch([rings] * 3)
    rows[1, 4] *= 1.07
    rows[2, 12] += 3.0
    sr, nv, descs, boxes = L.prepare(rows, rings, seed=1)
    L.run(sr, nv, descs)
    for k in range(3):
        (blo, bhi) = boxes[k]
        by, bx = bhi[1] - blo[1], bhi[0] - blo[0]
        got = np.zeros((by, bx, st.nsubs), np.float32)
        dm.ctx.check(dm.ctx.L.bbgpu_eval_model(dm.ctx.h, k, 0, _lib.ptr(got), by, bx, st.nsubs))
        ref = np.zeros((by, bx, st.nsubs))
        oracle_lib.galmod_mc(ref, sr[k], 0, sr.shape[2], 1, st.radsep, nv[k], st.cdens, st.cmode, st.pixarea,
                             st.cdelt[0], st.cdelt[1], st.crota2, blo[0], blo[1], bhi[0], bhi[1], st.ltype,
                             st.sig_instr, st.axtyp, st.velsys, st.lfreq0, st.crval3, st.cdelt3, st.crpix3, st.relint,
                             st.cd2i)
        assert np.array_equal(got != 0, ref != 0), k
        np.testing.assert_allclose(got, ref, rtol=1e-6, atol=0)


def _batch_vs_oracle(oracle_lib, cube, rings):
    """The batch path's float32 models of three ring sets against the oracle (same voxels, float32 values)."""
    from bbarolo2_gb300 import _lib, engine
    from bbarolo2_gb300.galmod import ring_rows_batch
    dm = engine.DiskModel(cube)
    st = dm.setup
    L = engine.BatchLikelihood(dm, np.ones(cube.array.shape, np.float32), None, maskmode=0, sigma=1.0)
    rows = ring_rows_batch([rings] * 3)
    rows[1, 4] *= 1.07
    rows[2, 12] += 3.0
    sr, nv, descs, boxes = L.prepare(rows, rings, seed=3)
    L.run(sr, nv, descs)
    for k in range(3):
        (blo, bhi) = boxes[k]
        by, bx = bhi[1] - blo[1], bhi[0] - blo[0]
        got = np.zeros((by, bx, st.nsubs), np.float32)
        dm.ctx.check(dm.ctx.L.bbgpu_eval_model(dm.ctx.h, k, 0, _lib.ptr(got), by, bx, st.nsubs))
        ref = np.zeros((by, bx, st.nsubs))
        oracle_lib.galmod_mc(ref, sr[k], 0, sr.shape[2], 3, st.radsep, nv[k], st.cdens, st.cmode, st.pixarea,
                             st.cdelt[0], st.cdelt[1], st.crota2, blo[0], blo[1], bhi[0], bhi[1], st.ltype,
                             st.sig_instr, st.axtyp, st.velsys, st.lfreq0, st.crval3, st.cdelt3, st.crpix3, st.relint,
                             st.cd2i)
        assert np.array_equal(got != 0, ref != 0), k
        np.testing.assert_allclose(got, ref, rtol=1e-6, atol=0)


@pytest.mark.parametrize("variant", ["narrow", "broad", "descending"])
def test_batch_path_line_widths_and_axis(gpu_lib, oracle_lib, variant):
    """The batch deposit counts each cloud's samples per channel in runs: lines so narrow that the 32 samples
    of a lane share one channel (vdisp 0.2 km/s in 5 km/s channels), so broad that a lane's samples spread over
    more than 12 channels (vdisp 90 km/s), and a channel axis that decreases with velocity (samples in
    descending order)."""
    from bbarolo2_gb300 import configs
    from bbarolo2_gb300.cube import Cube, Params
    cube, rings = configs.classic64(galmodtype="MC")
    if variant == "narrow":
        rings.vdisp[:] = 0.2
    elif variant == "broad":
        rings.vdisp[:] = 90.
    else:
        par = Params(CDENS=10, ISEED=1, LTYPE=1, galmodtype="MC")
        cube = Cube.empty(64, 64, 64, [-10. / 3600., 10. / 3600., -5.], beam=30. / 3600., par=par,
                          crpix=[33., 33., 33.], crval=[60., 0., 1000.], cunit=("deg", "deg", "km/s"))
    _batch_vs_oracle(oracle_lib, cube, rings)


@pytest.mark.parametrize("wl", ["classic64", "global160", "classic64_broad"])
def test_batch_path_gradient_members_shared(gpu_lib, oracle_lib, wl):
    """A finite-difference batch (one ring's VROT, VDISP, INC or PA stepped per member): the members that differ
    from member 0 in a few sub-rings are computed as member 0's model plus the difference of those sub-rings'
    clouds (member 0's taken out by its channel-count records, or, with lines broader than their window, deposited
    again negated); their unsmoothed models are, bit for bit, those of the full computation (option 3 off), and
    agree with the oracle's."""
    from bbarolo2_gb300 import _lib, configs, engine
    from bbarolo2_gb300.galmod import ring_rows_batch
    cube, rings = configs.WORKLOADS[wl.replace("_broad", "")](galmodtype="MC")
    if wl.endswith("_broad"):
        rings.vdisp[:] = 90.                       # (a cloud's channels spread beyond the records' window)
    dm = engine.DiskModel(cube)
    st = dm.setup
    L = engine.BatchLikelihood(dm, np.ones(cube.array.shape, np.float32), None, maskmode=0, sigma=1.0)
    base = ring_rows_batch([rings])[0]
    rows = [base]
    for j in sorted({0, rings.nr // 3, rings.nr - 1}):
        for row, step in ((4, 5.0), (5, 1.0), (12, 2.0), (13, 3.0)):
            r = base.copy()
            r[row, j] += step
            rows.append(r)
    rows = np.stack(rows)
    sr, nv, descs, boxes = L.prepare(rows, rings, seed=2)
    models = {}
    for share in (0, 1):
        dm.ctx.set_option(_lib.OPT_SHARE, share)
        ss, _ = L.run(sr, nv, descs)
        ms = []
        for k in range(len(rows)):
            (blo, bhi) = boxes[k]
            got = np.zeros((bhi[1] - blo[1], bhi[0] - blo[0], st.nsubs), np.float32)
            dm.ctx.check(dm.ctx.L.bbgpu_eval_model(dm.ctx.h, k, 0, _lib.ptr(got), got.shape[0], got.shape[1],
                                                   st.nsubs))
            ms.append(got)
        models[share] = (ss, ms)
    dm.ctx.set_option(_lib.OPT_SHARE, 1)
    np.testing.assert_array_equal(models[0][0], models[1][0])
    for k in range(len(rows)):
        np.testing.assert_array_equal(models[0][1][k], models[1][1][k], err_msg=str(k))
    for k in (1, 3, 5, len(rows) - 1):
        (blo, bhi) = boxes[k]
        got = models[1][1][k]
        ref = np.zeros(got.shape)
        oracle_lib.galmod_mc(ref, sr[k], 0, sr.shape[2], 2, st.radsep, nv[k], st.cdens, st.cmode, st.pixarea,
                             st.cdelt[0], st.cdelt[1], st.crota2, blo[0], blo[1], bhi[0], bhi[1], st.ltype,
                             st.sig_instr, st.axtyp, st.velsys, st.lfreq0, st.crval3, st.cdelt3, st.crpix3, st.relint,
                             st.cd2i)
        assert np.array_equal(got != 0, ref != 0), k
        np.testing.assert_allclose(got, ref, rtol=1e-6, atol=0)
