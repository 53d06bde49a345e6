"""Beams wider than the shared-memory templates of the float32 convolution (widths above 31 taps, or tiles above
220 KB): the 64x64x64 mock with circular beams of 90" and 200" FWHM on 10" pixels (33x33 and 73x73 kernels) and an
elliptical 120" x 60" beam at BPA 30 degrees (39x23), through the batch path (k_conv_wide: the taps in global memory).
Every voxel of the smoothed models within 1e-5 relative of the FP64 oracle's convolution above 1e-6 of the peak,
the sums of squares within SS_RTOL of the oracle pipeline's, and the flux normalisation (the ring maps convolved by
the same kernel) within the profile tests' tolerances."""
import numpy as np
import pytest

from test_gpu_likelihood import SS_RTOL, _oracle_ss

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5
FLOOR = 1e-6
BEAMS = {"c90": 90., "c200": 200., "e120x60": [120. / 3600., 60. / 3600., 30.]}


def _cube(beam):
    from bbarolo2_gb300.cube import Cube, Params
    par = Params(CDENS=10, ISEED=1, LTYPE=1)
    b = beam / 3600. if np.isscalar(beam) else beam
    return Cube.empty(64, 64, 64, [-10. / 3600., 10. / 3600., 5.], beam=b, par=par, crpix=[33., 33., 33.],
                      crval=[60., 0., 1000.], cunit=("deg", "deg", "km/s"))


def _setup(name, nb=3, seed=0):
    from bbarolo2_gb300 import engine
    from bbarolo2_gb300.galmod import ring_rows_batch
    from golden.cases import rings64
    dm = engine.DiskModel(_cube(BEAMS[name]), galmodtype="MC")
    rings = rings64()
    truth = dm.array(rings, seed=1)
    g = np.random.default_rng(seed)
    sigma = 0.01 * truth.max()
    data = (truth + g.normal(0, sigma, truth.shape)).astype(np.float32)
    mask = truth > 3 * sigma
    L = engine.BatchLikelihood(dm, data, mask, maskmode=2, sigma=sigma)
    rows = ring_rows_batch([rings] * nb)
    rows[1:, 4] *= 1 + 0.05 * g.standard_normal((nb - 1, rings.nr))
    rows[1:, 12] += 3.
    return dm, L, rings, rows, data, mask


@pytest.mark.parametrize("name", list(BEAMS))
def test_wide_beam_per_voxel_and_sums(gpu_lib, oracle_lib, name):
    from bbarolo2_gb300 import _lib
    dm, L, rings, rows, data, mask = _setup(name)
    ky, kx = dm.cfield.shape
    assert kx > 31 or ky > 23, dm.cfield.shape      # (outside the shared-memory templates)
    ctx = dm.ctx
    sr, nv, descs, boxes = L.prepare(rows, rings, seed=1)
    ctx.set_option(_lib.OPT_KEEP_SMOOTHED, 1)
    try:
        ss, _ = L.run(sr, nv, descs)
        used, _ = ctx.conv_variant()
        assert used == _lib.CONV_F32           # (no tensor-core template takes this kernel)
        nz = L.shape[0]
        worst = 0.0
        for k, (blo, bhi) in enumerate(boxes):
            by, bx = bhi[1] - blo[1], bhi[0] - blo[0]
            s = np.zeros((by, bx, nz), np.float32)
            m = np.zeros((by, bx, nz), np.float32)
            ctx.check(ctx.L.bbgpu_eval_model(ctx.h, k, 1, _lib.ptr(s), by, bx, nz))
            ctx.check(ctx.L.bbgpu_eval_model(ctx.h, k, 0, _lib.ptr(m), by, bx, nz))
            ref = oracle_lib.conv_same(m.astype(np.float64).transpose(2, 0, 1), dm.cfield, dm.scalefactor)
            ref = ref.transpose(1, 2, 0)
            big = ref > FLOOR * ref.max()
            rel = np.abs(s[big].astype(np.float64) - ref[big]) / ref[big]
            worst = max(worst, float(rel.max()))
            assert np.all(np.abs(s[~big] - ref[~big]) <= FLOOR * ref.max())
            ss_ref = _oracle_ss(dm, oracle_lib, sr[k], nv[k], boxes[k], 1, data, mask, 2)
            assert abs(ss[k] - ss_ref) <= SS_RTOL * ss_ref, (k, ss[k], ss_ref)
        print(name, dm.cfield.shape, "max relative error", worst)
        assert worst <= REL_TOL, worst
    finally:
        ctx.set_option(_lib.OPT_KEEP_SMOOTHED, 0)


def test_wide_beam_flux_normalisation(gpu_lib, oracle_lib):
    """The per-evaluation profile with the 90" beam (the ring maps convolved by the 33x33 kernel), members sharing
    member 0's maps and members that do not, against the oracle pipeline."""
    from oracle import cpu_baseline as CB
    dm, L, rings, rows, data, mask = _setup("c90", nb=4)
    mom0, mrms, ok = L.data_maps()
    L.set_profile(rings, mom0, mrms, ok, smooth=0.3, corr=2.0, beam_arcsec=90.)
    ll = L.evaluate(rows, rings, seed=1)
    x, st = L.last_profile()
    assert np.all(st == 0), st
    sr, nv, descs, boxes = L.prepare(rows, rings, seed=1)
    P = CB.setup_payload(dm, sr, nv, boxes, 1, data, L.mask, L.maskmode, like=L, rows=rows, proto=rings)
    CB._W.clear()
    CB._W.update(P)
    for k in range(len(rows)):
        xr = CB.profile_dens(k)
        np.testing.assert_allclose(x[k], xr, rtol=1e-6, atol=1e-6 * np.abs(xr).max())
        ll_ref = L.finish(np.array([CB.evaluate(k)]), np.zeros(1), [boxes[k]])[0]
        assert abs(ll[k] - ll_ref) <= SS_RTOL * abs(ll_ref), (k, ll[k], ll_ref)
