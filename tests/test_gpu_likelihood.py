"""GPU parity of the batched likelihood (MC model -> beam convolution -> masked residual -> log L) against the
CPU oracle pipeline: the oracle's bit-exact MC model, its FP64 direct convolution (the FFT of the reference to
1e-16) and the reference's residual. The device convolves in float32: the sums of squares agree within
SS_RTOL."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SS_RTOL = 1e-5


def _setup(wl, noise=0.01, seed=0):
    from bbarolo2_gb300 import configs, engine
    from oracle import oracle as O
    cube, rings = configs.WORKLOADS[wl](galmodtype="MC")
    dm = engine.DiskModel(cube)
    truth = dm.array(rings, seed=1)
    g = np.random.default_rng(seed)
    sigma = noise * truth.max()
    data = (truth + g.normal(0, sigma, truth.shape)).astype(np.float32)
    mask = truth > 3 * sigma
    return dm, rings, data, mask, sigma, O


def _oracle_ss(dm, O, sr, nv, box, seed, data, mask, maskmode, galmodtype="MC"):
    st = dm.setup
    (blo, bhi) = box
    m = np.zeros((bhi[1] - blo[1], bhi[0] - blo[0], st.nsubs))
    if galmodtype == "ANALYTIC":
        nzq = 1 if not np.any(sr[6] > 0) else 1024
        O.galmod_analytic(m, sr, 0, sr.shape[1], st.radsep, st.cdens, st.pixarea, st.cdelt[0], st.cdelt[1],
                          st.crota2, blo[0], blo[1], bhi[0], bhi[1], st.ltype, st.sig_instr, st._vedges_lines,
                          st.relint, st.cd2i, nzq, st.axtyp, st.velsys, st.lfreq0, st.crval3, st.cdelt3, st.crpix3,
                          st._chmin, None, st.zstep)
    else:
        O.galmod_mc(m, sr, 0, sr.shape[1], seed, st.radsep, nv, st.cdens, st.cmode, st.pixarea, st.cdelt[0],
                    st.cdelt[1], st.crota2, blo[0], blo[1], bhi[0], bhi[1], st.ltype, st.sig_instr, st.axtyp,
                    st.velsys, st.lfreq0, st.crval3, st.cdelt3, st.crpix3, st.relint, st.cd2i)
    sm = O.conv_same(m.transpose(2, 0, 1), dm.cfield, dm.scalefactor)
    sl = (slice(None), slice(blo[1], bhi[1]), slice(blo[0], bhi[0]))
    return O.sumsq_residuals(sm, data[sl], mask[sl], maskmode, None)


@pytest.mark.parametrize("wl,maskmode", [("classic64", 2), ("classic64", 1), ("global160", 2)])
def test_batch_likelihood_vs_oracle(gpu_lib, wl, maskmode):
    from bbarolo2_gb300 import engine
    from bbarolo2_gb300.galmod import ring_rows_batch
    dm, rings, data, mask, sigma, O = _setup(wl)
    L = engine.BatchLikelihood(dm, data, mask, maskmode=maskmode, sigma=sigma)
    g = np.random.default_rng(3)
    rows = ring_rows_batch([rings] * 5)
    rows[1:, 4] *= 1 + 0.05 * g.standard_normal((4, rings.nr))     # vrot
    rows[1:, 5] *= 1 + 0.2 * g.random((4, rings.nr))               # vdisp
    rows[3, 12] += 4.                                               # inc
    rows[4, 13] -= 6.                                               # phi
    sr, nv, descs, boxes = L.prepare(rows, rings, seed=1)
    ss, _ = L.run(sr, nv, descs)
    for k in range(5):
        ref = _oracle_ss(dm, O, sr[k], nv[k], boxes[k], 1, data, mask, maskmode)
        assert abs(ss[k] - ref) <= SS_RTOL * ref, (k, ss[k], ref)
    # deterministic
    ss2, _ = L.run(sr, nv, descs)
    np.testing.assert_array_equal(ss, ss2)
    lg = L.finish(ss, np.zeros(5), boxes)
    assert np.argmax(lg) == 0


@pytest.mark.parametrize("wl,nb", [("classic64", 5), ("global160", 3)])
def test_batch_likelihood_analytic_vs_oracle(gpu_lib, wl, nb):
    """The ANALYTIC model in the batch path: members that differ in every ring value but the radii (including the
    layer height, which changes the vertical grids and the boxes)."""
    from bbarolo2_gb300 import engine
    from bbarolo2_gb300.galmod import ring_rows_batch
    from bbarolo2_gb300.rings import RING_KEYS
    dm, rings, data, mask, sigma, O = _setup(wl)
    L = engine.BatchLikelihood(dm, data, mask, maskmode=2, sigma=sigma)
    g = np.random.default_rng(5)
    rows = ring_rows_batch([rings] * nb)
    rows[1:, 4] *= 1 + 0.05 * g.standard_normal((nb - 1, rings.nr))
    rows[1, 5] *= 1.3
    rows[2, RING_KEYS.index("z0")] += 6.
    if nb > 3:
        rows[3, 12] += 4.
        rows[4, 13] -= 6.
    sr, nv, descs, boxes = L.prepare(rows, rings, seed=1)
    ss, _ = L.run(sr, nv, descs, galmodtype="ANALYTIC")
    for k in range(nb):
        ref = _oracle_ss(dm, O, sr[k], nv[k], boxes[k], 1, data, mask, 2, galmodtype="ANALYTIC")
        assert abs(ss[k] - ref) <= SS_RTOL * ref, (k, ss[k], ref)
    ss2, _ = L.run(sr, nv, descs, galmodtype="ANALYTIC")
    np.testing.assert_array_equal(ss, ss2)


def test_fracerr_and_region(gpu_lib):
    from bbarolo2_gb300 import engine
    from bbarolo2_gb300.galmod import ring_rows_batch
    dm, rings, data, mask, sigma, O = _setup("classic64")
    region = np.ones(data.shape[1:], bool)
    region[:, :20] = False
    L = engine.BatchLikelihood(dm, data, mask, maskmode=2, sigma=sigma, region=region, fracerr=0.1)
    rows = ring_rows_batch([rings] * 2)
    rows[1, 4] *= 0.9
    sr, nv, descs, boxes = L.prepare(rows, rings, seed=1)
    ss, lg = L.run(sr, nv, descs)
    st = dm.setup
    for k in range(2):
        (blo, bhi) = boxes[k]
        m = np.zeros((bhi[1] - blo[1], bhi[0] - blo[0], st.nsubs))
        O.galmod_mc(m, sr[k], 0, sr.shape[2], 1, st.radsep, nv[k], st.cdens, st.cmode, st.pixarea, st.cdelt[0],
                    st.cdelt[1], st.crota2, blo[0], blo[1], bhi[0], bhi[1], st.ltype, st.sig_instr, st.axtyp,
                    st.velsys, st.lfreq0, st.crval3, st.cdelt3, st.crpix3, st.relint, st.cd2i)
        sm = O.conv_same(m.transpose(2, 0, 1), dm.cfield)
        sl = (slice(None), slice(blo[1], bhi[1]), slice(blo[0], bhi[0]))
        a, b = O.residuals_fracerr(sm, data[sl], mask[sl], 2, region[sl[1:]], sigma ** 2, 0.01)
        assert abs(ss[k] - a) <= SS_RTOL * a and abs(lg[k] - b) <= SS_RTOL * abs(b), (k, ss[k], a, lg[k], b)


def test_layout_mismatch_is_rejected(gpu_lib):
    """Members whose cloud layouts differ (other radii/seed/counts) are refused with a clear error."""
    from bbarolo2_gb300 import _lib, engine
    from bbarolo2_gb300.galmod import ring_rows_batch
    dm, rings, data, mask, sigma, O = _setup("classic64")
    L = engine.BatchLikelihood(dm, data, mask, maskmode=2, sigma=sigma)
    rows = ring_rows_batch([rings] * 2)
    sr, nv, descs, boxes = L.prepare(rows, rings, seed=1)
    descs[1]["seed"] = 7
    with pytest.raises(_lib.DeviceError, match="another cloud layout"):
        L.run(sr, nv, descs)


@pytest.mark.parametrize("galmodtype", ["MC", "ANALYTIC"])
def test_batch_members_equal_single_evaluations(gpu_lib, galmodtype):
    """Members whose sub-ring columns equal member 0's share its constants (the host marks them, the device fills
    them with the member's own fixed-point unit): each member of a mixed batch gives exactly the log L of its
    evaluation alone, with and without the flux normalisation."""
    from bbarolo2_gb300 import engine
    from bbarolo2_gb300.galmod import ring_rows_batch
    from bbarolo2_gb300.rings import RING_KEYS
    dm, rings, data, mask, sigma, O = _setup("classic64")
    L = engine.BatchLikelihood(dm, data, mask, maskmode=2, sigma=sigma)
    rows = ring_rows_batch([rings] * 4)
    rows[1, RING_KEYS.index("vrot"), 3] += 7.          # one column changed
    rows[2, RING_KEYS.index("inc"), :] += 2.           # every column changed
    rows[3, RING_KEYS.index("dens"), 5] *= 1.5         # another fixed-point unit
    for prof in (False, True):
        if prof:
            mom0, mrms, ok = L.data_maps()
            L.set_profile(rings, mom0, mrms, ok, smooth=0.3, corr=2.0, beam_arcsec=30.)
        whole = L.evaluate(rows, rings, seed=1, galmodtype=galmodtype)
        for k in range(4):
            alone = L.evaluate(rows[k:k + 1], rings, seed=1, galmodtype=galmodtype)
            assert whole[k] == alone[0], (prof, k, whole[k], alone[0])
