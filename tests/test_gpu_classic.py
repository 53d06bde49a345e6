"""GPU parity of the CLASSIC kernels: ``_conv_sparse`` (bit-exact with the reference's fixture) and ``_norm``
(same blank counts and normalised model; residual within NORM_RTOL of the reference, whose running sum over all
voxels the device reduces in a fixed tree)."""
import json

import numpy as np
import pytest

import golden_io as G

pytestmark = pytest.mark.gpu

# relative tolerance of the _norm residual and of the normalised model's sum (float64, rounding order only)
NORM_RTOL = 1e-12


def test_conv_sparse_bit_exact(gpu_lib):
    from bbarolo2_gb300 import galfit
    z = G.load("classic.npz")
    out = galfit._conv_sparse(z["conv_sparse/model"], z["conv_sparse/kernel"], 1.0)
    assert np.array_equal(out, z["conv_sparse/out"])
    out = galfit._conv_sparse(z["conv_sparse/model"], z["conv_sparse/kernel"], 2.5)
    assert np.array_equal(out, z["conv_sparse/out_scaled"])


def test_conv_sparse_ragged_vs_oracle(gpu_lib, oracle_lib):
    from bbarolo2_gb300 import galfit
    g = np.random.default_rng(3)
    for ny, nx, nz, ky, kx in ((1, 1, 1, 1, 1), (5, 9, 3, 7, 3), (13, 4, 17, 5, 9), (0, 4, 3, 3, 3)):
        m = np.abs(g.normal(size=(ny, nx, nz)))
        m[m < 0.8] = 0.
        k = np.abs(g.normal(size=(ky, kx)))
        k[0, 0] = 0.
        out = galfit._conv_sparse(m, k, 1.7)
        assert np.array_equal(out, oracle_lib.conv_sparse(m, k, 1.7)), (ny, nx, nz, ky, kx)


def _norm_cases():
    z = G.load("classic.npz")
    meta = json.loads(str(z["norm/meta"]))
    return z, meta


def test_norm_vs_reference(gpu_lib):
    from bbarolo2_gb300 import galfit
    z, meta = _norm_cases()
    ilo, ihi = z["norm/ilo"], z["norm/ihi"]
    assert np.isfinite(z["norm/results"][:, 6]).sum() >= 40          # (the cases have pixels in the ring)
    for normtype, ftype, wpow, side, foot, trunc, val, msum in z["norm/results"]:
        m = z["norm/model"].copy()
        pre = z["conv_sparse/model"] if trunc else None
        v = galfit._norm(m, z["norm/data_T"], z["norm/mask_T"], 0, 0, meta["x0"], meta["y0"], 45., 55., meta["r1"], meta["r2"],
                         wpow, int(side), int(ftype), z["norm/chan_noise"], 0.001, 1.0, int(normtype), pre,
                         ilo, ihi, z["norm/thr"] if trunc else np.zeros(0), None, int(foot), 4.0)
        case = (normtype, ftype, wpow, side, foot, trunc)
        if np.isinf(val):
            assert np.isinf(v), case
            continue
        assert abs(v - val) <= NORM_RTOL * abs(val), (case, v, val)
        assert abs(float(np.sum(m)) - msum) <= NORM_RTOL * abs(msum), case


def test_norm_counts_and_model_vs_oracle(gpu_lib, oracle_lib):
    """Blank counting decides the residual's weight: with BWEIGHT the count enters (1 + nb/n)^w, so two
    BWEIGHTs separate nb and n; the normalised model is compared voxel by voxel (LOCAL and NONE are exact)."""
    from bbarolo2_gb300 import galfit
    z, meta = _norm_cases()
    ilo, ihi = z["norm/ilo"], z["norm/ihi"]
    finite = 0
    for normtype in (0, 1, 2):
        for trunc in (0, 1):
            for foot in (0, 1):
                for bw in (0.0, 3.0):
                    args = (z["norm/data_T"], z["norm/mask_T"], 0, 0, meta["x0"], meta["y0"], 45., 55., 2.0, 7.5,
                            1., 0, 4, z["norm/chan_noise"], 0.001, bw, normtype,
                            z["conv_sparse/model"] if trunc else None, ilo, ihi,
                            z["norm/thr"] if trunc else np.zeros(0), None, foot, 3.0)
                    m_dev = z["norm/model"].copy()
                    m_ref = z["norm/model"].copy()
                    v = galfit._norm(m_dev, *args)
                    r = oracle_lib.norm(m_ref, *args)
                    case = (normtype, trunc, foot, bw)
                    if np.isinf(r):
                        assert np.isinf(v), case
                        continue
                    finite += 1
                    assert abs(v - r) <= NORM_RTOL * abs(r), (case, v, r)
                    if normtype == 1:
                        np.testing.assert_allclose(m_dev, m_ref, rtol=NORM_RTOL, atol=0)
                    else:
                        assert np.array_equal(m_dev, m_ref), case
    assert finite >= 20


def test_norm_offset_box_and_empty_ring(gpu_lib, oracle_lib):
    """A model box inside a larger data cube (blo != 0), and a ring with no pixel (inf)."""
    from bbarolo2_gb300 import galfit
    g = np.random.default_rng(11)
    dny, dnx, nz = 30, 40, 24
    data = np.abs(g.normal(size=(dny, dnx, nz))).astype(np.float32)
    mask = data > 0.6
    bsy, bsx = 17, 21
    model = np.abs(g.normal(size=(bsy, bsx, nz)))
    model[model < 0.5] = 0.
    cn = np.full(nz, 0.3)
    for r1, r2 in ((2., 9.), (50., 60.)):
        for normtype in (0, 1, 2):
            args = (data, mask, 11, 7, 9.5, 8.0, 30., 40., r1, r2, 2., 0, 1, cn, 0.01, 1.0, normtype, None,
                    np.zeros(0, np.int64), np.zeros(0, np.int64), np.zeros(0), None, 0, 4.0)
            m1, m2 = model.copy(), model.copy()
            v = galfit._norm(m1, *args)
            r = oracle_lib.norm(m2, *args)
            if np.isinf(r):
                assert np.isinf(v)
            else:
                assert abs(v - r) <= NORM_RTOL * abs(r), (r1, normtype, v, r)
            np.testing.assert_allclose(m1, m2, rtol=NORM_RTOL, atol=0)
