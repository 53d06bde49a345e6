"""The CPU oracle (oracle/bbref.c) against the golden fixtures generated by the reference's own kernels."""
import numpy as np
import pytest

import golden_io as G


def test_rng_stream(oracle_lib):
    z = G.load("rng.npz")
    for sd, st, words in zip(z["seeds"], z["init_states"], z["words"]):
        r = oracle_lib.RNG(int(sd))
        assert np.array_equal(r.s, st)
        assert [r.next() for _ in range(32)] == [int(w) for w in words]
    r = oracle_lib.RNG(12345)
    nrm, uni = [], []
    for _ in range(z["normals"].size):
        nrm.append(r.normal())
        uni.append(r.uniform())
    assert np.array_equal(np.array(nrm), z["normals"])
    assert np.array_equal(np.array(uni), z["uniforms"])
    assert np.array_equal(r.s, z["final_state"])
    kn, wn, fn = oracle_lib.zig_tables()
    assert np.array_equal(kn, z["KN"]) and np.array_equal(wn, z["WN"]) and np.array_equal(fn, z["FN"])
    assert np.array_equal(oracle_lib.phi_table(), z["PHI_TAB"])


def _mc_cases():
    z, idx = G.cases("mc.npz")
    return [(z, m) for m in idx]


@pytest.mark.parametrize("case", _mc_cases(), ids=lambda c: c[1]["name"])
def test_mc_model_bit_exact(oracle_lib, case):
    z, m = case
    nm = m["name"]
    sr = z[nm + "/sr"]
    out = np.zeros(m["shape"])
    oracle_lib.galmod_mc(out, sr, 0, sr.shape[1], *G.call_args_mc(m, z, nm))
    ref = G.dense(z[nm + "/idx"], z[nm + "/val"], m["shape"])
    assert np.array_equal(out, ref)


def _an_cases():
    z, idx = G.cases("analytic.npz")
    return [(z, m) for m in idx]


@pytest.mark.parametrize("case", _an_cases(), ids=lambda c: c[1]["name"])
def test_analytic_model_bit_exact(oracle_lib, case):
    z, m = case
    nm = m["name"]
    sr = z[nm + "/sr"]
    nzq = 1 if not np.any(sr[6] > 0) else 1024
    out = np.zeros(m["shape"])
    oracle_lib.galmod_analytic(out, sr, 0, sr.shape[1], *G.call_args_an(m, z, nm, nzq), None, m["zstep"])
    ref = G.dense(z[nm + "/idx"], z[nm + "/val"], m["shape"])
    assert np.array_equal(out, ref)


def test_fp64_convolution_vs_reference_fft(oracle_lib):
    """The FP64 direct convolution (the oracle of the smoothed cube) against the reference's FFT."""
    z = G.load("beam_conv.npz")
    shape = (64, 64, 64)
    unsm = G.dense(z["classic64/unsmoothed_idx"], z["classic64/unsmoothed_val"], shape)
    ref = G.dense(z["classic64/smoothed_idx"], z["classic64/smoothed_val"], shape)
    out = oracle_lib.conv_same(unsm, z["classic64/kernel"])
    assert np.abs(out - ref).max() <= 1e-13 * ref.max()
    # (the threshold at 1e-12 is on values where FFT and direct sums differ by ~1e-17: same zeros but a few)
    assert np.sum((out != 0) != (ref != 0)) <= 1e-4 * out.size
    refc = G.dense(z["classic64/coldens_smoothed_idx"], z["classic64/coldens_smoothed_val"], shape)
    outc = oracle_lib.conv_same(unsm, z["classic64/kernel"], float(z["classic64/coldens_scalefactor"]))
    assert np.abs(outc - refc).max() <= 1e-13 * refc.max()


def test_residual_kernels(oracle_lib):
    z = G.load("residuals.npz")
    for mm, reg, ss, fr0, fr1 in z["results"]:
        region = z["region"] if reg else None
        got = oracle_lib.sumsq_residuals(z["model"], z["data"], z["mask"], int(mm), region)
        assert got == ss
        a, b = oracle_lib.residuals_fracerr(z["model"], z["data"], z["mask"], int(mm), region, 0.09, 0.04)
        assert a == fr0 and b == fr1


def test_conv_sparse(oracle_lib):
    z = G.load("classic.npz")
    out = oracle_lib.conv_sparse(z["conv_sparse/model"], z["conv_sparse/kernel"], 1.0)
    assert np.array_equal(out, z["conv_sparse/out"])
    out = oracle_lib.conv_sparse(z["conv_sparse/model"], z["conv_sparse/kernel"], 2.5)
    assert np.array_equal(out, z["conv_sparse/out_scaled"])


def test_classic_norm(oracle_lib):
    import json
    z = G.load("classic.npz")
    meta = json.loads(str(z["norm/meta"]))
    ilo, ihi = z["norm/ilo"], z["norm/ihi"]
    for normtype, ftype, wpow, side, foot, trunc, val, msum in z["norm/results"]:
        m = z["norm/model"].copy()
        pre = z["conv_sparse/model"] if trunc else None
        thr = z["norm/thr"] if trunc else np.zeros(0)
        v = oracle_lib.norm(m, z["norm/data_T"], z["norm/mask_T"], 0, 0, meta["x0"], meta["y0"], 45., 55., meta["r1"], meta["r2"],
                            wpow, int(side), int(ftype), z["norm/chan_noise"], 0.001, 1.0, int(normtype), pre,
                            ilo if trunc else np.zeros(0, np.int64), ihi if trunc else np.zeros(0, np.int64), thr,
                            None, int(foot), 4.0)
        assert v == val, (normtype, ftype, wpow, side, foot, trunc)
        assert float(np.sum(m)) == msum


def test_ring_maps_raw(oracle_lib):
    z, idx = G.cases("ringmaps.npz")
    for m in idx:
        mode = m["mode"]
        raw = np.zeros_like(z[mode + "/raw"])
        oracle_lib.ring_maps_analytic(raw, z[mode + "/sr"], z[mode + "/widx"], z[mode + "/wval"], m["radsep"],
                                      m["pixarea"], m["cdelt0"], m["cdelt1"], m["crota2"], m["blo"][0], m["blo"][1],
                                      m["bhi"][0], m["bhi"][1], m["ltype"], m["nzq"], m["sig_instr"], m["chmin"],
                                      m["zstep"])
        assert np.array_equal(raw, z[mode + "/raw"]), mode


def test_profile_solve_matches_reference():
    """The oracle's restatement of solve_profile against the reference's densities (bbarolo/profile.py:91-138)."""
    import json
    from oracle import profile as P
    z = G.load("profile.npz")
    for m in json.loads(str(z["index"])):
        nm = m["name"]
        okk, rms, y = z[nm + "/okk"], z[nm + "/rms"], z[nm + "/y"]
        A = z[nm + "/maps"][:, okk].T / rms[okk, None]
        b = y[okk] / rms[okk]
        for smooth, corr in ((0.3, 1.0), (0.3, 4.0), (0.0, 1.0), (1.0, 2.0)):
            x = P.solve_profile(A, b, z[nm + "/Rc"], smooth, corr)
            ref = z[nm + f"/x_{smooth}_{corr}"]
            np.testing.assert_allclose(x, ref, rtol=1e-12, atol=1e-15 * np.abs(ref).max())
    z = G.load("ringmaps.npz")
    A, b, R = z["profile/A"], z["profile/b"], z["profile/radii"]
    np.testing.assert_allclose(P.solve_profile(A, b, R, 0.3, 4.0), z["profile/x_smooth"], rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(P.solve_profile(A, b, R, 0.0), z["profile/x_nosmooth"], rtol=1e-12, atol=1e-15)
