"""The drop-in binding of the device kernels in place of the reference's (``bbarolo2_gb300.dropin``).

CPU: install / uninstall swap exactly the reference's functions in modules that hold them (stand-in modules
with the reference's names, no GPU). GPU: the replacements, called with the reference kernels' own argument
lists (the golden fixtures' calls), give the reference's results."""
import types

import numpy as np
import pytest

import golden_io as G


def _fake_modules():
    def f(*a, **k):
        return "reference"

    class FFTConvolver:
        def __init__(self, kernel):
            self.kernel = kernel

        def __call__(self, data, workers=None):
            return "reference"
    mods = {}
    for name, attrs in (("bbarolo.galmod", ("_galmod_mc", "_galmod_analytic", "_ring_maps_analytic", "_conv_sparse",
                                            "_galmod_wind")),
                        ("bbarolo.galfit", ("_norm",)),
                        ("bbarolo.bayesian.likelihood", ("_sumsq_residuals", "_residuals_fracerr")),
                        ("bbarolo.galwind", ("_galmod_wind",)),
                        ("bbarolo.windmodel", ("WindModel", "WindCells", "WindPars", "Boxes")),
                        ("bbarolo.bayesian.wind", ("WindModel", "WindCells", "WindPars", "Boxes"))):
        m = types.ModuleType(name)
        for a in attrs:
            setattr(m, a, f)
        mods[name] = m
    sm = types.ModuleType("bbarolo.smooth")
    sm.FFTConvolver = FFTConvolver
    mods["bbarolo.smooth"] = sm
    return mods, f, FFTConvolver.__call__


def test_install_and_uninstall_swap_the_seams():
    from bbarolo2_gb300 import dropin
    mods, f, call = _fake_modules()
    done = dropin.install(mods)
    assert len(done) == len(dropin.SEAMS) + 1 + 8
    for mname, attr, fn in dropin.SEAMS:
        assert getattr(mods[mname], attr) is fn
    assert mods["bbarolo.smooth"].FFTConvolver.__call__ is dropin.FFTConvolver_call
    from bbarolo2_gb300 import wind
    for mname in dropin.WIND_MODULES:
        assert mods[mname].WindModel is wind.WindModel and mods[mname].Boxes is wind.Boxes
    dropin.uninstall(mods)
    for mname, attr, fn in dropin.SEAMS:
        assert getattr(mods[mname], attr) is f
    assert mods["bbarolo.smooth"].FFTConvolver.__call__ is call
    for mname in dropin.WIND_MODULES:
        assert mods[mname].WindModel is f


def test_install_skips_missing_modules():
    from bbarolo2_gb300 import dropin
    mods = {"bbarolo.galfit": types.ModuleType("bbarolo.galfit")}
    assert dropin.install(mods) == []


@pytest.mark.gpu
def test_dropin_kernels_with_reference_arguments(gpu_lib):
    from bbarolo2_gb300 import dropin
    z, idx = G.cases("mc.npz")
    for m in idx[:4]:
        nm = m["name"]
        sr = z[nm + "/sr"]
        out = np.zeros(m["shape"])
        dropin.galmod_mc(out, sr, 0, sr.shape[1], *G.call_args_mc(m, z, nm))
        ref = G.dense(z[nm + "/idx"], z[nm + "/val"], m["shape"])
        np.testing.assert_allclose(out, ref, rtol=1e-12, atol=0)
    z, idx = G.cases("analytic.npz")
    for m in idx[:3]:
        nm = m["name"]
        sr = z[nm + "/sr"]
        nzq = 1 if not np.any(sr[6] > 0) else 1024
        out = np.zeros(m["shape"])
        dropin.galmod_analytic(out, sr, 0, sr.shape[1], *G.call_args_an(m, z, nm, nzq), None, m["zstep"])
        ref = G.dense(z[nm + "/idx"], z[nm + "/val"], m["shape"])
        assert np.abs(out - ref).max() <= 1e-12 * np.abs(ref).max(), nm
    z, idx = G.cases("ringmaps.npz")
    for m in idx:
        mode = m["mode"]
        raw = np.zeros_like(z[mode + "/raw"])
        dropin.ring_maps_analytic(raw, z[mode + "/sr"], z[mode + "/widx"], z[mode + "/wval"], m["radsep"],
                                  m["pixarea"], m["cdelt0"], m["cdelt1"], m["crota2"], m["blo"][0], m["blo"][1],
                                  m["bhi"][0], m["bhi"][1], m["ltype"], m["nzq"], m["sig_instr"], m["chmin"], m["zstep"])
        ref = z[mode + "/raw"]
        assert np.abs(raw - ref).max() <= 1e-12 * np.abs(ref).max(), mode
    z = G.load("classic.npz")
    assert np.array_equal(dropin.conv_sparse(z["conv_sparse/model"], z["conv_sparse/kernel"], 2.5),
                          z["conv_sparse/out_scaled"])
    # _galmod_wind with the reference's arguments (the chunks of a GALWIND fixture, summed in chunk order)
    z, idx = G.cases("wind.npz")
    for nm in ("gw_velo", "gw_radii_freq"):
        m = idx[nm]
        (b0, b1), (e0, e1) = m["box"]
        out = np.zeros(m["shape"])
        for t, (lo, hi) in enumerate(z[nm + "/chunks"]):
            buf = dropin.galmod_wind(np.zeros(m["shape"]), z[nm + "/sr"], int(lo), int(hi),
                                     (m["seed"] + 7919 * t) & 0xFFFFFFFF, m["sep"], z[nm + "/nv"], m["cdens"], 1,
                                     m["pixarea"], m["cdelt0"], m["cdelt1"], m["crota2"], b0, b1, e0, e1,
                                     m["sig_instr"], m["axtyp"], m["velsys"], z[nm + "/lfreq0"], m["crval3"],
                                     m["cdelt3"], m["crpix3"], z[nm + "/relint"], z[nm + "/cd2i"])
            out += buf
        ref = G.dense(z[nm + "/idx"], z[nm + "/val"], m["shape"])
        np.testing.assert_allclose(out, ref, rtol=1e-12, atol=0)


@pytest.mark.gpu
def test_dropin_fftconvolver(gpu_lib):
    from bbarolo2_gb300 import dropin
    z = G.load("beam_conv.npz")
    shape = (64, 64, 64)
    unsm = G.dense(z["classic64/unsmoothed_idx"], z["classic64/unsmoothed_val"], shape)
    ref = G.dense(z["classic64/smoothed_idx"], z["classic64/smoothed_val"], shape)
    conv = types.SimpleNamespace(kernel=z["classic64/kernel"])
    out = dropin.FFTConvolver_call(conv, unsm)
    out[out < 1e-12] = 0.
    assert np.abs(out - ref).max() <= 1e-6 * ref.max()
