"""GPU parity of the beam convolution (float32 on the device) against the FP64 oracle and the reference's FFT,
and of the residual kernels against the reference's fixtures."""
import numpy as np
import pytest

import golden_io as G

pytestmark = pytest.mark.gpu

# the smoothed cube agrees with the FP64 oracle within this fraction of its peak (float32 accumulation)
CONV_TOL = 1e-6


def _dm():
    from bbarolo2_gb300 import configs, engine
    cube, rings = configs.classic64()
    return engine.DiskModel(cube), rings


def test_convolve_vs_reference_fft(gpu_lib):
    z = G.load("beam_conv.npz")
    dm, _ = _dm()
    shape = (64, 64, 64)
    unsm = G.dense(z["classic64/unsmoothed_idx"], z["classic64/unsmoothed_val"], shape)
    ref = G.dense(z["classic64/smoothed_idx"], z["classic64/smoothed_val"], shape)
    out = dm.convolve(unsm.transpose(1, 2, 0))
    err = np.abs(out - ref).max() / ref.max()
    assert err < CONV_TOL, err


@pytest.mark.parametrize("wl", ["global160", "bayes256"])
def test_convolve_vs_fp64_oracle(gpu_lib, oracle_lib, wl):
    from bbarolo2_gb300 import configs, engine
    cube, _ = configs.WORKLOADS[wl]()
    dm = engine.DiskModel(cube)
    g = np.random.default_rng(5)
    nz, ny, nx = cube.array.shape
    a = np.abs(g.normal(size=(nz, ny, nx)))
    a[:, :, : nx // 3] = 0.
    out = dm.convolve(a.transpose(1, 2, 0))
    ref = oracle_lib.conv_same(a, dm.cfield)
    err = np.abs(out - ref).max() / ref.max()
    assert err < CONV_TOL, err
    # planes without threshold (the FFTConvolver call itself)
    p = dm.convolve_planes(a[:5])
    r = oracle_lib.conv_same(a[:5], dm.cfield, 1.0, threshold=False)
    assert np.abs(p - r).max() < CONV_TOL * r.max()


def test_residual_kernels_vs_reference(gpu_lib):
    from bbarolo2_gb300 import _lib
    z = G.load("residuals.npz")
    ctx = _lib.Context(0)
    model = np.ascontiguousarray(z["model"])
    data = np.ascontiguousarray(z["data"])
    mask = np.ascontiguousarray(z["mask"]).view(np.uint8)
    nz, ny, nx = model.shape
    for mm, reg, ss, fr0, fr1 in z["results"]:
        region = np.ascontiguousarray(z["region"]).view(np.uint8) if reg else None
        out = np.zeros(1)
        ctx.check(ctx.L.bbgpu_sumsq_residuals(ctx.h, _lib.ptr(model), _lib.ptr(data), _lib.ptr(mask), int(mm),
                                              _lib.ptr(region), nz, ny, nx, _lib.ptr(out)))
        assert abs(out[0] - ss) <= 1e-13 * abs(ss)
        o2 = np.zeros(2)
        ctx.check(ctx.L.bbgpu_residuals_fracerr(ctx.h, _lib.ptr(model), _lib.ptr(data), _lib.ptr(mask), int(mm),
                                                _lib.ptr(region), nz, ny, nx, 0.09, 0.04, _lib.ptr(o2)))
        assert abs(o2[0] - fr0) <= 1e-12 * abs(fr0) and abs(o2[1] - fr1) <= 1e-12 * abs(fr1)


def test_residual_rejects_bad_arguments(gpu_lib):
    from bbarolo2_gb300 import _lib
    ctx = _lib.Context(0)
    m = np.zeros((2, 2, 2))
    d = np.zeros((2, 2, 2), np.float32)
    out = np.zeros(1)
    rc = ctx.L.bbgpu_sumsq_residuals(ctx.h, _lib.ptr(m), _lib.ptr(d), None, 2, None, 2, 2, 2, _lib.ptr(out))
    assert rc == _lib.ERR_ARG and b"mask" in ctx.L.bbgpu_last_error(ctx.h)
