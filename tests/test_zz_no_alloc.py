"""The allocation-free residual entry point (bbgpu_sumsq_residuals_noalloc) against the allocating one.

Callers that may not allocate device memory (their own pool, a fixed footprint) pass device buffers; the entry point keeps its partial sums in a scratch array of the library. Two
calls in a row must give the sums of bbgpu_sumsq_residuals / bbgpu_residuals_fracerr (same voxels, float64;
only the summation order differs). This file is collected last: it runs alone or after the other tests."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def _inputs(seed, nz=40, ny=57, nx=61):
    g = np.random.default_rng(seed)
    model = np.abs(g.normal(0, 1, (nz, ny, nx)))
    model[g.random(model.shape) < 0.3] = 0.
    data = (model + g.normal(0, 0.3, model.shape)).astype(np.float32)
    data[g.random(data.shape) < 0.05] = np.nan
    data[g.random(data.shape) < 0.05] = 0.
    mask = (g.random(data.shape) < 0.6).astype(np.uint8)
    region = (g.random((ny, nx)) < 0.8).astype(np.uint8)
    return model, data, mask, region


def _reference(ctx, _lib, model, data, mask, maskmode, region, s2, e2):
    nz, ny, nx = model.shape
    if e2 > 0:
        o = np.zeros(2)
        ctx.check(ctx.L.bbgpu_residuals_fracerr(ctx.h, _lib.ptr(model), _lib.ptr(data), _lib.ptr(mask), maskmode,
                                                _lib.ptr(region), nz, ny, nx, s2, e2, _lib.ptr(o)))
        return o
    o = np.zeros(1)
    ctx.check(ctx.L.bbgpu_sumsq_residuals(ctx.h, _lib.ptr(model), _lib.ptr(data), _lib.ptr(mask), maskmode,
                                          _lib.ptr(region), nz, ny, nx, _lib.ptr(o)))
    return np.array([o[0], 0.0])


def test_noalloc_matches_allocating_entry_point(gpu_lib):
    torch = pytest.importorskip("torch")
    from bbarolo2_gb300 import _lib
    ctx = _lib.Context(0)
    L = _lib.load()
    for seed, maskmode, use_region, s2, e2 in ((1, 2, True, 0.09, 0.0), (2, 1, False, 0.09, 0.04),
                                               (3, 0, True, 0.5, 0.01)):
        model, data, mask, region = _inputs(seed)
        ref = _reference(ctx, _lib, model, data, mask, maskmode, region if use_region else None, s2, e2)
        dev = {k: torch.from_numpy(v).cuda() for k, v in
               (("model", model), ("data", data), ("mask", mask), ("region", region))}
        out = torch.zeros(2, dtype=torch.float64, device="cuda")
        stream = torch.cuda.current_stream().cuda_stream
        nz, ny, nx = model.shape
        for _ in range(2):                          # two calls in a row share the scratch array
            out.zero_()
            rc = L.bbgpu_sumsq_residuals_noalloc(dev["model"].data_ptr(), dev["data"].data_ptr(),
                                                 dev["mask"].data_ptr(), maskmode,
                                                 dev["region"].data_ptr() if use_region else None, nz, ny, nx,
                                                 s2, e2, out.data_ptr(), stream)
            assert rc == _lib.OK
            torch.cuda.synchronize()
            got = out.cpu().numpy()
            assert abs(got[0] - ref[0]) <= RTOL * abs(ref[0]), (got, ref)
            assert abs(got[1] - ref[1]) <= RTOL * max(abs(ref[1]), 1e-300), (got, ref)


def test_noalloc_rejects_sizes_beyond_its_scratch(gpu_lib):
    torch = pytest.importorskip("torch")
    from bbarolo2_gb300 import _lib
    L = _lib.load()
    a = torch.zeros(8, dtype=torch.float64, device="cuda")
    b = torch.zeros(8, dtype=torch.float32, device="cuda")
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    # 4097 x 64 x 64 voxels: more blocks than the scratch array holds (the pointers are never read)
    rc = L.bbgpu_sumsq_residuals_noalloc(a.data_ptr(), b.data_ptr(), None, 0, None, 4097, 64, 64, 1.0, 0.0,
                                         out.data_ptr(), None)
    assert rc == _lib.ERR_ARG
    # a negative or NaN fractional error is refused, as the allocating entry point refuses it
    for eps2 in (-0.01, float("nan")):
        rc = L.bbgpu_sumsq_residuals_noalloc(a.data_ptr(), b.data_ptr(), None, 0, None, 2, 2, 2, 1.0, eps2,
                                             out.data_ptr(), None)
        assert rc == _lib.ERR_ARG, eps2


def test_noalloc_edge_sizes(gpu_lib):
    """No voxels: the sums are zero (written by the final kernel alone); exactly as many voxels as the scratch array
    holds sums for (4096 blocks of 4096): accepted, and equal to the allocating entry point."""
    torch = pytest.importorskip("torch")
    from bbarolo2_gb300 import _lib
    L = _lib.load()
    a = torch.zeros(8, dtype=torch.float64, device="cuda")
    b = torch.zeros(8, dtype=torch.float32, device="cuda")
    out = torch.full((2,), 7.0, dtype=torch.float64, device="cuda")
    rc = L.bbgpu_sumsq_residuals_noalloc(a.data_ptr(), b.data_ptr(), None, 0, None, 0, 64, 64, 1.0, 0.0,
                                         out.data_ptr(), None)
    assert rc == _lib.OK
    torch.cuda.synchronize()
    assert out.cpu().numpy().tolist() == [0.0, 0.0]
    nz, ny, nx = 1024, 128, 128                          # 16,777,216 voxels
    g = torch.Generator(device="cuda").manual_seed(5)
    model = torch.rand((nz, ny, nx), dtype=torch.float64, device="cuda", generator=g)
    data = (model + 0.1 * torch.randn((nz, ny, nx), dtype=torch.float64, device="cuda", generator=g)).float()
    rc = L.bbgpu_sumsq_residuals_noalloc(model.data_ptr(), data.data_ptr(), None, 0, None, nz, ny, nx, 1.0, 0.0,
                                         out.data_ptr(), None)
    assert rc == _lib.OK
    torch.cuda.synchronize()
    ref = float(((data.double() - model) ** 2).sum())
    assert abs(float(out[0]) - ref) <= 1e-10 * ref, (float(out[0]), ref)
