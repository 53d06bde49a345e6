"""Batch runs through CUDA graphs: the second run of an unchanged batch is captured, later runs replay it; the sums
are the ordinary runs' bit for bit, and an upload (a new batch) or an option change drops the graph."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _batch(prof):
    from bbarolo2_gb300 import configs, engine
    from bbarolo2_gb300.galmod import ring_rows_batch
    cube, rings = configs.global160(galmodtype="MC")
    dm = engine.DiskModel(cube)
    truth = dm.array(rings, seed=1)
    g = np.random.default_rng(0)
    sigma = 0.01 * truth.max()
    data = (truth + g.normal(0, sigma, truth.shape)).astype(np.float32)
    L = engine.BatchLikelihood(dm, data, truth > 3 * sigma, maskmode=2, sigma=sigma)
    if prof:
        mom0, mrms, ok = L.data_maps()
        L.set_profile(rings, mom0, mrms, ok, smooth=0.3, corr=4.0, beam_arcsec=30.)
    rows = ring_rows_batch([rings] * 9)
    for i in range(1, 9):
        rows[i, 4 if i % 2 else 12, (5 * i) % rings.nr] += 2.0 if i % 2 else 0.5
    return dm, L, rings, rows


def _run(ctx, L, rows, rings, galmodtype="MC"):
    from bbarolo2_gb300 import _lib
    sr, nv, descs, boxes = L.prepare(rows, rings, seed=1)
    code = _lib.ANALYTIC if galmodtype == "ANALYTIC" else _lib.MC
    ctx.check(ctx.L.bbgpu_eval_upload(ctx.h, code, len(rows), sr.shape[2], _lib.ptr(sr), _lib.ptr(nv),
                                      _lib.ptr(descs)))
    if L._prof is not None:
        ms = L._maps_sr
        ctx.check(ctx.L.bbgpu_eval_upload_profile(ctx.h, ms.shape[2], _lib.ptr(ms), _lib.ptr(L._prof["widx"]),
                                                  _lib.ptr(L._prof["wval"])))
    out = []
    for _ in range(4):
        ctx.check(ctx.L.bbgpu_eval_run(ctx.h))
        ss, lg = np.zeros(len(rows)), np.zeros(len(rows))
        ctx.check(ctx.L.bbgpu_eval_download(ctx.h, _lib.ptr(ss), _lib.ptr(lg)))
        out.append(ss)
    return out


@pytest.mark.parametrize("prof,galmodtype", [(False, "MC"), (True, "MC"), (True, "ANALYTIC")])
def test_graph_replays_equal_ordinary_runs(gpu_lib, prof, galmodtype):
    from bbarolo2_gb300 import _lib
    dm, L, rings, rows = _batch(prof)
    ctx = dm.ctx
    ctx.set_option(_lib.OPT_GRAPHS, 0)
    plain = _run(ctx, L, rows, rings, galmodtype)
    ctx.set_option(_lib.OPT_GRAPHS, 1)
    r0, _ = ctx.graph_stats()
    graphed = _run(ctx, L, rows, rings, galmodtype)
    r1, kernels = ctx.graph_stats()
    assert r1 - r0 == 2 and kernels > 0, (r1 - r0, kernels)     # run 2 captured, runs 3 and 4 replayed
    for a in plain + graphed:
        np.testing.assert_array_equal(a, plain[0])
    # an option change (and an upload) drops the graph of the old state
    ctx.set_option(_lib.OPT_SHARE, 1)
    assert ctx.graph_stats()[1] == 0
