"""Heterogeneous batches (``bbarolo2_gb300.ragged.GalaxyBatch``): galaxies of the heterogeneous population (cubes of
different sizes, channel widths, ring counts, geometries, scale heights and beams; the ANALYTIC model) evaluated
together, each galaxy's log L equal bit for bit to its own evaluation and within SS_RTOL of the oracle pipeline."""
import numpy as np
import pytest

from test_gpu_likelihood import SS_RTOL, _oracle_ss

pytestmark = pytest.mark.gpu


def _rows(rings, nb, g):
    from bbarolo2_gb300.galmod import ring_rows_batch
    rows = ring_rows_batch([rings] * nb)
    rows[1:, 4] *= 1 + 0.03 * g.standard_normal((nb - 1, rings.nr))
    rows[1:, 5] *= 1 + 0.1 * g.random((nb - 1, rings.nr))
    rows[1:, 12] += 2.
    return rows


def test_galaxy_batch_vs_own_and_oracle(gpu_lib, oracle_lib):
    from bbarolo2_gb300 import configs
    from bbarolo2_gb300.ragged import GalaxyBatch
    from oracle import oracle as O
    pop = configs.galaxy_population(8, seed=11, nmax=128, zmax=96)
    batch = GalaxyBatch.mock(pop, seed=3)
    g = np.random.default_rng(4)
    rows = [_rows(r, 3, g) for _, _, r in batch.items]
    for _ in range(3):                                  # (the runs after the first replay CUDA graphs)
        together = batch.evaluate(rows, seed=1)
    worst = 0.0
    for (dm, like, rings), rw, ll in zip(batch.items, rows, together):
        own = like.evaluate(rw, rings, seed=1, galmodtype="ANALYTIC")
        np.testing.assert_array_equal(ll, own)
        sr, nv, descs, boxes = like.prepare(rw, rings, seed=1)
        ss, _ = like.run(sr, nv, descs, galmodtype="ANALYTIC")
        for k in range(len(rw)):
            ref = _oracle_ss(dm, O, sr[k], nv[k], boxes[k], 1, like._data, like.mask, 2, galmodtype="ANALYTIC")
            worst = max(worst, abs(ss[k] - ref) / ref)
            assert abs(ss[k] - ref) <= SS_RTOL * ref, (dm.cin.DimX(), dm.cin.DimZ(), k, ss[k], ref)
    print("heterogeneous batch: max relative error of the sums of squares", worst)
