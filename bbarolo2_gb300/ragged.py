"""Heterogeneous batches: many galaxies whose cubes, grids, rings and beams all differ, evaluated together.

Each galaxy keeps its own device context (its grid, beam kernel, data and mask resident, its own streams), and a
batch queues every galaxy's evaluation (upload and launches, or the replay of its CUDA graph once its batch has run
unchanged) before it reads any result, so that the GPU runs the galaxies' kernels concurrently on their streams and
the host set-up of one galaxy overlaps the device work of the others. The result of each galaxy is, bit for bit,
that of its own ``BatchLikelihood.evaluate``.

This is not a single launch over all the galaxies: the kernels take one grid per context (``GridDev``), and a ragged
launch needs per-member grids, data cubes and beam kernels in every stage.
"""

import numpy as np

from . import _lib
from .engine import BatchLikelihood, DiskModel


class GalaxyBatch:
    """galaxies: a list of (cube, rings, data, mask, sigma); the ANALYTIC (default) or MC model."""

    def __init__(self, galaxies, galmodtype="ANALYTIC", maskmode=2, device=0):
        self.galmodtype = galmodtype.upper()
        self.items = []
        for cube, rings, data, mask, sigma in galaxies:
            dm = DiskModel(cube, galmodtype=self.galmodtype, device=device)
            like = BatchLikelihood(dm, data, mask, maskmode=maskmode, sigma=sigma)
            self.items.append((dm, like, rings))

    @classmethod
    def mock(cls, population, seed=0, galmodtype="ANALYTIC", device=0):
        """A batch of mock galaxies from (cube, rings, noise fraction) triples: each galaxy's data its model plus
        white noise of that fraction of the peak, its mask the model above three times the noise."""
        self = cls.__new__(cls)
        self.galmodtype = galmodtype.upper()
        self.items = []
        g = np.random.default_rng(seed)
        for cube, rings, frac in population:
            dm = DiskModel(cube, galmodtype=self.galmodtype, device=device)
            truth = dm.array(rings, seed=1)
            sigma = frac * float(truth.max())
            data = (truth + g.normal(0., sigma, truth.shape)).astype(np.float32)
            like = BatchLikelihood(dm, data, truth > 3 * sigma, maskmode=2, sigma=sigma)
            self.items.append((dm, like, rings))
        return self

    def __len__(self):
        return len(self.items)

    def upload(self, rows_list, seed=None):
        """The host set-up and upload of every galaxy's ring sets (rows_list[i]: (B_i, 17, nr_i)); returns the
        boxes per galaxy."""
        if len(rows_list) != len(self.items):
            raise ValueError("one array of ring sets per galaxy")
        code = _lib.ANALYTIC if self.galmodtype == "ANALYTIC" else _lib.MC
        boxes = []
        for (dm, like, rings), rows in zip(self.items, rows_list):
            sr, nv, descs, bx = like.prepare(rows, rings, seed)
            ctx = dm.ctx
            ctx.check(ctx.L.bbgpu_eval_upload(ctx.h, code, sr.shape[0], sr.shape[2], _lib.ptr(sr), _lib.ptr(nv),
                                              _lib.ptr(descs)))
            boxes.append(bx)
        return boxes

    def run(self):
        """Queues every galaxy's evaluation of its uploaded ring sets (no result is read)."""
        for dm, _, _ in self.items:
            dm.ctx.check(dm.ctx.L.bbgpu_eval_run(dm.ctx.h))

    def download(self, boxes):
        """log L of every galaxy's ring sets (waits for each galaxy's work in turn)."""
        out = []
        for (dm, like, _), bx in zip(self.items, boxes):
            n = len(bx)
            ss, lg = np.zeros(n), np.zeros(n)
            dm.ctx.check(dm.ctx.L.bbgpu_eval_download(dm.ctx.h, _lib.ptr(ss), _lib.ptr(lg)))
            out.append(like.finish(ss, lg, bx))
        return out

    def evaluate(self, rows_list, seed=None):
        """log L of every galaxy's ring sets: uploads, queues and reads them all."""
        boxes = self.upload(rows_list, seed)
        self.run()
        return self.download(boxes)
