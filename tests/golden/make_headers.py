"""Generates ``headers.json``: the reference's reading of the FITS headers of ``tests/fits_cases.py``
(``Header.fromAstropy``, ``bbarolo/header.py:195-407``, then the Stokes-axis swap and the velocity definition of
``Cube._readHeaderData``, ``bbarolo/cube.py:205-243``).

astropy is not installed here: the cards are read by ``bbarolo2_gb300.fits`` and handed to the reference in an
object with the astropy Header calls ``fromAstropy`` makes (get, in, cards by position and keyword, copy, item
assignment); ``astropy.wcs.WCS`` is a stand-in that fails, so the reference takes its no-WCS branch, which sets no
field recorded here.

Run: BBAROLO_REF=<reference tree> python tests/golden/make_headers.py
"""

import json
import os
import sys
import tempfile
import types

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import _refimport  # noqa: E402
import fits_cases  # noqa: E402
from bbarolo2_gb300 import fits  # noqa: E402


class _Cards(list):
    def __getitem__(self, k):
        if isinstance(k, str):
            return next(c for c in self if c.keyword == k)
        return list.__getitem__(self, k)


class _AstropyLikeHeader:
    def __init__(self, cards=()):
        self.cards = _Cards(cards)
        self._d = {}
        for c in self.cards:
            if c.keyword and c.keyword not in ("COMMENT", "HISTORY") and c.keyword not in self._d:
                self._d[c.keyword] = c.value

    def get(self, k, default=None):
        return self._d.get(k, default)

    def __contains__(self, k):
        return k in self._d

    def __iter__(self):
        return iter(list(self._d))

    def __getitem__(self, k):
        return self._d[k]

    def __setitem__(self, k, v):
        self._d[k] = v

    def __delitem__(self, k):
        del self._d[k]

    def copy(self):
        h = _AstropyLikeHeader(self.cards)
        h._d = dict(self._d)
        return h


def _stub_astropy():
    class _NoWCS:
        def __init__(self, *a, **k):
            raise RuntimeError("no astropy here")
    for name in ("astropy", "astropy.io", "astropy.io.fits", "astropy.wcs"):
        sys.modules.setdefault(name, types.ModuleType(name))
    sys.modules["astropy.io"].fits = sys.modules["astropy.io.fits"]
    sys.modules["astropy.io.fits"].Header = _AstropyLikeHeader
    sys.modules["astropy.wcs"].WCS = _NoWCS


def main():
    _refimport.load()
    _stub_astropy()
    import importlib
    H = importlib.import_module("bbarolo.header")
    out = {}
    with tempfile.TemporaryDirectory() as d:
        for i, (name, _, _, _) in enumerate(fits_cases.CASES):
            path, _ = fits_cases.write_case(d, i)
            fh, _ = fits.read_fits(path, data=False)
            h = H.Header(warning=False)
            assert h.fromAstropy(_AstropyLikeHeader(fh.cards)), name
            n = h.NumAx()
            ax = [0, 1, 2]
            if n > 3 and h.Ctype(2).lower() == "stokes":
                ax = [0, 1, 3]
            sp = h.SpectralType()
            veldef = {"velo-radio": "radio", "velo-opt": "optical", "freq": "radio", "wave": "relativistic"}.get(
                sp, "auto")
            out[name] = {"dims": [h.DimAx(i) for i in ax], "cdelt": [h.Cdelt(i) for i in ax],
                         "crpix": [h.Crpix(i) for i in ax], "crval": [h.Crval(i) for i in ax],
                         "ctype": [h.Ctype(i) for i in ax], "cunit": [h.Cunit(i) for i in ax],
                         "sptype": sp, "veldef": veldef, "freq0": h.Freq0(), "bmaj": h.Bmaj(), "bmin": h.Bmin(),
                         "bpa": h.Bpa(), "crota": h.Crota(), "bunit": h.Bunit(), "object": h.Name()}
    with open(os.path.join(HERE, "headers.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps(out, indent=0)[:3000])


if __name__ == "__main__":
    main()
