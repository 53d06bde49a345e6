"""FITS reading without astropy (``bbarolo2_gb300.fits``, ``Cube.from_fits``): the headers of ``fits_cases.py`` read
as the reference reads them (``tests/golden/headers.json``, made by ``tests/golden/make_headers.py`` from the
reference's ``Header.fromAstropy``), and the data as written (the first Stokes plane of a 4D cube, BSCALE/BZERO and
BLANK of integer data, blank voxels as 0)."""
import json
import os

import numpy as np
import pytest

import fits_cases as FC

with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "headers.json")) as _f:
    REF = json.load(_f)


@pytest.mark.parametrize("i", range(len(FC.CASES)), ids=[c[0] for c in FC.CASES])
def test_header_and_data_as_the_reference_reads_them(tmp_path, i):
    from bbarolo2_gb300.cube import Cube
    name = FC.CASES[i][0]
    path, data = FC.write_case(str(tmp_path), i)
    cube = Cube.from_fits(path)
    h, ref = cube.Head(), REF[name]
    assert h.dims == ref["dims"]
    for key in ("cdelt", "crpix", "crval"):
        np.testing.assert_allclose(getattr(h, key), ref[key], rtol=1e-15, atol=0, err_msg=f"{name} {key}")
    assert [c.lower() for c in h.cunit] == [c.lower() for c in ref["cunit"]], (h.cunit, ref["cunit"])
    assert list(h.ctype) == ref["ctype"]
    assert h.SpectralType() == ref["sptype"] and h.VelDef() == ref["veldef"]
    for key, got in (("freq0", h.Freq0()), ("bmaj", h.Bmaj()), ("bmin", h.Bmin()), ("bpa", h.Bpa()),
                     ("crota", h.Crota())):
        assert got == pytest.approx(ref[key], rel=1e-15, abs=0), (name, key, got, ref[key])
    assert h.Bunit() == ref["bunit"] and h.Name() == ref["object"]
    # the data: (nz, ny, nx) float32, blanks as 0
    d = data[:, 0] if data.ndim == 4 else data
    want = np.where(np.isnan(d), 0.0, d).astype(np.float32)
    assert cube.array.shape == want.shape and cube.array.dtype == np.float32
    np.testing.assert_array_equal(cube.array, want)


def test_cards_round_trip(tmp_path):
    from bbarolo2_gb300 import fits
    cards = [("OBJECT", "it's"), ("FLAG", True), ("N", -12), ("X", 1.5e-300), ("Y", -0.0), ("Z", 3.0),
             ("HISTORY", None, "a history line / with a slash"), ("COMMENT", None, "a comment")]
    a = np.arange(24, dtype=np.float64).reshape(2, 3, 4)
    p = str(tmp_path / "t.fits")
    fits.write_fits(p, a, cards, bitpix=-64)
    h, b = fits.read_fits(p)
    np.testing.assert_array_equal(a, b)
    assert h["OBJECT"] == "it's" and h["FLAG"] is True and h["N"] == -12 and h["X"] == 1.5e-300
    assert h["Z"] == 3.0 and isinstance(h["Z"], float) and h["NAXIS1"] == 4 and h["NAXIS3"] == 2
    assert h.history() == ["a history line / with a slash"]
    assert os.path.getsize(p) % 2880 == 0
    # integer storage with scaling and blanks; an unsigned byte cube
    for bitpix in (8, 16, 32, 64):
        v = np.array([[0.0, 1.25, np.nan, 2.5]], np.float64)
        fits.write_fits(p, v, bitpix=bitpix, bscale=0.25, bzero=0.0, blank=0 if bitpix == 8 else -1)
        _, w = fits.read_fits(p)
        want = v.copy()
        if bitpix == 8:
            want[0, 0] = np.nan        # (the blank value 0 of unsigned bytes is also the stored 0)
        np.testing.assert_array_equal(np.isnan(w), np.isnan(want))
        np.testing.assert_array_equal(w[~np.isnan(w)], want[~np.isnan(want)])


def test_header_errors(tmp_path):
    from bbarolo2_gb300 import fits
    from bbarolo2_gb300.cube import Cube
    p = str(tmp_path / "e.fits")
    fits.write_fits(p, np.zeros((2, 2, 2), np.float32), [("CRVAL1", 0.0), ("CRPIX1", 1.0)])
    with pytest.raises(ValueError, match="pixel spacing"):
        Cube.from_fits(p)
    fits.write_fits(p, np.zeros((2, 2, 2), np.float32), [("CDELT1", 1.0), ("CRVAL1", 0.0)])
    with pytest.raises(ValueError, match="CRPIX"):
        Cube.from_fits(p)
