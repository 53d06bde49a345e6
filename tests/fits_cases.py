"""FITS header cases of the reader tests: each a name, the cards after the structural ones, the data shape (C order)
and how the data are stored. ``write_case`` writes one with ``bbarolo2_gb300.fits.write_fits``; the data are seeded
random values with a few NaN voxels."""

import os

import numpy as np

from bbarolo2_gb300.fits import Raw

CASES = [
    ("velo", [("CTYPE1", "RA---SIN"), ("CTYPE2", "DEC--SIN"), ("CTYPE3", "VRAD"), ("CDELT1", -2.777777778E-03),
              ("CDELT2", 2.777777778E-03), ("CDELT3", -5000.0), ("CRPIX1", 17.0), ("CRPIX2", 16.5),
              ("CRPIX3", 9.0), ("CRVAL1", 114.21), ("CRVAL2", 65.60), ("CRVAL3", 132000.0), ("CUNIT1", "deg"),
              ("CUNIT2", "deg"), ("CUNIT3", "M/S"), ("BMAJ", 8.333333E-03), ("BMIN", 6.1E-03), ("BPA", 33.5),
              ("RESTFREQ", 1.420405752E9), ("OBJECT", "NGC 2403"), ("BUNIT", "JY/BEAM")], (16, 32, 33), -32),
    ("nocunit_kms", [("CTYPE1", "RA---NCP"), ("CTYPE2", "DEC--NCP"), ("CTYPE3", "VELO-LSR"), ("CDELT1", -0.004),
                     ("CDELT2", 0.004), ("CDELT3", 5.0), ("CRPIX1", 10.0), ("CRPIX2", 10.0), ("CRPIX3", 6.0),
                     ("CRVAL1", 20.0), ("CRVAL2", -30.0), ("CRVAL3", 1000.0), ("CROTA", 12.5),
                     ("HISTORY", None, "AIPS   CLEAN BMAJ=  8.3333E-03 BMIN=  5.5556E-03 BPA=  30.00"),
                     ("OBJECT", "ESO(1)/x")], (12, 20, 19), -32),
    ("nocunit_ms_gipsy", [("CTYPE1", "RA---SIN"), ("CTYPE2", "DEC--SIN"), ("CTYPE3", "VELO"), ("CDELT1", -0.002),
                          ("CDELT2", 0.002), ("CDELT3", 4000.0), ("CRPIX1", 8.0), ("CRPIX2", 8.0), ("CRPIX3", 4.0),
                          ("CRVAL1", 200.0), ("CRVAL2", 10.0), ("CRVAL3", 500000.0), ("CUNIT1", "DEGREE"),
                          ("CUNIT2", "DEGREE"), ("BMMAJ", Raw("3.0000000D+01")), ("BMMIN", Raw("2.0000000D+01")),
                          ("BMPA", 10.0)], (8, 16, 16), -64),
    ("freq", [("CTYPE1", "RA---SIN"), ("CTYPE2", "DEC--SIN"), ("CTYPE3", "FREQ"), ("CDELT1", -1.5E-03),
              ("CDELT2", 1.5E-03), ("CDELT3", 2.44140625E4), ("CRPIX1", 12.0), ("CRPIX2", 12.0), ("CRPIX3", 5.0),
              ("CRVAL1", 150.0), ("CRVAL2", 2.0), ("CRVAL3", 1.41555E9), ("CUNIT1", "deg"), ("CUNIT2", "deg"),
              ("CUNIT3", "Hz"), ("RESTFRQ", 1.420405752E9), ("BMAJ", 4.0E-03), ("BMIN", 4.0E-03), ("BPA", 0.0),
              ("BUNIT", "Jy beam-1")], (10, 24, 24), 16),
    ("freq_drval", [("CTYPE1", "RA---SIN"), ("CTYPE2", "DEC--SIN"), ("CTYPE3", "FREQ-LSR"), ("CDELT1", -1.0E-03),
                    ("CDELT2", 1.0E-03), ("CDELT3", -4.8828125E4), ("CRPIX1", 6.0), ("CRPIX2", 6.0),
                    ("CRPIX3", 3.0), ("CRVAL1", 10.0), ("CRVAL2", 45.0), ("CRVAL3", 1.41557E3), ("CUNIT1", "deg"),
                    ("CUNIT2", "deg"), ("CUNIT3", "MHz"), ("DRVAL3", 1200.0), ("DUNIT3", "KM/S"),
                    ("BMAJ", 3.0E-03), ("BMIN", 2.0E-03), ("BPA", -20.0)], (6, 10, 12), -32),
    ("arcsec", [("CTYPE1", "RA---TAN"), ("CTYPE2", "DEC--TAN"), ("CTYPE3", "VRAD"), ("CDELT1", -10.0),
                ("CDELT2", 10.0), ("CDELT3", 2.5), ("CRPIX1", 5.0), ("CRPIX2", 5.0), ("CRPIX3", 4.0),
                ("CRVAL1", -3600.0), ("CRVAL2", 7200.0), ("CRVAL3", 300.0), ("CUNIT1", "arcsec"),
                ("CUNIT2", "arcsec"), ("CUNIT3", "km s-1"), ("BMAJ", 8.0E-03), ("BMIN", 8.0E-03)], (7, 9, 10), -32),
    ("cd_matrix", [("CTYPE1", "RA---SIN"), ("CTYPE2", "DEC--SIN"), ("CTYPE3", "VRAD"), ("CD1_1", -2.0E-03),
                   ("CD2_2", 2.0E-03), ("CD3_3", 1.0E4), ("CRPIX1", 4.0), ("CRPIX2", 4.0), ("CRPIX3", 2.0),
                   ("CRVAL1", 30.0), ("CRVAL2", -5.0), ("CRVAL3", 0.0), ("CUNIT1", "deg"), ("CUNIT2", "deg"),
                   ("CUNIT3", "m/s"), ("CLBMMAJ", 25.0), ("CLBMMIN", 15.0)], (5, 8, 8), -32),
    ("stokes4d", [("CTYPE1", "RA---SIN"), ("CTYPE2", "DEC--SIN"), ("CTYPE3", "STOKES"), ("CTYPE4", "FREQ"),
                  ("CDELT1", -1.0E-03), ("CDELT2", 1.0E-03), ("CDELT3", 1.0), ("CDELT4", 1.0E5),
                  ("CRPIX1", 8.0), ("CRPIX2", 8.0), ("CRPIX3", 1.0), ("CRPIX4", 3.0), ("CRVAL1", 180.0),
                  ("CRVAL2", 30.0), ("CRVAL3", 1.0), ("CRVAL4", 1.4195E9), ("CUNIT1", "deg"), ("CUNIT2", "deg"),
                  ("CUNIT4", "Hz"), ("BMAJ", 5.0E-03), ("BMIN", 4.0E-03), ("BPA", 45.0),
                  ("BUNIT", "mJy beam-1")], (6, 1, 14, 15), -32),
    ("vopt", [("CTYPE1", "RA---SIN"), ("CTYPE2", "DEC--SIN"), ("CTYPE3", "VOPT"), ("CDELT1", -3.0E-03),
              ("CDELT2", 3.0E-03), ("CDELT3", 10.0), ("CRPIX1", 5.0), ("CRPIX2", 5.0), ("CRPIX3", 5.0),
              ("CRVAL1", 60.0), ("CRVAL2", 0.0), ("CRVAL3", 3000.0), ("CUNIT1", "deg"), ("CUNIT2", "deg"),
              ("CUNIT3", "km/sec"), ("BMAJ", 9.0E-03), ("BMIN", 9.0E-03), ("BPA", 0.0)], (9, 10, 10), -32),
    ("wave", [("CTYPE1", "RA---TAN"), ("CTYPE2", "DEC--TAN"), ("CTYPE3", "AWAV"), ("CDELT1", -5.5E-05),
              ("CDELT2", 5.5E-05), ("CDELT3", 1.25), ("CRPIX1", 10.0), ("CRPIX2", 10.0), ("CRPIX3", 1.0),
              ("CRVAL1", 340.0), ("CRVAL2", -20.0), ("CRVAL3", 6555.0), ("CUNIT1", "deg"), ("CUNIT2", "deg"),
              ("CUNIT3", "Angstrom"), ("BMAJ", 2.0E-04), ("BMIN", 2.0E-04), ("BPA", 0.0)], (12, 12, 12), -32),
]


def data_of(shape, seed):
    g = np.random.default_rng(seed)
    a = g.normal(0.0, 1.0, shape).astype(np.float32)
    a.reshape(-1)[::97] = np.nan
    return a


def write_case(directory, i):
    """Writes case i; returns (path, data written)."""
    from bbarolo2_gb300.fits import write_fits
    name, cards, shape, bitpix = CASES[i]
    data = data_of(shape, i)
    path = os.path.join(directory, name + ".fits")
    if bitpix > 0:
        # integers: stored as round((v - bzero) / bscale), NaN as the blank value
        write_fits(path, data, cards, bitpix=bitpix, bscale=1e-3, bzero=0.5, blank=-32768)
        stored = np.where(np.isnan(data), np.nan, np.round((data.astype(np.float64) - 0.5) / 1e-3) * 1e-3 + 0.5)
        return path, stored
    write_fits(path, data, cards, bitpix=bitpix)
    return path, data.astype(np.float64 if bitpix == -64 else np.float32)
