"""FITS images without astropy: the cards of an image HDU and its data (read and write), for ``Cube.from_fits``.

The reference reads its cubes with astropy (``bbarolo/header.py:21-50`` ``fits_image_hdu``/``read_fits_image``):
the image of the primary HDU, or, when that has no data, of the first image extension; ``file.fits[n]`` or
``file.fits[EXTNAME]`` name an HDU. This module reads the same images from the FITS standard itself: 2880-byte
blocks of 80-character cards up to END, then the data, big-endian, of the type BITPIX (8: unsigned bytes, 16/32/64:
signed integers, -32/-64: IEEE floats), the first axis (NAXIS1) fastest, physical values BZERO + BSCALE x stored,
integer BLANK values as NaN.
"""

import os
import re

import numpy as np

BLOCK = 2880
CARD = 80
_DTYPES = {8: ">u1", 16: ">i2", 32: ">i4", 64: ">i8", -32: ">f4", -64: ">f8"}


class Card:
    """A header card: keyword, value (str, bool, int, float, complex or None), comment, and the card's text
    (``image``, as written)."""

    __slots__ = ("keyword", "value", "comment", "image")

    def __init__(self, keyword, value=None, comment="", image=""):
        self.keyword, self.value, self.comment, self.image = keyword, value, comment, image


def _parse_value(text):
    """(value, comment) of the text after '= ' of a card (FITS standard 4.2)."""
    t = text.strip()
    if t.startswith("'"):
        # a string: '' inside is a quote; trailing blanks are not significant
        i, out = 1, []
        while i < len(t):
            if t[i] == "'":
                if i + 1 < len(t) and t[i + 1] == "'":
                    out.append("'")
                    i += 2
                    continue
                break
            out.append(t[i])
            i += 1
        rest = t[i + 1:]
        com = rest.split("/", 1)[1].strip() if "/" in rest else ""
        return "".join(out).rstrip(), com
    v, _, com = t.partition("/")
    v, com = v.strip(), com.strip()
    if v == "":
        return None, com
    if v in ("T", "F"):
        return v == "T", com
    if v.startswith("("):
        re_, im_ = v.strip("()").split(",")
        return complex(_number(re_), _number(im_)), com
    return _number(v), com


def _number(s):
    s = s.strip()
    if re.fullmatch(r"[+-]?\d+", s):
        return int(s)
    return float(s.replace("D", "E").replace("d", "e"))


def parse_card(image):
    """A Card of an 80-character card image."""
    key = image[:8].strip()
    if key in ("COMMENT", "HISTORY", "") or image[8:10] != "= ":
        return Card(key, None, image[8:].rstrip(), image)
    value, com = _parse_value(image[10:])
    return Card(key, value, com, image)


class FitsHeader:
    """The cards of an HDU with a dict-like access by keyword (the first card of a keyword): ``h["CDELT1"]``,
    ``h.get(key, default)``, ``key in h``, ``h.cards`` (all cards, in order)."""

    def __init__(self, cards):
        self.cards = list(cards)
        self._first = {}
        for c in self.cards:
            if c.keyword and c.keyword not in ("COMMENT", "HISTORY") and c.keyword not in self._first:
                self._first[c.keyword] = c

    def __contains__(self, key):
        return key in self._first

    def __getitem__(self, key):
        return self._first[key].value

    def get(self, key, default=None):
        c = self._first.get(key)
        return default if c is None or c.value is None else c.value

    def history(self):
        return [c.comment for c in self.cards if c.keyword == "HISTORY"]


def _read_header(f):
    cards = []
    while True:
        block = f.read(BLOCK)
        if len(block) < BLOCK:
            raise ValueError("FITS: the file ends inside a header")
        text = block.decode("ascii", errors="replace")
        for i in range(0, BLOCK, CARD):
            img = text[i:i + CARD]
            if img[:8].strip() == "END" and img[:3] == "END":
                return FitsHeader(cards)
            cards.append(parse_card(img))


def _data_bytes(h):
    n = int(h.get("NAXIS", 0))
    if n == 0:
        return 0
    size = 1
    for i in range(n):
        size *= int(h.get(f"NAXIS{i + 1}", 0))
    pc, gc = int(h.get("PCOUNT", 0)), int(h.get("GCOUNT", 1))
    return abs(int(h["BITPIX"])) // 8 * gc * (pc + size)


def _hdus(f):
    """(header, offset of its data) of every HDU of an open file."""
    out = []
    while True:
        try:
            h = _read_header(f)
        except ValueError:
            if out:
                return out
            raise
        off = f.tell()
        out.append((h, off))
        nb = _data_bytes(h)
        f.seek(off + (nb + BLOCK - 1) // BLOCK * BLOCK)
        if f.read(1) == b"":
            return out
        f.seek(-1, os.SEEK_CUR)


def _select(name):
    """(path, hdu selector or None) of a file name, with a CFITSIO-like [n] or [EXTNAME] suffix."""
    if os.path.isfile(name):
        return name, None
    m = re.match(r"^(.+?)\[([^][:,*]+)\]$", str(name))
    if m and os.path.isfile(m.group(1)):
        e = m.group(2).strip()
        return m.group(1), int(e) if e.isdigit() else e
    return name, None


def read_fits(name, data=True):
    """(FitsHeader, data array or None) of the image of a FITS file: the primary HDU, or the first extension with
    an image when the primary has none; ``file.fits[n]`` / ``file.fits[EXTNAME]`` choose the HDU. The data array is
    in C order (NAXISn, ..., NAXIS1), float32 for BITPIX -32 and float64 otherwise (physical values)."""
    path, sel = _select(name)
    with open(path, "rb") as f:
        hdus = _hdus(f)
        if sel is None:
            idx = 0
            if int(hdus[0][0].get("NAXIS", 0)) == 0:
                idx = next((i for i, (h, _) in enumerate(hdus[1:], 1)
                            if int(h.get("NAXIS", 0)) > 0 and str(h.get("XTENSION", "IMAGE")).strip() == "IMAGE"), 0)
        elif isinstance(sel, int):
            idx = sel
        else:
            idx = next(i for i, (h, _) in enumerate(hdus) if str(h.get("EXTNAME", "")).strip() == sel)
        h, off = hdus[idx]
        if not data or int(h.get("NAXIS", 0)) == 0:
            return h, None
        bitpix = int(h["BITPIX"])
        shape = tuple(int(h[f"NAXIS{i}"]) for i in range(int(h["NAXIS"]), 0, -1))
        f.seek(off)
        raw = np.fromfile(f, dtype=np.dtype(_DTYPES[bitpix]), count=int(np.prod(shape))).reshape(shape)
    bscale, bzero = float(h.get("BSCALE", 1.0)), float(h.get("BZERO", 0.0))
    if bitpix > 0:
        out = raw.astype(np.float64)
        if "BLANK" in h:
            out[raw == int(h["BLANK"])] = np.nan
        return h, out * bscale + bzero
    out = raw.astype(np.float32 if bitpix == -32 else np.float64)
    if bscale != 1.0 or bzero != 0.0:
        out = out * bscale + bzero
    return h, out


class Raw(str):
    """A card value written as it is (e.g. a Fortran exponent: 3.0000000D+01, which GIPSY writes)."""


def _format_value(v):
    if isinstance(v, Raw):
        return f"{str(v):>20}"
    if isinstance(v, bool):
        return f"{'T' if v else 'F':>20}"
    if isinstance(v, (int, np.integer)):
        return f"{int(v):>20d}"
    if isinstance(v, (float, np.floating)):
        s = repr(float(v)).upper()
        if "E" not in s and "." not in s and "N" not in s:
            s += "."
        return f"{s:>20}"
    s = "'" + str(v).replace("'", "''") + "'"
    return f"{s:<20}" if len(s) < 20 else s


def card_image(key, value=None, comment=""):
    """The 80-character image of a card (key = value / comment, or a COMMENT/HISTORY card when value is None)."""
    if key in ("COMMENT", "HISTORY", "") or value is None:
        img = f"{key:<8}{comment}"
    else:
        img = f"{key:<8}= {_format_value(value)}" + (f" / {comment}" if comment else "")
    if len(img) > CARD:
        raise ValueError(f"FITS card too long: {img!r}")
    return f"{img:<80}"


def write_fits(path, data, cards=(), bitpix=-32, bscale=None, bzero=None, blank=None):
    """A single-HDU FITS file: the array data (C order: NAXISn ... NAXIS1) with the cards (key, value[, comment])
    after the structural ones; bitpix -32, -64 (floats) or 8, 16, 32, 64 (integers: stored = round((value - bzero)
    / bscale), NaN as blank)."""
    a = np.asarray(data)
    head = [card_image("SIMPLE", True), card_image("BITPIX", int(bitpix)), card_image("NAXIS", a.ndim)]
    for i in range(a.ndim):
        head.append(card_image(f"NAXIS{i + 1}", int(a.shape[a.ndim - 1 - i])))
    if bitpix > 0:
        bscale = 1.0 if bscale is None else float(bscale)
        bzero = 0.0 if bzero is None else float(bzero)
        head += [card_image("BSCALE", bscale), card_image("BZERO", bzero)]
        if blank is not None:
            head.append(card_image("BLANK", int(blank)))
    for c in cards:
        head.append(card_image(*c))
    head.append(f"{'END':<80}")
    text = "".join(head)
    text += " " * (-len(text) % BLOCK)
    if bitpix > 0:
        v = (a.astype(np.float64) - bzero) / bscale
        bad = ~np.isfinite(v)
        v = np.where(bad, 0.0, np.round(v))
        st = v.astype(np.dtype(_DTYPES[bitpix]).newbyteorder("="))
        if blank is not None:
            st[bad] = blank
        payload = st.astype(_DTYPES[bitpix]).tobytes()
    else:
        payload = a.astype(_DTYPES[bitpix]).tobytes()
    payload += b"\0" * (-len(payload) % BLOCK)
    with open(path, "wb") as f:
        f.write(text.encode("ascii"))
        f.write(payload)
