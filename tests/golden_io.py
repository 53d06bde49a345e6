"""Loading of the golden fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py from the reference)."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


def cases(name):
    z = load(name)
    return z, json.loads(str(z["index"]))


def dense(idx, val, shape):
    a = np.zeros(int(np.prod(shape)))
    a[idx] = val
    return a.reshape(shape)


def call_args_mc(meta, arrs, nm):
    """The _galmod_mc arguments of a fixture case (after out, sr, ring_lo, ring_hi)."""
    m = meta
    return (m["seed32"], m["radsep"], arrs[nm + "/nv"], m["cdens"], m["cmode"], m["pixarea"], m["cdelt0"],
            m["cdelt1"], m["crota2"], m["blo"][0], m["blo"][1], m["bhi"][0], m["bhi"][1], m["ltype"],
            m["sig_instr"], m["axtyp"], m["velsys"], arrs[nm + "/lfreq0"], m["crval3"], m["cdelt3"], m["crpix3"],
            arrs[nm + "/relint"], arrs[nm + "/cd2i"])


def call_args_an(meta, arrs, nm, nzq):
    m = meta
    return (m["radsep"], m["cdens"], m["pixarea"], m["cdelt0"], m["cdelt1"], m["crota2"], m["blo"][0], m["blo"][1],
            m["bhi"][0], m["bhi"][1], m["ltype"], m["sig_instr"], arrs[nm + "/vedges"], arrs[nm + "/relint"],
            arrs[nm + "/cd2i"], nzq, m["axtyp"], m["velsys"], arrs[nm + "/lfreq0"], m["crval3"], m["cdelt3"],
            m["crpix3"], m["chmin"])
