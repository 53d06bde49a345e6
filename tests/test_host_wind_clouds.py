"""The host parse of the GALWIND stream (``bbh_wind_clouds`` in ``csrc/host_setup.cpp``), on the CPU: compiled with
a test shim (``tests/host/wind_clouds_shim.cpp``) and compared with the oracle's stream, draw by draw: the cloud
counts and the shells' constants of ``_galmod_wind`` (``bbarolo/galmod.py:546-566``), each cloud's radius, azimuth
and polar angle (``:567-573``), and each velocity deviate: the one-word ones from their first word and the
ziggurat's tables, the others from the side list."""
import ctypes as C
import math
import os
import subprocess

import numpy as np
import pytest

import wind_cases as WC
from golden_io import cases

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def shim(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("shim") / "libwindshim.so")
    subprocess.run(["g++", "-O2", "-fPIC", "-shared", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-o", out,
                    os.path.join(HERE, "host", "wind_clouds_shim.cpp"),
                    os.path.join(ROOT, "bbarolo2_gb300", "csrc", "host_setup.cpp")], check=True)
    return C.CDLL(out)


def _dump(L, seed, sr, lo, hi, sep, nv, cdens, pixarea, sig_instr, crota2):
    p = lambda a: None if a is None else a.ctypes.data_as(C.c_void_p)
    args = [C.c_uint64(seed), p(sr), C.c_int(sr.shape[1]), C.c_int(lo), C.c_int(hi), C.c_double(sep), p(nv),
            C.c_double(cdens), C.c_int(1), C.c_double(pixarea), C.c_double(sig_instr), C.c_double(crota2)]
    counts = np.zeros(4, np.int64)
    assert L.wind_clouds_dump(*args, p(counts), *[None] * 8) == 0
    ns, nc, nh, nsl = (int(v) for v in counts)
    shells = np.zeros((max(ns, 1), 12))
    shell, geo = np.zeros(max(nc, 1), np.int32), np.zeros((max(nc, 1), 5))
    nb, sb = np.zeros(max(nc, 1), np.int64), np.zeros(max(nc, 1), np.int64)
    hz, slow = np.zeros(max(nh, 1), np.int32), np.zeros(max(nsl, 1))
    assert L.wind_clouds_dump(*args, p(counts), p(shells), p(shell), p(geo), p(nb), p(sb), p(hz), p(slow)) == 0
    return shells[:ns], shell[:nc], geo[:nc], nb[:nc], sb[:nc], hz[:nh], slow[:nsl]


@pytest.mark.parametrize("name", list(WC.GW_CASES))
def test_host_stream_parse_matches_oracle(oracle_lib, shim, name):
    O = oracle_lib
    z, idx = cases("wind.npz")
    m = idx[name]
    sr, nv = z[name + "/sr"], z[name + "/nv"]
    kn, wn, _ = O.zig_tables()
    for t, (lo, hi) in enumerate(z[name + "/chunks"]):
        seed = (m["seed"] + 7919 * t) & 0xFFFFFFFF
        shells, shell, geo, nb, sb, hz, slow = _dump(shim, seed, sr, int(lo), int(hi), m["sep"], nv, m["cdens"],
                                                     m["pixarea"], m["sig_instr"], m["crota2"])
        rng = O.RNG(seed)
        ic_all, si = 0, 0
        for ir in range(int(lo), int(hi)):
            rtmp = sr[0, ir]
            nc = int(math.floor(m["cdens"] * sr[4, ir] ** 1 * 2 * math.pi * rtmp * m["sep"] / m["pixarea"] + 0.5))
            if nc == 0:
                continue
            # (fluxsc and vdisp of the shell; the record's first field is fluxsc, the second vdisp)
            assert shells[si, 0] == sr[4, ir] * 2 * math.pi * rtmp * m["sep"] / (nc * int(nv[ir]))
            assert shells[si, 1] == math.sqrt(sr[3, ir] * sr[3, ir] + m["sig_instr"] * m["sig_instr"])
            for ic in range(nc):
                rad = math.sqrt((rtmp - 0.5 * m["sep"]) ** 2 + 2 * m["sep"] * rtmp * abs(2.0 * rng.uniform() - 1.0))
                az = 2 * math.pi * abs(2.0 * rng.uniform() - 1.0)
                ph = sr[7, ir] / 2. * abs(2.0 * rng.uniform() - 1.0)
                if ic % 2 == 0:
                    ph = math.pi - ph
                assert shell[ic_all] == si
                assert tuple(geo[ic_all]) == (rad, math.cos(az), math.sin(az), math.sin(ph), math.cos(ph))
                js = int(sb[ic_all])
                for iv in range(int(nv[ir])):
                    ref = rng.normal()
                    h = int(hz[nb[ic_all] + iv])
                    if abs(h) < kn[h & 127]:
                        assert float(h) * wn[h & 127] == ref
                    else:
                        assert slow[js] == ref
                        js += 1
                ic_all += 1
            si += 1
        assert ic_all == shell.size and si == shells.shape[0]
