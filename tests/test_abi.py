"""The C-ABI library builds, loads without a GPU, and exports every function declared in include/bbgpu.h."""
import ctypes
import os
import re

from bbarolo2_gb300 import _lib, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    src = open(os.path.join(ROOT, "include", "bbgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(bbgpu_\w+)\s*\(", src)))


def test_exports_every_declared_symbol():
    path = build.build()
    lib = ctypes.CDLL(path)
    names = declared()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) == set(_lib.SYMBOLS)


def test_version_and_no_device_errors():
    L = _lib.load(build.build())
    assert L.bbgpu_version() >= 1
    assert L.bbgpu_kernel_name(0) == b"prof_maps" and L.bbgpu_kernel_name(4) == b"mc_bin"
    # a null context is rejected, not dereferenced
    assert L.bbgpu_set_kernel(None, None, 3, 3) == _lib.ERR_ARG
    assert L.bbgpu_eval_run(None) == _lib.ERR_ARG


def test_subrings_rows_argument_checks():
    """The host-only table builder (no context, no GPU) rejects what it cannot tabulate, writing nothing."""
    import numpy as np
    L = _lib.load(build.build())
    nb, nr, nsub = 2, 3, 4
    rows = np.zeros((nb, 17, nr))
    i1 = np.array([1, 1, 2, 2], np.int64)
    dr, dseg, radii = np.zeros(nsub), np.ones(nr - 1), np.arange(nsub, dtype=float)
    cst = np.zeros(nsub, np.uint8)
    side = np.ones((2, nsub))
    sr = np.full((nb, 16, nsub), 7.)
    nv = np.zeros((nb, nsub), np.int64)
    P = _lib.ptr

    def call(nr_=nr, i1_=i1, ms=None, nsm=0):
        return L.bbgpu_subrings_rows(P(rows), nb, nr_, nsub, P(i1_), P(dr), P(dseg), P(cst), P(radii), None,
                                     P(side), 16, P(sr), P(nv), P(ms), nsm)

    assert call(nr_=1) == _lib.ERR_ARG                              # one ring: the numpy path
    assert call(i1_=np.array([1, 1, 2, 3], np.int64)) == _lib.ERR_ARG  # a segment past the last ring
    assert call(ms=np.zeros((nb, 16, 2)), nsm=2) == _lib.ERR_ARG     # a maps table narrower than the tables
    assert np.all(sr == 7.)
    assert call() == _lib.OK
    assert np.array_equal(sr[:, 0], np.broadcast_to(radii, (nb, nsub))) and np.all(nv == 1)


def test_oracle_is_not_linked_by_the_product():
    """The product library does not reference the oracle's symbols (ref_*)."""
    import subprocess
    out = subprocess.run(["nm", "-D", build.build()], capture_output=True, text=True).stdout
    assert " ref_" not in out
