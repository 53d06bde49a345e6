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


def test_oracle_is_not_linked_by_the_product():
    """The product library does not reference the oracle's symbols (ref_*)."""
    import subprocess
    out = subprocess.run(["nm", "-D", build.build()], capture_output=True, text=True).stdout
    assert " ref_" not in out
