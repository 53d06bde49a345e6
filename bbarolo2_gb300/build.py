"""Builds ``libbbgpu.so`` in-tree (``bbarolo2_gb300/_build``) with nvcc for sm_103a: ``make -C csrc``.

A few translation units compiled in parallel; the host C++ without floating-point contraction. Used by
``__graft_entry__.build()`` and by the tests; a GPU machine builds its own copy (binaries do not travel).
"""

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "_build", "libbbgpu.so")


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    srcs = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    srcs.append(os.path.join(os.path.dirname(HERE), "include", "bbgpu.h"))
    return any(os.path.getmtime(s) > t for s in srcs)


def build(force=False, jobs=None):
    """Compiles the library if a source is newer than it (or force); returns its path."""
    if force or _stale():
        j = str(jobs or max(2, min(8, os.cpu_count() or 2)))
        subprocess.run(["make", "-s", "-C", CSRC, "-j", j], check=True)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
