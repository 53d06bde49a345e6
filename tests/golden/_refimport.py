"""Import the reference's hot-path modules as plain Python, for generating golden fixtures.

Used only by ``make_golden.py`` in a container that has the reference source tree. The reference
package ``bbarolo`` cannot be imported as a whole without astropy and numba, so:

* a stub ``numba`` module whose ``njit`` returns the function unchanged is put in ``sys.modules``;
* ``bbarolo`` and ``bbarolo.bayesian`` are registered as empty packages whose ``__path__`` points at
  the reference tree, so that ``bbarolo._rng``, ``bbarolo.galmod``, ``bbarolo.smooth``,
  ``bbarolo.galfit`` (its numba kernels) and ``bbarolo.bayesian.likelihood`` import as plain Python.

The kernels then run as the reference code itself (CPython ``math`` = the C library's libm, as numba
lowers them; numpy uint64 arithmetic wraps like numba's).
"""

import os
import sys
import types

def ref_root():
    """The reference source tree: the directory named by the BBAROLO_REF environment variable (required)."""
    root = os.environ.get("BBAROLO_REF")
    if not root or not os.path.isdir(os.path.join(root, "bbarolo")):
        raise RuntimeError("set BBAROLO_REF to the root of the reference source tree (the directory holding bbarolo/)")
    return root


def _stub_numba():
    if "numba" in sys.modules and getattr(sys.modules["numba"], "_is_stub", False):
        return
    nb = types.ModuleType("numba")
    nb._is_stub = True

    def njit(*args, **kw):
        if len(args) == 1 and callable(args[0]) and not kw:
            return args[0]
        return lambda f: f
    nb.njit = njit
    nb.jit = njit
    nb.prange = range
    nb.int64 = int
    nb.float64 = float
    nb.boolean = bool
    sys.modules["numba"] = nb


def load():
    """Returns a namespace with the reference modules (_rng, galmod, smooth, galfit, likelihood)."""
    _stub_numba()
    pkg = os.path.join(ref_root(), "bbarolo")
    if "bbarolo" not in sys.modules:
        m = types.ModuleType("bbarolo")
        m.__path__ = [pkg]
        sys.modules["bbarolo"] = m
    if "bbarolo.bayesian" not in sys.modules:
        m = types.ModuleType("bbarolo.bayesian")
        m.__path__ = [os.path.join(pkg, "bayesian")]
        sys.modules["bbarolo.bayesian"] = m
    import importlib
    ns = types.SimpleNamespace()
    ns.rng = importlib.import_module("bbarolo._rng")
    ns.galmod = importlib.import_module("bbarolo.galmod")
    ns.smooth = importlib.import_module("bbarolo.smooth")
    ns.rings = importlib.import_module("bbarolo.rings")
    ns.bbutils = importlib.import_module("bbarolo.bbutils")
    ns.likelihood = importlib.import_module("bbarolo.bayesian.likelihood")
    try:
        ns.galfit = importlib.import_module("bbarolo.galfit")
    except Exception as e:            # (galfit imports more of the package)
        ns.galfit = None
        ns.galfit_error = repr(e)
    try:
        ns.profile = importlib.import_module("bbarolo.profile")
    except Exception as e:
        ns.profile = None
        ns.profile_error = repr(e)
    return ns
