"""ctypes binding of ``libbbgpu.so`` (the C ABI declared in ``include/bbgpu.h``).

The library is built in-tree (``bbarolo2_gb300/_build/libbbgpu.so``, see ``bbarolo2_gb300.build``). There is no
CPU fallback: if the library is missing or no GPU is visible, the calls raise.
"""

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "_build", "libbbgpu.so")

OK, ERR_ARG, ERR_CUDA, ERR_NOMEM, ERR_STATE, ERR_KERNEL = 0, -1, -2, -3, -4, -5
MC, ANALYTIC = 0, 1
OPT_KEEP_SMOOTHED, OPT_TIMING, OPT_SHARE, OPT_CONV, OPT_GRAPHS = 1, 2, 3, 4, 5
CONV_AUTO, CONV_F32, CONV_BF16X3, CONV_TF32X3 = -1, 0, 1, 2
CONV_NAMES = {0: "f32", 1: "bf16x3", 2: "tf32x3"}

# every symbol of include/bbgpu.h (the ABI test checks that the library exports them all)
SYMBOLS = ("bbgpu_ctx_create", "bbgpu_ctx_destroy", "bbgpu_last_error", "bbgpu_version", "bbgpu_set_grid",
           "bbgpu_set_kernel", "bbgpu_set_cube", "bbgpu_galmod_mc", "bbgpu_galmod_analytic",
           "bbgpu_ring_maps_analytic", "bbgpu_convolve", "bbgpu_conv_sparse", "bbgpu_sumsq_residuals",
           "bbgpu_residuals_fracerr", "bbgpu_norm", "bbgpu_eval_upload", "bbgpu_eval_run", "bbgpu_eval_download",
           "bbgpu_eval_batch", "bbgpu_eval_model", "bbgpu_sync", "bbgpu_set_option", "bbgpu_launch_count",
           "bbgpu_last_run_times", "bbgpu_kernel_name", "bbgpu_transfer_bytes", "bbgpu_shared_members",
           "bbgpu_sumsq_residuals_noalloc", "bbgpu_set_profile", "bbgpu_eval_upload_profile", "bbgpu_eval_profile", "bbgpu_solve_profile",
           "bbgpu_subrings_rows", "bbgpu_conv_variant", "bbgpu_graph_stats", "bbgpu_mlp_create",
           "bbgpu_mlp_destroy", "bbgpu_mlp_nparams", "bbgpu_mlp_get_params", "bbgpu_mlp_set_params",
           "bbgpu_mlp_predict", "bbgpu_mlp_gradients", "bbgpu_mlp_train_step", "bbgpu_mlp_train",
           "bbgpu_galmod_wind", "bbgpu_galwind_spherical", "bbgpu_wind_create", "bbgpu_wind_destroy", "bbgpu_wind_last_error", "bbgpu_wind_launch_count",
           "bbgpu_wind_set_cells", "bbgpu_wind_points", "bbgpu_wind_set_points", "bbgpu_wind_boxes",
           "bbgpu_wind_columns", "bbgpu_wind_set_weights", "bbgpu_wind_normal", "bbgpu_wind_model")


class Grid(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("nlines", C.c_int), ("axtyp", C.c_int),
                ("velsys", C.c_int), ("ltype", C.c_int), ("cmode", C.c_int), ("radsep", C.c_double),
                ("cdens", C.c_double), ("pixarea", C.c_double), ("cdelt0", C.c_double), ("cdelt1", C.c_double),
                ("crota2", C.c_double), ("sig_instr", C.c_double), ("crval3", C.c_double),
                ("cdelt3", C.c_double), ("crpix3", C.c_double), ("chwidth", C.c_double), ("zstep", C.c_double),
                ("scalefactor", C.c_double)]


class WindGrid(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("nlines", C.c_int), ("axtyp", C.c_int),
                ("velsys", C.c_int), ("cdelt0", C.c_double), ("cdelt1", C.c_double), ("sig_instr", C.c_double),
                ("chmin", C.c_double), ("crval3", C.c_double), ("cdelt3", C.c_double), ("crpix3", C.c_double)]


class WindGeometry(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("x0", "y0", "vsys", "sinc", "cinc", "spa", "cpa", "th_in", "th_out",
                                          "rmax")]


class EvalDesc(C.Structure):
    _fields_ = [("blo0", C.c_int32), ("blo1", C.c_int32), ("bhi0", C.c_int32), ("bhi1", C.c_int32),
                ("seed", C.c_uint64), ("maskmode", C.c_int32), ("use_region", C.c_int32),
                ("sigma2", C.c_double), ("eps2", C.c_double)]


EVAL_DTYPE = np.dtype([("blo0", np.int32), ("blo1", np.int32), ("bhi0", np.int32), ("bhi1", np.int32),
                       ("seed", np.uint64), ("maskmode", np.int32), ("use_region", np.int32),
                       ("sigma2", np.float64), ("eps2", np.float64)], align=True)
assert EVAL_DTYPE.itemsize == C.sizeof(EvalDesc)

_lib = None


class DeviceError(RuntimeError):
    """A failure reported by the device library (status code and message)."""

    def __init__(self, code, msg):
        super().__init__(f"bbgpu error {code}: {msg}")
        self.code = code


def load(path=None):
    """The loaded library (ctypes.CDLL) with its prototypes; raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIBPATH
    if not os.path.exists(p):
        raise RuntimeError(f"libbbgpu.so not built ({p}): run bbarolo2_gb300.build.build() (no CPU fallback)")
    L = C.CDLL(p)
    vp, i, d, i64, u64 = C.c_void_p, C.c_int, C.c_double, C.c_int64, C.c_uint64
    proto = {
        "bbgpu_ctx_create": (i, [C.POINTER(vp), i]),
        "bbgpu_ctx_destroy": (i, [vp]),
        "bbgpu_subrings_rows": (i, [vp, i, i, i, vp, vp, vp, vp, vp, vp, vp, i64, vp, vp, vp, i]),
        "bbgpu_last_error": (C.c_char_p, [vp]),
        "bbgpu_version": (i, []),
        "bbgpu_set_grid": (i, [vp, C.POINTER(Grid), vp, vp, vp, vp]),
        "bbgpu_set_kernel": (i, [vp, vp, i, i]),
        "bbgpu_set_cube": (i, [vp, vp, vp, vp]),
        "bbgpu_galmod_mc": (i, [vp, vp, vp, i, i, i, u64, vp, i, i, i, i]),
        "bbgpu_galmod_analytic": (i, [vp, vp, vp, i, i, i, i, i, i, i, i]),
        "bbgpu_ring_maps_analytic": (i, [vp, vp, i, vp, i, vp, vp, i, i, i, i, i]),
        "bbgpu_convolve": (i, [vp, vp, vp, i, i, i, d, i]),
        "bbgpu_conv_sparse": (i, [vp, vp, vp, i, i, i, vp, i, i, d]),
        "bbgpu_sumsq_residuals": (i, [vp, vp, vp, vp, i, vp, i, i, i, vp]),
        "bbgpu_residuals_fracerr": (i, [vp, vp, vp, vp, i, vp, i, i, i, d, d, vp]),
        "bbgpu_norm": (i, [vp, vp, i, i, i, vp, vp, i, i, i64, i64, d, d, d, d, d, d, d, i, i, vp, d, d, i, vp,
                           vp, vp, i, vp, i, d, vp]),
        "bbgpu_eval_upload": (i, [vp, i, i, i, vp, vp, vp]),
        "bbgpu_eval_run": (i, [vp]),
        "bbgpu_eval_download": (i, [vp, vp, vp]),
        "bbgpu_eval_batch": (i, [vp, i, i, i, vp, vp, vp, vp, vp]),
        "bbgpu_eval_model": (i, [vp, i, i, vp, i, i, i]),
        "bbgpu_sync": (i, [vp]),
        "bbgpu_set_option": (i, [vp, i, i]),
        "bbgpu_launch_count": (i64, [vp]),
        "bbgpu_last_run_times": (i, [vp, vp, i]),
        "bbgpu_kernel_name": (C.c_char_p, [i]),
        "bbgpu_transfer_bytes": (i, [vp, vp, vp]),
        "bbgpu_shared_members": (i, [vp, vp, vp, vp, vp]),
        "bbgpu_conv_variant": (i, [vp, vp, vp]),
        "bbgpu_graph_stats": (i, [vp, vp, vp]),
        "bbgpu_mlp_create": (i, [C.POINTER(vp), i, i, i, u64]),
        "bbgpu_mlp_destroy": (i, [vp]),
        "bbgpu_mlp_nparams": (C.c_longlong, [vp]),
        "bbgpu_mlp_get_params": (i, [vp, vp]),
        "bbgpu_mlp_set_params": (i, [vp, vp]),
        "bbgpu_mlp_predict": (i, [vp, vp, i, vp]),
        "bbgpu_mlp_gradients": (i, [vp, vp, vp, i, vp, vp]),
        "bbgpu_mlp_train_step": (i, [vp, vp, vp, i, C.c_float, vp]),
        "bbgpu_mlp_train": (i, [vp, vp, vp, C.c_longlong, i, i, C.c_float, C.c_uint64, vp]),
        "bbgpu_sumsq_residuals_noalloc": (i, [vp, vp, vp, i, vp, i, i, i, d, d, vp, vp]),
        "bbgpu_set_profile": (i, [vp, i, i, i, i, i, vp, vp, vp, vp, d, d, d, d]),
        "bbgpu_eval_upload_profile": (i, [vp, i, vp, vp, vp]),
        "bbgpu_eval_profile": (i, [vp, vp, vp]),
        "bbgpu_solve_profile": (i, [vp, vp, vp, i, i, vp, d, d, d, vp, vp]),
        "bbgpu_galmod_wind": (i, [vp, vp, vp, i, i, i, u64, d, vp, i, i, i, i]),
        "bbgpu_galwind_spherical": (i, [vp, vp, vp, i, i, vp, vp, vp, d, vp, i, i, i, i, i]),
        "bbgpu_wind_create": (i, [C.POINTER(vp), i, C.POINTER(WindGrid), vp, vp, vp, vp, i, i, vp, vp, i]),
        "bbgpu_wind_destroy": (i, [vp]),
        "bbgpu_wind_last_error": (C.c_char_p, [vp]),
        "bbgpu_wind_launch_count": (i64, [vp]),
        "bbgpu_wind_set_cells": (i, [vp, i, vp, vp, vp]),
        "bbgpu_wind_points": (i, [vp, C.POINTER(WindGeometry), i, vp, vp, vp, vp] + [vp] * 8),
        "bbgpu_wind_set_points": (i, [vp, vp, vp, vp, vp, vp]),
        "bbgpu_wind_boxes": (i, [vp, vp, vp, vp, vp]),
        "bbgpu_wind_columns": (i, [vp, vp, vp]),
        "bbgpu_wind_set_weights": (i, [vp, vp, vp]),
        "bbgpu_wind_normal": (i, [vp, vp, d, vp, vp]),
        "bbgpu_wind_model": (i, [vp, vp, vp]),
    }
    for name, (res, args) in proto.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def ptr(a):
    """Data pointer of a numpy array (None for None)."""
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Context:
    """A device context (``bbgpu_ctx``): one GPU, one stream, the constants of one cube."""

    def __init__(self, device=0):
        self.L = load()
        h = C.c_void_p()
        rc = self.L.bbgpu_ctx_create(C.byref(h), int(device))
        if rc != OK:
            raise DeviceError(rc, "cannot create a context (no CUDA device visible?)")
        self.h = h

    def check(self, rc):
        if rc != OK:
            msg = self.L.bbgpu_last_error(self.h)
            raise DeviceError(rc, msg.decode() if msg else "")
        return rc

    def close(self):
        if getattr(self, "h", None):
            self.L.bbgpu_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def launches(self):
        return int(self.L.bbgpu_launch_count(self.h))

    def shared_members(self):
        """(profiles computed, MC members with all their clouds, MC members as a difference, MC members replaying
        member 0's clouds) of the last batch."""
        a, b, c, d = (C.c_int(0) for _ in range(4))
        self.check(self.L.bbgpu_shared_members(self.h, C.byref(a), C.byref(b), C.byref(c), C.byref(d)))
        return a.value, b.value, c.value, d.value

    def run_times(self):
        t = np.zeros(16)
        n = self.L.bbgpu_last_run_times(self.h, ptr(t), 16)
        return {self.L.bbgpu_kernel_name(i).decode(): float(t[i]) for i in range(n)}

    def transfer_bytes(self):
        a, b = np.zeros(1, np.int64), np.zeros(1, np.int64)
        self.check(self.L.bbgpu_transfer_bytes(self.h, ptr(a), ptr(b)))
        return int(a[0]), int(b[0])

    def set_option(self, opt, value):
        self.check(self.L.bbgpu_set_option(self.h, int(opt), int(value)))

    def graph_stats(self):
        """(graph replays so far, kernels per replay of the current batch's graph, 0 without one)."""
        a, b = np.zeros(1, np.int64), np.zeros(1, np.int64)
        self.check(self.L.bbgpu_graph_stats(self.h, ptr(a), ptr(b)))
        return int(a[0]), int(b[0])

    def conv_variant(self):
        """(variant of the last batch convolution, {variant: ms} of the autotuner's timings)."""
        u = C.c_int(0)
        t = np.zeros(3, np.float32)
        self.check(self.L.bbgpu_conv_variant(self.h, C.byref(u), ptr(t)))
        return u.value, {CONV_NAMES[i]: float(t[i]) for i in range(3) if t[i] >= 0}
