"""ctypes binding of the C ABI in include/wendy_gb300.h.

Loads ``_wendy_gb300.so`` from this package directory, the way wendy loads
``wendy_c`` (wendy/wendy.py:13-37), and declares the argument types of every
entry point.  There is no fallback: if the library is missing or the CUDA
runtime cannot load it, :func:`lib` raises.
"""
import ctypes
import os
import weakref

import numpy
from numpy.ctypeslib import ndpointer

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_wendy_gb300.so")

WG_OK = 0
WG_ERR_ARG, WG_ERR_CUDA, WG_ERR_NOMEM, WG_ERR_DEVICE = -1, -2, -3, -4
WG_ERR_EXT, WG_ERR_BUDGET, WG_ERR_NODEV, WG_ERR_MAXCOLL = -5, -6, -7, -8
STATUS_NAMES = {0: "WG_OK", -1: "WG_ERR_ARG", -2: "WG_ERR_CUDA", -3: "WG_ERR_NOMEM",
                -4: "WG_ERR_DEVICE", -5: "WG_ERR_EXT", -6: "WG_ERR_BUDGET", -7: "WG_ERR_NODEV",
                -8: "WG_ERR_MAXCOLL"}

EXT_NONE, EXT_HARMONIC, EXT_PULSE_TANH, EXT_EXPR = 0, 1, 2, 3

# Every symbol include/wendy_gb300.h declares.
EXPORTS = ("wg_version", "wg_status_string", "wg_last_error", "wg_device_info", "wg_create",
           "wg_step", "wg_step_begin", "wg_step_end", "wg_download", "wg_energy", "wg_get_stats", "wg_destroy", "wg_accel", "wg_ext_force_eval",
           "wg_nbody_approx_onestep", "wg_nbody_approx_stats", "wg_profile", "wg_host_register", "wg_host_unregister",
           "wg_host_alloc", "wg_host_free",
           "wg_accel_noalloc", "wg_pool_sim_bytes", "wg_pool_create", "wg_pool_add",
           "wg_pool_remove", "wg_pool_step", "wg_pool_step_begin", "wg_pool_step_end", "wg_pool_download", "wg_pool_download_many", "wg_pool_get_stats", "wg_pool_info",
           "wg_pool_destroy", "wg_set_tuning", "wg_get_tuning", "wg_set_debug_wait",
           "wg_exact_create", "wg_exact_step", "wg_exact_download", "wg_exact_destroy")

# Largest n wg_accel_noalloc accepts (its fixed device scratch array).
NOALLOC_MAX_SHEETS = 65536


class WgSheet(ctypes.Structure):
    """``wg_sheet`` == wendy's ``struct array_w_index`` (wendy/wendy.h:12-16)."""

    _fields_ = [("idx", ctypes.c_int), ("val", ctypes.c_double)]


SHEET_DTYPE = numpy.dtype({"names": ["idx", "val"], "formats": [numpy.int32, numpy.float64],
                           "offsets": [0, 8], "itemsize": 16})


class WgStats(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("substeps", ctypes.c_int64),
                ("sorts_full", ctypes.c_int64), ("sorts_skipped", ctypes.c_int64),
                ("sorts_window", ctypes.c_int64), ("last_max_disp", ctypes.c_double),
                ("device_bytes", ctypes.c_int64), ("launches", ctypes.c_int64),
                ("last_max_count", ctypes.c_int64), ("substeps_compact", ctypes.c_int64),
                ("big_buckets", ctypes.c_int64), ("substeps_predicted", ctypes.c_int64)]


class WgPoolStats(ctypes.Structure):
    _fields_ = [(f, ctypes.c_int64) for f in (
        "steps", "launches", "graph_builds", "members_sorted", "overflows", "recovery_rounds",
        "sheets_resorted", "substeps_relaunched")] + [
        ("graph_seconds", ctypes.c_double), ("recovery_seconds", ctypes.c_double),
        ("members_compact", ctypes.c_int64), ("substeps_compact", ctypes.c_int64)]


class WgTuning(ctypes.Structure):
    _fields_ = [("n_min", ctypes.c_int64), ("target", ctypes.c_int), ("window", ctypes.c_int),
                ("sort_bits", ctypes.c_int), ("ctas_per_sm", ctypes.c_int)]


class WendyGPUError(RuntimeError):
    def __init__(self, status, where, detail):
        self.status = status
        super().__init__("%s failed with %s (%d): %s" % (where, STATUS_NAMES.get(status, "?"),
                                                         status, detail))


_F64 = ndpointer(dtype=numpy.float64, flags=("C_CONTIGUOUS",))
_F64W = ndpointer(dtype=numpy.float64, flags=("C_CONTIGUOUS", "WRITEABLE"))
_I32W = ndpointer(dtype=numpy.int32, flags=("C_CONTIGUOUS", "WRITEABLE"))
_P = ctypes.c_void_p
_D = ctypes.c_double
_I = ctypes.c_int
_I64 = ctypes.c_int64

_lib = None


def load_raw(path=LIB_PATH):
    """Load the shared library without needing a GPU (symbols only)."""
    if not os.path.exists(path):
        raise ImportError("wendy_gb300 CUDA library not built: %s is missing "
                          "(run `python -m wendy_gb300.build`)" % path)
    return ctypes.CDLL(path)


def lib():
    global _lib
    if _lib is not None:
        return _lib
    L = load_raw()
    L.wg_version.restype = _I
    L.wg_status_string.argtypes = [_I]
    L.wg_status_string.restype = ctypes.c_char_p
    L.wg_last_error.restype = ctypes.c_char_p
    L.wg_device_info.argtypes = [ctypes.POINTER(_I), ctypes.POINTER(_I64), ctypes.POINTER(_I64)]
    L.wg_create.argtypes = [_I64, _F64, _F64, _F64, _D, _D, _I, _F64, _I,
                            ctypes.POINTER(_P)]
    L.wg_step.argtypes = [_P, _D, _I, ctypes.POINTER(_D), ctypes.POINTER(_D)]
    L.wg_step_begin.argtypes = [_P, _D, _I, ctypes.POINTER(_D)]
    L.wg_step_end.argtypes = [_P, ctypes.POINTER(_D)]
    L.wg_download.argtypes = [_P, _P, _P]
    L.wg_energy.argtypes = [_P, _D, _D, ctypes.POINTER(_D), ctypes.POINTER(_D)]
    L.wg_get_stats.argtypes = [_P, ctypes.POINTER(WgStats)]
    L.wg_nbody_approx_stats.argtypes = [ctypes.POINTER(WgStats)]
    L.wg_destroy.argtypes = [_P]
    L.wg_accel.argtypes = [_I64, _F64, _F64, _D, _D, _I, _F64, _I, _D, _P, _P]
    L.wg_ext_force_eval.argtypes = [_I64, _F64, _D, _I, _F64, _I, _F64W]
    L.wg_nbody_approx_onestep.argtypes = [_I, _P, _F64W, _F64W, _F64, _F64W, _D, _D, _I,
                                          ctypes.POINTER(_D), _D, _I, _F64, _I,
                                          ctypes.POINTER(_I), ctypes.POINTER(_D)]
    L.wg_profile.argtypes = [_P, _I, _I, ctypes.POINTER(_D)]
    L.wg_host_register.argtypes = [_P, _I64]
    L.wg_host_alloc.argtypes = [_I64, ctypes.POINTER(_P)]
    L.wg_host_free.argtypes = [_P]
    L.wg_host_unregister.argtypes = [_P]
    L.wg_accel_noalloc.argtypes = [_I64, _P, _P, _D, _D, _I, _F64, _I, _D, _P, _P, _P]
    L.wg_set_debug_wait.argtypes = [ctypes.c_uint, _I64]
    _I32 = ndpointer(dtype=numpy.int32, flags=("C_CONTIGUOUS",))
    L.wg_exact_create.argtypes = [_I64, _F64, _F64, _F64, _F64, _I32, _D, ctypes.POINTER(_P)]
    L.wg_exact_step.argtypes = [_P, _D, _I64, ctypes.POINTER(_I64), ctypes.POINTER(_D)]
    L.wg_exact_download.argtypes = [_P, _P, _P, _P, _P]
    L.wg_exact_destroy.argtypes = [_P]
    L.wg_pool_sim_bytes.argtypes = [_I64]
    L.wg_pool_create.argtypes = [_I64, ctypes.POINTER(_P)]
    L.wg_pool_add.argtypes = [_P, _I64, _F64, _F64, _F64, _D, _D, _I, _F64, _I,
                              ctypes.POINTER(_I)]
    L.wg_pool_remove.argtypes = [_P, _I]
    L.wg_pool_step.argtypes = [_P, _I, _P, _P, _I, _P, ctypes.POINTER(_D)]
    L.wg_pool_step_begin.argtypes = [_P, _I, _P, _P, _I, _P]
    L.wg_pool_step_end.argtypes = [_P, ctypes.POINTER(_D)]
    L.wg_pool_download.argtypes = [_P, _I, _P, _P]
    L.wg_pool_download_many.argtypes = [_P, _I, _P, _P, _P]
    L.wg_pool_get_stats.argtypes = [_P, ctypes.POINTER(WgPoolStats)]
    L.wg_pool_info.argtypes = [_P, ctypes.POINTER(_I64), ctypes.POINTER(_I64),
                               ctypes.POINTER(_I), ctypes.POINTER(_I64)]
    L.wg_pool_destroy.argtypes = [_P]
    L.wg_set_tuning.argtypes = [_P, _I]
    L.wg_get_tuning.argtypes = [_I64, ctypes.POINTER(WgTuning)]
    for name in EXPORTS:
        if name not in ("wg_status_string", "wg_last_error"):
            getattr(L, name).restype = _I
    L.wg_pool_sim_bytes.restype = _I64
    _lib = L
    # the tuning table measured on a GB300 that ships with the package
    from . import autotune
    autotune.apply_shipped()
    return L


def check(status, where):
    if status != WG_OK:
        detail = lib().wg_last_error().decode(errors="replace")
        raise WendyGPUError(status, where, detail)


def pinned_empty(shape, dtype=numpy.float64):
    """An uninitialised numpy array in page-locked host memory (wg_host_alloc),
    released when the array and every view of it are gone.  On the measured
    hosts, memory page-locked by registration (wg_host_register) loses most
    of its copy rate after tens of seconds of device load; this memory kept
    it in the same test."""
    dtype = numpy.dtype(dtype)
    count = int(numpy.prod(shape, dtype=numpy.int64))
    nbytes = max(count * dtype.itemsize, 1)
    ptr = ctypes.c_void_p()
    check(lib().wg_host_alloc(nbytes, ctypes.byref(ptr)), "wg_host_alloc")
    raw = (ctypes.c_char * nbytes).from_address(ptr.value)
    weakref.finalize(raw, lib().wg_host_free, ptr.value)
    return numpy.frombuffer(raw, dtype=dtype, count=count).reshape(shape)


def ext_params(params):
    """The parameters of an external force as the float64 array the C ABI
    takes (at least 4 entries, zero-padded)."""
    p = numpy.zeros(max(4, len(params)))
    p[:len(params)] = params
    return p
