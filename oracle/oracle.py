"""TEST INFRASTRUCTURE ONLY -- ctypes front end of the CPU oracle.

Loads ``oracle/libwendy_oracle.so`` (a C restatement of wendy's approximate
integrator, see ``wendy_oracle.c``) and, where it was built, the reference's
own library from ``oracle/_ref/``.  Only tests, ``__graft_entry__.smoke()``
and ``bench.py``'s CPU-baseline / reference legs import this module; the
product package ``wendy_gb300`` never does.

The generator :func:`nbody_approx` mirrors ``wendy._nbody_approx``
(wendy/wendy.py:336-437): it scales the masses by twopiG, sums them with
numpy for ``totmass``, builds the (idx, val) records in original order and
makes one C call per output, yielding the same (mutated in place) ``x, v``
arrays each time.
"""
import ctypes
import os
import subprocess
import sys
import sysconfig

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libwendy_oracle.so")
EXT_SUFFIX = sysconfig.get_config_var("EXT_SUFFIX")
REF_DIR = os.path.join(HERE, "_ref")

EXT_NONE, EXT_HARMONIC, EXT_PULSE_TANH, EXT_EXPR = 0, 1, 2, 3
SORT_IDS = {"quick": 0, "qsort": 3, "parallel": 4}

_F64 = numpy.ctypeslib.ndpointer(dtype=numpy.float64, flags=("C_CONTIGUOUS", "WRITEABLE"))
_F64R = numpy.ctypeslib.ndpointer(dtype=numpy.float64, flags=("C_CONTIGUOUS",))
_I32 = numpy.ctypeslib.ndpointer(dtype=numpy.int32, flags=("C_CONTIGUOUS", "WRITEABLE"))


class Sheet(ctypes.Structure):
    """Same layout as ``struct array_w_index`` (wendy/wendy.h:12-16)."""

    _fields_ = [("idx", ctypes.c_int), ("val", ctypes.c_double)]


SHEET_DTYPE = numpy.dtype({"names": ["idx", "val"], "formats": [numpy.int32, numpy.float64],
                           "offsets": [0, 8], "itemsize": 16})

_lib = None


def build():
    """Compile the oracle with its Makefile (needs gcc with OpenMP)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        build()
    lib = ctypes.CDLL(LIB_PATH)
    lib.wo_approx_onestep.argtypes = [
        ctypes.c_int, ctypes.c_void_p, _F64, _F64, _F64R, _F64, ctypes.c_double,
        ctypes.c_double, ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.c_double,
        ctypes.c_int, _F64R, ctypes.c_int, ctypes.POINTER(ctypes.c_double), _F64]
    lib.wo_approx_onestep.restype = None
    lib.wo_accel.argtypes = [ctypes.c_int, _F64R, _F64R, ctypes.c_double, ctypes.c_double,
                             ctypes.c_int, _F64R, ctypes.c_double, _F64, _I32, ctypes.c_int]
    lib.wo_accel.restype = None
    lib.wo_set_parallel_sort.argtypes = [ctypes.c_int, ctypes.c_long, ctypes.c_long]
    lib.wo_set_callback_force.argtypes = [ctypes.c_int, _F64R, ctypes.c_int]
    lib.wo_callback_force.restype = ctypes.c_double
    lib.wo_max_threads.restype = ctypes.c_int
    _lib = lib
    return lib


def _ext_args(ext):
    """(kind, params as float64) of ``ext``: None, (kind, params), or an
    object with ``kind`` and ``params`` (wendy_gb300's registered forces,
    compiled expressions included)."""
    if ext is None:
        return EXT_NONE, numpy.zeros(8)
    if hasattr(ext, "kind") and hasattr(ext, "params"):
        kind, params = ext.kind, ext.params
    else:
        kind, params = ext
    p = numpy.zeros(max(8, len(params)))
    p[:len(params)] = params
    return int(kind), p


def set_parallel_sort(nthreads, sort_switch=10000, merge_switch=50000):
    load().wo_set_parallel_sort(int(nthreads), int(sort_switch), int(merge_switch))


def max_threads():
    return int(load().wo_max_threads())


def make_sheets(x):
    xi = numpy.zeros(len(x), dtype=SHEET_DTYPE)
    xi["idx"] = numpy.arange(len(x), dtype=numpy.int32)
    xi["val"] = x
    return xi


def nbody_approx(x, v, m, dt, nleap, t0=0., omega=None, ext=None, sort="quick", twopiG=1.,
                 full_output=False):
    """Generator with the semantics of wendy._nbody_approx, run by the oracle.

    ``ext`` is ``None`` or ``(kind, params)`` with kind EXT_HARMONIC
    (params=[omega_ext**2]) or EXT_PULSE_TANH (params=[A, t0, tau, h]).
    """
    lib = load()
    omega2 = -1. if omega is None else omega ** 2.
    n = len(x)
    x = numpy.require(numpy.array(x, dtype=numpy.float64), requirements=["C", "W"])
    v = numpy.require(numpy.array(v, dtype=numpy.float64), requirements=["C", "W"])
    m = numpy.require(twopiG * numpy.array(m, dtype=numpy.float64), requirements=["C", "W"])
    a = numpy.zeros(n)
    cumulmass = numpy.zeros(n)
    totmass = numpy.sum(m)
    xi = make_sheets(x)
    kind, params = _ext_args(ext)
    tc = ctypes.c_double(t0)
    elapsed = ctypes.c_double(0.)
    dt_leap = dt / nleap
    while True:
        lib.wo_approx_onestep(n, xi.ctypes.data, x, v, m, a, totmass, dt_leap, nleap,
                              ctypes.byref(tc), omega2, kind, params, SORT_IDS[sort],
                              ctypes.byref(elapsed), cumulmass)
        if full_output:
            yield x, v, elapsed.value
        else:
            yield x, v


def onestep(xi, x, v, m, a, totmass, dt_leap, nleap, t0, omega2, ext=None, sort="quick",
            cumulmass=None):
    """One raw C call on caller-owned buffers; returns (t0, time_elapsed)."""
    lib = load()
    kind, params = _ext_args(ext)
    if cumulmass is None:
        cumulmass = numpy.zeros(len(x))
    tc = ctypes.c_double(t0)
    elapsed = ctypes.c_double(0.)
    lib.wo_approx_onestep(len(x), xi.ctypes.data, x, v, m, a, totmass, dt_leap, nleap,
                          ctypes.byref(tc), omega2, kind, params, SORT_IDS[sort],
                          ctypes.byref(elapsed), cumulmass)
    return tc.value, elapsed.value


def accel(x, m, totmass, omega2=-1., ext=None, t=0., sort="quick"):
    """One force evaluation in original order, plus the sort permutation
    (sort: "quick" as the reference's default, or "parallel" with the threads
    set by set_parallel_sort)."""
    lib = load()
    x = numpy.ascontiguousarray(x, dtype=numpy.float64)
    m = numpy.ascontiguousarray(m, dtype=numpy.float64)
    a = numpy.zeros(len(x))
    perm = numpy.zeros(len(x), dtype=numpy.int32)
    kind, params = _ext_args(ext)
    lib.wo_accel(len(x), x, m, totmass, omega2, kind, params, t, a, perm, SORT_IDS[sort])
    return a, perm


# --------------------------------------------------------------------------
# The reference itself (only where oracle/_ref was built from its sources).
# --------------------------------------------------------------------------
def ref_library(parallel=False):
    path = os.path.join(REF_DIR, "par" if parallel else "", "wendy_c%s" % EXT_SUFFIX)
    if not os.path.exists(path):
        return None
    lib = ctypes.CDLL(path)
    lib._wendy_nbody_approx_onestep.argtypes = [
        ctypes.c_int, ctypes.c_void_p, _F64, _F64, _F64R, _F64, ctypes.c_double,
        ctypes.c_double, ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.c_double,
        ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
        ctypes.POINTER(ctypes.c_double), _F64]
    lib._wendy_nbody_approx_onestep.restype = None
    return lib


def ref_onestep(lib, xi, x, v, m, a, totmass, dt_leap, nleap, t0, omega2, ext=None,
                sort="quick", cumulmass=None):
    """Drive the reference's _wendy_nbody_approx_onestep (wendy/wendy.c:385-418).

    An external force is passed as a C function pointer with the reference's
    callback signature (the oracle's ``wo_callback_force``), which is what
    numba's cfunc would hand it (wendy/wendy.py:389-404).
    """
    olib = load()
    fptr = None
    if ext is not None:
        kind, params = _ext_args(ext)
        olib.wo_set_callback_force(kind, params, len(params))
        fptr = ctypes.cast(olib.wo_callback_force, ctypes.c_void_p).value
    if cumulmass is None:
        cumulmass = numpy.zeros(len(x))
    tc = ctypes.c_double(t0)
    err = ctypes.c_int(0)
    elapsed = ctypes.c_double(0.)
    lib._wendy_nbody_approx_onestep(len(x), xi.ctypes.data, x, v, m, a, totmass, dt_leap,
                                    nleap, ctypes.byref(tc), omega2, fptr,
                                    {"quick": 0, "merge": 1, "tim": 2, "qsort": 3,
                                     "parallel": 4}[sort],
                                    ctypes.byref(err), ctypes.byref(elapsed), cumulmass)
    return tc.value, elapsed.value


def reference_root():
    """The reference checkout: $WENDY_REF_ROOT, else the one oracle/_ref was
    built from (recorded by the Makefile), else None."""
    root = os.environ.get("WENDY_REF_ROOT")
    if root:
        return root
    rec = os.path.join(REF_DIR, "ref_root.txt")
    if os.path.exists(rec):
        with open(rec) as f:
            return f.read().strip() or None
    return None


def import_reference_wendy(ref_root=None):
    """Import the reference's wendy.py with a stub numba (numba is absent).

    The stub's cfunc raises, which sends callables down the reference's own
    ctypes fallback (wendy/wendy.py:405-418).  Returns the module or None
    (also when no reference checkout is known, see reference_root).
    """
    if ref_root is None:
        ref_root = reference_root()
    if ref_root is None or not os.path.isdir(os.path.join(ref_root, "wendy")):
        return None
    if not os.path.exists(os.path.join(REF_DIR, "wendy_c%s" % EXT_SUFFIX)):
        return None
    import types as _types
    if "numba" not in sys.modules:
        stub = _types.ModuleType("numba")

        class _T:
            def __getattr__(self, name):
                return lambda *a, **k: None

        def cfunc(*a, **k):
            raise RuntimeError("numba stub")

        stub.types = _T()
        stub.cfunc = cfunc
        sys.modules["numba"] = stub
    if REF_DIR not in sys.path:
        sys.path.insert(0, REF_DIR)
    if ref_root not in sys.path:
        sys.path.insert(0, ref_root)
    import importlib
    return importlib.import_module("wendy")
