"""Ensembles: many simulations resident on one GPU, advanced together.

A :class:`Pool` wraps the C ABI's ``wg_pool``.  Each simulation added to it
is set up exactly like ``wendy.nbody(..., approx=True)`` sets up one run
(wendy/wendy.py:363-387: masses times twopiG, numpy ``totmass``, omega2 = -1
for no harmonic term), and :meth:`Pool.step` advances any subset of them by
one output interval of ``nleap`` leapfrog sub-steps with a single launch of
the fused sub-step kernel per sub-step.  Every simulation's result is
bit-identical to running it alone; the reference has no ensemble API, so
the per-simulation arithmetic is what is pinned to it.
"""
import ctypes

import numpy

from . import _lib
from .extforce import resolve


class Pool:
    def __init__(self, budget_bytes=0):
        self._L = _lib.lib()
        self._h = ctypes.c_void_p()
        _lib.check(self._L.wg_pool_create(int(budget_bytes), ctypes.byref(self._h)),
                   "wg_pool_create")
        self._n = {}

    @staticmethod
    def sim_bytes(n):
        """Device bytes a simulation of n sheets holds (for admission control)."""
        return int(_lib.lib().wg_pool_sim_bytes(int(n)))

    def add(self, x, v, m, omega=None, ext_force=None, twopiG=1.):
        """Add one simulation; returns its id.  Inputs are copied."""
        kind, params = resolve(ext_force)
        x = numpy.ascontiguousarray(x, dtype=numpy.float64)
        v = numpy.ascontiguousarray(v, dtype=numpy.float64)
        m = numpy.ascontiguousarray(twopiG * numpy.asarray(m, dtype=numpy.float64))
        omega2 = -1. if omega is None else omega ** 2.
        sid = ctypes.c_int(-1)
        _lib.check(self._L.wg_pool_add(self._h, len(x), x, v, m, float(numpy.sum(m)),
                                       float(omega2), int(kind), _lib.ext_params(params),
                                       len(params), ctypes.byref(sid)), "wg_pool_add")
        self._n[sid.value] = len(x)
        return sid.value

    def remove(self, sim_id):
        _lib.check(self._L.wg_pool_remove(self._h, int(sim_id)), "wg_pool_remove")
        self._n.pop(sim_id, None)

    def step(self, ids, dt_leap, nleap, t0=None):
        """Advance simulations ``ids`` by ``nleap`` sub-steps of ``dt_leap[k]``.

        ``t0`` (float64 array, one per id) is advanced in place as
        wendy_gb300.wg_step advances it.  Returns the device time in seconds.
        """
        ids = numpy.ascontiguousarray(ids, dtype=numpy.int32)
        dts = numpy.ascontiguousarray(numpy.broadcast_to(dt_leap, ids.shape), dtype=numpy.float64)
        if t0 is not None and (t0.dtype != numpy.float64 or not t0.flags.c_contiguous
                               or t0.shape != ids.shape):
            raise ValueError("t0 must be a contiguous float64 array, one entry per id")
        el = ctypes.c_double(0.)
        _lib.check(self._L.wg_pool_step(self._h, len(ids), ids.ctypes.data, dts.ctypes.data,
                                        int(nleap), None if t0 is None else t0.ctypes.data,
                                        ctypes.byref(el)), "wg_pool_step")
        return el.value

    def step_begin(self, ids, dt_leap, nleap, t0=None):
        """Enqueue ``step`` and return at once (``t0`` advances now).  Until
        ``step_end``, ``download`` returns each simulation's previous output."""
        ids = numpy.ascontiguousarray(ids, dtype=numpy.int32)
        dts = numpy.ascontiguousarray(numpy.broadcast_to(dt_leap, ids.shape), dtype=numpy.float64)
        if t0 is not None and (t0.dtype != numpy.float64 or not t0.flags.c_contiguous
                               or t0.shape != ids.shape):
            raise ValueError("t0 must be a contiguous float64 array, one entry per id")
        self._pend = (ids, dts)  # the arrays must outlive the call
        _lib.check(self._L.wg_pool_step_begin(self._h, len(ids), ids.ctypes.data, dts.ctypes.data,
                                              int(nleap), None if t0 is None else t0.ctypes.data),
                   "wg_pool_step_begin")

    def step_end(self):
        """Complete the step enqueued by ``step_begin``; returns its device time."""
        el = ctypes.c_double(0.)
        _lib.check(self._L.wg_pool_step_end(self._h, ctypes.byref(el)), "wg_pool_step_end")
        self._pend = None
        return el.value

    def download(self, sim_id, x=None, v=None):
        n = self._n[sim_id]
        x = numpy.empty(n) if x is None else x
        v = numpy.empty(n) if v is None else v
        _lib.check(self._L.wg_pool_download(self._h, int(sim_id), x.ctypes.data, v.ctypes.data),
                   "wg_pool_download")
        return x, v

    def download_many(self, ids, x=None, v=None):
        """``download`` of every simulation in ``ids`` in one call: their
        outputs one after another in ``x`` and ``v`` (float64, contiguous)."""
        ids = numpy.ascontiguousarray(ids, dtype=numpy.int32)
        total = sum(self._n[int(i)] for i in ids)
        x = numpy.empty(total) if x is None else x
        v = numpy.empty(total) if v is None else v
        for a in (x, v):
            if a.dtype != numpy.float64 or not a.flags.c_contiguous or a.size != total:
                raise ValueError("x and v must be contiguous float64 arrays of %d entries" % total)
        _lib.check(self._L.wg_pool_download_many(self._h, len(ids), ids.ctypes.data,
                                                 x.ctypes.data, v.ctypes.data),
                   "wg_pool_download_many")
        return x, v

    def stats(self):
        """The pool's counters (wg_pool_get_stats) as a dict."""
        st = _lib.WgPoolStats()
        _lib.check(self._L.wg_pool_get_stats(self._h, ctypes.byref(st)), "wg_pool_get_stats")
        return {name: getattr(st, name) for name, _ in st._fields_}

    def info(self):
        used, budget, nsim, launches = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int(), \
            ctypes.c_int64()
        _lib.check(self._L.wg_pool_info(self._h, ctypes.byref(used), ctypes.byref(budget),
                                        ctypes.byref(nsim), ctypes.byref(launches)),
                   "wg_pool_info")
        return {"used_bytes": used.value, "budget_bytes": budget.value, "sims": nsim.value,
                "launches": launches.value}

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._L.wg_pool_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
