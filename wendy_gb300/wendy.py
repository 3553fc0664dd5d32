"""wendy's public generator API, running the approximate integrator on the GPU.

``nbody(x, v, m, dt, approx=True, nleap=..., sort='cuda', ...)`` has the
signature, argument meaning, error behaviour and yield semantics of
``wendy.nbody`` (wendy/wendy.py:112-206) and ``wendy._nbody_approx``
(wendy/wendy.py:336-437): masses are multiplied by twopiG, ``totmass`` is
numpy's sum of them, ``omega=None`` means no harmonic term, and every
``next()`` advances one output interval of ``nleap`` leapfrog sub-steps and
yields the same ``x, v`` arrays, updated in place, in original particle
order (plus the elapsed time with ``full_output=True``).

The sheets stay on the device between outputs.  Each ``next()`` completes
the output interval enqueued before, copies x and v back into the yielded
(page-locked) arrays, and enqueues the next interval before yielding, so the
device computes output k + 1 while the caller works on output k.

One difference a caller can observe: wendy's C step reads the yielded ``v``
on every call (wendy/wendy.c:318-333; ``x`` is only written, at
wendy/wendy.c:413-415), so editing ``v`` in place between ``next()`` calls
changes the trajectory there.  Here the state lives on the device and the
next output is already being computed, so such edits are ignored unless
``follow_edits=True``: then every ``next()`` compares ``v`` with the copy
taken when it was yielded and, if it changed, drops the output computed
ahead and restarts from the yielded positions and the edited velocities (as
wendy does, edits of ``x`` still have no effect).  That costs a copy and a
comparison of ``x`` and ``v`` per output on the host.
"""
import copy
import ctypes

import numpy

from . import _lib
from .diagnostics import energy, momentum, potential  # noqa: F401  (public API)
from .extforce import resolve

CPU_SORTS = ("quick", "merge", "tim", "qsort", "parallel")


class Simulation:
    """One simulation resident on the GPU (a ``wg_sim`` handle)."""

    def __init__(self, x, v, m, totmass, omega2=-1., ext_force=None):
        L = _lib.lib()
        kind, params = resolve(ext_force)
        self._L = L
        self.n = len(x)
        self._h = ctypes.c_void_p()
        x = numpy.ascontiguousarray(x, dtype=numpy.float64)
        v = numpy.ascontiguousarray(v, dtype=numpy.float64)
        m = numpy.ascontiguousarray(m, dtype=numpy.float64)
        _lib.check(L.wg_create(self.n, x, v, m, float(totmass), float(omega2), int(kind),
                               _lib.ext_params(params), len(params), ctypes.byref(self._h)),
                   "wg_create")

    def step(self, dt_leap, nleap, t0):
        """One output interval; ``t0`` is a ctypes.c_double updated in place.
        Returns the device time in seconds."""
        elapsed = ctypes.c_double(0.)
        _lib.check(self._L.wg_step(self._h, float(dt_leap), int(nleap), ctypes.byref(t0),
                                   ctypes.byref(elapsed)), "wg_step")
        return elapsed.value

    def step_begin(self, dt_leap, nleap, t0):
        """Enqueue one output interval and return at once (``t0`` advances now).
        Until ``step_end``, ``download`` returns the output completed before it."""
        _lib.check(self._L.wg_step_begin(self._h, float(dt_leap), int(nleap), ctypes.byref(t0)),
                   "wg_step_begin")

    def step_end(self):
        """Complete the interval enqueued by step_begin; returns its device time."""
        elapsed = ctypes.c_double(0.)
        _lib.check(self._L.wg_step_end(self._h, ctypes.byref(elapsed)), "wg_step_end")
        return elapsed.value

    def energy(self, twopiG=1., omega=None):
        """Total energy and momentum of the last output, computed on the device.

        Same quantities as wendy.energy(x, v, m, twopiG, omega=omega) and
        wendy.momentum(v, m) (wendy/wendy.py:439-491) for the masses m this
        simulation was created with divided by twopiG; returns (energy,
        momentum).  Leaves the sheets compact: the next step re-sorts once.
        """
        e, p = ctypes.c_double(0.), ctypes.c_double(0.)
        omega2 = -1. if omega is None else float(omega) ** 2.
        _lib.check(self._L.wg_energy(self._h, float(twopiG), omega2, ctypes.byref(e),
                                     ctypes.byref(p)), "wg_energy")
        return e.value, p.value

    def download(self, x, v):
        """Positions and velocities of the last output, in original order, into
        ``x`` and ``v`` (float64[n]); during a step begun with ``step_begin``,
        those of the output completed before it, while the step runs."""
        for arr in (x, v):
            if not (arr.flags.c_contiguous and arr.flags.writeable and arr.dtype == numpy.float64
                    and len(arr) == self.n):
                raise ValueError("download buffers must be writeable contiguous float64[n]")
        _lib.check(self._L.wg_download(self._h, x.ctypes.data, v.ctypes.data), "wg_download")

    def stats(self):
        st = _lib.WgStats()
        _lib.check(self._L.wg_get_stats(self._h, ctypes.byref(st)), "wg_get_stats")
        return {k: getattr(st, k) for k, _ in st._fields_}

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._L.wg_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def nbody(x, v, m, dt, t0=0., twopiG=1., omega=None, ext_force=None, approx=False, nleap=None,
          sort="cuda", maxcoll=100000, warn_maxcoll=False, full_output=False,
          follow_edits=False):
    """Run a 1D N-body simulation (wendy/wendy.py:112-157 for the approximate path).

    ``approx=True`` runs the approximate leapfrog integrator (``sort`` must
    be ``'cuda'``: the CPU sorts are the reference's); ``approx=False`` runs
    the exact event-driven solver on one GPU warp (a cross-check for small N,
    wendy/wendy.py:158-206).
    ``follow_edits=True`` (not in wendy) honours in-place edits of the
    yielded ``v`` between outputs, as wendy's C step does; see the module
    documentation.
    """
    if approx:
        if nleap is None:
            raise ValueError("When approx is True, the number of leapfrog steps nleap= per output "
                             "time step needs to be set")
        # yield from: closing this generator closes the inner one (and its
        # simulation) at once
        yield from _nbody_approx(x, v, m, dt, nleap, t0=t0, sort=sort, omega=omega,
                                 ext_force=ext_force, twopiG=twopiG, full_output=full_output,
                                 follow_edits=follow_edits)
        return
    yield from _nbody_exact(x, v, m, dt, twopiG=twopiG, omega=omega, ext_force=ext_force,
                            maxcoll=maxcoll, warn_maxcoll=warn_maxcoll, full_output=full_output)


def _setup_exact(x, v, m):
    """Sort order and accelerations of wendy's _setup_arrays
    (wendy/wendy.py:208-238), with the same numpy operations; the pair
    crossing times are computed on the device."""
    sindx = numpy.argsort(x)
    mass_below = numpy.cumsum(m[sindx])
    mass_below[-1] = 0.
    mass_below = numpy.roll(mass_below, 1)
    mass_above = numpy.cumsum(m[sindx][::-1])[::-1]
    mass_above[0] = 0.
    mass_above = numpy.roll(mass_above, -1)
    a = (mass_above - mass_below)[numpy.argsort(sindx)]
    return (numpy.require(a, dtype=numpy.float64, requirements=["C", "W"]),
            numpy.require(sindx, dtype=numpy.int32, requirements=["C"]))


def _nbody_exact(x, v, m, dt, twopiG=1., omega=None, ext_force=None, maxcoll=100000,
                 warn_maxcoll=False, full_output=False):
    """Generator mirroring wendy's exact path (wendy/wendy.py:158-206) on the
    GPU event loop (wg_exact_*): one output interval per ``next()``, yielding
    the same x, v arrays updated in place (and the number of crossings and the
    event loop's time with ``full_output=True``)."""
    import warnings
    if ext_force is not None:
        raise ValueError("External forces (ext_force=) are not supported for the exact nbody "
                         "calculation")
    if omega is not None and omega * dt > numpy.pi / 2.:
        raise ValueError("When omega is set, omega*dt needs to be less than pi/2; please adjust "
                         "dt")
    if numpy.any(m < numpy.median(m) * 10. ** -8.):
        raise ValueError("Tiny masses m much smaller than the median mass are not supported, "
                         "please remove these from the inputs")
    x = numpy.require(copy.copy(x), dtype=numpy.float64, requirements=["C", "W"])
    v = numpy.require(copy.copy(v), dtype=numpy.float64, requirements=["C", "W"])
    m = numpy.require(twopiG * copy.copy(m), dtype=numpy.float64, requirements=["C", "W"])
    if omega is not None:
        m /= omega ** 2.
    L = _lib.lib()

    def create():
        a, sindx = _setup_exact(x, v, m)
        h = ctypes.c_void_p()
        _lib.check(L.wg_exact_create(len(x), x, v, a, m, sindx,
                                     float(omega) if omega is not None else 0., ctypes.byref(h)),
                   "wg_exact_create")
        return h

    h = create()
    ncoll = 0
    try:
        while True:
            nc, el = ctypes.c_int64(0), ctypes.c_double(0.)
            rc = L.wg_exact_step(h, float(dt), int(maxcoll), ctypes.byref(nc), ctypes.byref(el))
            ncoll += nc.value
            _lib.check(L.wg_exact_download(h, x.ctypes.data, v.ctypes.data, None, None),
                       "wg_exact_download")
            if rc == _lib.WG_ERR_MAXCOLL:
                if warn_maxcoll:
                    warnings.warn("Maximum number of collisions per time step exceeded",
                                  RuntimeWarning)
                    # re-compute the accelerations and crossing times
                    L.wg_exact_destroy(h)
                    h = create()
                else:
                    raise RuntimeError("Maximum number of collisions per time step exceeded")
            else:
                _lib.check(rc, "wg_exact_step")
            if full_output:
                yield (x, v, ncoll, el.value)
            else:
                yield (x, v)
    finally:
        L.wg_exact_destroy(h)


def _nbody_approx(x, v, m, dt, nleap, t0=0., omega=None, ext_force=None, sort="cuda", twopiG=1.,
                  full_output=False, follow_edits=False):
    """Generator mirroring wendy._nbody_approx (wendy/wendy.py:336-437)."""
    if sort != "cuda":
        if sort in CPU_SORTS:
            raise ValueError("sort=%r is a CPU sort of the reference wendy; wendy_gb300 runs "
                             "sort='cuda'" % (sort,))
        raise ValueError("unknown sort %r" % (sort,))
    if omega is None:
        omega2 = -1.
    else:
        omega2 = omega ** 2.
    x = numpy.require(copy.copy(x), dtype=numpy.float64, requirements=["C", "W"])
    v = numpy.require(copy.copy(v), dtype=numpy.float64, requirements=["C", "W"])
    m = numpy.require(twopiG * copy.copy(m), dtype=numpy.float64, requirements=["C", "W"])
    totmass = numpy.sum(m)
    sim = Simulation(x, v, m, totmass, omega2, ext_force)
    t = ctypes.c_double(t0)
    dt_leap = dt / nleap
    if x.nbytes >= (1 << 20):
        # the yielded copies live in page-locked memory, so that every
        # output downloads at the link's rate
        try:
            xp, vp = _lib.pinned_empty(x.shape), _lib.pinned_empty(v.shape)
            xp[:] = x
            vp[:] = v
            x, v = xp, vp
        except _lib.WendyGPUError:
            pass
    try:
        sim.step_begin(dt_leap, nleap, t)
        while True:
            elapsed = sim.step_end()
            # the next output is enqueued first; this one downloads while it runs
            t_ahead = t.value  # the time that next output starts from
            sim.step_begin(dt_leap, nleap, t)
            sim.download(x, v)
            if follow_edits:
                x_seen, v_seen = x.copy(), v.copy()
            if full_output:
                yield (x, v, elapsed)
            else:
                yield (x, v)
            if follow_edits and not numpy.array_equal(v.view(numpy.int64),
                                                      v_seen.view(numpy.int64)):
                # v was edited: the output computed ahead is dropped and the
                # run restarts from the yielded positions and the edited v
                sim.step_end()
                sim.close()
                x[:] = x_seen
                sim = Simulation(x, v, m, totmass, omega2, ext_force)
                t.value = t_ahead
                sim.step_begin(dt_leap, nleap, t)
    finally:
        # also runs when an unclosed generator is collected at interpreter exit
        try:
            sim.close()
        except Exception:
            pass


def accel(x, m, totmass, omega2=-1., ext_force=None, t=0.):
    """One force evaluation at positions x (original order).

    Returns (a, perm): accelerations in original order and the sort
    permutation (perm[i] = original index of the sheet at sorted slot i),
    the quantities of wendy's _nbody_force (wendy/wendy.c:334-384).  Masses
    are used as given (already times twopiG).
    """
    L = _lib.lib()
    kind, params = resolve(ext_force)
    x = numpy.ascontiguousarray(x, dtype=numpy.float64)
    m = numpy.ascontiguousarray(m, dtype=numpy.float64)
    a = numpy.empty(len(x))
    perm = numpy.empty(len(x), dtype=numpy.int32)
    _lib.check(L.wg_accel(len(x), x, m, float(totmass), float(omega2), int(kind),
                          _lib.ext_params(params), len(params), float(t), a.ctypes.data,
                          perm.ctypes.data), "wg_accel")
    return a, perm


def approx_onestep(xi, x, v, m, a, totmass, dt, nleap, t0, omega2=-1., ext_force=None):
    """The reference-shaped stateless step (wendy/wendy.c:385-418) on the GPU.

    ``xi`` is a structured array with fields idx (int32) and val (float64)
    laid out like ``struct array_w_index``; xi, x, v and a are updated in
    place exactly as the reference's C function updates them.  Returns
    (t0, time_elapsed).
    """
    L = _lib.lib()
    kind, params = resolve(ext_force)
    if xi.dtype != _lib.SHEET_DTYPE or not xi.flags.c_contiguous:
        raise ValueError("xi must be a contiguous array of dtype wendy_gb300._lib.SHEET_DTYPE")
    tc = ctypes.c_double(t0)
    el = ctypes.c_double(0.)
    err = ctypes.c_int(0)
    _lib.check(L.wg_nbody_approx_onestep(len(x), xi.ctypes.data, x, v, m, a, float(totmass),
                                         float(dt), int(nleap), ctypes.byref(tc), float(omega2),
                                         int(kind), _lib.ext_params(params), len(params),
                                         ctypes.byref(err), ctypes.byref(el)),
               "wg_nbody_approx_onestep")
    return tc.value, el.value


def approx_onestep_stats():
    """Counters of the state behind approx_onestep (wg_nbody_approx_stats):
    a call handed back exactly the previous call's outputs resumes from the
    resident sorted state and adds no full sort."""
    st = _lib.WgStats()
    _lib.check(_lib.lib().wg_nbody_approx_stats(ctypes.byref(st)), "wg_nbody_approx_stats")
    return {k: getattr(st, k) for k, _ in st._fields_}
