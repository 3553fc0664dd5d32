"""Serving: continuous batching of simulation requests on one GPU.

Requests (one simulation each: initial sheets, dt, nleap, number of
sub-steps, omega / registered external force) arrive over time.  The server
keeps every admitted simulation resident in HBM inside one
:class:`wendy_gb300.ensemble.Pool` and runs in rounds: each round admits the
requests that have arrived while the memory budget allows, advances *all*
resident simulations by one output interval (one launch of the fused
sub-step kernel per leapfrog sub-step, covering every simulation), streams
each simulation's previous output back while that runs, and retires the
simulations that are done.
Requests that arrive while a round is on the GPU join at the next round, so
work of new and old requests overlaps on the device.

Per simulation the arithmetic is that of wendy's approximate integrator and
the result is bit-identical whether the simulation runs alone or in the mix.

:func:`serve_one_at_a_time` is the plain alternative the server is measured
against: the same requests, first come first served, one simulation at a
time through ``wendy_gb300.Simulation``.
"""
import ctypes
import time
from dataclasses import dataclass, field

import numpy

from . import _lib
from .ensemble import Pool
from .wendy import Simulation


class _Pinned:
    """Output buffers of one request, page-locked for the stream of downloads."""

    def __init__(self, n):
        self.x = _lib.pinned_empty(n)
        self.v = _lib.pinned_empty(n)

    def release(self):
        self.x = self.v = None  # freed with the last view of them


@dataclass
class Request:
    x: numpy.ndarray
    v: numpy.ndarray
    m: numpy.ndarray            # masses, already times twopiG
    dt: float                   # output interval (dt_leap = dt / nleap)
    nleap: int
    noutputs: int
    omega: float = None
    ext_force: object = None
    t0: float = 0.0
    arrival: float = 0.0        # seconds after the start of the stream
    keep_outputs: bool = False
    # filled in by the server
    admitted_at: float = None
    done_at: float = None
    outputs: list = field(default_factory=list)
    last_x: numpy.ndarray = None
    last_v: numpy.ndarray = None

    @property
    def n(self):
        return len(self.x)

    @property
    def particle_steps(self):
        return self.n * self.nleap * self.noutputs


class Server:
    """Continuous-batching server over one Pool with an HBM budget (bytes)."""

    def __init__(self, budget_bytes, on_output=None):
        self.pool = Pool(budget_bytes=budget_bytes)
        self.budget = int(budget_bytes)
        self.on_output = on_output
        self.rounds = 0
        self.budget_waits = 0   # rounds in which an arrived request waited for memory
        self.peak_bytes = 0     # most device bytes the admitted simulations held at once

    def run(self, requests, clock=time.perf_counter):
        """Serve `requests` (sorted by arrival) in real time; returns them.

        Each round begins the pool step, then downloads and hands over the
        previous round's outputs while that step runs (the pool keeps each
        simulation's last output in a second pair of buffers), then completes
        the step.  Admission and retirement happen between steps.
        """
        pending = sorted(requests, key=lambda r: r.arrival)
        # sim id -> [request, outputs left to compute, t0, page-locked buffers,
        #            outputs delivered]
        active = {}
        unread = []  # simulations whose latest output is not delivered yet
        start = clock()
        i = 0
        used = 0

        def deliver(sids):
            for sid in sids:
                r, left, t, buf, done = active[sid]
                x, v = self.pool.download(sid, buf.x, buf.v)
                if r.keep_outputs:
                    r.outputs.append((x.copy(), v.copy()))
                if self.on_output:
                    self.on_output(r, x, v)
                active[sid][4] = done = done + 1
                if done == r.noutputs:
                    r.last_x, r.last_v = x.copy(), v.copy()
                    r.done_at = clock() - start

        while i < len(pending) or active:
            now = clock() - start
            # admit everything that has arrived and fits
            while i < len(pending) and pending[i].arrival <= now:
                r = pending[i]
                need = Pool.sim_bytes(r.n)
                if used + need > self.budget:
                    self.budget_waits += 1
                    break
                sid = self.pool.add(r.x, r.v, r.m, omega=r.omega, ext_force=r.ext_force,
                                    twopiG=1.)
                r.admitted_at = now
                active[sid] = [r, r.noutputs, r.t0, _Pinned(r.n), 0]
                used += need
                self.peak_bytes = max(self.peak_bytes, used)
                i += 1
            stepping = [sid for sid, a in active.items() if a[1] > 0]
            if not stepping and not unread:
                if i >= len(pending):
                    break
                # idle until the next arrival
                wait = pending[i].arrival - (clock() - start)
                if wait > 0:
                    time.sleep(min(wait, 0.05))
                continue
            # one round: every resident simulation with outputs left advances
            # one output interval; the previous round's outputs are delivered
            # while the first of its pool steps runs
            by_nleap = {}
            for sid in stepping:
                by_nleap.setdefault(active[sid][0].nleap, []).append(sid)
            to_read, unread = unread, []
            for nleap, ids in by_nleap.items():
                dts = numpy.array([active[s][0].dt / nleap for s in ids])
                t0 = numpy.array([active[s][2] for s in ids], dtype=numpy.float64)
                self.pool.step_begin(ids, dts, nleap, t0)
                deliver(to_read)
                to_read = []
                self.pool.step_end()
                for s, t in zip(ids, t0):
                    active[s][2] = float(t)
                    active[s][1] -= 1
                unread.extend(ids)
            deliver(to_read)  # a round with nothing left to step
            if by_nleap:
                self.rounds += 1
            # retire the simulations whose last output has been delivered
            for sid in list(active):
                r, left, t, buf, done = active[sid]
                if done == r.noutputs:
                    buf.release()
                    self.pool.remove(sid)
                    used -= Pool.sim_bytes(r.n)
                    del active[sid]
        return requests

    def close(self):
        self.pool.close()


def serve_one_at_a_time(requests, clock=time.perf_counter):
    """The plain path: first come first served, one simulation at a time."""
    pending = sorted(requests, key=lambda r: r.arrival)
    start = clock()
    for r in pending:
        now = clock() - start
        if r.arrival > now:
            time.sleep(r.arrival - now)
        r.admitted_at = clock() - start
        omega2 = -1. if r.omega is None else r.omega ** 2.
        sim = Simulation(r.x, r.v, r.m, float(numpy.sum(r.m)), omega2, r.ext_force)
        t = ctypes.c_double(r.t0)
        buf = _Pinned(r.n)
        x, v = buf.x, buf.v
        for _ in range(r.noutputs):
            sim.step(r.dt / r.nleap, r.nleap, t)
            sim.download(x, v)
            if r.keep_outputs:
                r.outputs.append((x.copy(), v.copy()))
        r.last_x, r.last_v = x.copy(), v.copy()
        r.done_at = clock() - start
        buf.release()
        sim.close()
    return requests


def latency_stats(requests):
    lat = numpy.array([r.done_at - r.arrival for r in requests])
    ps = sum(r.particle_steps for r in requests)
    span = max(r.done_at for r in requests) - min(r.arrival for r in requests)
    return {"p50_s": float(numpy.percentile(lat, 50)), "p99_s": float(numpy.percentile(lat, 99)),
            "mean_s": float(lat.mean()), "particle_steps": int(ps),
            "particle_steps_per_s": ps / span, "makespan_s": span}
