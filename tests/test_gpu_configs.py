"""Parity at the sizes the performance targets are stated on.

  * the HBM-scale configuration: 2^27 equal-mass sheets in a cold top-hat
    with the pulsed external force 0.3 exp(-(t-5)^2/2) tanh(x/0.5): one force
    evaluation at the pulse peak (t = 5) against the oracle's, and one output
    of 10 sub-steps (dt = 0.01) against the oracle's generator;
  * the large configuration: 2^24 sheets of a sech^2 disk with lognormal
    masses and omega = 1.1: one output of nleap = 20 sub-steps (dt = 0.02);
  * the regime after the top-hat's collapse (t = pi/2), where buckets
    overflow and sub-steps fall back to the compact path: a 2^22 top-hat run
    past it on the GPU, and three consecutive outputs each compared with the
    oracle started from the same state.

Bars (the reference's approximate step, wendy/wendy.c:334-418): sort
permutation bit-exact for distinct positions; accelerations within 1e-12 of
the acceleration scale max(totmass, max|a|); positions and velocities after
one output within 1e-10.  Sheets that share a position with another are
left out of the permutation and acceleration checks: the reference's
quicksort leaves their order to its pivots, and their forces follow that
order.  The oracle runs the reference's task-parallel merge sort on all host
threads here (the same order for distinct positions), which keeps each
case within a minute of host time.
"""
import ctypes
import os

import numpy
import pytest

import wendy_gb300
from oracle import oracle as O
from wendy_gb300 import ics
from wendy_gb300.extforce import PulseTanh

pytestmark = pytest.mark.gpu

PULSE_P = [0.3, 5.0, 1.0, 0.5]
PULSE = PulseTanh(*PULSE_P)
ORACLE_PULSE = (O.EXT_PULSE_TANH, PULSE_P)


@pytest.fixture(scope="module", autouse=True)
def all_host_threads():
    O.set_parallel_sort(os.cpu_count() or 1)


def _tied(xs):
    """Mask of sorted positions whose value a neighbour shares."""
    eq = xs[1:] == xs[:-1]
    t = numpy.zeros(len(xs), dtype=bool)
    t[1:] |= eq
    t[:-1] |= eq
    return t


def _check_force(x, a, perm, ra, rperm, totmass):
    xs = x[rperm]
    assert numpy.array_equal(x[perm], xs)          # the same order of positions
    tie = _tied(xs)
    assert numpy.array_equal(perm[~tie], rperm[~tie])  # bit-exact where distinct
    keep = numpy.ones(len(x), dtype=bool)
    keep[rperm[tie]] = False
    scale = max(float(totmass), float(numpy.max(numpy.abs(ra))))
    err = float(numpy.max(numpy.abs(a[keep] - ra[keep])))
    assert err <= 1e-12 * scale, (err, scale)
    return int(tie.sum()), err


def test_hbm_scale_top_hat_force_at_the_pulse_peak():
    n = 1 << 27
    x, v, m = ics.top_hat(n, seed=0)
    del v
    tot = numpy.sum(m)
    a, perm = wendy_gb300.accel(x, m, tot, omega2=-1., ext_force=PULSE, t=5.0)
    ra, rperm = O.accel(x, m, tot, -1., ORACLE_PULSE, 5.0, sort="parallel")
    _check_force(x, a, perm, ra, rperm, tot)


def test_hbm_scale_top_hat_one_output():
    n = 1 << 27
    x, v, m = ics.top_hat(n, seed=0)
    g = wendy_gb300.nbody(x, v, m, 0.01, approx=True, nleap=10, ext_force=PULSE, t0=4.95)
    gx, gv = next(g)
    g.close()
    r = O.nbody_approx(x, v, m, 0.01, 10, t0=4.95, ext=ORACLE_PULSE, sort="parallel")
    rx, rv = next(r)
    assert numpy.max(numpy.abs(gx - rx)) <= 1e-10
    assert numpy.max(numpy.abs(gv - rv)) <= 1e-10


def test_large_sech2_lognormal_one_output():
    n = 1 << 24
    x, v, m = ics.sech2_disk(n, seed=0, masses="lognormal", sigma_ln=0.5)
    g = wendy_gb300.nbody(x, v, m, 0.02, approx=True, nleap=20, omega=1.1)
    gx, gv = next(g)
    g.close()
    r = O.nbody_approx(x, v, m, 0.02, 20, omega=1.1, sort="parallel")
    rx, rv = next(r)
    assert numpy.max(numpy.abs(gx - rx)) <= 1e-10
    assert numpy.max(numpy.abs(gv - rv)) <= 1e-10


def test_top_hat_after_the_collapse():
    n = 1 << 22
    x, v, m = ics.top_hat(n, seed=5)
    tot = numpy.sum(m)
    sim = wendy_gb300.Simulation(x, v, m, tot, -1., PULSE)
    t = ctypes.c_double(0.)
    for _ in range(158):  # t = 1.58, just past the collapse at pi/2
        sim.step(0.001, 10, t)
    gx, gv = numpy.empty(n), numpy.empty(n)
    sim.download(gx, gv)
    compact0 = sim.stats()["substeps_compact"]
    resorts0 = sim.stats()["sorts_full"]
    for _ in range(3):
        xs, vs, ts = gx.copy(), gv.copy(), t.value
        sim.step(0.001, 10, t)
        sim.download(gx, gv)
        # the oracle from the same state: sheets in original order, the
        # reference's generator set-up (wendy/wendy.py:363-387)
        r = O.nbody_approx(xs, vs, m, 0.01, 10, t0=ts, ext=ORACLE_PULSE, sort="parallel")
        rx, rv = next(r)
        assert numpy.max(numpy.abs(gx - rx)) <= 1e-10
        assert numpy.max(numpy.abs(gv - rv)) <= 1e-10
    st = sim.stats()
    sim.close()
    # the compared outputs ran in the regime this test is about: sub-steps
    # that needed a full re-sort, on the compact path or as a restart
    assert st["substeps_compact"] > 0
    assert st["sorts_full"] - resorts0 > 0 or st["substeps_compact"] - compact0 > 0
