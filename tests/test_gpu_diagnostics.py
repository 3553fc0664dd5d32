"""Output-side entries: device energy and momentum (wg_energy) against the
reference's formulas, and the split step (wg_step_begin / wg_step_end) the
generator uses to compute the next output while the caller holds this one.

The reference computes energy and momentum on the host from the yielded
arrays (wendy/wendy.py:439-491); wendy_gb300.diagnostics restates them in
numpy with the same operation order.  The device sums differ only in
summation order.
"""
import ctypes

import numpy
import pytest

import wendy_gb300
from wendy_gb300 import diagnostics, ics

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,masses,omega,twopiG,rtol", [
    (10000, "equal", None, 1.0, 1e-12),
    (10000, "lognormal", 1.1, 2.0, 1e-12),
    (1 << 20, "lognormal", 0.5, 1.0, 1e-10),
])
def test_device_energy_matches_reference_formula(n, masses, omega, twopiG, rtol):
    x, v, m = ics.sech2_disk(n, seed=3, masses=masses)
    omega2 = -1. if omega is None else omega ** 2
    sim = wendy_gb300.Simulation(x, v, twopiG * m, float(numpy.sum(twopiG * m)), omega2)
    t = ctypes.c_double(0.)
    for _ in range(2):
        sim.step(0.002, 5, t)
    gx, gv = numpy.empty(n), numpy.empty(n)
    sim.download(gx, gv)
    e_dev, p_dev = sim.energy(twopiG=twopiG, omega=omega)
    e_ref = diagnostics.energy(gx, gv, m, twopiG=twopiG, omega=omega)
    p_ref = diagnostics.momentum(gv, m)
    assert abs(e_dev - e_ref) <= rtol * abs(e_ref)
    assert abs(p_dev - p_ref) <= 1e-12 * numpy.sum(numpy.abs(m * gv))
    sim.close()


def test_energy_call_leaves_the_trajectory_unchanged():
    n = 30000
    x, v, m = ics.sech2_disk(n, seed=4, masses="lognormal")
    a = wendy_gb300.Simulation(x, v, m, float(numpy.sum(m)), 1.21)
    b = wendy_gb300.Simulation(x, v, m, float(numpy.sum(m)), 1.21)
    ta, tb = ctypes.c_double(0.), ctypes.c_double(0.)
    a.step(0.002, 5, ta)
    b.step(0.002, 5, tb)
    a.energy(omega=1.1)
    a.step(0.002, 5, ta)
    b.step(0.002, 5, tb)
    ax, av, bx, bv = (numpy.empty(n) for _ in range(4))
    a.download(ax, av)
    b.download(bx, bv)
    assert numpy.array_equal(ax, bx) and numpy.array_equal(av, bv)
    a.close()
    b.close()


def test_energy_of_a_fresh_simulation_and_bad_arguments():
    x, v, m = ics.sech2_disk(5000, seed=5)
    sim = wendy_gb300.Simulation(x, v, m, float(numpy.sum(m)))
    e, p = sim.energy()
    assert abs(e - diagnostics.energy(x, v, m)) <= 1e-12 * abs(e)
    with pytest.raises(wendy_gb300._lib.WendyGPUError):
        sim.energy(twopiG=0.)
    sim.close()


def test_step_begin_end_equals_step_and_guards_the_handle():
    n = 20000
    x, v, m = ics.sech2_disk(n, seed=6, masses="lognormal")
    a = wendy_gb300.Simulation(x, v, m, float(numpy.sum(m)), 1.21)
    b = wendy_gb300.Simulation(x, v, m, float(numpy.sum(m)), 1.21)
    ta, tb = ctypes.c_double(1.0), ctypes.c_double(1.0)
    prev = None
    for _ in range(3):
        b.step_begin(0.002, 5, tb)
        # with a step in flight, download returns the output completed before
        # it (none before the first), and every other entry refuses the handle
        bx, bv = numpy.empty(n), numpy.empty(n)
        if prev is None:
            with pytest.raises(wendy_gb300._lib.WendyGPUError):
                b.download(bx, bv)
        else:
            b.download(bx, bv)
            assert numpy.array_equal(bx, prev[0]) and numpy.array_equal(bv, prev[1])
        a.step(0.002, 5, ta)
        ax, av = numpy.empty(n), numpy.empty(n)
        a.download(ax, av)
        prev = (ax, av)
        with pytest.raises(wendy_gb300._lib.WendyGPUError):
            b.step(0.002, 5, tb)
        with pytest.raises(wendy_gb300._lib.WendyGPUError):
            b.energy()
        assert b.step_end() > 0.0
    with pytest.raises(wendy_gb300._lib.WendyGPUError):
        b.step_end()
    assert ta.value == tb.value
    ax, av, bx, bv = (numpy.empty(n) for _ in range(4))
    a.download(ax, av)
    b.download(bx, bv)
    assert numpy.array_equal(ax, bx) and numpy.array_equal(av, bv)
    b.step_begin(0.002, 5, tb)
    b.close()  # destroying a handle with a step in flight waits for it
    a.close()


def test_generator_computes_ahead_and_stops_cleanly():
    x, v, m = ics.sech2_disk(50000, seed=7)
    g = wendy_gb300.nbody(x, v, m, 0.01, approx=True, nleap=5)
    outs = [tuple(a.copy() for a in next(g)) for _ in range(3)]
    g.close()
    sim = wendy_gb300.Simulation(x, v, m, float(numpy.sum(m)))
    t = ctypes.c_double(0.)
    for ox, ov in outs:
        sim.step(0.002, 5, t)
        gx, gv = numpy.empty(len(x)), numpy.empty(len(x))
        sim.download(gx, gv)
        assert numpy.array_equal(gx, ox) and numpy.array_equal(gv, ov)
    sim.close()
