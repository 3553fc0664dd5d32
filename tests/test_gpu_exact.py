"""The exact event-driven solver on the GPU (nbody(..., approx=False))
against the reference's exact solver (tests/golden/exact.npz and
exact_more.npz, made by wendy/wendy.c:53-315 itself) and the reference's own
tests of that path (tests/test_wendy.py, tests/test_harm.py).

The GPU event loop follows the reference's arithmetic operation by
operation, without FMA contraction, and processes crossings in the same
order, so without a harmonic potential the trajectories are expected to be
the same bits; with one, CUDA's sin/asin/atan2/acos differ from libm's in the
last bits, hence the 1e-10 bar there.
"""
import numpy
import pytest

import wendy_gb300
from wendy_gb300 import ics

pytestmark = pytest.mark.gpu


def test_matches_the_reference_exact_solver(golden):
    g = golden("exact")
    gen = wendy_gb300.nbody(g["x0"], g["v0"], g["m"], 0.05)
    for k in range(1, 21):
        tx, tv = next(gen)
        assert numpy.max(numpy.abs(tx - g["x%d" % k])) <= 1e-12, k
        assert numpy.max(numpy.abs(tv - g["v%d" % k])) <= 1e-12, k


@pytest.mark.parametrize("name,tol", [("harm", 1e-10), ("large", 1e-12)])
def test_matches_the_reference_with_omega_and_at_larger_n(golden, name, tol):
    # "large" (6000 sheets) runs from global memory: the state does not fit in
    # one block's shared memory
    g = golden("exact_more")
    dt, nout, omega = g[name + "/par"]
    gen = wendy_gb300.nbody(g[name + "/x0"], g[name + "/v0"], g[name + "/m"], dt,
                            omega=None if omega < 0 else omega, full_output=True)
    for k in range(1, int(nout) + 1):
        tx, tv, nc, el = next(gen)
        assert nc == int(g["%s/ncoll%d" % (name, k)][0]), k
        assert numpy.max(numpy.abs(tx - g["%s/x%d" % (name, k)])) <= tol, k
        assert numpy.max(numpy.abs(tv - g["%s/v%d" % (name, k)])) <= tol, k
        assert el > 0


@pytest.mark.parametrize("m", [[1., 1., 1.], [1., 2., 3.]])
def test_energy_and_momentum_conservation(m):
    # tests/test_wendy.py:6-34,69-82 of the reference
    x = numpy.array([-1.1, 0.1, 1.3])
    v = numpy.array([3., 2., -5.])
    m = numpy.array(m)
    g = wendy_gb300.nbody(x, v, m, 0.05)
    E = wendy_gb300.energy(x, v, m)
    p = wendy_gb300.momentum(v, m)
    for _ in range(100):
        tx, tv = next(g)
        assert numpy.fabs(wendy_gb300.energy(tx, tv, m) - E) < 1e-10
        assert numpy.fabs(wendy_gb300.momentum(tv, m) - p) < 1e-10


def test_energy_conservation_sech2_disk():
    # tests/test_wendy.py:36-53 (and tests/test_harm.py for omega)
    x, v, m = ics.sech2_disk(101, seed=8)
    v = v - numpy.mean(v)
    m = m * (1. + 0.1 * (2. * numpy.random.default_rng(8).uniform(size=101) - 1))
    for omega in (None, 1.1):
        g = wendy_gb300.nbody(x, v, m, 0.05, omega=omega)
        E = wendy_gb300.energy(x, v, m, omega=omega)
        for _ in range(100):
            tx, tv = next(g)
            assert numpy.fabs(wendy_gb300.energy(tx, tv, m, omega=omega) - E) < 1e-10


def test_collision_count_two_body():
    # tests/test_wendy.py:106-123: first crossing at t = sqrt(2), then every 2 sqrt(2)
    g = wendy_gb300.nbody(numpy.array([-1., 1.]), numpy.zeros(2), numpy.ones(2), 1,
                          full_output=True)
    counts = [next(g)[2] for _ in range(5)]
    assert counts == [0, 1, 1, 1, 2]


def test_maxcoll_error_and_warning():
    # tests/test_wendy.py:125-148
    x, v, m = numpy.array([-1., 1.]), numpy.zeros(2), numpy.ones(2)
    g = wendy_gb300.nbody(x, v, m, 2, maxcoll=0, full_output=True)
    with pytest.raises(RuntimeError) as e:
        next(g)
    assert str(e.value) == "Maximum number of collisions per time step exceeded"
    g = wendy_gb300.nbody(x, v, m, 2, maxcoll=0, full_output=True, warn_maxcoll=True)
    with pytest.warns(RuntimeWarning) as record:
        next(g)
    assert len(record) == 1
    assert record[0].message.args[0] == "Maximum number of collisions per time step exceeded"


def test_exact_and_approximate_paths_agree():
    # tests/test_approx.py:213-232 of the reference: both paths on the GPU
    x, v, m = ics.sech2_disk(101, seed=9)
    v = v - numpy.mean(v)
    ge = wendy_gb300.nbody(x, v, m, 0.05)
    ga = wendy_gb300.nbody(x, v, m, 0.05, approx=True, nleap=2000)
    for _ in range(20):
        ex, ev = next(ge)
        ax, av = next(ga)
        assert numpy.all(numpy.fabs(ex - ax) < 1e-5)
        assert numpy.all(numpy.fabs(ev - av) < 1e-5)
