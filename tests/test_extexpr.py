"""Expression forces: the compiler (wendy_gb300/extforce.py) and the
oracle's evaluation of its programs, against the reference's own runs with
the same forces given as Python functions (tests/golden/extexpr.npz, made by
its ctypes callback route, wendy/wendy.py:405-418).  No GPU needed."""
import math
import sys
import os

import numpy
import pytest

from oracle import oracle as O
from wendy_gb300 import ics
from wendy_gb300.extforce import Expression, Harmonic, resolve

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import forces  # noqa: E402


@pytest.mark.parametrize("case", forces.CASES, ids=[c[0] for c in forces.CASES])
def test_program_matches_the_function(case):
    fn = case[1]
    e = Expression(fn)
    rng = numpy.random.default_rng(5)
    x = rng.normal(0., 2., 1000)
    for t in (0.0, 0.37, 3.1):
        got, ref = e.run_program(x, t), fn(x, t)
        assert numpy.max(numpy.abs(got - ref)) <= 4e-16 * numpy.max(numpy.abs(ref)) + 1e-300
    # the header of the C-ABI parameters
    assert e.params[0] == len(e.ops) and e.params[1] == e.n_time
    assert len(e.params) == 2 + 5 * len(e.ops)


def test_time_only_parts_are_hoisted_and_constants_folded():
    e = Expression("0.3*exp(-(t-5)**2/(2*1.0**2))*tanh(x/0.5)")
    space = e.ops[e.n_time:]
    assert [op[0] for op in space] == [0, 7, 16, 6]  # x, /, tanh, *: four ops per sheet
    assert all(op[0] != 0 for op in e.ops[:e.n_time])  # no x in the time phase
    e = Expression(forces.harmonic_lambda)
    assert e.ops[0][:2] == (2, 0) and e.ops[0][4] == -forces.OMEGA ** 2.


def test_names_are_read_when_compiled():
    scale = 2.0

    def f(x, t):
        return scale * x
    e = Expression(f)
    scale = 3.0  # noqa: F841  (numba freezes globals the same way)
    assert e.run_program(numpy.array([1.0]), 0.0)[0] == 2.0


class _Eforce:
    # the callable-class form of wendy's tests/test_approx_external.py:22-42
    def __init__(self, omega):
        self.omega = omega

    def __call__(self, x, t):
        return -self.omega ** 2. * x


def test_callable_objects_and_plain_functions_resolve():
    kind, params = resolve(_Eforce(1.1))
    assert kind == 3 and params[2 + 4] == -1.1 ** 2.
    kind, params = resolve(forces.iso_force)
    assert kind == 3
    assert resolve(Harmonic(1.1)) == (1, (1.1 ** 2.,))


@pytest.mark.parametrize("bad", ["x if t > 0 else x", "x[0]", "undefined_name * x",
                                 "numpy.maximum(x, t)", "x.sum()", "(x, t)", "x < 1",
                                 "exp(x, t)", "lambda: x"])
def test_outside_the_subset_is_rejected(bad):
    with pytest.raises(ValueError):
        Expression(bad)


def test_too_long_programs_are_rejected():
    with pytest.raises(ValueError):
        Expression("+".join("sin(x*%d)" % k for k in range(1, 40)))


def test_oracle_matches_the_reference_with_python_functions(golden):
    g = golden("extexpr")
    for name, fn, fam, n, seed, dt, nleap, nout, t0 in forces.CASES:
        x0, v0, m = g[name + "/x0"], g[name + "/v0"], g[name + "/m"]
        r = O.nbody_approx(x0, v0, m, dt, nleap, t0=t0, ext=Expression(fn))
        for k in range(1, nout + 1):
            rx, rv = next(r)
            if k in (1, nout):
                gx, gv = g["%s/x%d" % (name, k)], g["%s/v%d" % (name, k)]
                # the reference evaluates the function with numpy, the oracle
                # the program with libm: the forces differ in the last bits
                assert numpy.max(numpy.abs(rx - gx)) <= 1e-11, (name, k)
                assert numpy.max(numpy.abs(rv - gv)) <= 1e-11, (name, k)


def test_the_forces_move_the_sheets(golden):
    # the golden runs did go through the callables: without them the same
    # runs end elsewhere
    g = golden("extexpr")
    name, fn, fam, n, seed, dt, nleap, nout, t0 = forces.CASES[3]
    r = O.nbody_approx(g[name + "/x0"], g[name + "/v0"], g[name + "/m"], dt, nleap, t0=t0)
    for _ in range(nout):
        rx, rv = next(r)
    assert numpy.max(numpy.abs(rv - g["%s/v%d" % (name, nout)])) > 1e-4
