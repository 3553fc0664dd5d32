"""The integer-pipe tanh of the pulsed external force (wendy_gb300/csrc/wg_tanh.cuh):
tanh_q62 fills a table of Taylor polynomials, tanh_tab evaluates them.

CPU: the constants of tanh_q62, recomputed with 60-digit decimal arithmetic.  GPU: the
device evaluation of the registered forces (wg_ext_force_eval, the force
kernels' own code) against numpy, which is how the reference evaluates its
ext_force callables (wendy/wendy.py:389-418).
"""
import os
import re
from decimal import Decimal, getcontext

import numpy
import pytest

import wendy_gb300
from wendy_gb300.extforce import Harmonic, PulseTanh, evaluate_on_device

HEADER = os.path.join(os.path.dirname(__file__), "..", "wendy_gb300", "csrc", "wg_tanh.cuh")


def _header():
    with open(HEADER) as f:
        return f.read()


def test_tanh_constants_are_correctly_rounded():
    getcontext().prec = 60
    ln2 = Decimal(2).ln()
    q62 = Decimal(2) ** 62
    src = _header()
    table = src[src.index("kExp2Tab[256]"):src.index("};", src.index("kExp2Tab[256]"))]
    tab = [int(h, 16) for h in re.findall(r"0x([0-9a-f]{16})ull", table)]
    assert tab == [int((q62 * (-(Decimal(j) / 256) * ln2).exp()).to_integral_value())
                   for j in range(256)]
    body = src[src.index("inv_fact_q62(int n)"):src.index("kLn2Q64")]
    fact = [int(h, 16) for h in re.findall(r"0x([0-9a-f]{16})ull", body)]
    want = [int((q62 / Decimal(f)).to_integral_value()) for f in (1, 2, 6, 24, 120, 720, 5040)]
    assert fact == want  # n = 0 and 1 share the first
    ln2q = int(re.search(r"kLn2Q64 = 0x([0-9a-f]{16})ull", src).group(1), 16)
    l2q = int(re.search(r"kTwoLog2eQ61 = 0x([0-9a-f]{16})ull", src).group(1), 16)
    assert ln2q == int((ln2 * Decimal(2) ** 64).to_integral_value())
    assert l2q == int((2 / ln2 * Decimal(2) ** 61).to_integral_value())


def _inputs():
    rng = numpy.random.default_rng(0)
    mag = 10.0 ** rng.uniform(-12, 1.5, 1 << 20)
    special = numpy.array([0., -0., 2. ** -27, numpy.nextafter(2. ** -27, 0.),
                           numpy.nextafter(2. ** -27, 1.), 2. ** -5, 0.5, 1., -1., 19.06,
                           numpy.nextafter(20., 0.), 20., 25., 709., 1e-300, 5e-324,
                           numpy.inf, -numpy.inf])
    return numpy.concatenate([rng.uniform(-25., 25., 1 << 20),
                              mag * rng.choice([-1., 1.], len(mag)), special])


@pytest.mark.gpu
def test_tanh_matches_numpy_within_its_error_bound():
    # A = 1, t = t0, h = 1: F(x) = tanh(x) with no other rounding
    x = _inputs()
    got = evaluate_on_device(PulseTanh(1., 0., 1., 1.), x, 0.)
    ref = numpy.tanh(x)
    # the table's rows carry tanh at the cell starts within 2^-57, the degree-5
    # polynomials add below 2^-61 before rounding to double; plus half an
    # ulp, plus the host libm's own error (one ulp)
    bound = 2. ** -57 + 2. ** -61 + 1.5 * numpy.spacing(numpy.abs(ref))
    err = numpy.abs(got - ref)
    assert numpy.all(err <= bound), (x[numpy.argmax(err - bound)], numpy.max(err - bound))
    small = numpy.abs(x) < 2. ** -27
    assert numpy.array_equal(got[small], x[small])          # tanh(x) rounds to x there
    assert numpy.all(numpy.abs(got) <= 1.)
    assert numpy.array_equal(numpy.signbit(got), numpy.signbit(x))
    assert numpy.isnan(evaluate_on_device(PulseTanh(1., 0., 1., 1.), [numpy.nan], 0.)[0])


@pytest.mark.gpu
@pytest.mark.parametrize("t", [4.2, 5.0, 9.0])
def test_pulse_force_matches_the_reference_formula(t):
    f = PulseTanh(0.3, 5.0, 1.0, 0.5)
    x = _inputs()[:-2]
    got = evaluate_on_device(f, x, t)
    ref = f(x, t)
    amp = 0.3 * numpy.exp(-(t - 5.0) ** 2 / 2.)
    # x * (1/h) instead of x / h moves the argument by at most one rounding
    # (|d tanh| <= 0.45 * 2^-52), the device and host exp(.) of the amplitude
    # differ by at most a few ulp
    assert numpy.max(numpy.abs(got - ref)) <= 6e-16 * amp


@pytest.mark.gpu
def test_harmonic_force_is_exact():
    x = _inputs()[:-2]
    f = Harmonic(1.3)
    assert numpy.array_equal(evaluate_on_device(f, x, 0.), f(x, 0.))


@pytest.mark.gpu
def test_no_force_and_bad_arguments():
    assert numpy.array_equal(evaluate_on_device(None, [1., 2.], 0.), [0., 0.])
    with pytest.raises(wendy_gb300._lib.WendyGPUError):
        evaluate_on_device(PulseTanh(1., 0., 1., 1.), [1.], numpy.nan)
