"""External forces given as plain Python functions of (x, t), the way wendy
takes them (wendy/wendy.py:389-418).  tests/golden/make_golden.py hands them
to the reference itself (its ctypes callback route) to make
tests/golden/extexpr.npz; the tests compile the same functions with
wendy_gb300.extforce.Expression and compare.  Test infrastructure only.
"""
import numpy

ALPHA, SIGMA2, ZH = 0.3, 1.0, 0.5
OMEGA = 1.1


def iso_force(x, t):
    """The form of the external force of wendy's GaiaPhaseSpaceSpiral
    example: the non-live fraction of an isothermal disk."""
    return -(1. - ALPHA) * SIGMA2 * numpy.tanh(0.5 * x / ZH) / ZH


# the form of wendy's own external-force test (tests/test_approx_external.py:12)
harmonic_lambda = lambda x, t: -OMEGA ** 2. * x  # noqa: E731


def breathing(x, t):
    """An anharmonic, time-modulated restoring force."""
    return -0.5 * (1. + 0.3 * numpy.sin(2. * t)) * x ** 3 / (1. + x ** 2)


def satellite(x, t):
    """A softened point mass passing through the slab at constant speed."""
    return -0.05 * (x - (2. - 0.5 * t)) / ((x - (2. - 0.5 * t)) ** 2 + 0.09) ** 1.5


# (name, force, initial-condition family, n, seed, dt, nleap, outputs, t0)
CASES = [
    ("iso", iso_force, "sech2", 2000, 31, 0.05, 10, 10, 0.0),
    ("harmonic_lambda", harmonic_lambda, "sech2", 101, 32, 0.05, 100, 10, 0.0),
    ("breathing", breathing, "gaussian", 1500, 33, 0.02, 10, 10, 0.3),
    ("satellite", satellite, "tophat", 3000, 34, 0.05, 10, 10, 0.0),
]
