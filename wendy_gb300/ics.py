"""Seeded initial conditions for the workloads this package is measured on.

All generators draw from ``numpy.random.default_rng(seed)`` in the order
x, v, m and return float64 arrays (x, v, m).  Units follow wendy's
(twopiG = 1): a self-gravitating isothermal sheet of total surface mass
Sigma and scale height z0 has velocity dispersion sigma^2 = 2 pi G Sigma z0,
which is 1.0 for Sigma = z0 = 1 (the convention of wendy's own sech^2 tests,
tests/test_approx.py:36-40 in the reference).
"""
import numpy


def _masses(rng, n, kind, sigma_ln=0.5, totmass=1.0):
    if kind == "equal":
        return numpy.full(n, totmass / n)
    if kind == "lognormal":
        m = rng.lognormal(0.0, sigma_ln, size=n)
        return m * (totmass / numpy.sum(m))
    raise ValueError("unknown mass law %r" % kind)


def sech2_disk(n, seed=0, z0=1.0, sigma2=1.0, masses="equal", sigma_ln=0.5, totmass=1.0):
    """Isothermal sech^2 sheet: x = 2 z0 artanh(2u - 1), v ~ N(0, sigma2)."""
    rng = numpy.random.default_rng(seed)
    x = 2.0 * z0 * numpy.arctanh(2.0 * rng.uniform(size=n) - 1.0)
    v = rng.normal(0.0, numpy.sqrt(sigma2), size=n)
    m = _masses(rng, n, masses, sigma_ln, totmass)
    return x, v, m


def top_hat(n, seed=0, half_width=1.0, sigma_v=1e-3, masses="equal", totmass=1.0):
    """Cold top-hat slab: x ~ U(-w, w), v ~ N(0, sigma_v^2)."""
    rng = numpy.random.default_rng(seed)
    x = rng.uniform(-half_width, half_width, size=n)
    v = rng.normal(0.0, sigma_v, size=n)
    m = _masses(rng, n, masses, totmass=totmass)
    return x, v, m


def gaussian(n, seed=0, sigma_x=1.0, sigma_v=1.0, masses="equal", totmass=1.0):
    """Gaussian blob in phase space: x ~ N(0, sigma_x^2), v ~ N(0, sigma_v^2)."""
    rng = numpy.random.default_rng(seed)
    x = rng.normal(0.0, sigma_x, size=n)
    v = rng.normal(0.0, sigma_v, size=n)
    m = _masses(rng, n, masses, totmass=totmass)
    return x, v, m


FAMILIES = {"sech2": sech2_disk, "tophat": top_hat, "gaussian": gaussian}
