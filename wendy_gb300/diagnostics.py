"""Host-side diagnostics with the semantics of wendy.energy / momentum /
potential (wendy/wendy.py:439-517).

These are numpy, as in the reference: they run on the (x, v) arrays the
generator yields.  ``energy`` uses the same sorted cumulative sums as the
reference (wendy/wendy.py:467-475), so for identical inputs it returns the
identical float.
"""
import numpy


def energy(x, v, m, twopiG=1., individual=False, omega=None):
    """Total energy, or each sheet's energy with ``individual=True``.

    Mirrors wendy/wendy.py:439-475: the potential term of the total is
    sum_i m_i (M_below(i) x_i - (m x)_below(i)) over sorted order, times
    twopiG; the individual form is the O(N^2) pairwise sum.
    """
    if omega is not None:
        harm = m * omega ** 2. * x ** 2. / 2.
    else:
        harm = 0.
    if individual:
        return harm + twopiG * m * numpy.sum(m * numpy.fabs(x - numpy.atleast_2d(x).T),
                                             axis=1) + m * v ** 2. / 2.
    order = numpy.argsort(x)
    below = numpy.roll(numpy.cumsum(m[order]), 1)
    below[0] = 0.
    xbelow = numpy.roll(numpy.cumsum((m * x)[order]), 1)
    xbelow[0] = 0.
    return (numpy.sum(harm)
            + twopiG * numpy.sum(m[order] * (below * x[order] - xbelow))
            + numpy.sum(m * v ** 2. / 2.))


def momentum(v, m):
    """Total momentum (wendy/wendy.py:477-491)."""
    return numpy.sum(m * v)


def potential(y, x, v, m, twopiG=1., omega=None):
    """Potential at the points y (wendy/wendy.py:493-517)."""
    if omega is not None:
        harm = omega ** 2. * y ** 2. / 2.
    else:
        harm = 0.
    return harm + twopiG * numpy.sum(m * numpy.fabs(x - numpy.atleast_2d(y).T), axis=1)
