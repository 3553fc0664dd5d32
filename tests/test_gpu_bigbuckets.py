"""Buckets that receive more sheets than one shared-memory pass holds.

A single simulation's layouts have room for kBucketCapBig sheets per bucket;
a bucket above kBucketCap (2048) is taken in chunks along its keys by
k_bucket_big, and one whose keys crowd into a single bin beyond what a chunk
holds is handed back to the host, which re-sorts the layout that sub-step
read and runs it again.  Both must give the reference's trajectory (the
oracle, within 1e-10 per output, wendy/wendy.c:385-418).
"""
import ctypes

import numpy
import pytest

import wendy_gb300
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _compare(x, v, m, dt, nleap, nout):
    n = len(x)
    sim = wendy_gb300.Simulation(x, v, m, numpy.sum(m), -1.)
    r = O.nbody_approx(x, v, m, dt * nleap, nleap, sort="quick")
    t = ctypes.c_double(0.)
    gx, gv = numpy.empty(n), numpy.empty(n)
    for _ in range(nout):
        sim.step(dt, nleap, t)
        sim.download(gx, gv)
        rx, rv = next(r)
        assert numpy.max(numpy.abs(gx - rx)) <= 1e-10
        assert numpy.max(numpy.abs(gv - rv)) <= 1e-10
    st = sim.stats()
    sim.close()
    return st


def test_a_block_moving_into_a_region_doubles_its_buckets():
    # uniform sheets at rest, and those in (0.5, 0.6) moving left by 0.05 per
    # sub-step: where the block passes, buckets laid out for the old density
    # receive about twice their target (> 2048), and are taken in chunks
    n = 1 << 20
    rng = numpy.random.default_rng(3)
    x = rng.uniform(-1, 1, n)
    v = numpy.where((x > 0.5) & (x < 0.6), -50.0, 0.0)
    m = numpy.full(n, 1.0 / n)
    st = _compare(x, v, m, 0.001, 4, 1)
    assert st["big_buckets"] > 0
    assert st["sorts_full"] == 1  # the first sort only: no bucket overflowed


def test_a_dense_cluster_is_sent_back_and_recovered():
    # 1100 sheets within 1e-9 of each other move with the block: a bucket
    # then holds more sheets in one key bin than a chunk can take, the host
    # re-sorts the layout the sub-step read and runs it again
    n = 1 << 20
    rng = numpy.random.default_rng(4)
    x = rng.uniform(-1, 1, n)
    cl = rng.choice(n, 1100, replace=False)
    x[cl] = 0.55 + 1e-9 * rng.uniform(size=1100)
    v = numpy.where((x > 0.5) & (x < 0.6), -50.0, 0.0)
    m = numpy.full(n, 1.0 / n)
    st = _compare(x, v, m, 0.001, 4, 2)
    assert st["sorts_full"] > 1


def test_predicted_splitters_follow_the_block():
    # the first output meets buckets above one shared-memory pass, so the
    # next outputs take their splitters from the sheets' positions moved on
    # by two drifts at their bucket's mean velocity (sorted after every
    # sub-step); any sorted splitters give the same trajectory
    n = 1 << 20
    rng = numpy.random.default_rng(5)
    x = rng.uniform(-1, 1, n)
    v = numpy.where((x > 0.5) & (x < 0.6), -50.0, 0.0)
    m = rng.lognormal(0.0, 0.5, n)
    m /= m.sum()
    st = _compare(x, v, m, 0.001, 4, 4)
    assert st["substeps_predicted"] > 0
