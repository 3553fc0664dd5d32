"""Expression forces on the GPU: functions of (x, t) compiled into register
programs (wendy_gb300.extforce.Expression) and interpreted by the force
kernels, against the reference's own runs with the same Python functions
(tests/golden/extexpr.npz, its ctypes callback route, wendy/wendy.py:405-418)
and against the oracle evaluating the same programs.

Bars as elsewhere: accelerations within 1e-12 of the acceleration scale,
positions and velocities within 1e-11 over these runs (the reference
evaluates the functions with numpy, the GPU with CUDA's math library: the
forces differ in their last bits), ensembles bit-identical to solo runs.
"""
import ctypes
import os
import sys

import numpy
import pytest

import wendy_gb300
from oracle import oracle as O
from wendy_gb300 import _lib, ics
from wendy_gb300.ensemble import Pool
from wendy_gb300.extforce import Expression, PulseTanh, evaluate_on_device

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import forces  # noqa: E402

pytestmark = pytest.mark.gpu


def test_python_functions_match_the_reference(golden):
    g = golden("extexpr")
    for name, fn, fam, n, seed, dt, nleap, nout, t0 in forces.CASES:
        x0, v0, m = g[name + "/x0"], g[name + "/v0"], g[name + "/m"]
        # a plain function, as wendy takes it: compiled on the way in
        gen = wendy_gb300.nbody(x0, v0, m, dt, approx=True, nleap=nleap, t0=t0, ext_force=fn)
        for k in range(1, nout + 1):
            tx, tv = next(gen)
            if k in (1, nout):
                assert numpy.max(numpy.abs(tx - g["%s/x%d" % (name, k)])) <= 1e-11, (name, k)
                assert numpy.max(numpy.abs(tv - g["%s/v%d" % (name, k)])) <= 1e-11, (name, k)
        gen.close()


@pytest.mark.parametrize("case", forces.CASES, ids=[c[0] for c in forces.CASES])
def test_device_evaluation_matches_the_function(case):
    fn = case[1]
    x = numpy.random.default_rng(3).normal(0., 2., 100000)
    for t in (0.0, 1.7):
        got = evaluate_on_device(Expression(fn), x, t)
        ref = fn(x, t)
        assert numpy.max(numpy.abs(got - ref)) <= 1e-14 * max(1.0, numpy.max(numpy.abs(ref)))


def test_accel_with_an_expression_matches_oracle():
    n = 1 << 20
    x, v, m = ics.top_hat(n, seed=12)
    tot = numpy.sum(m)
    e = Expression(forces.satellite)
    a, perm = wendy_gb300.accel(x, m, tot, ext_force=e, t=1.3)
    ra, rperm = O.accel(x, m, tot, -1., e, 1.3)
    assert numpy.array_equal(perm, rperm)
    assert numpy.max(numpy.abs(a - ra)) <= 1e-12 * max(tot, float(numpy.max(numpy.abs(ra))))


def test_bucket_path_with_an_expression_matches_oracle():
    n = 1 << 20
    x, v, m = ics.sech2_disk(n, seed=13, masses="lognormal")
    e = Expression(forces.breathing)
    g = wendy_gb300.nbody(x, v, m, 0.01, approx=True, nleap=10, ext_force=e, t0=0.2)
    r = O.nbody_approx(x, v, m, 0.01, 10, t0=0.2, ext=e)
    for _ in range(2):
        gx, gv = next(g)
        rx, rv = next(r)
        assert numpy.max(numpy.abs(gx - rx)) <= 1e-10
        assert numpy.max(numpy.abs(gv - rv)) <= 1e-10
    g.close()


def test_dropin_with_an_expression_matches_oracle():
    n = 3000
    x, v, m = ics.top_hat(n, seed=14)
    tot = numpy.sum(m)
    e = Expression(forces.satellite)
    outs = []
    for which in ("gpu", "oracle"):
        xx, vv, a = x.copy(), v.copy(), numpy.zeros(n)
        xi = O.make_sheets(xx)
        t = 0.0
        for _ in range(3):
            if which == "gpu":
                t, _el = wendy_gb300.approx_onestep(xi, xx, vv, m, a, tot, 0.005, 10, t,
                                                    ext_force=e)
            else:
                t, _el = O.onestep(xi, xx, vv, m, a, tot, 0.005, 10, t, -1., e)
        outs.append((xi.copy(), xx, vv, a, t))
    (gxi, gx, gv, ga, gt), (rxi, rx, rv, ra, rt) = outs
    assert gt == rt
    assert numpy.array_equal(gxi["idx"], rxi["idx"])
    for p, q in ((gx, rx), (gv, rv), (ga, ra)):
        assert numpy.max(numpy.abs(p - q)) <= 1e-10


def test_ensemble_with_expression_members_matches_solo_bit_for_bit():
    cases = [(700, "sech2", 1, 0.004, Expression(forces.iso_force)),
             (5000, "tophat", 2, 0.002, PulseTanh(0.3, 5.0, 1.0, 0.5)),
             (20000, "gaussian", 3, 0.003, Expression(forces.breathing)),
             (3000, "sech2", 4, 0.002, None)]
    nleap, nout = 5, 3
    with Pool() as pool:
        ids = []
        for n, fam, seed, dt, ext in cases:
            x, v, m = ics.FAMILIES[fam](n, seed=seed)
            ids.append(pool.add(x, v, m, ext_force=ext))
        dts = numpy.array([c[3] for c in cases])
        t0 = numpy.full(len(cases), 0.5)
        got = [[] for _ in cases]
        for _ in range(nout):
            pool.step(ids, dts, nleap, t0)
            for k, sid in enumerate(ids):
                got[k].append(pool.download(sid))
    for k, (n, fam, seed, dt, ext) in enumerate(cases):
        x, v, m = ics.FAMILIES[fam](n, seed=seed)
        sim = wendy_gb300.Simulation(x, v, m, numpy.sum(m), -1., ext)
        t = ctypes.c_double(0.5)
        for gx_gv in got[k]:
            sim.step(dt, nleap, t)
            sx, sv = numpy.empty(n), numpy.empty(n)
            sim.download(sx, sv)
            assert numpy.array_equal(gx_gv[0], sx) and numpy.array_equal(gx_gv[1], sv), (n, fam)
        assert t.value == t0[k]
        sim.close()


def test_malformed_programs_are_refused_by_the_library():
    L = _lib.lib()
    x = numpy.zeros(4)
    out = numpy.empty(4)
    bad = [
        [1, 0, 99, 0, 0, 0, 0.0],         # unknown op code
        [1, 0, 4, 0, 1, 2, 0.0],          # reads registers nothing wrote
        [1, 1, 0, 0, 0, 0, 0.0],          # x in the time phase
        [2, 0, 0, 16, 0, 0, 0.0],         # register out of range (and too short)
        [65, 0] + [2, 0, 0, 0, 1.0] * 65,  # too many ops
    ]
    for p in bad:
        params = numpy.array(p, dtype=numpy.float64)
        rc = L.wg_ext_force_eval(4, x, 0.0, 3, params, len(params), out)
        assert rc == _lib.WG_ERR_EXT, p
