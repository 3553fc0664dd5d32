"""The CPU oracle against the reference's golden vectors and, where it was
built here from its own sources, against the reference library itself."""
import numpy
import pytest

from oracle import oracle as O


def _ext(par):
    kind = int(par[3])
    if kind == 0:
        return None
    if kind == O.EXT_HARMONIC:
        return (kind, [par[4]])
    return (kind, list(par[4:8]))


def test_accel_matches_reference_golden(golden):
    g = golden("accel")
    for name in g["names"]:
        name = str(name)
        x, m, par = g[name + "/x"], g[name + "/m"], g[name + "/par"]
        a, perm = O.accel(x, m, par[0], par[1], _ext(par), par[2])
        assert numpy.array_equal(perm, g[name + "/perm"]), name
        assert numpy.array_equal(a, g[name + "/a"]), name


def test_trajectories_match_reference_golden(golden):
    g = golden("traj")
    for name in g["names"]:
        name = str(name)
        x0, v0, m, par = g[name + "/x0"], g[name + "/v0"], g[name + "/m"], g[name + "/par"]
        dt, nleap, nout, omega, t0 = par
        keep = set(int(k) for k in g[name + "/keep"])
        ext = (O.EXT_PULSE_TANH, [0.3, 5.0, 1.0, 0.5]) if name == "tophat_pulse" else None
        gen = O.nbody_approx(x0, v0, m, dt, int(nleap), t0=t0,
                             omega=None if omega < 0 else omega, ext=ext)
        for k in range(1, int(nout) + 1):
            tx, tv = next(gen)
            if k in keep:
                assert numpy.array_equal(tx, g["%s/x%d" % (name, k)]), (name, k)
                assert numpy.array_equal(tv, g["%s/v%d" % (name, k)]), (name, k)


def test_energy_series_matches_reference_golden(golden):
    from wendy_gb300 import ics
    from wendy_gb300.diagnostics import energy
    g = golden("energy")
    n, _, dt, nleap, nout = g["par"]
    x, v, m = ics.sech2_disk(int(n), seed=0)
    E0 = energy(x, v, m)
    assert E0 == g["E0"][0]
    gen = O.nbody_approx(x, v, m, dt, int(nleap))
    for k in range(50):  # the first 50 outputs keep the CPU suite short
        tx, tv = next(gen)
        dE = (energy(tx, tv, m) - E0) / E0
        assert dE == g["dE"][k], k


@pytest.mark.parametrize("sort", ["quick", "qsort", "parallel"])
def test_sorts_agree_for_distinct_positions(sort):
    from wendy_gb300 import ics
    O.set_parallel_sort(2, 10, 10)  # exercise the recursive branches, as the reference CI
    x, v, m = ics.sech2_disk(257, seed=12)
    ref = O.nbody_approx(x, v, m, 0.05, 10, sort="quick")
    got = O.nbody_approx(x, v, m, 0.05, 10, sort=sort)
    for _ in range(5):
        rx, rv = next(ref)
        gx, gv = next(got)
        assert numpy.array_equal(rx, gx) and numpy.array_equal(rv, gv)
    O.set_parallel_sort(32, 10000, 50000)


def test_oracle_equals_reference_library_directly():
    lib = O.ref_library()
    if lib is None:
        pytest.skip("reference library not built from its sources on this machine")
    rng = numpy.random.default_rng(5)
    for n, omega2, ext, sort in [(3, -1.0, None, "quick"), (64, 1.21, None, "qsort"),
                                 (500, -1.0, (O.EXT_PULSE_TANH, [0.3, 5.0, 1.0, 0.5]), "quick"),
                                 (8, -1.0, (O.EXT_HARMONIC, [0.7]), "quick"),
                                 (300, -1.0, None, "parallel")]:
        x = rng.normal(size=n)
        v = rng.normal(size=n)
        m = rng.uniform(0.5, 1.5, size=n) / n
        res = []
        for which in ("oracle", "ref"):
            xx, vv, a = x.copy(), v.copy(), numpy.zeros(n)
            xi = O.make_sheets(xx)
            t0 = 3.9
            for _ in range(3):
                if which == "oracle":
                    t0, _el = O.onestep(xi, xx, vv, m, a, m.sum(), 0.002, 7, t0, omega2, ext, sort)
                else:
                    t0, _el = O.ref_onestep(lib, xi, xx, vv, m, a, m.sum(), 0.002, 7, t0, omega2,
                                            ext, sort)
            res.append((xx, vv, a, xi["idx"].copy(), t0))
        for p, q in zip(res[0], res[1]):
            assert numpy.array_equal(numpy.asarray(p), numpy.asarray(q)), (n, sort)


def test_time_sequence_lags_by_repeated_addition():
    # wendy/wendy.c:403-404,409-410: t0 advances by dt per force evaluation.
    x = numpy.array([-1.0, 0.5, 2.0])
    v = numpy.zeros(3)
    m = numpy.ones(3) / 3
    xi = O.make_sheets(x.copy())
    t0, _ = O.onestep(xi, x.copy(), v, m, numpy.zeros(3), 1.0, 0.025, 3, 1.0, -1.0,
                      (O.EXT_HARMONIC, [1.0]))
    t = 1.0
    for _ in range(3):
        t += 0.025
    assert t0 == t == 1.0749999999999997 or t0 == t
