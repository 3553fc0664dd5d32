"""Continuous-batching server: same results alone and in the mix."""
import numpy
import pytest

from wendy_gb300 import ics
from wendy_gb300.ensemble import Pool
from wendy_gb300.extforce import PulseTanh
from wendy_gb300.serve import Request, Server, latency_stats, serve_one_at_a_time

pytestmark = pytest.mark.gpu


def _requests(seed, count):
    rng = numpy.random.default_rng(seed)
    fams = ["sech2", "tophat", "gaussian"]
    out = []
    t = 0.0
    for k in range(count):
        n = int(numpy.exp(rng.uniform(numpy.log(50), numpy.log(30000))))
        fam = fams[k % 3]
        x, v, m = ics.FAMILIES[fam](n, seed=1000 + k)
        omega = [None, 0.5, 1.1][k % 3]
        ext = PulseTanh(0.3, 5.0, 1.0, 0.5) if k % 5 == 0 else None
        t += rng.exponential(0.01)
        out.append(Request(x=x, v=v, m=m, dt=float(rng.uniform(0.005, 0.05)), nleap=10,
                           noutputs=int(rng.integers(2, 7)), omega=omega, ext_force=ext,
                           t0=4.0, arrival=t, keep_outputs=True))
    return out


def _clone(reqs):
    return [Request(x=r.x, v=r.v, m=r.m, dt=r.dt, nleap=r.nleap, noutputs=r.noutputs,
                    omega=r.omega, ext_force=r.ext_force, t0=r.t0, arrival=r.arrival,
                    keep_outputs=True) for r in reqs]


def test_served_results_equal_solo_results():
    reqs = _requests(1, 14)
    solo = serve_one_at_a_time(_clone(reqs))
    srv = Server(budget_bytes=8 << 30)
    try:
        served = srv.run(_clone(reqs))
    finally:
        srv.close()
    for a, b in zip(solo, served):
        assert len(a.outputs) == len(b.outputs) == a.noutputs
        for (ax, av), (bx, bv) in zip(a.outputs, b.outputs):
            assert numpy.array_equal(ax, bx) and numpy.array_equal(av, bv)
    st = latency_stats(served)
    assert st["p99_s"] >= st["p50_s"] > 0


def test_budget_limits_residency_but_serves_everything():
    reqs = _requests(2, 8)
    budget = int(max(Pool.sim_bytes(r.n) for r in reqs) * 2.2)
    srv = Server(budget_bytes=budget)
    try:
        served = srv.run(_clone(reqs))
    finally:
        srv.close()
    assert all(r.done_at is not None for r in served)
    solo = serve_one_at_a_time(_clone(reqs))
    for a, b in zip(solo, served):
        assert numpy.array_equal(a.last_x, b.last_x) and numpy.array_equal(a.last_v, b.last_v)
