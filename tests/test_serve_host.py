"""Host logic of the continuous-batching server (wendy_gb300/serve.py), run
against a fake pool on the CPU: admission under the budget, one pool step per
round, each round's outputs delivered while the next round's step is in
flight, retirement after the last output.  The fake pool follows the device
pool's contract: during a step, download returns a member's output before it."""
import numpy
import pytest

from wendy_gb300 import serve


class FakePool:
    BYTES_PER_SHEET = 100

    def __init__(self, budget_bytes=0):
        self.sims = {}
        self.next_id = 0
        self.inflight = None
        self.steps = 0
        self.max_used = 0

    @staticmethod
    def sim_bytes(n):
        return FakePool.BYTES_PER_SHEET * n

    def add(self, x, v, m, omega=None, ext_force=None, twopiG=1.):
        assert self.inflight is None, "members change only between steps"
        sid = self.next_id
        self.next_id += 1
        self.sims[sid] = {"x": numpy.array(x, float), "v": numpy.array(v, float), "done": 0}
        self.max_used = max(self.max_used, sum(len(s["x"]) for s in self.sims.values()))
        return sid

    def remove(self, sid):
        assert self.inflight is None, "members change only between steps"
        del self.sims[sid]

    def step_begin(self, ids, dts, nleap, t0):
        assert self.inflight is None
        self.inflight = list(ids)
        for k in range(len(ids)):
            t0[k] += 1.0  # the step advances t0 at once

    def step_end(self):
        for sid in self.inflight:
            self.sims[sid]["done"] += 1
        self.inflight = None
        self.steps += 1
        return 1e-3

    def download(self, sid, x, v):
        s = self.sims[sid]
        done = s["done"]  # during a step: the output before it
        if done == 0:
            raise RuntimeError("no completed output")
        x[:] = s["x"] + done
        v[:] = s["v"] - done
        return x, v

    def close(self):
        pass


class FakePinned:
    def __init__(self, n):
        self.x = numpy.empty(n)
        self.v = numpy.empty(n)

    def release(self):
        pass


@pytest.fixture
def fake(monkeypatch):
    monkeypatch.setattr(serve, "Pool", FakePool)
    monkeypatch.setattr(serve, "_Pinned", FakePinned)


def _requests(rng, count):
    reqs = []
    for k in range(count):
        n = int(rng.integers(1, 6))
        reqs.append(serve.Request(x=rng.normal(size=n), v=rng.normal(size=n), m=numpy.ones(n),
                                  dt=0.1, nleap=10 if k % 3 else 5,
                                  noutputs=int(rng.integers(1, 7)), arrival=0.0,
                                  keep_outputs=True))
    return reqs


def test_every_output_delivered_once_in_order(fake):
    rng = numpy.random.default_rng(0)
    reqs = _requests(rng, 12)
    srv = serve.Server(budget_bytes=10 ** 9)
    srv.run(reqs, clock=lambda: 0.0)
    for r in reqs:
        assert len(r.outputs) == r.noutputs
        for k, (x, v) in enumerate(r.outputs, start=1):
            assert numpy.array_equal(x, r.x + k) and numpy.array_equal(v, r.v - k)
        assert numpy.array_equal(r.last_x, r.x + r.noutputs)
        assert r.done_at is not None
    assert not srv.pool.sims  # everything retired
    # rounds: as many as the longest request has outputs, and at most one step per
    # nleap group per round
    assert srv.rounds == max(r.noutputs for r in reqs)


def test_budget_bounds_the_resident_sheets(fake):
    rng = numpy.random.default_rng(1)
    reqs = _requests(rng, 20)
    budget = FakePool.BYTES_PER_SHEET * 8
    srv = serve.Server(budget_bytes=budget)
    srv.run(reqs, clock=lambda: 0.0)
    assert srv.pool.max_used <= 8
    assert all(len(r.outputs) == r.noutputs for r in reqs)
