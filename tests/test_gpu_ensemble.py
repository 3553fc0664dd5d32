"""Ensembles on one GPU: each simulation bit-identical to its solo run."""
import ctypes

import numpy
import pytest

import wendy_gb300
from oracle import oracle as O
from wendy_gb300 import ics
from wendy_gb300.ensemble import Pool
from wendy_gb300.extforce import Harmonic, PulseTanh

pytestmark = pytest.mark.gpu

CASES = [  # (n, family, seed, dt_leap, omega, ext)
    (1, "gaussian", 1, 0.01, None, None),
    (7, "sech2", 2, 0.004, 1.1, None),
    (500, "tophat", 3, 0.001, None, PulseTanh(0.3, 5.0, 1.0, 0.5)),
    (3000, "gaussian", 4, 0.002, 0.5, None),
    (20000, "sech2", 5, 0.003, None, Harmonic(0.7)),
    (70001, "sech2", 6, 0.001, 1.1, None),
]


def _solo(n, fam, seed, dt, omega, ext, nleap, nout):
    x, v, m = ics.FAMILIES[fam](n, seed=seed)
    omega2 = -1. if omega is None else omega ** 2
    sim = wendy_gb300.Simulation(x, v, m, numpy.sum(m), omega2, ext)
    t = ctypes.c_double(4.0)
    outs = []
    for _ in range(nout):
        sim.step(dt, nleap, t)
        gx, gv = numpy.empty(n), numpy.empty(n)
        sim.download(gx, gv)
        outs.append((gx, gv))
    return outs, t.value


def test_ensemble_matches_solo_bit_for_bit():
    nleap, nout = 5, 3
    with Pool() as pool:
        ids = []
        for n, fam, seed, dt, omega, ext in CASES:
            x, v, m = ics.FAMILIES[fam](n, seed=seed)
            ids.append(pool.add(x, v, m, omega=omega, ext_force=ext))
        dts = numpy.array([c[3] for c in CASES])
        t0 = numpy.full(len(CASES), 4.0)
        got = [[] for _ in CASES]
        for _ in range(nout):
            pool.step(ids, dts, nleap, t0)
            for k, sid in enumerate(ids):
                got[k].append(pool.download(sid))
    for k, (n, fam, seed, dt, omega, ext) in enumerate(CASES):
        solo, tsolo = _solo(n, fam, seed, dt, omega, ext, nleap, nout)
        assert t0[k] == tsolo
        for (gx, gv), (sx, sv) in zip(got[k], solo):
            assert numpy.array_equal(gx, sx) and numpy.array_equal(gv, sv), (n, fam)


def test_ensemble_matches_oracle():
    n, dt, nleap = 4000, 0.002, 8
    x, v, m = ics.sech2_disk(n, seed=11, masses="lognormal")
    with Pool() as pool:
        a = pool.add(x, v, m, omega=1.1)
        b = pool.add(x[:900], v[:900], m[:900])
        pool.step([a, b], [dt, dt], nleap)
        gx, gv = pool.download(a)
    r = O.nbody_approx(x, v, m, dt * nleap, nleap, omega=1.1)
    rx, rv = next(r)
    assert numpy.max(numpy.abs(gx - rx)) <= 1e-10
    assert numpy.max(numpy.abs(gv - rv)) <= 1e-10


def test_members_join_and_leave_without_changing_results():
    nleap = 4
    x, v, m = ics.sech2_disk(12000, seed=21)
    xo, vo, mo = ics.top_hat(5000, seed=22)
    with Pool() as alone, Pool() as mixed:
        a = alone.add(x, v, m)
        b = mixed.add(x, v, m)
        other = mixed.add(xo, vo, mo)
        for k in range(4):
            alone.step([a], [0.002], nleap)
            if k == 1:
                mixed.remove(other)
                other = mixed.add(xo[:3000], vo[:3000], mo[:3000])
            ids = [other, b] if k % 2 else [b, other]
            mixed.step(ids, [0.002, 0.002], nleap)
            ax, av = alone.download(a)
            bx, bv = mixed.download(b)
            assert numpy.array_equal(ax, bx) and numpy.array_equal(av, bv), k


def test_budget_is_enforced():
    need = Pool.sim_bytes(10000)
    with Pool(budget_bytes=int(need * 1.5)) as pool:
        x, v, m = ics.sech2_disk(10000, seed=3)
        pool.add(x, v, m)
        with pytest.raises(wendy_gb300._lib.WendyGPUError) as e:
            pool.add(x, v, m)
        assert e.value.status == -6
        assert pool.info()["sims"] == 1


def _converging(n, seed):
    # every sheet reaches the origin within one sub-step: the bucket layout
    # overflows and the call finishes on a full re-sort
    rng = numpy.random.default_rng(seed)
    x = rng.uniform(-1, 1, size=n)
    return x, -x / 0.01 * 0.999, numpy.full(n, 1.0 / n)


def test_members_overflowing_in_one_call_recover_independently():
    # two members overflow in the same call, a third does not; each must
    # still equal the oracle (the recoveries share the pool's workspace)
    cases = [_converging(50000, 7), _converging(30001, 8), ics.sech2_disk(20000, seed=9)]
    pool = Pool()
    ids = [pool.add(x, v, m) for (x, v, m) in cases]
    gens = [O.nbody_approx(x, v, m, 0.05, 5) for (x, v, m) in cases]
    t0 = numpy.zeros(len(ids))
    for _ in range(2):
        pool.step(ids, 0.01, 5, t0)
        for sid, g, (x, _, _) in zip(ids, gens, cases):
            gx, gv = pool.download(sid)
            rx, rv = next(g)
            assert numpy.max(numpy.abs(gx - rx)) <= 1e-9
            assert numpy.max(numpy.abs(gv - rv)) <= 1e-9
    pool.close()


def test_download_during_a_step_returns_the_previous_output():
    # wg_pool_step_begin / wg_pool_step_end: while a step runs, each member's
    # download is its output before that step (none before the first); the
    # pool refuses to change its members; results equal synchronous steps
    members = [ics.sech2_disk(20000, seed=s, masses="lognormal") for s in (1, 2)]
    p, q = Pool(), Pool()
    ids = [p.add(x, v, m, omega=1.1) for x, v, m in members]
    qids = [q.add(x, v, m, omega=1.1) for x, v, m in members]
    for k in range(3):
        p.step_begin(ids, 0.002, 5)
        for sid, qid in zip(ids, qids):
            if k == 0:
                with pytest.raises(wendy_gb300._lib.WendyGPUError):
                    p.download(sid)
            else:
                x, v = p.download(sid)
                qx, qv = q.download(qid)
                assert numpy.array_equal(x, qx) and numpy.array_equal(v, qv)
        with pytest.raises(wendy_gb300._lib.WendyGPUError):
            p.remove(ids[0])
        with pytest.raises(wendy_gb300._lib.WendyGPUError):
            p.add(*members[0])
        assert p.step_end() > 0.0
        q.step(qids, 0.002, 5)
    for sid, qid in zip(ids, qids):
        x, v = p.download(sid)
        qx, qv = q.download(qid)
        assert numpy.array_equal(x, qx) and numpy.array_equal(v, qv)
    p.close()
    q.close()


def test_download_many_equals_downloads_one_by_one():
    # wg_pool_download_many: the members' outputs one after another, in the
    # order of ids, during a step (the output before it) and after it; a bad
    # id fails the call before anything is copied
    members = [ics.sech2_disk(n, seed=s, masses="lognormal") for n, s in ((3000, 1), (20000, 2),
                                                                          (777, 3))]
    p = Pool()
    ids = [p.add(x, v, m, omega=1.1) for x, v, m in members]
    order = [ids[2], ids[0], ids[1]]
    p.step(ids, 0.002, 5)
    for running in (False, True):
        if running:
            p.step_begin(ids, 0.002, 5)
        one = [p.download(sid) for sid in order]
        total = sum(len(a) for a, _ in one)
        # into page-locked memory of the library's own (wg_host_alloc)
        x, v = p.download_many(order, wendy_gb300._lib.pinned_empty(total),
                               wendy_gb300._lib.pinned_empty(total))
        assert numpy.array_equal(x, numpy.concatenate([a for a, _ in one]))
        assert numpy.array_equal(v, numpy.concatenate([b for _, b in one]))
        xs = numpy.full(len(x), 7.0)
        bad = numpy.array([ids[0], 99], numpy.int32)
        assert p._L.wg_pool_download_many(p._h, 2, bad.ctypes.data, xs.ctypes.data,
                                          xs.ctypes.data) == wendy_gb300._lib.WG_ERR_ARG
        assert numpy.all(xs == 7.0)
        if running:
            p.step_end()
    p.close()


def test_collapsing_members_match_their_solo_runs():
    # cold top-hats run through their collapse (t = pi/2) in one pool: their
    # buckets overflow, the pool recovers them and switches them to predicted
    # splitters; every output must still be the solo run's, bit for bit
    members = [(20000, 11), (60000, 12), (150000, 13)]
    dt, nleap, nout = 0.002, 10, 100  # t = 0 .. 2
    with Pool() as pool:
        ids = []
        for n, seed in members:
            x, v, m = ics.top_hat(n, seed=seed)
            ids.append(pool.add(x, v, m))
        t0 = numpy.zeros(len(ids))
        got = [[] for _ in members]
        for k in range(nout):
            pool.step(ids, numpy.full(len(ids), dt), nleap, t0)
            if k % 10 == 9:
                for j, sid in enumerate(ids):
                    got[j].append(pool.download(sid))
        st = pool.stats()
    # the collapse overflowed buckets and the pool recovered them
    # (members below 2^20 sheets never finish on the compact path)
    assert st["steps"] == nout and st["members_sorted"] == len(members)
    assert st["members_compact"] == 0 and st["substeps_compact"] == 0
    assert st["overflows"] > 0 and st["recovery_rounds"] > 0
    assert st["sheets_resorted"] >= st["overflows"] * min(n for n, _ in members)
    assert 0 < st["substeps_relaunched"] <= st["overflows"] * (nleap - 1)
    for j, (n, seed) in enumerate(members):
        x, v, m = ics.top_hat(n, seed=seed)
        sim = wendy_gb300.Simulation(x, v, m, numpy.sum(m), -1.)
        t = ctypes.c_double(0.)
        for k in range(nout):
            sim.step(dt, nleap, t)
            if k % 10 == 9:
                sx, sv = numpy.empty(n), numpy.empty(n)
                sim.download(sx, sv)
                gx, gv = got[j][k // 10]
                assert numpy.array_equal(gx, sx) and numpy.array_equal(gv, sv), (n, k)
        sim.close()


def test_a_large_collapsing_member_matches_its_solo_run():
    # a collapsing member of 2^20 sheets and a smaller one, re-sorted together
    # after their overflows: both bit for bit
    members = [(1 << 20, 21), (30000, 22)]
    dt, nleap, nout = 0.002, 10, 100  # t = 0 .. 2, through the collapse
    with Pool() as pool:
        ids = []
        for n, seed in members:
            x, v, m = ics.top_hat(n, seed=seed)
            ids.append(pool.add(x, v, m))
        t0 = numpy.zeros(len(ids))
        got = [[] for _ in members]
        for k in range(nout):
            pool.step(ids, numpy.full(len(ids), dt), nleap, t0)
            if k % 20 == 19:
                for j, sid in enumerate(ids):
                    got[j].append(pool.download(sid))
        st = pool.stats()
    assert st["overflows"] > 0 and st["recovery_rounds"] > 0
    for j, (n, seed) in enumerate(members):
        x, v, m = ics.top_hat(n, seed=seed)
        sim = wendy_gb300.Simulation(x, v, m, numpy.sum(m), -1.)
        t = ctypes.c_double(0.)
        for k in range(nout):
            sim.step(dt, nleap, t)
            if k % 20 == 19:
                sx, sv = numpy.empty(n), numpy.empty(n)
                sim.download(sx, sv)
                gx, gv = got[j][k // 20]
                assert numpy.array_equal(gx, sx) and numpy.array_equal(gv, sv), (n, k)
        sim.close()
