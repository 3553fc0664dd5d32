"""Benchmark of the GPU approximate integrator (one JSON line on stdout).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload sech2_2p24|sech2_1e4|tophat_2p27]

Workload (default, the HBM-scale single-simulation configuration): N = 2^27
equal-mass sheets (total mass 1, twopiG = 1) in a cold top-hat, x ~ U(-1, 1),
v ~ N(0, 1e-3^2), no harmonic term, the registered pulsed external force
F(x, t) = 0.3 exp(-(t - 5)^2 / 2) tanh(x / 0.5), dt = 0.01 per output,
nleap = 10 sub-steps, 500 outputs from t = 0.  The slab collapses at
t = pi/2 (inside it a = -x) and relaxes violently afterwards.  Seeded
synthetic inputs (numpy default_rng(0), draw order x, v, m).  The other
single-simulation workloads (--workload sech2_2p24 ...) follow the same
rules.

A step is one output interval (nleap sub-steps); steps are counted from
t = 0, the first W of them untimed.  `value` is particle-steps/s
(N x nleap x steps / device time) with the sheets resident in HBM, timed with
CUDA events on the library's stream.  `full_run` then continues the same
simulation through all of the configuration's outputs (for the top-hat: the
collapse and the relaxation after it) and reports its particle-steps/s over
the whole run, per phase, and how many sub-steps ran on the bucket path and
how many on the compact (full re-sort) path.  `e2e` is the same metric
through the reference-shaped C-ABI call wg_nbody_approx_onestep with
page-locked host buffers, so every step uploads its inputs and downloads x,
v, a and the sorted records.  The resident state (28 B/sheet, 3.8 GB at
2^27) is larger than L2, so no flush is needed between steps.

--impl reference times the CPU implementation of the same path on this
host's cores: the oracle restatement of wendy's C (oracle/), with all host
threads and the task-parallel merge sort, on a bounded sample of the same
workload (the sheets sorted once, then timed sub-steps in the steady state,
as in the reference's generator loop).
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: (n, ics, ics kwargs, dt, nleap, omega, ext)
    "sech2_2p24": dict(n=1 << 24, family="sech2", kw=dict(masses="lognormal", sigma_ln=0.5),
                       dt=0.02, nleap=20, omega=1.1, ext=None, outputs=200),
    "sech2_2p23": dict(n=1 << 23, family="sech2", kw=dict(masses="lognormal", sigma_ln=0.5),
                       dt=0.02, nleap=20, omega=1.1, ext=None, outputs=200),
    "sech2_1e4": dict(n=10000, family="sech2", kw=dict(masses="equal"), dt=0.05, nleap=10,
                      omega=None, ext=None, outputs=1000),
    "tophat_2p27": dict(n=1 << 27, family="tophat", kw=dict(masses="equal"), dt=0.01,
                        nleap=10, omega=None, ext=("pulse", (0.3, 5.0, 1.0, 0.5)), outputs=500),
    "tophat_2p23": dict(n=1 << 23, family="tophat", kw=dict(masses="equal"), dt=0.01,
                        nleap=10, omega=None, ext=("pulse", (0.3, 5.0, 1.0, 0.5)), outputs=500),
    # ensemble / serving workloads (see run_ensemble, run_serve)
    "ensemble_4096": dict(sims=4096, nmin=1e3, nmax=1e6, nleap=10),
    "serve_poisson": dict(rate=200.0, nmin=1e3, nmax=4e6, smin=100, smax=10000, nleap=10,
                          budget=150e9, requests=1000),
}


def replica_reduce(elapsed, units):
    """Max of the elapsed times and sum of the units over the ranks of the
    default process group (replicas: every rank runs its own simulation; this
    is the only cross-rank exchange, for reporting)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(elapsed)], dtype=torch.float64)
    u = torch.tensor([float(units)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), float(u.item())


def ensemble_members(count, nmin, nmax, seed=0):
    """(n, family, seed, dt, omega) of `count` simulations drawn from `seed`:
    N log-uniform in [nmin, nmax], initial conditions cycling over the sech^2
    disk, the cold top-hat and the Gaussian blob (sigma_x = sigma_v = 1), dt
    uniform in [0.005, 0.05], omega in {0, 0.5, 1.1}."""
    rng = numpy.random.default_rng(seed)
    fams = ["sech2", "tophat", "gaussian"]
    out = []
    for k in range(count):
        n = int(round(numpy.exp(rng.uniform(numpy.log(nmin), numpy.log(nmax)))))
        out.append((n, fams[k % 3], int(rng.integers(1 << 30)), float(rng.uniform(0.005, 0.05)),
                    [0.0, 0.5, 1.1][int(rng.integers(3))]))
    return out


def member_inputs(n, fam, seed):
    from wendy_gb300 import ics
    if fam == "gaussian":
        return ics.gaussian(n, seed=seed, sigma_x=1.0, sigma_v=1.0)
    return ics.FAMILIES[fam](n, seed=seed)


def run_ensemble(args, w):
    """Many simulations in one pool: one launch per sub-step for all of them."""
    import wendy_gb300
    from wendy_gb300.ensemble import Pool
    mem = ensemble_members(w["sims"], w["nmin"], w["nmax"])
    nleap = w["nleap"]
    pool = Pool()
    ids, dts = [], []
    total = 0
    for (n, fam, seed, dt, omega) in mem:
        x, v, m = member_inputs(n, fam, seed)
        ids.append(pool.add(x, v, m, omega=omega))
        dts.append(dt / nleap)
        total += n
    dts = numpy.array(dts)
    t0 = numpy.zeros(len(ids))
    for _ in range(args.warmup):
        pool.step(ids, dts, nleap, t0)
    st0 = pool.stats()
    # the K timed steps, end to end: every output copied back (x, v of every
    # simulation, wg_pool_download_many) into page-locked host memory while
    # the next step computes (wg_pool_step_begin / wg_pool_step_end), the last
    # one after it, wall clock; `value` is the device time of the same steps
    from wendy_gb300 import _lib as LL
    xall, vall = LL.pinned_empty(total), LL.pinned_empty(total)
    with Clocks(0) as clk:
        el = 0.0
        t_start = time.perf_counter()
        for k in range(args.steps):
            pool.step_begin(ids, dts, nleap, t0)
            if k:
                pool.download_many(ids, xall, vall)
            el += pool.step_end()
        pool.download_many(ids, xall, vall)
        wall = time.perf_counter() - t_start
    st = {k: v - st0[k] for k, v in pool.stats().items()}
    launches = st["launches"]
    pool.close()
    value = total * nleap * args.steps / el
    e2e_value = total * nleap * args.steps / wall
    # the plain path: a sample of the same simulations, one at a time
    # the plain path on a random sample of the same simulations, one at a
    # time: each simulation's step timed on the device (CUDA events, like the
    # pool's `value`) and end to end (step + download into page-locked
    # memory, wall clock, like the pool's `e2e`)
    rng = numpy.random.default_rng(1)
    sample = rng.choice(len(mem), size=min(args.plain_sample, len(mem)), replace=False)
    solo_ps, solo_dev, solo_wall = 0, 0.0, 0.0
    for k in sample:
        n, fam, seed, dt, omega = mem[k]
        x, v, m = member_inputs(n, fam, seed)
        sim = wendy_gb300.Simulation(x, v, m, numpy.sum(m), omega ** 2)
        tt = ctypes.c_double(0.0)
        xx, vv = LL.pinned_empty(n), LL.pinned_empty(n)
        for _ in range(args.warmup):
            sim.step(dt / nleap, nleap, tt)
        for _ in range(args.steps):
            t1 = time.perf_counter()
            solo_dev += sim.step(dt / nleap, nleap, tt)
            sim.download(xx, vv)
            solo_wall += time.perf_counter() - t1
            solo_ps += n * nleap
        sim.close()
    solo = solo_ps / solo_dev
    solo_e2e = solo_ps / solo_wall
    line = {"metric": "particle-steps/s", "value": value, "unit": "particle-steps/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": el / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded initial conditions)",
            "config": {"workload": args.workload, "sims": len(mem), "sheets": total,
                       "nleap": nleap, "n_range": [w["nmin"], w["nmax"]],
                       "l2": "resident state larger than L2; no flush"},
            "e2e": {"value": e2e_value, "unit": "particle-steps/s",
                    "h2d_bytes_per_step": 16 * len(ids), "d2h_bytes_per_step": 16 * total,
                    "overlap": "every member's x, v downloaded every step into page-locked "
                               "memory while the next step runs; the last step's after it",
                    "steps": args.steps},
            "value_timing": "device time (CUDA events) of the same timed steps",
            "pool_stats": {k: st[k] for k in ("overflows", "recovery_rounds", "sheets_resorted",
                                             "substeps_relaunched", "graph_builds")},
            "plain_one_at_a_time": {"value": solo, "unit": "particle-steps/s",
                                    "e2e": solo_e2e, "sample_sims": int(len(sample)),
                                    "steps_per_sim": args.steps,
                                    "ratio_device_to_device": value / solo,
                                    "ratio_e2e_to_e2e": e2e_value / solo_e2e},
            "clocks": clk.summary(), "gpu_launches": launches}
    print(json.dumps(line))


def run_serve(args, w):
    """Poisson stream of simulation requests: continuous batching vs the plain path."""
    from wendy_gb300.serve import Request, Server, latency_stats, serve_one_at_a_time
    rng = numpy.random.default_rng(0)
    nreq = args.requests or w["requests"]
    fams = ["sech2", "tophat", "gaussian"]
    reqs = []
    t = 0.0
    for k in range(nreq):
        t += rng.exponential(1.0 / w["rate"])
        n = int(round(numpy.exp(rng.uniform(numpy.log(w["nmin"]), numpy.log(w["nmax"])))))
        steps = int(round(numpy.exp(rng.uniform(numpy.log(w["smin"]), numpy.log(w["smax"])))))
        nout = max(1, steps // w["nleap"])
        x, v, m = member_inputs(n, fams[k % 3], int(rng.integers(1 << 30)))
        reqs.append(dict(x=x, v=v, m=m, dt=float(rng.uniform(0.005, 0.05)), nleap=w["nleap"],
                         noutputs=nout, omega=[None, 0.5, 1.1][int(rng.integers(3))], arrival=t))
    budget = args.budget_gb * 1e9 if args.budget_gb else w["budget"]
    srv = Server(budget_bytes=int(budget))
    with Clocks(0) as clk:
        served = srv.run([Request(**r) for r in reqs])
    rounds, waits, peak = srv.rounds, srv.budget_waits, srv.peak_bytes
    pool_stats = srv.pool.stats()
    srv.close()
    b, clk_plain = None, None
    if not args.skip_plain:
        with Clocks(0) as clk_plain:
            plain = serve_one_at_a_time([Request(**r) for r in reqs])
        b = latency_stats(plain)
    a = latency_stats(served)
    line = {"metric": "served p50/p99 latency and particle-steps/s", "value": a["p99_s"],
            "unit": "s (p99 latency)", "n_gpus": 1, "steps": nreq, "warmup": 0,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded Poisson stream, seeded initial conditions)",
            "config": {"workload": args.workload, "requests": nreq, "rate_per_s": w["rate"],
                       "arrivals_s": reqs[-1]["arrival"],
                       "n_range": [w["nmin"], w["nmax"]], "steps_range": [w["smin"], w["smax"]],
                       "budget_bytes": budget, "rounds": rounds,
                       "rounds_with_a_request_waiting_for_memory": waits,
                       "peak_admitted_bytes": peak},
            "continuous_batching": a, "plain_one_at_a_time": b,
            "throughput_ratio": a["particle_steps_per_s"] / b["particle_steps_per_s"] if b else None,
            "pool_stats": {k: pool_stats[k] for k in (
                "overflows", "recovery_rounds", "sheets_resorted", "members_compact",
                "graph_seconds", "recovery_seconds")},
            "clocks": clk.summary(), "clocks_plain": clk_plain.summary() if clk_plain else None}
    print(json.dumps(line))

HBM_FALLBACK_GBS = 6800.0
# dram__bytes_read.sum + dram__bytes_write.sum of one k_bucket_step launch
# from an ncu capture of a smaller case of the same family, per sheet
TRAFFIC_PER_SHEET = {
    "sech2": ((237.496576e6 + 185.93152e6) / (1 << 23),
              "ncu capture of one sub-step of the sech2 disk at N = 2^23"),
    "tophat": ((237.603328e6 + 187.855872e6) / (1 << 23),
               "ncu capture of one sub-step of the cold top-hat with the pulsed force at "
               "N = 2^23"),
}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return HBM_FALLBACK_GBS, "fallback"


class Clocks:
    """Samples the GPU's clocks and throttle reasons every 50 ms (one
    `nvidia-smi -lms 50` process) while the timed region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []  # (time, fields)
        self._p = None
        self._t = None
        self._t_in = self._t_out = None

    def _read(self):
        for line in self._p.stdout:
            self.rows.append((time.perf_counter(), [c.strip() for c in line.split(",")]))

    def __enter__(self):
        try:
            self._p = subprocess.Popen(["nvidia-smi", "-i", str(self.index),
                                        "--query-gpu=" + self.QUERY,
                                        "--format=csv,noheader,nounits", "-lms", "50"],
                                       stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self._p = None
        if self._p is not None:
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
            # the sampler is running before the timed region starts
            t0 = time.perf_counter()
            while not self.rows and self._p.poll() is None and time.perf_counter() - t0 < 5:
                time.sleep(0.005)
        self._t_in = time.perf_counter()
        return self

    def __exit__(self, *a):
        self._t_out = time.perf_counter()
        if self._p is not None:
            self._p.terminate()  # the process this object started
            try:
                self._p.wait(timeout=5)
            except Exception:
                self._p.kill()
            self._t.join(timeout=5)

    def summary(self):
        inside = [r for t, r in self.rows if self._t_in is not None and self._t_in <= t
                  and (self._t_out is None or t <= self._t_out)]
        if not inside and self.rows:
            # a region shorter than the sampling interval: the sample nearest to it
            ref = self._t_in if self._t_in is not None else 0.0
            inside = [min(self.rows, key=lambda tr: abs(tr[0] - ref))[1]]
        rows = inside
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in rows if len(r) > 1 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4)
                          if len(r) > 5 + i and r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows), "interval_ms": 50}


def make_inputs(w, seed=0):
    from wendy_gb300 import ics
    return ics.FAMILIES[w["family"]](w["n"], seed=seed, **w["kw"])


def ext_of(w):
    if w["ext"] is None:
        return None
    from wendy_gb300.extforce import PulseTanh
    return PulseTanh(*w["ext"][1])


class CpuSample:
    """The oracle (C restatement of wendy's approximate step) on this host's
    cores, in the reference's steady state: one untimed call sorts the sheets
    (the reference's generator does that once, on its first call), then
    timed calls continue from the sorted records, as wendy's loop does."""

    def __init__(self, w, x, v, m):
        from oracle import oracle as O
        O.load()
        self.O = O
        self.w = w
        self.ext = None if w["ext"] is None else (O.EXT_PULSE_TANH, list(w["ext"][1]))
        self.omega2 = -1.0 if w["omega"] is None else w["omega"] ** 2
        self.dt_leap = w["dt"] / w["nleap"]
        self.m = m
        self.tot = numpy.sum(m)
        self.x, self.v = x.copy(), v.copy()
        self.a = numpy.zeros(len(x))
        self.xi = O.make_sheets(self.x)
        self.t = 0.0
        self.cores = os.cpu_count() or 1
        O.set_parallel_sort(self.cores)
        self.t, _ = O.onestep(self.xi, self.x, self.v, m, self.a, self.tot, self.dt_leap, 1,
                              self.t, self.omega2, self.ext, "parallel")

    def snapshot(self):
        return (self.xi.copy(), self.x.copy(), self.v.copy(), self.t)

    def restore(self, snap):
        xi, x, v, t = snap
        self.xi[:] = xi
        self.x[:] = x
        self.v[:] = v
        self.t = t

    def run(self, nsub, sort):
        """nsub sub-steps in one call; returns the call's own elapsed time."""
        self.O.set_parallel_sort(self.cores)
        self.t, el = self.O.onestep(self.xi, self.x, self.v, self.m, self.a, self.tot,
                                    self.dt_leap, nsub, self.t, self.omega2, self.ext, sort)
        return el


def cpu_baseline(w, x, v, m, budget_s=20.0):
    """Bounded sample of the CPU path on this host (rank 0 only)."""
    cs = CpuSample(w, x, v, m)
    snap = cs.snapshot()
    res = {}
    for sort in ("parallel", "quick"):
        cs.restore(snap)
        # one sub-step first, to size the sample within the budget
        el1 = cs.run(1, sort)
        k = int(max(1, min(w["nleap"], (budget_s / 2) // max(el1, 1e-9))))
        el = cs.run(k, sort) if k > 1 else el1
        res[sort] = (w["n"] * k / el, k, el)
    best = max(res, key=lambda s: res[s][0])
    val, k, el = res[best]
    return {"value": val, "unit": "particle-steps/s", "cores": cs.cores, "kind": "port",
            "sample": "oracle (C restatement of wendy's approx step), sort=%s, OMP threads=%d, "
                      "N=%d, %d sub-steps in one call from sorted records (%.1f s)"
                      % (best, cs.cores, w["n"], k, el),
            "variants": {s: {"value": r[0], "substeps": r[1], "seconds": r[2]}
                         for s, r in res.items()}}


def run_reference(args, w):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    x, v, m = make_inputs(w)
    # sub-steps per timed step: keeps K + W steps within minutes at N = 2^24 .. 2^27
    per_step = w["nleap"] if w["n"] <= 100000 else (2 if w["n"] <= (1 << 24) else 1)
    cs = CpuSample(w, x, v, m)
    for _ in range(args.warmup):
        cs.run(per_step, "parallel")
    tot = 0.0
    for _ in range(args.steps):
        tot += cs.run(per_step, "parallel")
    val = w["n"] * per_step * args.steps / tot
    line = {"metric": "particle-steps/s", "value": val, "unit": "particle-steps/s",
            "impl": "reference", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": tot / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload, "n": w["n"], "nleap": w["nleap"],
                       "dt": w["dt"], "omega": w["omega"], "ext_force": w["ext"],
                       "timed_substeps_per_step": per_step},
            "cpu_baseline": {"value": val, "unit": "particle-steps/s", "cores": cores,
                             "kind": "port",
                             "sample": "oracle restatement of wendy's approx step, "
                                       "sort=parallel, %d threads, %d sub-steps per step, "
                                       "from sorted records (steady state)" % (cores, per_step)},
            "e2e": {"value": val, "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def full_run_summary(w, per_output, world):
    """particle-steps/s of a whole run (every output from t = 0), per phase of
    100 outputs, and which path its sub-steps took."""
    n, nleap = w["n"], w["nleap"]
    dev = sum(r[0] for r in per_output)
    wall = sum(r[1] for r in per_output)
    nout = len(per_output)
    last = per_output[-1][2]
    phases = []
    prev = {"substeps_compact": 0, "sorts_full": 0, "substeps_predicted": 0}
    for lo in range(0, nout, 100):
        rows = per_output[lo:lo + 100]
        st = rows[-1][2]
        d = sum(r[0] for r in rows)
        phases.append({"outputs": [lo, lo + len(rows)],
                       "t": [lo * w["dt"], (lo + len(rows)) * w["dt"]],
                       "ms_per_substep": d / (len(rows) * nleap) * 1e3,
                       "particle_steps_per_s": n * nleap * len(rows) / d,
                       "substeps_compact": st["substeps_compact"] - prev["substeps_compact"],
                       "substeps_predicted": st["substeps_predicted"] - prev["substeps_predicted"],
                       "resorts": st["sorts_full"] - prev["sorts_full"],
                       "largest_bucket_count": max(r[2]["last_max_count"] for r in rows)})
        prev = st
    out = {"outputs": nout, "substeps": nout * nleap, "t_end": nout * w["dt"],
           "value": world * n * nleap * nout / dev, "unit": "particle-steps/s",
           "device_s": dev, "wall_s": wall, "wall_value": world * n * nleap * nout / wall,
           "substeps_bucket": nout * nleap - last["substeps_compact"],
           "substeps_compact": last["substeps_compact"], "sorts_full": last["sorts_full"],
           "substeps_predicted": last["substeps_predicted"],
           "phases": phases}
    if w["family"] == "tophat":
        # inside the uniform slab a = -x (total mass 1): it collapses at t = pi/2
        kc = int(numpy.ceil((numpy.pi / 2) / w["dt"]))
        post = per_output[kc - 1:] if kc < nout else []
        if post:
            c0 = per_output[kc - 1][2]["substeps_compact"]
            out["post_collapse"] = {
                "from_output": kc, "substeps": len(post[1:]) * nleap,
                "substeps_compact": last["substeps_compact"] - c0,
                "particle_steps_per_s": n * nleap * len(post[1:]) /
                                        max(sum(r[0] for r in post[1:]), 1e-12)}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="tophat_2p27", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-full-run", action="store_true")
    ap.add_argument("--plain-sample", type=int, default=48,
                    help="ensemble_4096: simulations of the plain one-at-a-time comparison")
    ap.add_argument("--requests", type=int, default=0,
                    help="serve_poisson: requests in the stream (default 1000)")
    ap.add_argument("--skip-plain", action="store_true",
                    help="serve_poisson: continuous batching only (no one-at-a-time arm)")
    ap.add_argument("--budget-gb", type=float, default=0.0,
                    help="serve_poisson: HBM budget in GB (default: the configuration's 150)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    w = WORKLOADS[args.workload]
    if args.impl == "reference":
        if "family" not in w:
            print(json.dumps({"impl": "reference", "unavailable":
                              "the reference runs one simulation per call; its ensemble rate is "
                              "the single-simulation CPU rate"}))
            return
        return run_reference(args, w)
    if args.workload == "ensemble_4096":
        return run_ensemble(args, w)
    if args.workload == "serve_poisson":
        return run_serve(args, w)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        # replicas: one independent simulation per GPU, no data-path collective
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
        import torch.distributed as dist
        dist.init_process_group("gloo")

    import wendy_gb300
    from wendy_gb300 import _lib
    L = _lib.lib()
    x, v, m = make_inputs(w, seed=rank)
    n, nleap, dt = w["n"], w["nleap"], w["dt"]
    omega2 = -1.0 if w["omega"] is None else w["omega"] ** 2
    ext = ext_of(w)
    tot = numpy.sum(m)
    sim = wendy_gb300.Simulation(x, v, m, tot, omega2, ext)
    t0 = ctypes.c_double(0.0)  # steps are outputs counted from t = 0
    dt_leap = dt / nleap
    per_output = []  # (device s, wall s, stats) of every output from t = 0

    def one_output():
        tw = time.perf_counter()
        el = sim.step(dt_leap, nleap, t0)
        per_output.append((el, time.perf_counter() - tw, sim.stats()))
        return el

    for _ in range(args.warmup):
        one_output()
    st0 = sim.stats()
    if world > 1:
        dist.barrier()
    with Clocks(local) as clk:
        elapsed = 0.0
        for _ in range(args.steps):
            elapsed += one_output()
    st1 = sim.stats()
    # energy / momentum of the last output: on the device (wg_energy) and with
    # the reference's formula on the host, outside the timed region
    diag = None
    if rank == 0 and not args.no_cpu_baseline and ext is None:
        from wendy_gb300 import diagnostics
        gx, gv = numpy.empty(n), numpy.empty(n)
        sim.download(gx, gv)
        tq = time.perf_counter()
        e_dev, p_dev = sim.energy(omega=w["omega"])
        t_dev = time.perf_counter() - tq
        tq = time.perf_counter()
        e_host = diagnostics.energy(gx, gv, m, omega=w["omega"])
        t_host = time.perf_counter() - tq
        diag = {"device_energy_s": t_dev, "host_energy_s": t_host, "energy": e_dev,
                "energy_rel_diff_vs_host": abs(e_dev - e_host) / abs(e_host),
                "momentum": p_dev, "host": "numpy, reference formula (argsort + cumsum)"}
    units = n * nleap * args.steps
    if world > 1:
        elapsed, units = replica_reduce(elapsed, units)
    value = units / elapsed
    launches = st1["launches"] - st0["launches"]

    # The timed region launches k_bucket_step once per sub-step and, per
    # call, one short k_split_out (x, v out of the last sub-step's records)
    # and a few small copies, so its CUDA-event time divided by the sub-steps
    # is the bucket kernel's average launch duration to within that.
    hbm, hbm_kind = peaks()
    sub_s = elapsed / (args.steps * nleap)
    bucket_gbs = 56.0 * n / sub_s / 1e9

    def prof(what, reps):
        out = ctypes.c_double()
        _lib.check(L.wg_profile(sim._h, what, reps, ctypes.byref(out)), "wg_profile")
        return out.value
    f_s = prof(0, 10)   # fused force kernel on compact sets (initial call, fallback)
    s_s = prof(1, 3)    # full radix re-sort (initial sort, fallback)
    comps = {"k_bucket_step": {"ms": sub_s * 1e3, "algorithmic_bytes_per_sheet": 56,
                               "achieved_gbs": bucket_gbs, "share_of_timed_region": 1.0},
             "k_force_kick_drift": {"ms": f_s * 1e3, "algorithmic_bytes_per_sheet": 40,
                                    "achieved_gbs": 40.0 * n / f_s / 1e9},
             "radix_resort": {"ms": s_s * 1e3, "algorithmic_bytes_per_sheet": 250,
                              "achieved_gbs": 250.0 * n / s_s / 1e9}}
    traffic_per_sheet, traffic_src = TRAFFIC_PER_SHEET.get(
        w["family"], TRAFFIC_PER_SHEET["sech2"])
    traffic = traffic_per_sheet * n
    roof = {"bound": "hbm", "kernel": "k_bucket_step", "achieved": bucket_gbs, "peak": hbm,
            "unit": "GB/s", "frac": bucket_gbs / hbm, "peak_kind": hbm_kind,
            "traffic": traffic, "traffic_unit": "bytes per launch",
            "traffic_source": traffic_src + ", scaled to N by the sheets",
            "algorithmic_bytes_per_launch": 56.0 * n,
            "components": comps, "substep_ms": sub_s * 1e3,
            "stats": {k: st1[k] - st0[k] for k in ("sorts_full", "sorts_window", "substeps",
                                                   "substeps_compact")}}

    # end to end through the reference-shaped call, buffers in page-locked
    # host memory (wg_host_alloc: on the measured GB300 hosts memory page-locked
    # by registration falls from about 190 to about 5 GB/s after tens of
    # seconds of sustained device load, allocated page-locked memory does not)
    e2e = None
    if not args.no_e2e:
        from wendy_gb300 import _lib as LL
        xi = LL.pinned_empty(n, LL.SHEET_DTYPE)
        xi["idx"] = numpy.arange(n, dtype=numpy.int32)
        xi["val"] = x
        xx, vv, a, mm = (LL.pinned_empty(n) for _ in range(4))
        xx[:] = x
        vv[:] = v
        a[:] = 0.0
        mm[:] = m
        # outputs counted from t = 0 as above: W untimed, then K timed
        tt = 0.0
        for _ in range(args.warmup):
            tt, _el = wendy_gb300.approx_onestep(xi, xx, vv, mm, a, tot, dt_leap, nleap, tt,
                                                 omega2, ext)
        from wendy_gb300.wendy import approx_onestep_stats
        sorts0 = approx_onestep_stats()["sorts_full"]
        t_start = time.perf_counter()
        k_e2e = args.steps
        for _ in range(k_e2e):
            tt, _el = wendy_gb300.approx_onestep(xi, xx, vv, mm, a, tot, dt_leap, nleap, tt,
                                                 omega2, ext)
        wall = time.perf_counter() - t_start
        resorted = approx_onestep_stats()["sorts_full"] - sorts0
        del xi, xx, vv, a, mm
        e2e = {"value": world * n * nleap * k_e2e / wall, "unit": "particle-steps/s",
               "h2d_bytes_per_step": 32 * n, "d2h_bytes_per_step": 40 * n,
               "call": "wg_nbody_approx_onestep", "steps": k_e2e,
               "calls_resorted": resorted,
               "overlap": "every call uploads xi, v, m and downloads xi, x, v, a (page-locked, "
                          "wall clock); as in wendy's generator each call is handed the previous "
                          "call's outputs, which it verifies bit for bit on the device, so its "
                          "sub-steps, enqueued by the previous call, run under these transfers"}

    # the same simulation on through all of the configuration's outputs: the
    # whole run from t = 0, collapse and relaxation included
    full = None
    if not args.no_full_run and w.get("outputs"):
        while len(per_output) < w["outputs"]:
            one_output()
        full = full_run_summary(w, per_output, world)

    sim.close()

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(w, x, v, m)

    if rank == 0:
        line = {"metric": "particle-steps/s", "value": value, "unit": "particle-steps/s",
                "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": elapsed / args.steps * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded initial conditions, no dataset)",
                "config": {"workload": args.workload, "n": n, "nleap": nleap, "dt": dt,
                           "omega": w["omega"], "ext_force": w["ext"], "ics": w["family"],
                           "parallelism": "replicas" if world > 1 else "single",
                           "l2": "resident state larger than L2; no flush"},
                "e2e": e2e, "roofline": roof, "full_run": full, "cpu_baseline": cpu,
                "clocks": clk.summary(), "diagnostics": diag,
                "gpu_launches": launches}
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
