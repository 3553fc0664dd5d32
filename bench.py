"""Benchmark of the GPU approximate integrator (one JSON line on stdout).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload sech2_2p24|sech2_1e4|tophat_2p27]

Workload (default, the large single-simulation configuration): N = 2^24
sheets, isothermal sech^2 disk (z0 = 1, sigma^2 = 2 pi G Sigma z0 = 1.0 with
twopiG = 1), lognormal masses (sigma_ln = 0.5) normalised to 1, harmonic
omega = 1.1, dt = 0.02 per output, nleap = 20 sub-steps.  Seeded synthetic
inputs (numpy default_rng(0), draw order x, v, m).

A step is one output interval (nleap sub-steps).  `value` is particle-steps/s
(N x nleap x steps / device time) with the sheets resident in HBM, timed with
CUDA events on the library's stream; `e2e` is the same metric through the
reference-shaped C-ABI call wg_nbody_approx_onestep with page-locked host
buffers, so every step uploads its inputs and downloads x, v, a and the
sorted records.  The resident state (28 B/sheet x 2^24 = 470 MB) is larger
than L2, so no flush is needed between steps.

--impl reference times the CPU implementation of the same path on this
host's cores: the oracle restatement of wendy's C (oracle/), with all host
threads and the task-parallel merge sort, on a bounded sample of the same
workload.
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
                       dt=0.02, nleap=20, omega=1.1, ext=None),
    "sech2_2p23": dict(n=1 << 23, family="sech2", kw=dict(masses="lognormal", sigma_ln=0.5),
                       dt=0.02, nleap=20, omega=1.1, ext=None),
    "sech2_1e4": dict(n=10000, family="sech2", kw=dict(masses="equal"), dt=0.05, nleap=10,
                      omega=None, ext=None),
    "tophat_2p27": dict(n=1 << 27, family="tophat", kw=dict(masses="equal"), dt=0.01,
                        nleap=10, omega=None, ext=("pulse", (0.3, 5.0, 1.0, 0.5))),
}

HBM_FALLBACK_GBS = 6800.0


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return HBM_FALLBACK_GBS, "fallback"


class Clocks:
    """Samples nvidia-smi every 200 ms while the timed region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self._stop = threading.Event()
        self._t = threading.Thread(target=self._run, daemon=True)

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index),
                                      "--query-gpu=" + self.QUERY, "--format=csv,noheader,nounits"],
                                     capture_output=True, text=True, timeout=5).stdout
                for line in out.strip().splitlines():
                    self.rows.append([c.strip() for c in line.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4)
                          if len(r) > 5 + i and r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


def make_inputs(w, seed=0):
    from wendy_gb300 import ics
    return ics.FAMILIES[w["family"]](w["n"], seed=seed, **w["kw"])


def ext_of(w):
    if w["ext"] is None:
        return None
    from wendy_gb300.extforce import PulseTanh
    return PulseTanh(*w["ext"][1])


def cpu_run(w, x, v, m, nleap_sample, sort, threads):
    """Time the oracle on one output of nleap_sample sub-steps (seconds)."""
    from oracle import oracle as O
    O.set_parallel_sort(threads)
    ext = None if w["ext"] is None else (O.EXT_PULSE_TANH, list(w["ext"][1]))
    omega2 = -1.0 if w["omega"] is None else w["omega"] ** 2
    xx, vv = x.copy(), v.copy()
    a = numpy.zeros(len(x))
    xi = O.make_sheets(xx)
    _t0, el = O.onestep(xi, xx, vv, m, a, numpy.sum(m), w["dt"] / w["nleap"], nleap_sample, 4.0,
                        omega2, ext, sort)
    return el


def cpu_baseline(w, x, v, m, budget_s=20.0):
    """Bounded sample of the CPU path on this host (rank 0 only)."""
    from oracle import oracle as O
    O.load()
    cores = os.cpu_count() or 1
    res = {}
    for sort in ("parallel", "quick"):
        # one sub-step first, to size the sample within the budget
        el1 = cpu_run(w, x, v, m, 1, sort, cores)
        k = int(max(1, min(w["nleap"], (budget_s / 2) // max(el1, 1e-9))))
        el = cpu_run(w, x, v, m, k, sort, cores) if k > 1 else el1
        res[sort] = (w["n"] * k / el, k, el)
    best = max(res, key=lambda s: res[s][0])
    val, k, el = res[best]
    return {"value": val, "unit": "particle-steps/s", "cores": cores, "kind": "port",
            "sample": "oracle (C restatement of wendy's approx step), sort=%s, OMP threads=%d, "
                      "N=%d, one output of %d sub-steps (%.1f s)" % (best, cores, w["n"], k, el),
            "variants": {s: {"value": r[0], "substeps": r[1], "seconds": r[2]}
                         for s, r in res.items()}}


def run_reference(args, w):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle as O
    O.load()
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    x, v, m = make_inputs(w)
    per_step = 2  # sub-steps per timed step: keeps K + W steps within minutes at N = 2^24
    if w["n"] <= 100000:
        per_step = w["nleap"]
    for _ in range(args.warmup):
        cpu_run(w, x, v, m, per_step, "parallel", cores)
    tot = 0.0
    for _ in range(args.steps):
        tot += cpu_run(w, x, v, m, per_step, "parallel", cores)
    val = w["n"] * per_step * args.steps / tot
    line = {"metric": "particle-steps/s", "value": val, "unit": "particle-steps/s",
            "impl": "reference", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": tot / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload, "n": w["n"], "nleap": w["nleap"],
                       "dt": w["dt"], "omega": w["omega"],
                       "timed_substeps_per_step": per_step},
            "cpu_baseline": {"value": val, "unit": "particle-steps/s", "cores": cores,
                             "kind": "port",
                             "sample": "oracle restatement of wendy's approx step, "
                                       "sort=parallel, %d threads, %d sub-steps per step"
                                       % (cores, per_step)},
            "e2e": {"value": val, "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="sech2_2p24", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    w = WORKLOADS[args.workload]
    if args.impl == "reference":
        return run_reference(args, w)

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
    t0 = ctypes.c_double(4.0 if ext else 0.0)
    dt_leap = dt / nleap
    for _ in range(args.warmup):
        sim.step(dt_leap, nleap, t0)
    st0 = sim.stats()
    if world > 1:
        dist.barrier()
    with Clocks(local) as clk:
        elapsed = 0.0
        for _ in range(args.steps):
            elapsed += sim.step(dt_leap, nleap, t0)
    st1 = sim.stats()
    if world > 1:
        import torch
        t = torch.tensor([elapsed], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed = float(t.item())
    value = world * n * nleap * args.steps / elapsed
    launches = st1["launches"] - st0["launches"]

    # kernel-level timing (CUDA events inside the library, same stream)
    f_s, s_s = ctypes.c_double(), ctypes.c_double()
    _lib.check(L.wg_profile(sim._h, 0, 20, ctypes.byref(f_s)), "wg_profile")
    _lib.check(L.wg_profile(sim._h, 1, 5, ctypes.byref(s_s)), "wg_profile")
    hbm, hbm_kind = peaks()
    force_gbs = 40.0 * n / f_s.value / 1e9
    sort_gbs = 224.0 * n / s_s.value / 1e9
    sub_ms = elapsed / (args.steps * nleap) * 1e3
    comps = {"force_kick_drift": {"ms": f_s.value * 1e3, "algorithmic_bytes_per_sheet": 40,
                                  "achieved_gbs": force_gbs},
             "radix_resort": {"ms": s_s.value * 1e3, "algorithmic_bytes_per_sheet": 224,
                              "achieved_gbs": sort_gbs}}
    dom = max(comps, key=lambda k: comps[k]["ms"])
    dk = comps[dom]
    roof = {"bound": "hbm", "kernel": dom, "achieved": dk["achieved_gbs"], "peak": hbm,
            "unit": "GB/s", "frac": dk["achieved_gbs"] / hbm, "peak_kind": hbm_kind,
            "traffic": None, "components": comps, "substep_ms": sub_ms}
    sim.close()

    # end to end through the reference-shaped call, page-locked host buffers
    e2e = None
    if not args.no_e2e:
        from wendy_gb300 import _lib as LL
        xi = numpy.zeros(n, dtype=LL.SHEET_DTYPE)
        xi["idx"] = numpy.arange(n, dtype=numpy.int32)
        xi["val"] = x
        xx, vv, a = x.copy(), v.copy(), numpy.zeros(n)
        mm = m.copy()
        bufs = [xi, xx, vv, a, mm]
        for b in bufs:
            _lib.check(L.wg_host_register(b.ctypes.data, b.nbytes), "wg_host_register")
        tt = 4.0 if ext else 0.0
        for _ in range(2):
            tt, _el = wendy_gb300.approx_onestep(xi, xx, vv, mm, a, tot, dt_leap, nleap, tt,
                                                 omega2, ext)
        t_start = time.perf_counter()
        k_e2e = max(3, min(args.steps, 5))
        for _ in range(k_e2e):
            tt, _el = wendy_gb300.approx_onestep(xi, xx, vv, mm, a, tot, dt_leap, nleap, tt,
                                                 omega2, ext)
        wall = time.perf_counter() - t_start
        for b in bufs:
            L.wg_host_unregister(b.ctypes.data)
        e2e = {"value": world * n * nleap * k_e2e / wall, "unit": "particle-steps/s",
               "h2d_bytes_per_step": 32 * n, "d2h_bytes_per_step": 40 * n,
               "call": "wg_nbody_approx_onestep", "steps": k_e2e}

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
                "e2e": e2e, "roofline": roof, "cpu_baseline": cpu, "clocks": clk.summary(),
                "gpu_launches": launches}
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
