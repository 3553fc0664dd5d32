"""bench.py's CPU legs run here (no GPU): the reference arm and the CPU baseline."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_json_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--workload", "sech2_1e4", "--steps", "2", "--warmup", "3"],
                         capture_output=True, text=True, timeout=300, cwd=ROOT,
                         env=dict(os.environ, OMP_NUM_THREADS="2"))
    assert out.returncode == 0, out.stderr
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["cpu_baseline"]["kind"] == "port"
    assert d["e2e"]["h2d_bytes_per_step"] == 0


def test_reference_arm_for_ensembles_is_marked_unavailable():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--workload", "ensemble_4096"], capture_output=True, text=True,
                         timeout=120, cwd=ROOT)
    assert out.returncode == 0
    assert "unavailable" in json.loads(out.stdout.strip().splitlines()[-1])


def test_bench_module_parses_and_defines_the_workloads():
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench", os.path.join(ROOT, "bench.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    assert {"sech2_2p24", "tophat_2p27", "ensemble_4096", "serve_poisson"} <= set(b.WORKLOADS)
    mem = b.ensemble_members(16, 1e3, 1e6)
    assert len(mem) == 16 and all(1000 <= m[0] <= 1e6 for m in mem)


def test_clock_summary_keeps_the_samples_of_the_timed_region():
    sys.path.insert(0, ROOT)
    import bench
    c = bench.Clocks(0)
    row = lambda mhz, slow="Not Active", cap="Not Active": [
        "0", str(mhz), "2070", "900.0", "0x1", slow, "Not Active", "Not Active", cap]
    c.rows = [(0.9, row(135)), (1.05, row(2070)), (1.10, row(2040, cap="Active")),
              (1.15, row(2070)), (1.40, row(300, slow="Active"))]
    c._t_in, c._t_out = 1.0, 1.2
    s = c.summary()
    assert s["samples"] == 3 and s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"]  # the idle and later samples are left out
    # a region shorter than the interval: the nearest sample stands in
    c._t_in, c._t_out = 1.06, 1.07
    s = c.summary()
    assert s["samples"] == 1 and s["sm_mhz"] == 2070.0


def test_full_run_summary_counts_paths_and_phases():
    sys.path.insert(0, ROOT)
    import bench
    w = dict(bench.WORKLOADS["tophat_2p27"], n=1000)
    rows = []
    compact = sorts = pred = 0
    for k in range(500):
        # the compact path from the collapse (output 158) to output 300,
        # predicted splitters on the bucket path from output 300 to 316
        step_c = 10 if 158 <= k < 300 else 0
        compact += step_c
        sorts += step_c + (1 if k == 0 else 0)
        pred += 10 if 300 <= k < 316 else 0
        rows.append((0.02 if step_c else 0.01, 0.011,
                     {"substeps_compact": compact, "sorts_full": sorts,
                      "substeps_predicted": pred,
                      "last_max_count": 0 if step_c else 1800}))
    s = bench.full_run_summary(w, rows, 1)
    assert s["outputs"] == 500 and s["substeps"] == 5000
    assert s["substeps_compact"] == 1420 and s["substeps_bucket"] == 3580
    assert len(s["phases"]) == 5 and s["phases"][0]["substeps_compact"] == 0
    assert s["phases"][1]["substeps_compact"] == 420
    assert s["phases"][3]["substeps_predicted"] == 160 and s["substeps_predicted"] == 160
    assert abs(s["value"] - 1000 * 5000 / (0.01 * 358 + 0.02 * 142)) < 1e-6 * s["value"]
    pc = s["post_collapse"]
    assert pc["from_output"] == 158 and pc["substeps_compact"] == 1420
    assert pc["substeps"] == (500 - 158) * 10


def test_default_workload_is_the_hbm_scale_top_hat():
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench2", os.path.join(ROOT, "bench.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    w = b.WORKLOADS["tophat_2p27"]
    assert w["n"] == 1 << 27 and w["outputs"] == 500 and w["nleap"] == 10 and w["dt"] == 0.01
    assert w["ext"][1] == (0.3, 5.0, 1.0, 0.5)
