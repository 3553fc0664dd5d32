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
