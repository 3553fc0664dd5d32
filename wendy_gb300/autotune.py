"""Autotuner of the fused bucket sub-step.

The sub-step kernel has four tunables whose best values depend on the
number of sheets of a simulation (how many buckets there are to keep the SMs
busy, how far sheets travel in bucket units, how clustered the keys inside a
bucket are):

  target       sheets per bucket right after a re-sort (capacity 2048, at most 1536)
  window       splitters searched in shared memory on each side of a bucket
  sort_bits    2^sort_bits bins of the in-bucket counting sort
  ctas_per_sm  persistent CTAs per SM

:func:`tune` times candidate settings by coordinate descent from the
defaults, for a few simulation sizes n.  Each timing advances a pool of
identical seeded sech^2 disks of n sheets, as many as make about 2^23 sheets
in all (a single simulation from that size up), by real output intervals
(CUDA-event device time through ``wg_pool_step``): the objective is the
throughput of a full GPU, which is what both a large simulation and an
ensemble of small ones need.  It returns a table of rows
``(n_min, target, window, sort_bits, ctas_per_sm)``; :func:`apply` installs
a table in the library (``wg_set_tuning``), which uses the row with the
largest ``n_min <= n`` for every simulation created afterwards.  A table
measured on a GB300 ships as ``tuning_gb300.json`` and is applied when the
library is first loaded; results do not depend on the tuning, only speed
does.
"""
import ctypes
import json
import os

import numpy

from . import _lib

HERE = os.path.dirname(os.path.abspath(__file__))
TABLE_PATH = os.path.join(HERE, "tuning_gb300.json")
DEFAULT = dict(target=1536, window=64, sort_bits=12, ctas_per_sm=2)
SPACE = dict(target=(768, 1024, 1280, 1536), window=(16, 32, 64), sort_bits=(11, 12, 13),
             ctas_per_sm=(1, 2))


def apply(rows):
    """Install rows [{n_min, target, window, sort_bits, ctas_per_sm}, ...]."""
    L = _lib.lib()
    rows = sorted(rows, key=lambda r: r["n_min"])
    arr = (_lib.WgTuning * max(1, len(rows)))()
    for i, r in enumerate(rows):
        arr[i].n_min = int(r["n_min"])
        arr[i].target = int(r["target"])
        arr[i].window = int(r["window"])
        arr[i].sort_bits = int(r["sort_bits"])
        arr[i].ctas_per_sm = int(r["ctas_per_sm"])
    _lib.check(L.wg_set_tuning(ctypes.cast(arr, ctypes.c_void_p), len(rows)), "wg_set_tuning")


def current(n):
    t = _lib.WgTuning()
    _lib.check(_lib.lib().wg_get_tuning(int(n), ctypes.byref(t)), "wg_get_tuning")
    return dict(target=t.target, window=t.window, sort_bits=t.sort_bits,
                ctas_per_sm=t.ctas_per_sm)


def load_table(path=TABLE_PATH):
    if not os.path.exists(path):
        return None
    with open(path) as f:
        return json.load(f)["rows"]


def apply_shipped():
    rows = load_table()
    if rows:
        apply(rows)
    return rows


def _time(n, setting, nleap=10, outputs=2, seed=0, total=1 << 23):
    """Device seconds per sub-step of a pool of max(1, total // n) simulations of n sheets."""
    from .ensemble import Pool
    from .ics import sech2_disk
    apply([dict(n_min=0, **setting)])
    x, v, m = sech2_disk(n, seed=seed, masses="lognormal")
    pool = Pool()
    try:
        ids = [pool.add(x, v, m, omega=1.1) for _ in range(max(1, total // n))]
        pool.step(ids, 0.001, nleap)
        el = 0.0
        for _ in range(outputs):
            el += pool.step(ids, 0.001, nleap)
    finally:
        pool.close()
    return el / (outputs * nleap)


def tune(sizes=(1 << 11, 1 << 14, 1 << 17, 1 << 20, 1 << 24), rounds=2, verbose=False):
    """Coordinate descent over SPACE for each size; returns the table rows."""
    rows = []
    for n in sizes:
        best = dict(DEFAULT)
        best_t = _time(n, best)
        for _ in range(rounds):
            improved = False
            for key, values in SPACE.items():
                for val in values:
                    if val == best[key]:
                        continue
                    cand = dict(best)
                    cand[key] = val
                    t = _time(n, cand)
                    if verbose:
                        print(n, cand, "%.1f us/substep" % (t * 1e6))
                    if t < best_t * 0.98:
                        best, best_t, improved = cand, t, True
            if not improved:
                break
        rows.append(dict(n_min=0 if not rows else int(n), substep_us=best_t * 1e6,
                         size=int(n), **best))
    # boundaries half-way (in log) between the tuned sizes
    for i in range(1, len(rows)):
        rows[i]["n_min"] = int(numpy.sqrt(rows[i - 1]["size"] * rows[i]["size"]))
    apply(rows)
    return rows


def save_table(rows, path=TABLE_PATH, gpu=None):
    with open(path, "w") as f:
        json.dump({"gpu": gpu, "rows": rows}, f, indent=1)


if __name__ == "__main__":
    import sys
    r = tune(verbose=True)
    name = sys.argv[1] if len(sys.argv) > 1 else None
    save_table(r, gpu=name)
    print(json.dumps(r, indent=1))
