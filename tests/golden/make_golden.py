"""Generate the golden vectors in tests/golden/ from the reference itself.

Run in a checkout where the reference's sources are present and its library
has been compiled from them (``make -C oracle ref``):

    python tests/golden/make_golden.py [--ref-root /path/to/wendy/checkout]

Every number stored here comes out of the reference's own code: its C step
function ``_wendy_nbody_approx_onestep`` (wendy/wendy.c:385-418) driven
through ctypes, its Python generator ``wendy.nbody`` (wendy/wendy.py:112-206,
336-437, imported with a stub numba) and, for the physics cross-check, its
exact event-driven solver (wendy/wendy.c:53-315).  The CPU oracle is not
used to make any of them.  Inputs are seeded synthetic initial conditions
from wendy_gb300.ics.

Files:
  accel.npz     one force evaluation per case: inputs, a (original order),
                and the sort permutation
  traj.npz      x, v after selected outputs of short runs
  energy.npz    relative energy error per output of a 1000-output run
                (N=10,000 sech^2 disk, dt=0.05, nleap=10)
  exact.npz     reference exact solver, N=101 sech^2 disk, 20 outputs
  exact_more.npz  reference exact solver with a harmonic potential (N=101,
                omega=1.1, 20 outputs) and at N=6000 (3 outputs), with the
                number of crossings per output
  extexpr.npz   x, v after outputs 1 and 10 of runs with external forces
                given as Python functions (tests/golden/forces.py), through
                the reference's own callable route

    python tests/golden/make_golden.py --only extexpr   # just that file
"""
import argparse
import os
import sys

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402  (reference loader helpers only)
from wendy_gb300 import ics  # noqa: E402

PULSE = [0.3, 5.0, 1.0, 0.5]  # A, t0, tau, h


def accel_cases():
    """(name, x, m, omega2, ext, t) for single force evaluations."""
    cases = []
    for n in (1, 2, 3, 10, 11, 16, 17, 101, 1000, 2048, 4097, 10000):
        x, v, m = ics.sech2_disk(n, seed=100 + n, masses="lognormal")
        cases.append(("sech2_ln_%d" % n, x, m, -1.0, None, 0.0))
    x, v, m = ics.sech2_disk(5000, seed=7)
    cases.append(("sech2_eq_omega", x, m, 1.21, None, 0.0))
    x, v, m = ics.top_hat(3000, seed=8)
    cases.append(("tophat_pulse", x, m, -1.0, (O.EXT_PULSE_TANH, PULSE), 4.2))
    cases.append(("tophat_pulse_small", x[:9], m[:9], -1.0, (O.EXT_PULSE_TANH, PULSE), 5.3))
    x, v, m = ics.gaussian(2500, seed=9, masses="lognormal")
    cases.append(("gauss_harm", x, m, -1.0, (O.EXT_HARMONIC, [1.21]), 0.0))
    x, v, m = ics.sech2_disk(999, seed=10)
    m = m.copy()
    m[::3] = 0.0  # tracer sheets
    cases.append(("tracers", x, m, -1.0, None, 0.0))
    x, v, m = ics.gaussian(777, seed=11)
    cases.append(("wide_range", x * numpy.logspace(-30, 30, 777), m, 0.25, None, 0.0))
    return cases


def ref_accel(lib, x, m, omega2, ext, t):
    n = len(x)
    xx = numpy.array(x, dtype=numpy.float64)
    vv = numpy.zeros(n)
    a = numpy.zeros(n)
    xi = O.make_sheets(xx)
    totmass = numpy.sum(m)
    # v = 0 makes the opening half drift a no-op; with nleap = 1 the call then
    # evaluates the force once at x and leaves it in `a` (original order) and
    # the permutation it sorted by in xi.idx.
    O.ref_onestep(lib, xi, xx, vv, numpy.ascontiguousarray(m), a, totmass, 1e-3, 1, t,
                  omega2, ext)
    return a, xi["idx"].copy(), totmass


def make_exact_more(wendy):
    """The reference's exact solver with a harmonic potential and at a size
    beyond what one GPU thread block's shared memory holds."""
    out = {}
    for name, n, seed, dt, nout, omega in (("harm", 101, 6, 0.05, 20, 1.1),
                                           ("large", 6000, 7, 0.02, 3, None)):
        x, v, m = ics.sech2_disk(n, seed=seed)
        v = v - numpy.mean(v)
        g = wendy.nbody(x.copy(), v.copy(), m.copy(), dt, omega=omega, full_output=True)
        out[name + "/x0"], out[name + "/v0"], out[name + "/m"] = x, v, m
        out[name + "/par"] = numpy.array([dt, nout, -1.0 if omega is None else omega])
        for k in range(1, nout + 1):
            tx, tv, nc, _el = next(g)
            out["%s/x%d" % (name, k)] = tx.copy()
            out["%s/v%d" % (name, k)] = tv.copy()
            out["%s/ncoll%d" % (name, k)] = numpy.array([nc])
    numpy.savez_compressed(os.path.join(HERE, "exact_more.npz"), **out)


def make_extexpr(wendy):
    """Runs of the reference's generator with Python-function forces: with
    numba stubbed out, wendy wraps each function in its ctypes callback
    (wendy/wendy.py:405-418) and its C step calls it per force evaluation."""
    import forces
    out = {}
    for name, fn, fam, n, seed, dt, nleap, nout, t0 in forces.CASES:
        x, v, m = ics.FAMILIES[fam](n, seed=seed)
        g = wendy.nbody(x.copy(), v.copy(), m.copy(), dt, approx=True, nleap=nleap, t0=t0,
                        sort="quick", ext_force=fn)
        for k in range(1, nout + 1):
            tx, tv = next(g)
            if k in (1, nout):
                out["%s/x%d" % (name, k)] = tx.copy()
                out["%s/v%d" % (name, k)] = tv.copy()
        out[name + "/x0"], out[name + "/v0"], out[name + "/m"] = x, v, m
    out["names"] = numpy.array([c[0] for c in forces.CASES])
    numpy.savez_compressed(os.path.join(HERE, "extexpr.npz"), **out)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-root", default=None,
                    help="reference checkout (default: $WENDY_REF_ROOT, else the one "
                         "oracle/_ref was built from)")
    ap.add_argument("--only", default=None, choices=["extexpr", "exact_more"],
                    help="write just this file")
    args = ap.parse_args()
    lib = O.ref_library()
    wendy = O.import_reference_wendy(args.ref_root)
    if lib is None or wendy is None:
        sys.exit("reference library not built: run `make -C oracle ref` first")
    sys.path.insert(0, HERE)
    if args.only:
        {"extexpr": make_extexpr, "exact_more": make_exact_more}[args.only](wendy)
        print("golden vectors written to", HERE)
        return

    # ---- single force evaluations
    out = {}
    names = []
    for name, x, m, omega2, ext, t in accel_cases():
        a, perm, totmass = ref_accel(lib, x, m, omega2, ext, t)
        names.append(name)
        out[name + "/x"] = x
        out[name + "/m"] = m
        out[name + "/a"] = a
        out[name + "/perm"] = perm
        out[name + "/par"] = numpy.array([totmass, omega2, t,
                                          0 if ext is None else ext[0]] +
                                         list((ext[1] if ext else []) + [0.0] * 4)[:4])
    out["names"] = numpy.array(names)
    numpy.savez_compressed(os.path.join(HERE, "accel.npz"), **out)

    # ---- short trajectories through the reference's own generator
    traj = {}
    tnames = []

    def run_gen(name, x, v, m, dt, nleap, nout, keep, **kw):
        g = wendy.nbody(x.copy(), v.copy(), m.copy(), dt, approx=True, nleap=nleap,
                        sort="quick", **kw)
        for k in range(1, nout + 1):
            tx, tv = next(g)
            if k in keep:
                traj["%s/x%d" % (name, k)] = tx.copy()
                traj["%s/v%d" % (name, k)] = tv.copy()
        traj[name + "/x0"] = x
        traj[name + "/v0"] = v
        traj[name + "/m"] = m
        traj[name + "/par"] = numpy.array([dt, nleap, nout, kw.get("omega") or -1.0,
                                           kw.get("t0", 0.0)])
        traj[name + "/keep"] = numpy.array(sorted(keep))
        tnames.append(name)

    x, v, m = ics.sech2_disk(101, seed=1)
    run_gen("sech2_101", x, v, m, 0.05, 10, 10, {1, 2, 5, 10})
    run_gen("sech2_101_omega", x, v, m, 0.05, 10, 10, {1, 10}, omega=1.1)
    x, v, m = ics.sech2_disk(1000, seed=2, masses="lognormal")
    run_gen("cfg2_small", x, v, m, 0.02, 20, 10, {1, 10}, omega=1.1)
    x, v, m = ics.sech2_disk(10000, seed=0)
    run_gen("cfg1", x, v, m, 0.05, 10, 10, {1, 10})
    x = numpy.array([-1.1, 0.1, 1.3])
    v = numpy.array([3.0, 2.0, -5.0])
    m = numpy.array([1.0, 2.0, 3.0])
    run_gen("three", x, v, m, 0.05, 1000, 10, {1, 10})
    x, v, m = ics.sech2_disk(101, seed=3)
    m = m.copy()
    m[50:] = 0.0
    run_gen("tracers_101", x, v, m, 0.05, 10, 10, {10})
    # config-3-shaped small case: pulsed external force through the C step
    # function with a C callback (the numba-cfunc route of the reference).
    x, v, m = ics.top_hat(2000, seed=4)
    xx, vv = x.copy(), v.copy()
    mm = m.copy()
    a = numpy.zeros(len(x))
    xi = O.make_sheets(xx)
    t0 = 4.0
    totmass = numpy.sum(mm)
    for k in range(1, 11):
        t0, _ = O.ref_onestep(lib, xi, xx, vv, mm, a, totmass, 0.01 / 10, 10, t0, -1.0,
                              (O.EXT_PULSE_TANH, PULSE))
        if k in (1, 10):
            traj["tophat_pulse/x%d" % k] = xx.copy()
            traj["tophat_pulse/v%d" % k] = vv.copy()
            traj["tophat_pulse/t%d" % k] = numpy.array([t0])
    traj["tophat_pulse/x0"] = x
    traj["tophat_pulse/v0"] = v
    traj["tophat_pulse/m"] = m
    traj["tophat_pulse/par"] = numpy.array([0.01, 10, 10, -1.0, 4.0])
    traj["tophat_pulse/keep"] = numpy.array([1, 10])
    tnames.append("tophat_pulse")
    traj["names"] = numpy.array(tnames)
    numpy.savez_compressed(os.path.join(HERE, "traj.npz"), **traj)

    # ---- long-run energy drift (configuration of the small CPU workload)
    x, v, m = ics.sech2_disk(10000, seed=0)
    E0 = wendy.energy(x, v, m)
    g = wendy.nbody(x.copy(), v.copy(), m.copy(), 0.05, approx=True, nleap=10, sort="quick")
    dE = numpy.empty(1000)
    for k in range(1000):
        tx, tv = next(g)
        dE[k] = (wendy.energy(tx, tv, m) - E0) / E0
    numpy.savez_compressed(os.path.join(HERE, "energy.npz"), dE=dE, E0=numpy.array([E0]),
                           par=numpy.array([10000, 0, 0.05, 10, 1000]))

    # ---- exact event-driven solver as a physics cross-check
    x, v, m = ics.sech2_disk(101, seed=5)
    v = v - numpy.mean(v)
    ge = wendy.nbody(x.copy(), v.copy(), m.copy(), 0.05)
    ex = {"x0": x, "v0": v, "m": m}
    for k in range(1, 21):
        tx, tv = next(ge)
        ex["x%d" % k] = tx.copy()
        ex["v%d" % k] = tv.copy()
    numpy.savez_compressed(os.path.join(HERE, "exact.npz"), **ex)
    make_exact_more(wendy)
    make_extexpr(wendy)
    print("golden vectors written to", HERE)


if __name__ == "__main__":
    main()
