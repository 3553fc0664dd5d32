"""The bounded waits of the kernels, made to run out on purpose.

The compact path's force kernel finds each tile's mass prefix by looking
back over the records of earlier tiles; every such wait has an iteration
limit, after which the kernel records the expiry in the device error word
and carries on.  The test hook wg_set_debug_wait lowers that limit and keeps
one tile from ever publishing its record (a flag that nothing sets), so the
waits on it run out after a few microseconds.  The prefix is a mass sum, not
an address: the kernel's memory accesses do not depend on it, so nothing is
written out of place.  The call must report WG_ERR_DEVICE, name the expired
wait, refuse every later call on the same simulation but wg_destroy, and a
fresh simulation must compute the right result.  (The reference has no
device and no such error channel: its step function cannot fail,
wendy/wendy.c:385-418.)
"""
import ctypes

import numpy
import pytest

import wendy_gb300
from oracle import oracle as O
from wendy_gb300 import _lib, ics

pytestmark = pytest.mark.gpu

N = 1 << 16            # 32 tiles of the force kernel
WITHHELD_TILE = 5
SPIN_LIMIT = 64        # iterations of 32 ns back-off: a few microseconds


@pytest.fixture
def L():
    lib = _lib.lib()
    yield lib
    assert lib.wg_set_debug_wait(0, -1) == 0  # production limits again


def test_expired_lookback_gives_up_the_simulation(L):
    x, v, m = ics.sech2_disk(N, seed=71, masses="lognormal")
    tot = numpy.sum(m)
    good = wendy_gb300.Simulation(x, v, m, tot, 1.21)
    e_ref = good.energy(omega=1.1)
    good.close()

    sim = wendy_gb300.Simulation(x, v, m, tot, 1.21)
    assert L.wg_set_debug_wait(SPIN_LIMIT, WITHHELD_TILE) == 0
    with pytest.raises(_lib.WendyGPUError) as ei:
        sim.energy(omega=1.1)  # sort + one force evaluation on the compact sets
    assert ei.value.status == _lib.WG_ERR_DEVICE
    assert "force look-back wait expired" in str(ei.value)
    assert L.wg_set_debug_wait(0, -1) == 0
    # the simulation's state is no longer trusted: later calls are refused
    with pytest.raises(_lib.WendyGPUError) as ei:
        sim.step(1e-3, 2, ctypes.c_double(0.))
    assert ei.value.status == _lib.WG_ERR_DEVICE
    with pytest.raises(_lib.WendyGPUError):
        sim.energy(omega=1.1)
    sim.close()  # wg_destroy still works

    fresh = wendy_gb300.Simulation(x, v, m, tot, 1.21)
    assert fresh.energy(omega=1.1)[0] == e_ref[0]
    fresh.close()


def test_expired_lookback_in_a_stateless_call_then_recovery(L):
    x, v, m = ics.top_hat(N, seed=72)
    tot = numpy.sum(m)
    assert L.wg_set_debug_wait(SPIN_LIMIT, WITHHELD_TILE) == 0
    with pytest.raises(_lib.WendyGPUError) as ei:
        wendy_gb300.accel(x, m, tot, omega2=-1.)
    assert ei.value.status == _lib.WG_ERR_DEVICE
    assert L.wg_set_debug_wait(0, -1) == 0
    a, perm = wendy_gb300.accel(x, m, tot, omega2=-1.)
    ra, rperm = O.accel(x, m, tot, -1.)
    assert numpy.array_equal(perm, rperm)
    assert numpy.max(numpy.abs(a - ra)) <= 1e-12 * max(tot, float(numpy.max(numpy.abs(ra))))


def test_a_withheld_tile_beyond_the_launch_changes_nothing(L):
    x, v, m = ics.sech2_disk(N, seed=73)
    tot = numpy.sum(m)
    a0, p0 = wendy_gb300.accel(x, m, tot, omega2=1.21)
    assert L.wg_set_debug_wait(SPIN_LIMIT, 1 << 40) == 0
    a1, p1 = wendy_gb300.accel(x, m, tot, omega2=1.21)
    assert numpy.array_equal(p0, p1)
    assert numpy.array_equal(a0.view(numpy.int64), a1.view(numpy.int64))
