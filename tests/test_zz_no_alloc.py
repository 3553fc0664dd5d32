"""wg_accel_noalloc: the force evaluation for callers that cannot allocate.

Callers whose device memory is owned by another framework's allocator, or
that must not trigger the device-wide synchronisation of cudaMalloc/cudaFree,
pass their own device buffers and get the result without the library
allocating anything; its intermediates live in a fixed device array of the
library.  This file is collected last so that a run stopping at the first
failure has run every other test before it.

The test allocates the caller-side device buffers itself, through the CUDA
runtime's shared library, and compares two calls in a row with the existing
entry point wg_accel.  Both run the same sort and force kernels on the same
sheets, so the permutation and the accelerations must be identical bit for
bit; the result is also compared with the CPU oracle under the parity
tolerance of the other tests (permutation bit-exact, accelerations within
1e-12 of the acceleration scale).  Around the second call the device's free
memory is read before and after: the call must not change it.
"""
import ctypes
import ctypes.util
import glob
import os

import numpy
import pytest

import wendy_gb300
from wendy_gb300 import _lib, ics
from wendy_gb300.extforce import PulseTanh

pytestmark = pytest.mark.gpu


def _cudart():
    cands = []
    name = ctypes.util.find_library("cudart")
    if name:
        cands.append(name)
    cands += sorted(glob.glob("/usr/local/cuda/lib64/libcudart.so*"))
    cands += sorted(glob.glob("/usr/local/cuda/targets/*/lib/libcudart.so*"))
    for c in cands:
        try:
            rt = ctypes.CDLL(c)
        except OSError:
            continue
        rt.cudaMalloc.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_size_t]
        rt.cudaFree.argtypes = [ctypes.c_void_p]
        rt.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
        rt.cudaMemGetInfo.argtypes = [ctypes.POINTER(ctypes.c_size_t),
                                      ctypes.POINTER(ctypes.c_size_t)]
        rt.cudaDeviceSynchronize.argtypes = []
        return rt
    pytest.skip("CUDA runtime shared library not found")


H2D, D2H = 1, 2


class DeviceBuffer:
    def __init__(self, rt, nbytes):
        self.rt = rt
        self.ptr = ctypes.c_void_p()
        assert rt.cudaMalloc(ctypes.byref(self.ptr), nbytes) == 0
        self.nbytes = nbytes

    def upload(self, arr):
        assert self.rt.cudaMemcpy(self.ptr, arr.ctypes.data, arr.nbytes, H2D) == 0

    def download(self, arr):
        assert self.rt.cudaMemcpy(arr.ctypes.data, self.ptr, arr.nbytes, D2H) == 0

    def free(self):
        self.rt.cudaFree(self.ptr)


def _free_bytes(rt):
    free, total = ctypes.c_size_t(0), ctypes.c_size_t(0)
    assert rt.cudaDeviceSynchronize() == 0
    assert rt.cudaMemGetInfo(ctypes.byref(free), ctypes.byref(total)) == 0
    return free.value


def _noalloc_accel(L, rt, x, m, totmass, omega2, force, t):
    """One call through the C ABI; returns (a, perm, free bytes before, after)."""
    n = len(x)
    dx, dm = DeviceBuffer(rt, 8 * n), DeviceBuffer(rt, 8 * n)
    da, dp = DeviceBuffer(rt, 8 * n), DeviceBuffer(rt, 4 * n)
    try:
        dx.upload(numpy.ascontiguousarray(x))
        dm.upload(numpy.ascontiguousarray(m))
        kind, params = (0, ()) if force is None else (force.kind, force.params)
        free0 = _free_bytes(rt)
        rc = L.wg_accel_noalloc(n, dx.ptr, dm.ptr, totmass, omega2, kind,
                                _lib.ext_params(params), len(params), t, da.ptr, dp.ptr, None)
        free1 = _free_bytes(rt)
        _lib.check(rc, "wg_accel_noalloc")
        a = numpy.empty(n)
        perm = numpy.empty(n, dtype=numpy.int32)
        da.download(a)
        dp.download(perm)
        return a, perm, free0, free1
    finally:
        for b in (dx, dm, da, dp):
            b.free()


def test_noalloc_matches_wg_accel_on_two_calls_in_a_row():
    from oracle import oracle as O
    L = _lib.lib()
    rt = _cudart()
    cases = [
        (ics.sech2_disk(_lib.NOALLOC_MAX_SHEETS, seed=61, masses="lognormal"), 1.21, None, 0.0),
        (ics.top_hat(20001, seed=62), -1.0, PulseTanh(0.3, 5.0, 1.0, 0.5), 4.7),
    ]
    for (x, v, m), omega2, force, t in cases:
        tot = numpy.sum(m)
        ref_a, ref_perm = wendy_gb300.accel(x, m, tot, omega2=omega2, ext_force=force, t=t)
        ext = None if force is None else (O.EXT_PULSE_TANH, list(force.params))
        o_a, o_perm = O.accel(x, m, tot, omega2, ext, t)
        scale = max(tot, float(numpy.max(numpy.abs(o_a))))
        for call in range(2):
            a, perm, free0, free1 = _noalloc_accel(L, rt, x, m, tot, omega2, force, t)
            # same kernels as wg_accel on the same sheets: identical bits
            assert numpy.array_equal(perm, ref_perm)
            assert numpy.array_equal(a.view(numpy.int64), ref_a.view(numpy.int64))
            # and the oracle's result within the parity tolerance
            assert numpy.array_equal(perm, o_perm)
            assert numpy.max(numpy.abs(a - o_a)) <= 1e-12 * scale
            if call == 1:
                # the first call may load the library's device code; the
                # second one takes no device memory at all
                assert free1 == free0, (free0, free1)


def test_noalloc_rejects_sizes_beyond_its_array():
    L = _lib.lib()
    rc = L.wg_accel_noalloc(_lib.NOALLOC_MAX_SHEETS + 1, None, None, 1.0, -1.0, 0,
                            _lib.ext_params(()), 0, 0.0, None, None, None)
    assert rc == -1
    assert b"outside" in L.wg_last_error()
