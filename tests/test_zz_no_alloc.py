"""wg_accel_noalloc: the force evaluation for callers that cannot allocate.

Callers whose device memory is owned by another framework's allocator, or
that must not trigger the device-wide synchronisation of cudaMalloc/cudaFree,
pass their own device buffers and get the result without the library
allocating anything; its intermediates live in a fixed device array of the
library.  This file is collected last so that a run stopping at the first
failure has run every other test before it.

The test allocates the caller-side device buffers itself, through the CUDA
runtime's shared library, and compares two calls in a row with the existing
entry point wg_accel under the parity tolerance of the other tests
(permutation bit-exact, accelerations within 1e-12 of the acceleration scale).
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


def _noalloc_accel(L, rt, x, m, totmass, omega2, force, t):
    n = len(x)
    dx, dm = DeviceBuffer(rt, 8 * n), DeviceBuffer(rt, 8 * n)
    da, dp = DeviceBuffer(rt, 8 * n), DeviceBuffer(rt, 4 * n)
    try:
        dx.upload(numpy.ascontiguousarray(x))
        dm.upload(numpy.ascontiguousarray(m))
        kind, params = (0, ()) if force is None else (force.kind, force.params)
        rc = L.wg_accel_noalloc(n, dx.ptr, dm.ptr, totmass, omega2, kind,
                                _lib.ext_params(params), len(params), t, da.ptr, dp.ptr, None)
        _lib.check(rc, "wg_accel_noalloc")
        a = numpy.empty(n)
        perm = numpy.empty(n, dtype=numpy.int32)
        da.download(a)
        dp.download(perm)
        return a, perm
    finally:
        for b in (dx, dm, da, dp):
            b.free()


def test_noalloc_matches_wg_accel_on_two_calls_in_a_row():
    L = _lib.lib()
    rt = _cudart()
    cases = [
        (ics.sech2_disk(_lib.NOALLOC_MAX_SHEETS, seed=61, masses="lognormal"), 1.21, None, 0.0),
        (ics.top_hat(20001, seed=62), -1.0, PulseTanh(0.3, 5.0, 1.0, 0.5), 4.7),
    ]
    for (x, v, m), omega2, force, t in cases:
        tot = numpy.sum(m)
        ref_a, ref_perm = wendy_gb300.accel(x, m, tot, omega2=omega2, ext_force=force, t=t)
        scale = max(tot, float(numpy.max(numpy.abs(ref_a))))
        for _ in range(2):
            a, perm = _noalloc_accel(L, rt, x, m, tot, omega2, force, t)
            assert numpy.array_equal(perm, ref_perm)
            assert numpy.max(numpy.abs(a - ref_a)) <= 1e-12 * scale


def test_noalloc_rejects_sizes_beyond_its_array():
    L = _lib.lib()
    rc = L.wg_accel_noalloc(_lib.NOALLOC_MAX_SHEETS + 1, None, None, 1.0, -1.0, 0,
                            _lib.ext_params(()), 0, 0.0, None, None, None)
    assert rc == -1
    assert b"outside" in L.wg_last_error()
