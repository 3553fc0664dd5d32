"""CPU-side checks of the C ABI library and the host logic (no GPU needed)."""
import os
import re

import numpy
import pytest

import wendy_gb300
from wendy_gb300 import _lib
from wendy_gb300.extforce import Harmonic, PulseTanh, resolve

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                      "wendy_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(wg_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_bound_symbols():
    assert declared_symbols() == sorted(_lib.EXPORTS)


def test_library_exports_every_declared_symbol():
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("CUDA library not built here")
    L = _lib.load_raw()
    for name in declared_symbols():
        assert hasattr(L, name), name


def test_library_reports_missing_device_cleanly():
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("CUDA library not built here")
    import ctypes
    L = _lib.lib()
    sm = ctypes.c_int(0)
    rc = L.wg_device_info(ctypes.byref(sm), None, None)
    assert rc in (0, -7)
    assert L.wg_status_string(-7).decode() == "no CUDA device"


def test_nleap_error_message_matches_reference():
    g = wendy_gb300.nbody(numpy.array([-1., 1.]), numpy.zeros(2), numpy.ones(2), 2, approx=True)
    with pytest.raises(ValueError) as e:
        next(g)
    assert str(e.value) == ("When approx is True, the number of leapfrog steps nleap= per "
                            "output time step needs to be set")


def test_cpu_sorts_are_rejected_not_emulated():
    g = wendy_gb300.nbody(numpy.array([-1., 1.]), numpy.zeros(2), numpy.ones(2), 2, approx=True,
                          nleap=2, sort="quick")
    with pytest.raises(ValueError):
        next(g)


def test_callables_compile_or_are_rejected():
    # a plain function in the supported subset compiles into an expression
    # force; anything else (here: a comparison) is refused
    assert resolve(lambda x, t: -x)[0] == _lib.EXT_EXPR
    with pytest.raises(ValueError):
        resolve(lambda x, t: x > t)
    with pytest.raises(ValueError):
        resolve(3.0)
    assert resolve(Harmonic(1.1))[0] == _lib.EXT_HARMONIC
    k, p = resolve(PulseTanh(0.3, 5., 1., 0.5))
    assert k == _lib.EXT_PULSE_TANH and p == (0.3, 5., 1., 0.5)


def test_registered_forces_evaluate_like_numpy():
    x = numpy.linspace(-2, 2, 9)
    f = PulseTanh(0.3, 5., 1., 0.5)
    assert numpy.array_equal(f(x, 4.2), 0.3 * numpy.exp(-(4.2 - 5.) ** 2 / 2.) * numpy.tanh(x / .5))
    assert numpy.array_equal(Harmonic(1.1)(x, 0.), -(1.1 ** 2.) * x)


def test_exact_solver_rejects_what_the_reference_rejects():
    # wendy/wendy.py:159-165, checked before the GPU is touched
    x, v = numpy.array([-1., 1.]), numpy.zeros(2)
    cases = [(dict(ext_force=lambda x, t: -x), "External forces (ext_force=) are not supported "
                                                "for the exact nbody calculation"),
             (dict(omega=40.), "When omega is set, omega*dt needs to be less than pi/2; please "
                               "adjust dt")]
    for kw, msg in cases:
        with pytest.raises(ValueError) as e:
            next(wendy_gb300.nbody(x, v, numpy.ones(2), 0.05, **kw))
        assert str(e.value) == msg
    for m in (numpy.array([1., 0.]), numpy.array([1., 1e-10])):
        with pytest.raises(ValueError) as e:
            next(wendy_gb300.nbody(x, v, m, 2))
        assert str(e.value) == ("Tiny masses m much smaller than the median mass are not "
                                "supported, please remove these from the inputs")


def test_tuning_table_rows_select_by_size():
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("CUDA library not built here")
    from wendy_gb300 import autotune
    saved = [dict(n_min=0, **autotune.current(0))]
    try:
        rows = [dict(n_min=0, target=512, window=32, sort_bits=11, ctas_per_sm=2),
                dict(n_min=1 << 16, target=1024, window=64, sort_bits=12, ctas_per_sm=2)]
        autotune.apply(rows)
        assert autotune.current(1000)["target"] == 512
        assert autotune.current((1 << 16) - 1)["window"] == 32
        assert autotune.current(1 << 16)["target"] == 1024
        assert autotune.current(1 << 30)["sort_bits"] == 12
        for bad in (dict(n_min=0, target=4096, window=64, sort_bits=12, ctas_per_sm=2),
                    dict(n_min=0, target=1024, window=65, sort_bits=12, ctas_per_sm=2),
                    dict(n_min=0, target=1024, window=64, sort_bits=14, ctas_per_sm=2),
                    dict(n_min=0, target=1024, window=64, sort_bits=12, ctas_per_sm=3)):
            with pytest.raises(_lib.WendyGPUError):
                autotune.apply([bad])
    finally:
        autotune.apply(autotune.load_table() or saved)


def test_shipped_tuning_table_is_valid():
    from wendy_gb300 import autotune
    rows = autotune.load_table()
    if rows is None:
        pytest.skip("no shipped table")
    assert rows[0]["n_min"] == 0
    assert all(a["n_min"] <= b["n_min"] for a, b in zip(rows, rows[1:]))
    for r in rows:
        assert 64 <= r["target"] <= 1536 and 1 <= r["window"] <= 64
        assert 9 <= r["sort_bits"] <= 13 and r["ctas_per_sm"] in (1, 2)


def header_struct(name):
    """(type, field) pairs of `typedef struct name { ... } name;` in the header."""
    text = open(HEADER).read()
    body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), text, re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    return re.findall(r"(int64_t|int|double)\s+(\w+)\s*;", body)


@pytest.mark.parametrize("name,mirror", [("wg_stats", _lib.WgStats),
                                         ("wg_pool_stats", _lib.WgPoolStats),
                                         ("wg_tuning", _lib.WgTuning)])
def test_ctypes_structs_mirror_the_header(name, mirror):
    # the Python mirrors of the ABI's structs: same fields, order and types
    import ctypes
    ctype = {"int64_t": ctypes.c_int64, "int": ctypes.c_int, "double": ctypes.c_double}
    fields = header_struct(name)
    assert [f for _, f in fields] == [f for f, _ in mirror._fields_]
    assert [ctype[t] for t, _ in fields] == [t for _, t in mirror._fields_]


def test_pinned_arrays_fail_loudly_without_a_device():
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("CUDA library not built here")
    import ctypes
    sm = ctypes.c_int(0)
    if _lib.lib().wg_device_info(ctypes.byref(sm), None, None) == 0:
        pytest.skip("a device is present")
    with pytest.raises(_lib.WendyGPUError):
        _lib.pinned_empty(16)
