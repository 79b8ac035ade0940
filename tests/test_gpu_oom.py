"""Out-of-memory handling, made on the host: acg_inject_alloc_failure fails the
n-th device allocation the library makes, for every n up to the number of
allocations of the call, and each time the call returns
ACG_ERR_OUT_OF_MEMORY and leaves the device memory in use where it was
(nothing leaked: partial objects are freed, temporaries go back).  The
reference checks none of its cudaMalloc calls (main.cu:85-99).

No GPU fault is involved: the failing allocation is never made."""
import ctypes as C

import numpy as np
import pytest

from conftest import load_golden
from application_classification_gb300 import _lib, matcher

pytestmark = pytest.mark.gpu

OOM = 2


def _in_use():
    b = C.c_int64(0)
    _lib.check(_lib.lib().acg_device_memory_in_use(C.byref(b)), "in use")
    return b.value


def _sweep(attempt, limit=400):
    """Run attempt() with the n-th allocation failing, n = 1, 2, ... until it
    succeeds; returns the number of failed attempts."""
    L = _lib.lib()
    for n in range(1, limit):
        start = _in_use()
        L.acg_inject_alloc_failure(n)
        st = attempt()
        L.acg_inject_alloc_failure(0)
        if st == 0:
            return n - 1
        assert st == OOM, (n, st, L.acg_last_error())
        assert _in_use() == start, f"allocation {n}: device memory leaked"
    raise AssertionError("the call never succeeded")


@pytest.fixture(scope="module")
def graphs():
    d, p, _ = load_golden("irregular")
    return matcher.DeviceGraph(d), matcher.DeviceGraph(p)


def test_data_create_out_of_memory(cuda, graphs):
    dg, _ = graphs
    L = _lib.lib()
    cg = dg.c_graph()

    def attempt():
        h = C.c_void_p()
        st = L.acg_data_create(C.byref(cg), None, C.byref(h))
        if st == 0:
            L.acg_data_destroy(h)
        return st

    start = _in_use()
    assert _sweep(attempt) >= 3
    assert _in_use() == start


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_plan_create_out_of_memory(cuda, graphs, prec):
    """Each attempt makes a fresh data graph (no injection), then a plan with the
    n-th allocation failing (the data graph's cached work splits and FP32 copies
    count too), then destroys the data graph: memory in use returns to its start."""
    dg, pg = graphs
    L = _lib.lib()
    cd, cp = dg.c_graph(), pg.c_graph()
    opt = _lib.Options()
    L.acg_options_default(C.byref(opt))
    opt.precision = matcher.PRECISIONS[prec]
    start = _in_use()
    n = 0
    while True:
        n += 1
        assert n < 400
        h = C.c_void_p()
        _lib.check(L.acg_data_create(C.byref(cd), None, C.byref(h)), "data")
        L.acg_inject_alloc_failure(n)
        plan = C.c_void_p()
        st = L.acg_plan_create(h, C.byref(cp), C.byref(opt), None, C.byref(plan))
        L.acg_inject_alloc_failure(0)
        if st == 0:
            L.acg_plan_destroy(plan)
        else:
            assert st == OOM, (n, st, L.acg_last_error())
        L.acg_data_destroy(h)
        assert _in_use() == start, f"allocation {n}: device memory leaked"
        if st == 0:
            break
    assert n > 10


def test_batch_create_out_of_memory(cuda):
    """As for plans: a fresh data graph per attempt, destroyed after it."""
    d, p, _ = load_golden("er300")
    dev = matcher.DeviceGraph(d)
    cd = dev.c_graph()
    pats = [matcher.DeviceGraph(p), matcher.DeviceGraph(p)]
    arr = (_lib.Graph * 2)(*[x.c_graph() for x in pats])
    L = _lib.lib()
    opt = _lib.Options()
    L.acg_options_default(C.byref(opt))
    opt.precision = matcher.PRECISIONS["mixed"]
    start = _in_use()
    n = 0
    while True:
        n += 1
        assert n < 400
        h = C.c_void_p()
        _lib.check(L.acg_data_create(C.byref(cd), None, C.byref(h)), "data")
        L.acg_inject_alloc_failure(n)
        b = C.c_void_p()
        st = L.acg_batch_create(h, C.cast(arr, C.c_void_p), 2, C.byref(opt), None, C.byref(b))
        L.acg_inject_alloc_failure(0)
        if st == 0:
            L.acg_batch_destroy(b)
        else:
            assert st == OOM, (n, st, L.acg_last_error())
        L.acg_data_destroy(h)
        assert _in_use() == start, f"allocation {n}: device memory leaked"
        if st == 0:
            break
    assert n > 10


def test_match_after_failed_creates(cuda, graphs):
    """The library still works after the injected failures."""
    d, p, ref = load_golden("irregular")
    mu = matcher.match(d, p, "fp64")
    assert np.abs(mu - ref).max() <= 1e-10 * max(1.0, np.abs(ref).max())
