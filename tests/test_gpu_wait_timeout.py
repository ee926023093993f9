"""Failure detection of the device-side waits (GB300): every mbarrier wait of the
tensor-core kernels is bounded in time; a wait that runs out stops the kernel,
which reports it through its error flag, and the context stays usable. The
self-test withholds one tile copy so that a wait runs out; nothing faults."""
import ctypes as C

import pytest

pytestmark = pytest.mark.gpu


def test_withheld_copy_times_out_and_context_survives():
    from mestrado_gb300 import _lib

    lib = _lib.load()
    timed_out, ms, clean = C.c_int(), C.c_float(), C.c_int()
    rc = lib.gbivf_selftest_wait_timeout(0, C.byref(timed_out), C.byref(ms), C.byref(clean))
    assert rc == 0, lib.gbivf_last_error().decode()
    assert timed_out.value == 1
    assert 1500.0 < ms.value < 20000.0, ms.value  # the 2 s wait limit, not a hang and not an early exit
    assert clean.value == 1


def test_search_after_timeout_is_exact():
    """A search after the stalled launch still matches the oracle bit for bit."""
    import numpy as np

    import oracle
    from mestrado_gb300 import _lib
    from mestrado_gb300.engine import GpuIndex
    from tests import golden_cases

    lib = _lib.load()
    timed_out, ms, clean = C.c_int(), C.c_float(), C.c_int()
    assert lib.gbivf_selftest_wait_timeout(0, C.byref(timed_out), C.byref(ms), C.byref(clean)) == 0
    assert timed_out.value == 1
    g = golden_cases.load("cfg1")
    gi = GpuIndex(g.ix, base=g.base)
    w = g.meta["w"]
    ids, dis = gi.search(g.queries, 10, w, rerank=False)
    o_ids, o_dis = oracle.ivfpq_search(g.ix, g.queries, k=10, w=w, rerank=False, ties=oracle.TIES_KEYED)
    np.testing.assert_array_equal(ids, o_ids)
    np.testing.assert_array_equal(dis.view(np.uint32), o_dis.view(np.uint32))
    gi.close()
