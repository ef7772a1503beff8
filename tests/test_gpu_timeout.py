"""Bounded device waits, run out on purpose without faulting or hanging anything.

Every cross-CTA wait of the library (the decoupled look-back of the outlier gather, the encoder's
chunk scan and the device-wide scans) polls a bounded number of times, then records
VSZ_ERR_TIMEOUT in the call's status word and returns.  Here the device-wide scan runs with its
tile ticket started past tile 0, so one tile waits on a predecessor that never publishes; with the
spin limit lowered to a few thousand polls, that wait gives up at once.  The status must say
VSZ_ERR_TIMEOUT, and the context must stay usable: an ordinary round trip afterwards is bit-exact.
"""
import ctypes as C
import time

import numpy as np
import pytest

import oracle as O
import vecsz_gb300 as V
from vecsz_gb300 import _lib as L
from vecsz_gb300 import fields

pytestmark = pytest.mark.gpu


def test_lookback_wait_runs_out_and_reports_timeout(cuda):
    lib = L.lib()
    L.check(lib.vsz_debug_set_spin_limit(2000), "set spin limit")
    try:
        st = C.c_int(-1)
        t0 = time.perf_counter()
        L.check(lib.vsz_debug_scan_stalled_predecessor(4 * 4096, C.byref(st)), "stalled scan")
        dt = time.perf_counter() - t0
        assert st.value == L.VSZ_ERR_TIMEOUT
        assert dt < 10.0  # a few thousand polls, not the default 2^22
    finally:
        L.check(lib.vsz_debug_set_spin_limit(0), "restore spin limit")
    # the ordinary entry points are unaffected: a round trip right after is bit-exact
    x = fields.grf_3d(16, 24, 40, seed=5).ravel()
    dims = (40, 24, 16)
    c = V.compress(x, dims, eb=1e-3, mode="r2r", dict_size=1024, block_size=8)
    oa, _ = O.compress(x, dims, 8, 1024, 1e-3, True)
    assert c.data[: c.data_size] == oa
    y = V.decompress(c)
    np.testing.assert_array_equal(y.view(np.uint32), O.decompress(oa, 8, 1024, O.value_range(x)).view(np.uint32))


def test_spin_limit_argument_checks(cuda):
    lib = L.lib()
    st = C.c_int(-1)
    assert lib.vsz_debug_scan_stalled_predecessor(0, C.byref(st)) == L.VSZ_ERR_INVALID
    assert lib.vsz_debug_scan_stalled_predecessor((1 << 24) + 1, C.byref(st)) == L.VSZ_ERR_INVALID
    assert lib.vsz_debug_set_spin_limit(0) == L.VSZ_OK


def test_tree_handoff_wait_runs_out_and_reports_timeout(cuda):
    """The host tree build is a handoff: a kernel posts the histogram and waits, bounded, for the
    host worker's answer.  With the worker holding its answers and the bound lowered to 50 ms, a
    compress records VSZ_ERR_TIMEOUT instead of hanging; once the worker answers again, the next
    compress is the oracle's archive."""
    lib = L.lib()
    x = fields.grf_3d(16, 24, 40, seed=6).ravel()
    dims = (40, 24, 16)
    L.check(lib.vsz_debug_set_tree_wait_ns(50_000_000), "set tree wait")
    L.check(lib.vsz_debug_tree_hold(1), "hold")
    try:
        t0 = time.perf_counter()
        with pytest.raises(V.VszError) as e:
            V.compress(x, dims, eb=1e-3, mode="r2r", dict_size=1024, block_size=8)
        assert e.value.status == L.VSZ_ERR_TIMEOUT
        assert time.perf_counter() - t0 < 10.0
    finally:
        L.check(lib.vsz_debug_tree_hold(0), "release")
        L.check(lib.vsz_debug_set_tree_wait_ns(0), "restore tree wait")
    c = V.compress(x, dims, eb=1e-3, mode="r2r", dict_size=1024, block_size=8)
    oa, _ = O.compress(x, dims, 8, 1024, 1e-3, True)
    assert c.data[: c.data_size] == oa
