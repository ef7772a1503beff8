"""The allocation-free outlier gather (vsz_outlier_gather_noalloc) against the allocating one.

Callers that cannot call cudaMalloc -- a serving process whose device memory another allocator
owns, a latency-critical loop that cannot take an allocation's implicit synchronisation, a plugin
host that only hands over input and output buffers -- use the no-alloc entry point, whose scratch
is a static device array shared by all calls.  Two calls in a row (the second on a different field,
so stale scratch from the first would show) must give exactly what vsz_outlier_gather gives.
This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from vecsz_gb300 import _lib as L
from vecsz_gb300 import api, fields

pytestmark = pytest.mark.gpu


def _noalloc_gather(torch, dims, segc, scratch):
    nseg = L.lib().vsz_outlier_segments(len(dims), L.dims_arg(dims))
    out = torch.zeros(nseg * 128 + 4, dtype=torch.float32, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int64, device="cuda")
    rc = L.lib().vsz_outlier_gather_noalloc(len(dims), L.dims_arg(dims), C.c_void_p(segc.data_ptr()),
                                            C.c_void_p(scratch.data_ptr()), C.c_void_p(out.data_ptr()),
                                            C.c_void_p(cnt.data_ptr()), api._stream_ptr())
    L.check(rc, "outlier_gather_noalloc")
    torch.cuda.synchronize()
    return out[: int(cnt.item())]


def _stage_outputs(torch, x_np, dims, eb):
    x = torch.from_numpy(np.ascontiguousarray(x_np.ravel())).cuda()
    consts, _, st = api.eb_setup(x, eb, "abs")
    assert st == 0
    code, hist, scratch, segc = api.dualquant(x, dims, 8, 1024, consts)
    return segc, scratch


def test_noalloc_gather_matches_allocating_gather_twice(cuda):
    torch = cuda
    cases = [
        (fields.adversarial_3d(20, 33, 47, seed=1), (47, 33, 20), 1e-5),  # many outliers
        (fields.grf_3d(12, 40, 300, seed=2), (300, 40, 12), 1e-4),        # a different shape, few
    ]
    for x_np, dims, eb in cases:
        segc, scratch = _stage_outputs(torch, x_np, dims, eb)
        want = api.outlier_gather(dims, segc, scratch)
        got = _noalloc_gather(torch, dims, segc, scratch)
        assert got.numel() == want.numel() and want.numel() > 0
        assert torch.equal(got.view(torch.int32), want.view(torch.int32))


def test_noalloc_gather_rejects_oversize_field(cuda):
    # 2^29 rows of one 128-wide segment each exceeds the 2^28-segment static scratch
    dims = (1, 1 << 15, 1 << 14)
    dummy = cuda.zeros(16, dtype=cuda.uint8, device="cuda")
    rc = L.lib().vsz_outlier_gather_noalloc(3, L.dims_arg(dims), C.c_void_p(dummy.data_ptr()),
                                            C.c_void_p(dummy.data_ptr()), C.c_void_p(dummy.data_ptr()),
                                            C.c_void_p(dummy.data_ptr()), None)
    assert rc == L.VSZ_ERR_CAPACITY
