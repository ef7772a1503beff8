"""The request server (vsz_server_*): compress and decompress requests admitted under a device
memory budget, overlapping on the device.  Each result must be the same alone and in the mix, a
request larger than the budget is refused, and a budget smaller than the whole set forces requests
to wait for memory (outputs released as they complete)."""
import numpy as np
import pytest

import vecsz_gb300 as V
from vecsz_gb300 import fields
from vecsz_gb300.api import DecompressOpts, make_params

pytestmark = pytest.mark.gpu


def _requests(torch, seed, n):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        nd = int(rng.choice([2, 3]))
        if nd == 2:
            dims = (int(rng.integers(64, 700)), int(rng.integers(64, 500)))
        else:
            dims = tuple(int(v) for v in rng.integers(16, 90, 3))
        x = fields.grf_torch(tuple(reversed(dims)), seed=seed * 1000 + i).reshape(-1)
        out.append({"x": x, "dims": dims, "eb": float(10 ** rng.uniform(-5, -2)), "mode": "r2r"})
    return out


def _alone_compress(f):
    codec = V.DeviceCodec(f["dims"], eb=f["eb"], mode=f["mode"], dict_size=1024, block_size=8)
    codec.compress(f["x"])
    return codec.archive_bytes()


def test_results_same_alone_and_in_the_mix(cuda):
    torch = cuda
    reqs = _requests(torch, 5, 24)
    alone = [_alone_compress(f) for f in reqs]
    srv = V.Server(budget_bytes=2 << 30, slots=6)
    # the mix: all compress requests at once, plus decompress requests of the archives made alone
    tickets = [srv.submit_compress(f["x"], f["dims"], f["eb"], f["mode"], 1024, 8) for f in reqs]
    d_archives, dtickets = [], []
    for a in alone[:12]:
        buf = torch.from_numpy(np.frombuffer(a + bytes(64), np.uint8).copy()).cuda()
        d_archives.append(buf)
        desc = V.parse_archive(a)
        dtickets.append(srv.submit_decompress(buf, desc, DecompressOpts(1024, 8, 1, 0.0)))
    for i, t in enumerate(tickets):
        c = srv.wait(t)
        assert c.status == 0
        assert srv.output_bytes(c) == alone[i], f"request {i}"
        assert c.t_submit <= c.t_start <= c.t_done
        srv.release(t)
    for i, t in enumerate(dtickets):
        c = srv.wait(t)
        assert c.status == 0
        got = srv.output_view(c, "float32").cpu().numpy()
        want = V.decompress(alone[i])
        np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))
        srv.release(t)
    s = srv.stats()
    assert s["completed"] == len(tickets) + len(dtickets) and s["queued"] == 0 and s["arena_bytes_in_use"] == 0
    srv.close()


def test_budget_admission(cuda):
    torch = cuda
    reqs = _requests(torch, 9, 10)
    alone = [_alone_compress(f) for f in reqs]
    # a budget that holds one or two requests at a time: the rest wait for memory
    import ctypes as C
    need = 0
    for f in reqs:
        p, ws, cap = make_params(f["eb"], f["mode"], 1024, 8), C.c_size_t(0), C.c_size_t(0)
        V.lib().vsz_compress_bounds(C.byref(p), len(f["dims"]), V.api.dims_arg(f["dims"]), C.byref(ws), C.byref(cap))
        need = max(need, ws.value + cap.value + 1024)
    srv = V.Server(budget_bytes=max(3 * need // 2, 1 << 20), slots=4)
    big = torch.zeros(64 << 20, dtype=torch.float32, device="cuda")
    with pytest.raises(V.VszError) as e:
        srv.submit_compress(big, (64 << 20,), 1e-3, "abs", 1024, 8)  # could never fit
    assert e.value.status == 4
    tickets = [srv.submit_compress(f["x"], f["dims"], f["eb"], f["mode"], 1024, 8) for f in reqs]
    for i, t in enumerate(tickets):
        c = srv.wait(t)
        assert c.status == 0 and srv.output_bytes(c) == alone[i]
        srv.release(t)  # frees memory for the requests still queued
    assert srv.stats()["arena_bytes_in_use"] == 0
    srv.close()


def test_cancel_queued_request(cuda):
    """A request held back by the memory budget can be withdrawn: it completes at once as
    cancelled with no output; an admitted or finished request cannot be; the rest are unaffected."""
    import ctypes as C
    torch = cuda
    x = fields.grf_torch((64, 64, 64), seed=77).reshape(-1)
    dims = (64, 64, 64)
    p, ws, cap = make_params(1e-4, "r2r", 1024, 8), C.c_size_t(0), C.c_size_t(0)
    V.lib().vsz_compress_bounds(C.byref(p), 3, V.api.dims_arg(dims), C.byref(ws), C.byref(cap))
    # room for one request, not for a second while the first one's archive is kept
    budget = max(ws.value + cap.value + (64 << 10), 1 << 20)
    alone = _alone_compress({"x": x, "dims": dims, "eb": 1e-4, "mode": "r2r"})
    srv = V.Server(budget_bytes=budget, slots=2)
    t1 = srv.submit_compress(x, dims, 1e-4, "r2r", 1024, 8)
    t2 = srv.submit_compress(x, dims, 1e-4, "r2r", 1024, 8)
    c1 = srv.wait(t1)
    assert c1.status == 0 and srv.output_bytes(c1) == alone
    assert srv.stats()["queued"] == 1  # t2 waits for t1's archive to be released
    assert srv.cancel(t2) == 0
    c2 = srv.wait(t2, timeout_s=5)
    assert c2.status == 10  # VSZ_ERR_CANCELLED
    assert c2.out_bytes == 0
    assert srv.cancel(t1) == 6  # already ran
    assert srv.cancel(987654) == 1
    srv.release(t1)
    srv.release(t2)
    t3 = srv.submit_compress(x, dims, 1e-4, "r2r", 1024, 8)
    c3 = srv.wait(t3)
    assert c3.status == 0 and srv.output_bytes(c3) == alone
    srv.release(t3)
    s = srv.stats()
    assert s["queued"] == 0 and s["arena_bytes_in_use"] == 0
    srv.close()
