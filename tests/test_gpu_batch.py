"""The batched compressor (vsz_batch_*): many fields of uneven shapes, dimensionalities, error
bounds, dictionaries and block sizes in one launch sequence.  Every field's archive and result must
be byte-identical to single-field vsz_compress of the same input; a field that fails (zero value
range in r2r) fails alone; the sequence replays from a CUDA graph on new inputs."""
import numpy as np
import pytest

import oracle as O
import vecsz_gb300 as V
from vecsz_gb300 import fields

pytestmark = pytest.mark.gpu


def _mixed_fields(torch, seed, n):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        nd = int(rng.choice([1, 2, 3], p=[0.2, 0.4, 0.4]))
        if nd == 1:
            dims = (int(rng.integers(1, 300000)),)
            x = (np.cumsum(rng.standard_normal(dims[0])) * 0.01).astype(np.float32)
        elif nd == 2:
            dims = (int(rng.integers(1, 900)), int(rng.integers(1, 600)))
            x = fields.bump_field_2d(dims[1], dims[0], seed=seed * 100 + i).ravel()
        else:
            dims = tuple(int(v) for v in rng.integers(1, 90, 3))
            x = fields.grf_3d(dims[2], dims[1], dims[0], seed=seed * 100 + i).ravel()
        mode = "r2r" if rng.random() < 0.7 else "abs"
        if mode == "r2r" and (x.size < 2 or float(x.max()) == float(x.min())):
            mode = "abs"
        out.append({"x": torch.from_numpy(np.ascontiguousarray(x, dtype=np.float32)).cuda(), "dims": dims,
                    "eb": float(10 ** rng.uniform(-5, -2)), "mode": mode,
                    "dict_size": int(rng.choice([256, 1024, 1024, 4096, 65536])),
                    "block_size": int(rng.choice([8, 8, 16, 32, 64]))})
    return out


def _plain(f):
    codec = V.DeviceCodec(f["dims"], eb=f["eb"], mode=f["mode"], dict_size=f["dict_size"],
                          block_size=f["block_size"])
    codec.compress(f["x"])
    return codec.archive_bytes(), codec.result_host()


def test_batch_matches_single_field_compress(cuda):
    fs = _mixed_fields(cuda, 3, 40)
    # a constant field in r2r: zero value range, the reference exits; only this field fails
    fs.append({"x": cuda.full((4096,), 2.5, dtype=cuda.float32, device="cuda"), "dims": (4096,), "eb": 1e-3,
               "mode": "r2r", "dict_size": 1024, "block_size": 8})
    b = V.BatchCompressor(fs)
    b.compress()
    cuda.cuda.synchronize()
    for i, f in enumerate(fs[:-1]):
        want, r = _plain(f)
        got = b.archive_bytes(i)
        assert got == want, f"field {i} {f['dims']} {f['mode']} dict {f['dict_size']} bs {f['block_size']}"
        rb = b.result(i)
        assert (rb.data_size, rb.n_outlier, rb.payload_bits) == (r.data_size, r.n_outlier, r.payload_bits)
    assert b.result(len(fs) - 1).status == 7
    # a few against the oracle directly
    for i in (0, 7, 19):
        f = fs[i]
        a_or, _ = O.compress(f["x"].cpu().numpy(), f["dims"], f["block_size"], f["dict_size"], f["eb"],
                             f["mode"] == "r2r")
        assert b.archive_bytes(i)[: len(a_or)] == a_or
    b.close()


def test_batch_replays_from_cuda_graph(cuda):
    torch = cuda
    fs = _mixed_fields(torch, 8, 12)
    b = V.BatchCompressor(fs)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        b.compress(s)
    s.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        b.compress(s)
    for rnd in range(2):
        for f in fs:
            f["x"].mul_(1.5 if rnd == 0 else 0.25)
        g.replay()
        torch.cuda.synchronize()
        for i, f in enumerate(fs):
            want, _ = _plain(f)
            assert b.archive_bytes(i) == want
    b.close()


def test_batch_autotune_keeps_archives(cuda):
    """Task sizes change how units are handed out, never the archives."""
    fs = _mixed_fields(cuda, 11, 10)
    b = V.BatchCompressor(fs)
    dq, enc = b.autotune(iterations=1)
    assert dq in (8, 16, 32, 64, 128) and enc in (16, 32, 64, 128, 256)
    for sizes in ((8, 16), (128, 256), (dq, enc)):
        b.set_task_sizes(*sizes)
        b.compress()
        cuda.cuda.synchronize()
        for i, f in enumerate(fs):
            assert b.archive_bytes(i) == _plain(f)[0]
    b.close()


def test_block_size_autotuner(cuda):
    from vecsz_gb300.api import autotune_block_size
    x = fields.grf_torch((96, 80, 128), seed=4).reshape(-1)
    best, t = autotune_block_size(x, (128, 80, 96), eb=1e-4, mode="r2r", sample_percent=50.0, iterations=2)
    assert best in (8, 16, 32, 64) and all(v > 0 for v in t.values())
    assert t[best] == min(t.values())


def test_field_autotuner_scores_whole_round_trip_and_caches(cuda):
    """vsz_autotune times compress + decompress per block size, scores the archive's transfer at
    the given link rate, and caches the choice per field class: a second field of the same class
    (same dimensionality, size class and eb class) returns the cached result without timing."""
    from vecsz_gb300.api import autotune, autotune_cache_clear
    autotune_cache_clear()
    x = cuda.from_numpy(fields.grf_3d(96, 80, 128, seed=4).ravel()).cuda()
    r1 = autotune(x, (128, 80, 96), eb=1e-4, mode="r2r", sample_percent=50.0, iterations=2, link_gbs=25.0)
    assert not r1["cached"] and r1["block_size"] in (8, 16, 32, 64)
    for k in range(4):
        assert r1["compress_ms"][k] > 0 and r1["decompress_ms"][k] > 0 and r1["archive_bytes"][k] > 0
        want = r1["compress_ms"][k] + r1["decompress_ms"][k] + r1["archive_bytes"][k] / 25e9 * 1e3
        assert abs(r1["score_ms"][k] - want) < 1e-9 * max(1.0, want)
    assert r1["score_ms"][[8, 16, 32, 64].index(r1["block_size"])] == min(r1["score_ms"])
    # the same class (96 x 80 x 120: same log2 size class, same eb class): a cache hit, same choice
    y = cuda.from_numpy(fields.grf_3d(80, 80, 120, seed=5).ravel()).cuda()
    r2 = autotune(y, (120, 80, 80), eb=2e-4, mode="r2r", sample_percent=50.0, iterations=2, link_gbs=25.0)
    assert r2["cached"] and r2["block_size"] == r1["block_size"] and r2["score_ms"] == r1["score_ms"]
    # another class (2D): timed afresh; speed alone (no link) is a separate class too
    z = cuda.from_numpy(fields.bump_field_2d(300, 500, seed=6).ravel()).cuda()
    r3 = autotune(z, (500, 300), eb=1e-4, mode="r2r", sample_percent=100.0, iterations=1, link_gbs=25.0)
    assert not r3["cached"]
    r4 = autotune(x, (128, 80, 96), eb=1e-4, mode="r2r", sample_percent=50.0, iterations=1, link_gbs=0.0)
    assert not r4["cached"]
    assert r4["score_ms"] == [c + d for c, d in zip(r4["compress_ms"], r4["decompress_ms"])]
    autotune_cache_clear()
    r5 = autotune(x, (128, 80, 96), eb=1e-4, mode="r2r", sample_percent=50.0, iterations=1, link_gbs=25.0)
    assert not r5["cached"]
