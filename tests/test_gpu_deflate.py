"""The gzip pass on the device (vsz_deflate): every stream must inflate, with Python's zlib (the
same inflate the reference's lossless pass calls, src/lossless.hh:144-177), to the exact input,
including the Adler-32 check zlib performs; the reference's format detection must accept it."""
import zlib

import numpy as np
import pytest

import oracle as O
import vecsz_gb300 as V
from vecsz_gb300 import api, fields

pytestmark = pytest.mark.gpu
CH = 16384  # vsz_deflate_chunk_bytes(); checked below


def roundtrip(data):
    out, stats = api.deflate(data)
    assert out[:2] == b"\x78\x01"
    assert V.lib().vsz_lossless_detect(out, len(out)) == 2  # isZlibFormat(120, 1)
    assert zlib.decompress(out) == bytes(data)
    return out, stats


def test_chunk_size(cuda):
    assert V.lib().vsz_deflate_chunk_bytes() == CH


@pytest.mark.parametrize("n", [0, 1, 2, 3, 4, 5, 63, 64, 65, 127, 128, 129, 4095, 4096, 4100, CH - 1, CH, CH + 1,
                               2 * CH + 7, 32768, 65536, 100003])
def test_deflate_sizes_random_and_runs(cuda, n):
    rng = np.random.default_rng(n)
    roundtrip(rng.integers(0, 256, n, dtype=np.uint8).tobytes())
    roundtrip(bytes(n))
    # runs of a few byte values with a skewed distribution
    roundtrip(np.repeat(rng.choice([0, 1, 255, 7], size=n // 7 + 1, p=[0.7, 0.1, 0.1, 0.1]).astype(np.uint8),
                        7)[:n].tobytes())


def test_deflate_block_types(cuda):
    rng = np.random.default_rng(5)
    _, st = roundtrip(rng.integers(0, 256, 5 * CH, dtype=np.uint8).tobytes())
    assert (st["chunks"], st["stored"], st["fixed"], st["dynamic"]) == (5, 5, 0, 0)
    assert list(st["chunk_bytes"]) == [CH + 5] * 5  # stored: 5 header bytes + the chunk
    _, st = roundtrip(bytes(3 * CH))
    assert st["chunks"] == 3 and st["stored"] == 0
    text = (b"the quick brown fox jumps over the lazy dog " * 2000)[:70000]
    out, st = roundtrip(text)
    assert st["dynamic"] + st["fixed"] == (len(text) + CH - 1) // CH and len(out) < len(text) // 12


def test_deflate_patterns_and_long_matches(cuda):
    rng = np.random.default_rng(9)
    for period in (1, 2, 3, 5, 17, 258, 259, 1000, 4097, 20000):
        unit = rng.integers(0, 256, period, dtype=np.uint8).tobytes()
        data = (unit * (100000 // period + 2))[:100000]
        out, _ = roundtrip(data)
        if period <= 1000:
            assert len(out) < len(data) // 4
        elif period <= 4097:  # each chunk's first period is literals
            assert len(out) < len(data) * (period + 2048) // CH
    # text with many 3-byte repeats at large distances, and a skewed literal alphabet
    words = [bytes(rng.integers(97, 123, int(k), dtype=np.uint8)) for k in rng.integers(2, 9, 400)]
    roundtrip(b" ".join(words[int(i)] for i in rng.integers(0, 400, 30000)))
    roundtrip(np.clip(rng.normal(128, 6, 300000), 0, 255).astype(np.uint8).tobytes())


def test_deflate_archives(cuda):
    """The archives the pass is for: a smooth 2D field compresses well (Huffman runs), a 3D
    turbulent one hardly at all; both inflate to the packed block."""
    x = fields.bump_field_2d(600, 1200, seed=1).ravel()
    a = V.compress(x, (1200, 600), eb=1e-4, mode="abs", dict_size=1024, block_size=8)
    block = a.data[: a.data_size]
    out, st = roundtrip(block)
    z3 = len(zlib.compress(block, 3))
    assert len(out) < 0.85 * len(block)
    assert len(out) < 1.15 * z3
    g = fields.grf_3d(64, 64, 64, seed=2).ravel()
    b = V.compress(g, (64, 64, 64), eb=1e-4, mode="r2r", dict_size=1024, block_size=8)
    roundtrip(b.data[: b.data_size])


def test_deflate_large_input(cuda):
    torch = cuda
    rng = np.random.default_rng(11)
    base = np.repeat(rng.integers(0, 4, 2_000_000, dtype=np.uint8), 3)
    base[::97] = rng.integers(0, 256, base[::97].size, dtype=np.uint8)
    out, st = api.deflate(torch.from_numpy(base).cuda())
    assert st["chunks"] == (base.size + CH - 1) // CH
    assert zlib.decompress(out) == base.tobytes()


@pytest.mark.parametrize("mode,eb", [("abs", 1e-4), ("r2r", 1e-3)])
def test_host_compress_with_device_gzip(cuda, mode, eb):
    """-L gzip on the device through the host entry points: the frame inflates to the same packed
    block as the plain archive's, and the archive decompresses to the same floats."""
    x = fields.bump_field_2d(300, 700, seed=4).ravel()
    plain = V.compress(x, (700, 300), eb=eb, mode=mode, dict_size=1024, block_size=8)
    dev = V.compress(x, (700, 300), eb=eb, mode=mode, dict_size=1024, block_size=8, lossless="gzip-device")
    assert dev.lossless_size > 0 and dev.data[:2] == b"\x78\x01"
    assert dev.data_size == plain.data_size
    assert zlib.decompress(dev.data[: dev.lossless_size]) == plain.data[: plain.data_size]
    trailer = plain.data[plain.data_size:]
    assert dev.data[dev.lossless_size:dev.lossless_size + len(trailer)] == trailer  # the same trailer
    index = dev.data[dev.lossless_size + len(trailer):]
    assert index[:4] == b"VSZD" and len(index) % 8 == 0
    np.testing.assert_array_equal(V.decompress(dev).view(np.uint32), V.decompress(plain).view(np.uint32))
    # the oracle reads the inflated block
    y = O.decompress(zlib.decompress(dev.data[: dev.lossless_size]), 8, 1024,
                     O.value_range(x) if mode == "r2r" else 0.0)
    np.testing.assert_array_equal(y.view(np.uint32), V.decompress(plain).view(np.uint32))


def inflate_roundtrip(data):
    out, st = api.deflate(data)
    y, status = api.inflate(out, st["chunk_bytes"], len(data))
    assert status == 0
    assert y == bytes(data)
    return out, st


@pytest.mark.parametrize("n", [0, 1, 3, 4096, CH - 1, CH, CH + 1, 32769, 100003, 1 << 20])
def test_inflate_device_streams(cuda, n):
    rng = np.random.default_rng(100 + n)
    inflate_roundtrip(rng.integers(0, 256, n, dtype=np.uint8).tobytes())
    inflate_roundtrip(bytes(n))
    inflate_roundtrip(np.repeat(rng.choice([0, 1, 255, 7], size=n // 5 + 1, p=[0.7, 0.1, 0.1, 0.1]).astype(np.uint8),
                                5)[:n].tobytes())
    words = [bytes(rng.integers(97, 123, int(k), dtype=np.uint8)) for k in rng.integers(2, 9, 300)]
    text = b" ".join(words[int(i)] for i in rng.integers(0, 300, n // 5 + 1))[:n]
    inflate_roundtrip(text)


def test_inflate_archives_and_fixed_blocks(cuda):
    x = fields.bump_field_2d(600, 1200, seed=1).ravel()
    a = V.compress(x, (1200, 600), eb=1e-4, mode="abs", dict_size=1024, block_size=8)
    _, st = inflate_roundtrip(a.data[: a.data_size])
    assert st["dynamic"] > 0
    rng = np.random.default_rng(3)
    # a skewed but wide literal alphabet with short runs, where fixed codes can win
    inflate_roundtrip(np.clip(rng.normal(100, 30, 200000), 0, 255).astype(np.uint8).tobytes())


def test_inflate_rejects_other_streams(cuda):
    """Damaged streams and streams of other encoders: VSZ_ERR_CORRUPT, never a fault."""
    x = fields.bump_field_2d(300, 700, seed=5).ravel()
    block = V.compress(x, (700, 300), eb=1e-4, mode="abs", dict_size=1024, block_size=8).data
    out, st = api.deflate(block)
    sizes = st["chunk_bytes"]
    rng = np.random.default_rng(7)
    for k in range(12):
        bad = bytearray(out)
        pos = int(rng.integers(2, len(out) - 6))
        bad[pos] ^= int(rng.integers(1, 256))
        y, status = api.inflate(bytes(bad), sizes, len(block))
        assert status in (0, 3)
        if status == 0:  # a flip that still decodes is caught by the Adler-32, so only a no-op passes
            assert y == block
    bad = bytearray(out)
    bad[-1] ^= 1  # Adler-32
    assert api.inflate(bytes(bad), sizes, len(block))[1] == 3
    z = zlib.compress(block, 6)  # zlib's stream: a final block inside the "chunk"
    assert api.inflate(z, np.array([len(z) - 6], np.uint32), min(len(block), CH))[1] == 3
    wrong = sizes.copy()
    wrong[0] += 1
    assert api.inflate(out, wrong, len(block))[1] == 3
    huge = sizes.copy()
    huge[-1] = 1 << 30
    assert api.inflate(out, huge, len(block))[1] == 3


def test_host_decompress_inflates_on_device(cuda):
    """With the deflate index the host entry point inflates on the device (two more launches than
    the plain archive's decompress); without it, through the host library; the same floats."""
    x = fields.bump_field_2d(400, 900, seed=6).ravel()
    plain = V.compress(x, (900, 400), eb=1e-4, mode="abs", dict_size=1024, block_size=8)
    dev = V.compress(x, (900, 400), eb=1e-4, mode="abs", dict_size=1024, block_size=8, lossless="gzip-device")
    lib = V.lib()
    want = V.decompress(plain)
    l0 = lib.vsz_launch_count()
    V.decompress(plain)
    l1 = lib.vsz_launch_count()
    got = V.decompress(dev)
    l2 = lib.vsz_launch_count()
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))
    assert (l2 - l1) - (l1 - l0) == 2
    trailer_len = len(plain.data) - plain.data_size
    stripped = api.Compressed(dev.data[: dev.lossless_size + trailer_len], dev.data_size, dev.lossless_size,
                              dev.n_outlier)
    l3 = lib.vsz_launch_count()
    np.testing.assert_array_equal(V.decompress(stripped).view(np.uint32), want.view(np.uint32))
    assert lib.vsz_launch_count() - l3 == l1 - l0
