"""The C-ABI library without a GPU: it builds, loads, exports every entry point that
include/vecsz_gb300.h declares, and its host-only entry points (argument checks, archive parsing,
the lossless pass) behave.  No device compute is called here."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import oracle as O
import vecsz_gb300 as V
from vecsz_gb300 import _lib as L
from conftest import ROOT, golden_cases, load_golden

HEADER = os.path.join(ROOT, "include", "vecsz_gb300.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s*(vsz_[a-z0-9_]+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "vsz_compress" in names and "vsz_decompress" in names and "vsz_dualquant" in names
    assert len(names) >= 30


def test_library_exports_every_declared_symbol():
    lib = V.lib()
    for name in declared_functions():
        assert hasattr(lib, name), f"{name} declared in include/vecsz_gb300.h but not exported"
    assert set(declared_functions()) <= set(L.exported_symbols())


def test_status_strings():
    lib = V.lib()
    for s in range(11):
        assert lib.vsz_status_string(s)
    assert b"sm_103a" in lib.vsz_version()


def _bounds(eb=1e-4, mode=0, dict_size=1024, bs=8, dims=(64, 64, 64)):
    p = L.Params(eb, mode, dict_size, bs, 0)
    ws, cap = C.c_size_t(0), C.c_size_t(0)
    rc = V.lib().vsz_compress_bounds(C.byref(p), len(dims), L.dims_arg(dims), C.byref(ws), C.byref(cap))
    return rc, ws.value, cap.value


def test_argument_checks():
    assert _bounds()[0] == L.VSZ_OK
    assert _bounds(eb=0.0)[0] == L.VSZ_ERR_INVALID
    assert _bounds(eb=-1.0)[0] == L.VSZ_ERR_INVALID
    assert _bounds(eb=float("nan"))[0] == L.VSZ_ERR_INVALID
    assert _bounds(mode=3)[0] == L.VSZ_ERR_INVALID
    assert _bounds(dict_size=1023)[0] == L.VSZ_ERR_INVALID
    assert _bounds(dict_size=131072)[0] == L.VSZ_ERR_INVALID
    assert _bounds(bs=12)[0] == L.VSZ_ERR_UNSUPPORTED
    assert _bounds(bs=0)[0] == L.VSZ_ERR_INVALID
    assert _bounds(dims=(0, 4))[0] == L.VSZ_ERR_INVALID
    # size limits: each dimension fits the archive's i32, at most 2^36 elements in all
    assert _bounds(dims=(1 << 31,))[0] == L.VSZ_ERR_INVALID
    assert _bounds(dims=((1 << 31) - 1,))[0] == L.VSZ_OK
    assert _bounds(dims=(65536, 65536, 16))[0] == L.VSZ_OK
    assert _bounds(dims=(65536, 65536, 17))[0] == L.VSZ_ERR_INVALID
    rc, ws, cap = _bounds(dims=(512, 512, 512))
    assert rc == 0 and ws > 512 ** 3 * 2 and cap > 512 ** 3 * 4


def test_noalloc_gather_refuses_dims_before_any_device_call():
    """The allocation-free gather applies the same field limits as the allocating one, on the host,
    before it touches the device: dims above 2^31 - 1 or a product above 2^36 elements are refused."""
    lib = V.lib()
    fake = C.c_void_p(16)  # never dereferenced: the checks come first
    for dims in ((65536, 65536, 17), (1 << 31, 1, 1), (0, 5, 5), ((1 << 31) - 1, (1 << 31) - 1, 2)):
        rc = lib.vsz_outlier_gather_noalloc(3, L.dims_arg(dims), fake, fake, fake, fake, None)
        assert rc == L.VSZ_ERR_INVALID, dims


@pytest.mark.parametrize("name", golden_cases())
def test_archive_parse_matches_oracle(name):
    g = load_golden(name)
    d = V.parse_archive(g["archive"].tobytes())
    h = O.parse_header(g["archive"].tobytes())
    assert d.ndim == h["ndim"] and tuple(d.dims[: d.ndim]) == h["dims"] and d.eb == h["eb"]
    assert (d.n_pad, d.huff_bytes, d.n_outlier) == h["lens"]
    assert d.data_size == g["data_size"] and not d.has_trailer
    nc = int.from_bytes(g["huff"][:4].tobytes(), "big")
    assert d.node_count == nc
    assert d.payload_offset + d.payload_bytes == d.outlier_offset


def test_archive_parse_rejects_garbage():
    lib = V.lib()
    d = L.ArchiveDesc()
    for buf in (b"", b"\x07\x00\x00\x00" + b"\x00" * 60, b"\x02\x00\x00\x00" + b"\xff" * 60):
        a = np.frombuffer(buf + b"\x00" * 8, np.uint8)
        rc = lib.vsz_archive_parse(a.ctypes.data_as(C.c_void_p), len(buf), C.byref(d))
        assert rc == L.VSZ_ERR_CORRUPT
    g = load_golden("d2_bump_64x45")
    a = g["archive"]
    rc = lib.vsz_archive_parse(a.ctypes.data_as(C.c_void_p), a.size - 1, C.byref(d))  # truncated
    assert rc == L.VSZ_ERR_CORRUPT


def test_lossless_reads_reference_zstd_frame():
    g = load_golden("d2_bump_64x45")
    frame = g["zstd_frame"]
    lib = V.lib()
    assert lib.vsz_lossless_detect(frame.ctypes.data_as(C.c_void_p), frame.size) == 1
    out, ol = C.c_void_p(0), C.c_size_t(0)
    rc = lib.vsz_lossless_decompress(frame.ctypes.data_as(C.c_void_p), frame.size, g["data_size"], C.byref(out),
                                     C.byref(ol))
    if rc == L.VSZ_ERR_UNSUPPORTED:
        pytest.skip("libzstd not present on this machine")
    assert rc == 0 and ol.value == g["data_size"]
    assert C.string_at(out.value, ol.value) == g["archive"].tobytes()
    lib.vsz_free_host(out)


@pytest.mark.parametrize("which", [L.LOSSLESS_ZSTD, L.LOSSLESS_GZIP])
def test_lossless_roundtrip(which):
    g = load_golden("d3_tail_19x23x29")
    a = g["archive"]
    lib = V.lib()
    out, ol = C.c_void_p(0), C.c_size_t(0)
    rc = lib.vsz_lossless_compress(which, a.ctypes.data_as(C.c_void_p), a.size, C.byref(out), C.byref(ol))
    if rc == L.VSZ_ERR_UNSUPPORTED:
        pytest.skip("lossless library not present")
    assert rc == 0
    frame = np.frombuffer(C.string_at(out.value, ol.value), np.uint8).copy()
    lib.vsz_free_host(out)
    assert lib.vsz_lossless_detect(frame.ctypes.data_as(C.c_void_p), frame.size) == (1 if which == 1 else 2)
    back, bl = C.c_void_p(0), C.c_size_t(0)
    assert lib.vsz_lossless_decompress(frame.ctypes.data_as(C.c_void_p), frame.size, a.size, C.byref(back),
                                       C.byref(bl)) == 0
    assert C.string_at(back.value, bl.value) == a.tobytes()
    lib.vsz_free_host(back)


def _host_build(hist, dict_size):
    hist = np.ascontiguousarray(hist, np.uint64)
    cb = np.zeros(9 * dict_size, np.uint8)
    head = np.zeros(V.lib().vsz_huff_head_max(dict_size), np.uint8)
    info = np.zeros(4, np.uint32)
    rc = V.lib().vsz_huffman_build_host(hist.ctypes.data, dict_size, cb.ctypes.data, head.ctypes.data,
                                        info.ctypes.data)
    return rc, cb[:8 * dict_size].view(np.uint64), cb[8 * dict_size:], head, info


def _hist_cases():
    rng = np.random.default_rng(11)
    yield "zipf", 1024, np.minimum(rng.zipf(1.3, 1024), 5000).astype(np.uint64) * (rng.random(1024) < 0.7)
    yield "ties", 256, np.full(256, 7, np.uint64)                     # every comparison a tie
    yield "two_level_ties", 512, np.where(np.arange(512) % 3 == 0, 4, 2).astype(np.uint64)
    yield "single", 1024, np.eye(1, 1024, 513, dtype=np.uint64)[0] * 99
    yield "pair", 2, np.array([5, 1], np.uint64)
    yield "wide_w2", 4096, rng.integers(0, 40, 4096).astype(np.uint64)        # 256 < nodes <= 65536
    yield "wide_w4", 65536, rng.integers(1, 3, 65536).astype(np.uint64)       # nodes > 65536: 4-byte indices
    yield "peaked", 1024, np.concatenate([np.zeros(500), [3, 90, 100000, 80, 2], np.zeros(519)]).astype(np.uint64)


@pytest.mark.parametrize("case", list(_hist_cases()), ids=lambda c: c[0])
def test_host_tree_build_matches_oracle(case):
    """The host tree builder used inside vsz_compress gives the reference's tree and codebook."""
    _, dict_size, hist = case
    rc, words, lens, head, info = _host_build(hist, dict_size)
    assert rc == L.VSZ_OK
    o_lens, o_w0, _, o_nc = O.huffman_codebook(hist, dict_size)
    np.testing.assert_array_equal(lens, o_lens)
    assert int(info[0]) == o_nc and int(info[2]) == int(o_lens.max())
    short = (o_lens > 0) & (o_lens <= 64)
    want = o_w0[short] >> (64 - o_lens[short].astype(np.uint64))
    np.testing.assert_array_equal(words[short], want)
    # serialised tree: the oracle's encode_withTree section head for codes with this histogram
    codes = np.repeat(np.arange(dict_size, dtype=np.int32), hist.astype(np.int64))
    sec = np.frombuffer(O.huffman_encode(codes, dict_size), np.uint8)
    n_head = 8 + int(info[1])
    assert head[:n_head].tobytes() == sec[:n_head].tobytes()


def test_host_tree_build_deep_and_empty():
    # Fibonacci frequencies give a path-shaped tree with codes longer than 64 bits: lengths and
    # node count still match; the encoder refuses max length > 64 (info[2])
    fib = [1, 1]
    while len(fib) < 90:
        fib.append(fib[-1] + fib[-2])
    hist = np.zeros(128, np.uint64)
    hist[:90] = np.array(fib, np.uint64)
    rc, _, lens, _, info = _host_build(hist, 128)
    o_lens, _, _, o_nc = O.huffman_codebook(hist, 128)
    assert rc == L.VSZ_OK and int(info[0]) == o_nc and int(info[2]) > 64
    np.testing.assert_array_equal(lens, o_lens)
    rc, *_ , info = _host_build(np.zeros(64, np.uint64), 64)
    assert rc == L.VSZ_ERR_INVALID and not info.any()


def test_tree_builder_switch():
    lib = V.lib()
    prev = lib.vsz_set_tree_builder(-1)
    assert prev in (L.TREE_DEVICE, L.TREE_HOST)
    assert lib.vsz_set_tree_builder(L.TREE_DEVICE) == prev
    assert lib.vsz_set_tree_builder(-1) == L.TREE_DEVICE
    lib.vsz_set_tree_builder(prev)


@pytest.mark.parametrize("spec,want", [
    ("block,max", (L.PAD_BLOCK, L.PADV_MAX, 0.0)),
    ("global", (L.PAD_GLOBAL, L.PADV_CONST, 0.0)),
    ("edge,avg", (L.PAD_EDGE, L.PADV_AVG, 0.0)),
    ("block,edge,min", (L.PAD_BLOCK, L.PADV_MIN, 0.0)),        # block wins over edge
    ("global,block,avg", (L.PAD_GLOBAL, L.PADV_AVG, 0.0)),     # global wins over block / edge
    ("block,constant,12.5", (L.PAD_BLOCK, L.PADV_CONST, 12.5)),
    ("edge,constant,-3.25", (L.PAD_EDGE, L.PADV_CONST, 3.25)),  # the reference's regex reads no sign
    ("global,constant,.5", (L.PAD_GLOBAL, L.PADV_CONST, 0.5)),
    ("block,constant,7.x", (L.PAD_BLOCK, L.PADV_CONST, 7.0)),
    ("max,min", (L.PAD_NONE, L.PADV_MIN, 0.0)),                # later type names win; no mode named
])
def test_parse_padding_like_reference_cli(spec, want):
    p = V.make_params(padding=spec)
    assert (p.pad_mode, p.pad_type) == want[:2]
    assert p.pad_constant == pytest.approx(want[2])


def test_padding_argument_checks_and_counts():
    def bounds(ndim, dims, dict_size=1024, padding="block,max", strict=False):
        p = V.make_params(eb=1e-3, dict_size=dict_size, block_size=8, padding=padding, strict=strict)
        ws, cap = C.c_size_t(0), C.c_size_t(0)
        rc = V.lib().vsz_compress_bounds(C.byref(p), ndim, L.dims_arg(dims), C.byref(ws), C.byref(cap))
        return rc, cap.value
    rc0, cap0 = bounds(2, (64, 64), padding=None)
    rc1, cap1 = bounds(2, (64, 64), padding="edge,max")
    assert rc0 == rc1 == L.VSZ_OK
    assert cap1 >= cap0 + 4 * 2 * 9 * 9   # 9 x 9 blocks of the reference grid, 2 values each
    assert bounds(1, (1000,), dict_size=65536)[0] == L.VSZ_ERR_UNSUPPORTED      # code 2R must fit u16
    assert bounds(1, (1000,), dict_size=65536, padding="global,max")[0] == L.VSZ_OK
    assert bounds(2, (64, 64), strict=True)[0] == L.VSZ_ERR_UNSUPPORTED
    p = V.make_params(padding="block,max")
    p.pad_type = 9
    ws, cap = C.c_size_t(0), C.c_size_t(0)
    assert V.lib().vsz_compress_bounds(C.byref(p), 1, L.dims_arg((100,)), C.byref(ws), C.byref(cap)) == \
        L.VSZ_ERR_INVALID
    for dims, mode in [((16,), "block"), ((14,), "block"), ((16, 17), "edge"), ((8, 8, 8), "edge"),
                       ((100, 7, 3), "global"), ((100,), None)]:
        mcode = {"block": O.PAD_BLOCK, "edge": O.PAD_EDGE, "global": O.PAD_GLOBAL, None: O.PAD_NONE}[mode]
        assert V.pad_count(dims, 8, mode and mode + ",max") == O.pad_count(dims, 8, mcode)
